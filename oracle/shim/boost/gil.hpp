// Test-infrastructure shim: the reference includes <boost/gil.hpp>
// (src/types/constants.hpp:9) but uses nothing from it on the buffer path.
#pragma once
