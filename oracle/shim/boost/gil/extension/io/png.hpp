// Test-infrastructure shim, written for this project: the reference's
// src/utils/image.hpp includes Boost.GIL's PNG extension; the oracle
// replaces the PNG writer (oracle/img_driver.cpp), so nothing is needed here.
#pragma once
