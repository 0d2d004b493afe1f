// Test infrastructure (never linked into the product): the image writer for
// the reference's own ffr-img (src/ffr_img.cpp), built into
// oracle/_ref/ffr_img_ref by oracle/build_ref.sh.  The reference writes PNG
// through Boost.GIL and libpng (src/utils/image.cpp:8-21), neither of which
// is installed; this definition of tkoz::flame::writePng writes the pixels
// the reference's ImageRenderer produced, unencoded, so the golden-image
// fixtures pin the reference's pixel mapping itself:
//   "FFRIMG1\n", then u32 width, height, channels, bytes per channel
//   (little endian), then the rows top to bottom as the reference's view
//   holds them, each channel little endian.
#include "utils/image.hpp"

#include <cstdint>
#include <ostream>

namespace tkoz::flame {

template <typename img_t>
bool writePng(const img_t& img, std::ostream& os)
{
    using C = typename img_t::channel_t;
    const uint32_t head[4] = {(uint32_t)img.width(), (uint32_t)img.height(),
                              (uint32_t)img_t::channels, (uint32_t)sizeof(C)};
    os.write("FFRIMG1\n", 8);
    os.write(reinterpret_cast<const char*>(head), sizeof head);
    os.write(reinterpret_cast<const char*>(img.data()),
             (std::streamsize)(img.width() * img.height() * img_t::channels * sizeof(C)));
    return os.good();
}

template bool writePng<gray_img_t<u8>>(const gray_img_t<u8>&, std::ostream&);
template bool writePng<gray_img_t<u16>>(const gray_img_t<u16>&, std::ostream&);
template bool writePng<rgb_img_t<u8>>(const rgb_img_t<u8>&, std::ostream&);
template bool writePng<rgb_img_t<u16>>(const rgb_img_t<u16>&, std::ostream&);

} // namespace tkoz::flame
