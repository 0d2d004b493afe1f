// Test-infrastructure shim, written for this project: the few pieces of
// Boost.GIL the reference's image path touches, so that its own
// ImageRenderer (src/renderers/image_renderer.hpp) and ffr-img
// (src/ffr_img.cpp) compile into the oracle where Boost is not installed.
// The buffer path includes this header (src/types/constants.hpp:9) and uses
// none of it.
//
// What the reference uses: image types constructed from (width, height)
// (gray8/gray16/rgb8/rgb16, and the gray1 typedef of utils/image.hpp),
// boost::gil::view(image), view.row_begin(y) indexed by x, and pixel
// assignment from an integer (gray) or a brace list {r, g, b} (rgb).
// Images here are plain row-major pixel arrays.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace boost::gil {

template <typename C>
struct gray_pixel
{
    C v;
    gray_pixel& operator=(C x)
    {
        v = x;
        return *this;
    }
};

template <typename C>
struct rgb_pixel
{
    C r, g, b;
};

template <typename Pixel>
class shim_view
{
    Pixel* base_;
    std::size_t w_;

public:
    shim_view(Pixel* base, std::size_t w) : base_(base), w_(w) {}
    Pixel* row_begin(std::size_t y) const { return base_ + y * w_; }
};

template <typename Pixel, int Channels, typename C>
class shim_image
{
    std::size_t w_, h_;
    std::vector<Pixel> px_;

public:
    using pixel_t = Pixel;
    using channel_t = C;
    static constexpr int channels = Channels;
    shim_image(std::size_t w, std::size_t h) : w_(w), h_(h), px_(w * h) {}
    std::size_t width() const { return w_; }
    std::size_t height() const { return h_; }
    Pixel* data() { return px_.data(); }
    const Pixel* data() const { return px_.data(); }
};

using gray1_image_t = shim_image<gray_pixel<std::uint8_t>, 1, std::uint8_t>;
using gray8_image_t = shim_image<gray_pixel<std::uint8_t>, 1, std::uint8_t>;
using gray16_image_t = shim_image<gray_pixel<std::uint16_t>, 1, std::uint16_t>;
using rgb8_image_t = shim_image<rgb_pixel<std::uint8_t>, 3, std::uint8_t>;
using rgb16_image_t = shim_image<rgb_pixel<std::uint16_t>, 3, std::uint16_t>;

template <typename Pixel, int Channels, typename C>
shim_view<Pixel> view(shim_image<Pixel, Channels, C>& img)
{
    return shim_view<Pixel>(img.data(), img.width());
}

} // namespace boost::gil
