// ffr-img's pixel mapping on the device: the count buffer (and, for colour
// images, the three colour sums) of every cell becomes one gray or RGB pixel,
// as the reference's render_image does on the CPU
// (src/ffr_img.cpp:199-309 with ImageRenderer::renderGrayImage /
// renderColorImageRGB, src/renderers/image_renderer.hpp:139-191):
//
//   monochrome  (u8)((count != 0 ? 1.0 : 0.0) * pix_scale)
//   grayscale   l = log(1 + count) / max_l;  (pix)(pow(l, 1/gamma) * pix_scale)
//   colour      ll = pow(l, 1/gamma);  (pix)((ll * (colour_c / count)) * pix_scale)
//
// with max_l = max over cells of log(1 + count) and pix_scale = 2^bits *
// (1 - 2^-52) (pix_scale<u8|u16, double>, src/types/constants.hpp:77-91),
// all in double as the reference (num_t = double).  Pixels come out in
// buffer order (x fastest, then rows), the reference's image row order.
//
// Where the reference converts an out-of-range or NaN double to an integer
// pixel (undefined behaviour: an empty cell's colour is 0/0), the pixel is
// saturated to [0, 2^bits - 1] and NaN maps to 0.
//
// One grid-stride pass, HBM-bound: 4 B (+ 4 B high words) per cell read for
// gray, + 24 B colours for RGB; 1 or 2 B per channel written.
#include "launch.h"

namespace ffr {

namespace {

template <typename P>
__device__ __forceinline__ P to_pixel(double x, double top)
{
    if (!(x > 0.0))            // also NaN
        return P(0);
    return (P)(unsigned int)(x < top ? x : top);
}

template <typename P>
__global__ void image_kernel(P* __restrict__ out, unsigned long long cells, int mode, int r,
                             const unsigned int* __restrict__ counts,
                             const unsigned int* __restrict__ hi,
                             const double* __restrict__ colors, double max_l, double gp,
                             double scale, double top)
{
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         i < cells; i += (unsigned long long)gridDim.x * blockDim.x)
    {
        const unsigned long long h = ((unsigned long long)(hi ? hi[i] : 0u) << 32) | counts[i];
        if (mode == 0)
        {
            out[i] = to_pixel<P>((h != 0ull ? 1.0 : 0.0) * scale, top);
            continue;
        }
        const double l = log(1.0 + (double)h) / max_l;
        const double ll = pow(l, gp);
        if (mode == 1)
        {
            out[i] = to_pixel<P>(ll * scale, top);
            continue;
        }
        const double hd = (double)h;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[3 * i + c] = to_pixel<P>((ll * (colors[i * r + c] / hd)) * scale, top);
    }
}

int grid_for_cells(unsigned long long n, int block)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long want = (n + block - 1) / block;
    const unsigned long long cap = (unsigned long long)(sms > 0 ? sms : 1) * 8;
    if (want > cap)
        want = cap;
    return want ? (int)want : 1;
}

} // namespace

cudaError_t launch_image(void* out, int bits, unsigned long long cells, int mode,
                         int color_dims, const unsigned int* counts, const unsigned int* hi,
                         const double* colors, double max_l, double gp, cudaStream_t st)
{
    // pix_scale<u8|u16, double> = 2^bits * (1 - 2^-52)
    const double adj = 1.0 - 0x1p-52;
    const int grid = grid_for_cells(cells, 256);
    if (bits == 8)
        image_kernel<unsigned char><<<grid, 256, 0, st>>>(
            static_cast<unsigned char*>(out), cells, mode, color_dims, counts, hi, colors, max_l,
            gp, 256.0 * adj, 255.0);
    else
        image_kernel<unsigned short><<<grid, 256, 0, st>>>(
            static_cast<unsigned short*>(out), cells, mode, color_dims, counts, hi, colors, max_l,
            gp, 65536.0 * adj, 65535.0);
    return cudaGetLastError();
}

} // namespace ffr
