// Instantiates the chaos kernels for one (precision, dims) pair; compiled
// once per pair and kind with -DFFR_P=<0|1> -DFFR_D=<1|2|3>
// -DFFR_KIND=<0..7>, so the objects compile in parallel:
//   0  plain render kernel without colour (and the colour dispatch)
//   1  xform-sorted render kernel
//   2  plain render kernel with colour
//   3  persistent batch kernel without colour (and the colour dispatch)
//   4  persistent batch kernel with colour
//   5  single-step and trace kernels
//   6  FP32 only: plain render kernels for merged-form programs (both colour
//      variants, variation sets 1 and 2; ProgHeader::merged, only the seven
//      benchmark variations)
//   7  FP32 only: persistent batch kernels for merged-form programs
// Each general render kernel inlines every variation, so one kernel per
// object keeps the slowest object (FP64 without contraction) short.  The FP64 objects are
// built with --fmad=false so no multiply-add is contracted: the reference
// (and the oracle) round every product and sum separately.
#include "chaos_kernel.cuh"
#include "chaos_sorted.cuh"

#if !defined(FFR_P) || !defined(FFR_D) || !defined(FFR_KIND)
#error "compile with -DFFR_P=<0|1> -DFFR_D=<1|2|3> -DFFR_KIND=<0..7>"
#endif

#define FFR_CAT2(a, b, c, d) a##_p##b##_d##c##d
#define FFR_CAT(a, b, c) FFR_CAT2(a, b, c, )
#define FFR_NAME(a) FFR_CAT(a, FFR_P, FFR_D)

namespace ffr {

#if FFR_P == 0
using Real = double;
#else
using Real = float;
#endif

// the colour instantiations live in their own objects (kinds 2 and 4)
cudaError_t FFR_NAME(launch_render_color)(const RenderArgs& a, int grid, cudaStream_t st);
cudaError_t FFR_NAME(occupancy_color)(int rsl_words, int hot, int* blocks_per_sm,
                                      unsigned int prog_bytes, int nxf, size_t* smem);
cudaError_t FFR_NAME(launch_batch_color)(const BatchArgs& b, int grid, size_t smem,
                                         cudaStream_t st);
cudaError_t FFR_NAME(occupancy_batch_color)(int* blocks_per_sm, size_t smem);
// the merged-form instantiations (FP32, kinds 6 and 7)
cudaError_t FFR_NAME(launch_render_merged)(const RenderArgs& a, int grid, cudaStream_t st);
cudaError_t FFR_NAME(occupancy_merged)(int color, int vs, int rsl_words, int hot,
                                       int* blocks_per_sm, unsigned int prog_bytes, int nxf,
                                       size_t* smem);
cudaError_t FFR_NAME(launch_batch_merged)(const BatchArgs& b, int color, int vs, int grid,
                                          size_t smem, cudaStream_t st);
cudaError_t FFR_NAME(occupancy_batch_merged)(int color, int vs, int* blocks_per_sm, size_t smem);

constexpr int kBlock = 128;

#if FFR_KIND == 0 || FFR_KIND == 2 || FFR_KIND == 6

template <bool C, int V = 0>
static cudaError_t launch_one(const RenderArgs& a, int grid, cudaStream_t st)
{
    const size_t smem = chaos_smem_bytes<kBlock>(a.prog_bytes, a.nxf, a.rsl_words,
                                                 a.hot_keys != nullptr);
    auto k = chaos_kernel<FFR_D, Real, C, kBlock, V>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    k<<<grid, kBlock, smem, st>>>(a);
    return cudaGetLastError();
}

template <bool C, int V = 0>
static cudaError_t occ_one(int* bps, unsigned int prog_bytes, int nxf, int rsl_words, int hot,
                           size_t* smem_out)
{
    const size_t smem = chaos_smem_bytes<kBlock>(prog_bytes, nxf, rsl_words, hot != 0);
    auto k = chaos_kernel<FFR_D, Real, C, kBlock, V>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    *smem_out = smem;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, kBlock, smem);
}

#endif

#if FFR_KIND == 0

cudaError_t FFR_NAME(launch_render)(const RenderArgs& a, int grid, cudaStream_t st)
{
#if FFR_P == 1
    if (a.merged)
        return FFR_NAME(launch_render_merged)(a, grid, st);
#endif
    return a.color_dims > 0 ? FFR_NAME(launch_render_color)(a, grid, st)
                            : launch_one<false>(a, grid, st);
}

cudaError_t FFR_NAME(occupancy)(int color, int merged, int rsl_words, int hot,
                                int* blocks_per_sm, int* block, unsigned int prog_bytes,
                                int nxf, size_t* smem)
{
    *block = kBlock;
#if FFR_P == 1
    if (merged)
        return FFR_NAME(occupancy_merged)(color, merged, rsl_words, hot, blocks_per_sm,
                                          prog_bytes, nxf, smem);
#else
    (void)merged;
#endif
    return color ? FFR_NAME(occupancy_color)(rsl_words, hot, blocks_per_sm, prog_bytes, nxf, smem)
                 : occ_one<false>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem);
}

#elif FFR_KIND == 2

cudaError_t FFR_NAME(launch_render_color)(const RenderArgs& a, int grid, cudaStream_t st)
{
    return launch_one<true>(a, grid, st);
}

cudaError_t FFR_NAME(occupancy_color)(int rsl_words, int hot, int* blocks_per_sm,
                                      unsigned int prog_bytes, int nxf, size_t* smem)
{
    return occ_one<true>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem);
}

#elif FFR_KIND == 6 && FFR_P == 1

cudaError_t FFR_NAME(launch_render_merged)(const RenderArgs& a, int grid, cudaStream_t st)
{
    if (a.merged == 2)
        return a.color_dims > 0 ? launch_one<true, 2>(a, grid, st)
                                : launch_one<false, 2>(a, grid, st);
    return a.color_dims > 0 ? launch_one<true, 1>(a, grid, st)
                            : launch_one<false, 1>(a, grid, st);
}

cudaError_t FFR_NAME(occupancy_merged)(int color, int vs, int rsl_words, int hot,
                                       int* blocks_per_sm, unsigned int prog_bytes, int nxf,
                                       size_t* smem)
{
    if (vs == 2)
        return color ? occ_one<true, 2>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem)
                     : occ_one<false, 2>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem);
    return color ? occ_one<true, 1>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem)
                 : occ_one<false, 1>(blocks_per_sm, prog_bytes, nxf, rsl_words, hot, smem);
}

#endif

#if FFR_KIND == 3 || FFR_KIND == 4 || FFR_KIND == 7

template <bool C, int V = 0>
static cudaError_t batch_attr(size_t smem)
{
    return cudaFuncSetAttribute(chaos_batch_kernel<FFR_D, Real, C, kBlock, V>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <bool C, int V = 0>
static cudaError_t batch_launch(const BatchArgs& b, int grid, size_t smem, cudaStream_t st)
{
    chaos_batch_kernel<FFR_D, Real, C, kBlock, V><<<grid, kBlock, smem, st>>>(b);
    return cudaGetLastError();
}

template <bool C, int V = 0>
static cudaError_t batch_occ(int* blocks_per_sm, size_t smem)
{
    cudaError_t e = batch_attr<C, V>(smem);
    if (e != cudaSuccess)
        return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        blocks_per_sm, chaos_batch_kernel<FFR_D, Real, C, kBlock, V>, kBlock, smem);
}

#if FFR_KIND == 3

cudaError_t FFR_NAME(launch_batch)(const BatchArgs& b, int color, int merged, int grid,
                                   size_t smem, cudaStream_t st)
{
#if FFR_P == 1
    if (merged)
        return FFR_NAME(launch_batch_merged)(b, color, merged, grid, smem, st);
#else
    (void)merged;
#endif
    return color ? FFR_NAME(launch_batch_color)(b, grid, smem, st)
                 : batch_launch<false>(b, grid, smem, st);
}

cudaError_t FFR_NAME(occupancy_batch)(int color, int merged, int* blocks_per_sm, int* block,
                                      size_t smem)
{
    *block = kBlock;
#if FFR_P == 1
    if (merged)
        return FFR_NAME(occupancy_batch_merged)(color, merged, blocks_per_sm, smem);
#else
    (void)merged;
#endif
    return color ? FFR_NAME(occupancy_batch_color)(blocks_per_sm, smem)
                 : batch_occ<false>(blocks_per_sm, smem);
}

#elif FFR_KIND == 7

#if FFR_P == 1
cudaError_t FFR_NAME(launch_batch_merged)(const BatchArgs& b, int color, int vs, int grid,
                                          size_t smem, cudaStream_t st)
{
    if (vs == 2)
        return color ? batch_launch<true, 2>(b, grid, smem, st)
                     : batch_launch<false, 2>(b, grid, smem, st);
    return color ? batch_launch<true, 1>(b, grid, smem, st)
                 : batch_launch<false, 1>(b, grid, smem, st);
}

cudaError_t FFR_NAME(occupancy_batch_merged)(int color, int vs, int* blocks_per_sm, size_t smem)
{
    if (vs == 2)
        return color ? batch_occ<true, 2>(blocks_per_sm, smem)
                     : batch_occ<false, 2>(blocks_per_sm, smem);
    return color ? batch_occ<true, 1>(blocks_per_sm, smem)
                 : batch_occ<false, 1>(blocks_per_sm, smem);
}
#endif

#else

cudaError_t FFR_NAME(launch_batch_color)(const BatchArgs& b, int grid, size_t smem,
                                         cudaStream_t st)
{
    return batch_launch<true>(b, grid, smem, st);
}

cudaError_t FFR_NAME(occupancy_batch_color)(int* blocks_per_sm, size_t smem)
{
    return batch_occ<true>(blocks_per_sm, smem);
}

#endif

#elif FFR_KIND == 5

cudaError_t FFR_NAME(launch_step)(const StepArgs& a, cudaStream_t st)
{
    if (a.npts == 0)
        return cudaSuccess;
    const size_t smem = align16u(a.prog_bytes) + 2 * 16 * 128 * sizeof(uint64_t);
    auto k = step_kernel<FFR_D, Real>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    unsigned long long blocks = (a.npts + 127) / 128;
    if (blocks > 65535)
        blocks = 65535;
    k<<<(unsigned int)blocks, 128, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t FFR_NAME(launch_trace)(const TraceArgs& a, cudaStream_t st)
{
    const size_t smem = align16u(a.prog_bytes) + 2 * 16 * sizeof(uint64_t);
    auto k = trace_kernel<FFR_D, Real>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    k<<<1, 1, smem, st>>>(a);
    return cudaGetLastError();
}

#elif FFR_KIND == 1

template <bool C>
static cudaError_t launch_sorted_one(const RenderArgs& a, int grid, cudaStream_t st)
{
    const size_t smem = sorted_smem_bytes<kSortedBlock>(
        a.prog_bytes, a.nxf, a.rng_words, FFR_D, (int)sizeof(Real));
    auto k = chaos_sorted_kernel<FFR_D, Real, C, kSortedBlock>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    k<<<grid, kSortedBlock, smem, st>>>(a);
    return cudaGetLastError();
}

template <bool C>
static cudaError_t occ_sorted_one(int* bps, unsigned int prog_bytes, int nxf, int words,
                                  size_t* smem_out)
{
    const size_t smem = sorted_smem_bytes<kSortedBlock>(prog_bytes, nxf, words, FFR_D,
                                                        (int)sizeof(Real));
    auto k = chaos_sorted_kernel<FFR_D, Real, C, kSortedBlock>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    *smem_out = smem;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, kSortedBlock, smem);
}

cudaError_t FFR_NAME(launch_sorted)(const RenderArgs& a, int grid, cudaStream_t st)
{
    return a.color_dims > 0 ? launch_sorted_one<true>(a, grid, st)
                            : launch_sorted_one<false>(a, grid, st);
}

cudaError_t FFR_NAME(occupancy_sorted)(int color, int spill, int* blocks_per_sm, int* block,
                                       unsigned int prog_bytes, int nxf, int words,
                                       size_t* smem)
{
    *block = kSortedBlock;
    if (nxf > kSortedMaxXforms)
    {
        *blocks_per_sm = 0;
        return cudaSuccess;
    }
    (void)spill;
    return color ? occ_sorted_one<true>(blocks_per_sm, prog_bytes, nxf, words, smem)
                 : occ_sorted_one<false>(blocks_per_sm, prog_bytes, nxf, words, smem);
}

#endif

} // namespace ffr
