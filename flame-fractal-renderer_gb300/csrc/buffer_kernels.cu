// Buffer kernels: file-layout import/export, histogram reduction and the
// raw ISAAC word generator used by the verification entry point.
//
// Device buffer layout (planar, chosen for the binning kernel): counts as
// u32 low words [cells], optional u32 high words [cells] (present once any
// count can pass 2^32), colours f64 [cells][color_dims].  File layout (the
// reference's, buffer_renderer.hpp:476-480): per cell one u64 count then
// color_dims f64 colours.
//
//   launch_accumulate  BufferRenderer::addBuffer / readBuffer (overwrite)
//                      buffer_renderer.hpp:375-475
//   launch_export      BufferRenderer::writeBuffer, buffer_renderer.hpp:476-480
//   launch_hist_reduce histogramSum/Min/Max, buffer_renderer.hpp:483-507
//   launch_hot_collect cells at or above a count (the render kernel's
//                      hot-cell table; no reference counterpart)
// All are grid-stride loops sized to the SM count: HBM-bound streaming.
#include "isaac64.cuh"
#include "launch.h"

namespace ffr {

namespace {

int grid_for(unsigned long long n, int block)
{
    static int sms = 0;
    if (sms == 0)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0)
            sms = 1;
    }
    unsigned long long want = (n + block - 1) / block;
    unsigned long long cap = (unsigned long long)sms * 8;
    if (want > cap)
        want = cap;
    return want ? (int)want : 1;
}

__global__ void isaac_words_kernel(unsigned long long key, unsigned long long n,
                                   unsigned long long* out, IsaacInit init)
{
    __shared__ uint64_t st[32];
    DevIsaac<1> g;
    g.mem = st;
    g.rsl = st + 16;
    g.seed(key, init.w);
    for (unsigned long long i = 0; i < n; ++i)
        out[i] = g.next();
}

// one thread per cell; colour f64 values move as raw 64-bit words
__global__ void accumulate_kernel(const unsigned long long* __restrict__ file,
                                  unsigned long long cells, int r,
                                  unsigned int* __restrict__ counts,
                                  unsigned int* __restrict__ hi,
                                  double* __restrict__ colors, int overwrite)
{
    const unsigned long long stride = 1ull + (unsigned long long)r;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         i < cells; i += (unsigned long long)gridDim.x * blockDim.x)
    {
        const unsigned long long add = file[i * stride];
        if (overwrite)
        {
            counts[i] = (unsigned int)add;
            if (hi)
                hi[i] = (unsigned int)(add >> 32);
        }
        else
        {
            const unsigned long long cur = ((unsigned long long)(hi ? hi[i] : 0u) << 32) | counts[i];
            const unsigned long long sum = cur + add;      // u64 wrap, as hist_t
            counts[i] = (unsigned int)sum;
            if (hi)
                hi[i] = (unsigned int)(sum >> 32);
        }
        for (int c = 0; c < r; ++c)
        {
            const double v = __longlong_as_double((long long)file[i * stride + 1 + c]);
            if (overwrite)
                colors[i * r + c] = v;
            else
                colors[i * r + c] += v;
        }
    }
}

// largest u64 count in a file-layout buffer (atomicMax into *out)
__global__ void file_max_kernel(const unsigned long long* __restrict__ file,
                                unsigned long long cells, int r,
                                unsigned long long* out)
{
    const unsigned long long stride = 1ull + (unsigned long long)r;
    unsigned long long mx = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         i < cells; i += (unsigned long long)gridDim.x * blockDim.x)
        mx = max(mx, file[i * stride]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31u) == 0 && mx)
        atomicMax(out, mx);
}

__global__ void export_kernel(unsigned long long* __restrict__ file,
                              unsigned long long cells, int r,
                              const unsigned int* __restrict__ counts,
                              const unsigned int* __restrict__ hi,
                              const double* __restrict__ colors)
{
    const unsigned long long stride = 1ull + (unsigned long long)r;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         i < cells; i += (unsigned long long)gridDim.x * blockDim.x)
    {
        file[i * stride] = ((unsigned long long)(hi ? hi[i] : 0u) << 32) | counts[i];
        for (int c = 0; c < r; ++c)
            file[i * stride + 1 + c] =
                (unsigned long long)__double_as_longlong(colors[i * r + c]);
    }
}

// out[0] += sum, out[1] = min, out[2] = max (out preset to 0, ~0, 0)
__global__ void hist_reduce_kernel(const uint4* __restrict__ counts4,
                                   const unsigned int* __restrict__ counts,
                                   const unsigned int* __restrict__ hi,
                                   unsigned long long cells, unsigned long long* out)
{
    unsigned long long sum = 0, mn = ~0ull, mx = 0;
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long nth = (unsigned long long)gridDim.x * blockDim.x;
    if (!hi)
    {
        const unsigned long long n4 = cells / 4;
        for (unsigned long long i = tid; i < n4; i += nth)
        {
            const uint4 v = counts4[i];
            sum += (unsigned long long)v.x + v.y + v.z + v.w;
            mn = min(mn, (unsigned long long)min(min(v.x, v.y), min(v.z, v.w)));
            mx = max(mx, (unsigned long long)max(max(v.x, v.y), max(v.z, v.w)));
        }
        for (unsigned long long i = n4 * 4 + tid; i < cells; i += nth)
        {
            const unsigned long long v = counts[i];
            sum += v;
            mn = min(mn, v);
            mx = max(mx, v);
        }
    }
    else
    {
        for (unsigned long long i = tid; i < cells; i += nth)
        {
            const unsigned long long v = ((unsigned long long)hi[i] << 32) | counts[i];
            sum += v;
            mn = min(mn, v);
            mx = max(mx, v);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
        sum += __shfl_down_sync(0xffffffffu, sum, off);
        mn = min(mn, __shfl_down_sync(0xffffffffu, mn, off));
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, off));
    }
    if ((threadIdx.x & 31u) == 0)
    {
        atomicAdd(&out[0], sum);
        atomicMin(&out[1], mn);
        atomicMax(&out[2], mx);
    }
}

// Roofline microbenchmark: fire-and-forget 4-byte atomic adds (RED) at
// uniformly distributed cells of a `cells`-long buffer; the index comes from
// a 32-bit integer hash of (thread, iteration), a few integer instructions.
__global__ void atomic_rate_kernel(unsigned int* __restrict__ buf, unsigned int cells,
                                   unsigned int iters, unsigned int salt)
{
    const unsigned int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int x = t * 0x9E3779B9u + salt;
    for (unsigned int j = 0; j < iters; ++j)
    {
        x += 0x6D2B79F5u;
        unsigned int h = x;
        h ^= h >> 15;
        h *= 0x2C1B3C6Du;
        h ^= h >> 12;
        h *= 0x297A2D39u;
        h ^= h >> 15;
        atomicAdd(&buf[__umulhi(h, cells)], 1u);
    }
}

// zero one statistics head and its per-xform counts, extreme keys to
// +inf / -inf (one CTA)
__device__ void reset_one(DevStats* st, int nxf)
{
    if (threadIdx.x == 0)
    {
        st->s_iter = st->s_plot = st->bad_total = st->dropped = st->bad_claim = 0ull;
        st->stop = st->cancelled = 0u;
        for (int i = 0; i < kMaxDims; ++i)
        {
            st->ext_lo[i] = order_key(__longlong_as_double(0x7ff0000000000000ll));
            st->ext_hi[i] = order_key(__longlong_as_double((long long)0xfff0000000000000ull));
        }
    }
    for (int i = threadIdx.x; i < nxf; i += blockDim.x)
        st->xf_dist[i] = 0ull;
}

// one CTA per job: reset its statistics; CTA 0 also rewinds the claim cursor
__global__ void batch_reset_kernel(const JobDesc* jobs, int njobs, BatchHead* head)
{
    const int j = blockIdx.x;
    if (j == 0 && threadIdx.x == 0)
        head->cursor = 0ull;
    if (j >= njobs)
        return;
    reset_one(jobs[j].a.stats, jobs[j].a.nxf);
}

__global__ void stats_reset_kernel(DevStats* st, int nxf)
{
    reset_one(st, nxf);
}

} // namespace

cudaError_t launch_batch_reset(const JobDesc* jobs, int njobs, BatchHead* head,
                               cudaStream_t st)
{
    batch_reset_kernel<<<njobs > 0 ? njobs : 1, 128, 0, st>>>(jobs, njobs, head);
    return cudaGetLastError();
}

cudaError_t launch_stats_reset(DevStats* st, int nxf, cudaStream_t s)
{
    stats_reset_kernel<<<1, 128, 0, s>>>(st, nxf);
    return cudaGetLastError();
}

cudaError_t launch_atomic_rate(unsigned int* buf, unsigned int cells, unsigned int iters,
                               int grid, int block, unsigned int salt, cudaStream_t st)
{
    atomic_rate_kernel<<<grid, block, 0, st>>>(buf, cells, iters, salt);
    return cudaGetLastError();
}

cudaError_t launch_isaac_words(unsigned long long key, unsigned long long n,
                               unsigned long long* out, const unsigned long long* init16,
                               cudaStream_t st)
{
    IsaacInit init;
    for (int i = 0; i < 16; ++i)
        init.w[i] = init16[i];
    isaac_words_kernel<<<1, 1, 0, st>>>(key, n, out, init);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const unsigned long long* file, unsigned long long cells,
                              int color_dims, unsigned int* counts, unsigned int* hi,
                              double* colors, int overwrite, cudaStream_t st)
{
    accumulate_kernel<<<grid_for(cells, 256), 256, 0, st>>>(file, cells, color_dims,
                                                             counts, hi, colors, overwrite);
    return cudaGetLastError();
}

cudaError_t launch_file_max(const unsigned long long* file, unsigned long long cells,
                            int color_dims, unsigned long long* out, cudaStream_t st)
{
    file_max_kernel<<<grid_for(cells, 256), 256, 0, st>>>(file, cells, color_dims, out);
    return cudaGetLastError();
}

cudaError_t launch_export(unsigned long long* file, unsigned long long cells,
                          int color_dims, const unsigned int* counts,
                          const unsigned int* hi, const double* colors, cudaStream_t st)
{
    export_kernel<<<grid_for(cells, 256), 256, 0, st>>>(file, cells, color_dims,
                                                         counts, hi, colors);
    return cudaGetLastError();
}

namespace {

__global__ void hot_collect_kernel(const volatile unsigned int* counts, unsigned int cells,
                                   unsigned int thr, unsigned long long* out, unsigned int cap)
{
    // out[0]: number of cells found; out[1 ..]: (count << 32 | cell), the
    // first cap of them in no particular order.  Volatile loads are relaxed
    // accesses, not racing with the atomic adds of a render still running.
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < cells;
         i += gridDim.x * blockDim.x)
    {
        const unsigned int v = counts[i];
        if (v >= thr)
        {
            const unsigned long long k = atomicAdd(out, 1ull);
            if (k < cap)
                out[1 + k] = ((unsigned long long)v << 32) | i;
        }
    }
}

} // namespace

cudaError_t launch_hot_collect(const unsigned int* counts, unsigned int cells, unsigned int thr,
                               unsigned long long* out, unsigned int cap, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
    hot_collect_kernel<<<grid_for(cells, 256), 256, 0, st>>>(counts, cells, thr, out, cap);
    return cudaGetLastError();
}

cudaError_t collect_hot_candidates(const unsigned int* counts, unsigned int cells,
                                   unsigned long long thr, unsigned long long thr_max,
                                   unsigned long long* out, cudaStream_t st,
                                   std::vector<unsigned long long>& found, bool* got,
                                   unsigned int* launches)
{
    *got = false;
    found.clear();
    thr = thr ? thr : 1;
    for (; thr <= thr_max && thr <= 0xFFFFFFFFull; thr *= 4)
    {
        unsigned long long n = 0;
        cudaError_t e = launch_hot_collect(counts, cells, (unsigned int)thr, out, kHotCollectCap,
                                           st);
        if (e == cudaSuccess && launches)
            ++*launches;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&n, out, sizeof n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return e;
        if (n > kHotCollectCap)
            continue;           // too many at this threshold: raise it
        found.resize(n);
        if (n)
        {
            e = cudaMemcpyAsync(found.data(), out + 1, n * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (e != cudaSuccess)
                return e;
        }
        *got = true;
        return cudaSuccess;
    }
    return cudaSuccess;
}

cudaError_t launch_hist_reduce(const unsigned int* counts, const unsigned int* hi,
                               unsigned long long cells, unsigned long long* out,
                               cudaStream_t st)
{
    hist_reduce_kernel<<<grid_for(cells / 4 + 1, 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(counts), counts, hi, cells, out);
    return cudaGetLastError();
}

} // namespace ffr
