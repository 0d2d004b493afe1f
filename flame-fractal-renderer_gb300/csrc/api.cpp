// C ABI of libffr_gpu.so (include/ffr_gpu.h): context lifetime, device
// memory admission, launches on a context-owned stream, bounded waits and
// statistics.  No exception crosses the boundary.
#include "ffr_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "flame.hpp"
#include "isaac64.cuh"
#include "jit.h"
#include "launch.h"

namespace ffr {

// Isaac::init with flag = false (src/rng/isaac.hpp:93-131): randmem is the
// golden-ratio constant mixed 4 times, then mixed once per 8 words.
void isaac_init_table(unsigned long long out[16])
{
    uint64_t a, b, c, d, e, f, g, h;
    a = b = c = d = e = f = g = h = kIsaacGolden;
    auto mix = [&]() {
        a -= e; f ^= h >> 9;  h += a;
        b -= f; g ^= a << 9;  a += b;
        c -= g; h ^= b >> 23; b += c;
        d -= h; a ^= c << 15; c += d;
        e -= a; b ^= d >> 14; d += e;
        f -= b; c ^= e << 20; e += f;
        g -= c; d ^= f >> 17; f += g;
        h -= d; e ^= g << 14; g += h;
    };
    for (int i = 0; i < 4; ++i)
        mix();
    for (int i = 0; i < 16; i += 8)
    {
        mix();
        out[i + 0] = a; out[i + 1] = b; out[i + 2] = c; out[i + 3] = d;
        out[i + 4] = e; out[i + 5] = f; out[i + 6] = g; out[i + 7] = h;
    }
}

} // namespace ffr

using namespace ffr;

namespace {

thread_local std::string g_create_error = "no error";

} // namespace

void ffr::set_global_error(const std::string& m)
{
    g_create_error = m;
}

namespace {

const Launchers kLaunchers[2][4] = {
    {
        {launch_render_p0_d1, occupancy_p0_d1, launch_sorted_p0_d1,
         occupancy_sorted_p0_d1, launch_batch_p0_d1, occupancy_batch_p0_d1,
         launch_step_p0_d1, launch_trace_p0_d1},
        {launch_render_p0_d2, occupancy_p0_d2, launch_sorted_p0_d2,
         occupancy_sorted_p0_d2, launch_batch_p0_d2, occupancy_batch_p0_d2,
         launch_step_p0_d2, launch_trace_p0_d2},
        {launch_render_p0_d3, occupancy_p0_d3, launch_sorted_p0_d3,
         occupancy_sorted_p0_d3, launch_batch_p0_d3, occupancy_batch_p0_d3,
         launch_step_p0_d3, launch_trace_p0_d3},
        {launch_render_p0_d4, occupancy_p0_d4, nullptr, nullptr, nullptr, nullptr,
         launch_step_p0_d4, launch_trace_p0_d4},
    },
    {
        {launch_render_p1_d1, occupancy_p1_d1, launch_sorted_p1_d1,
         occupancy_sorted_p1_d1, launch_batch_p1_d1, occupancy_batch_p1_d1,
         launch_step_p1_d1, launch_trace_p1_d1},
        {launch_render_p1_d2, occupancy_p1_d2, launch_sorted_p1_d2,
         occupancy_sorted_p1_d2, launch_batch_p1_d2, occupancy_batch_p1_d2,
         launch_step_p1_d2, launch_trace_p1_d2},
        {launch_render_p1_d3, occupancy_p1_d3, launch_sorted_p1_d3,
         occupancy_sorted_p1_d3, launch_batch_p1_d3, occupancy_batch_p1_d3,
         launch_step_p1_d3, launch_trace_p1_d3},
        {launch_render_p1_d4, occupancy_p1_d4, nullptr, nullptr, nullptr, nullptr,
         launch_step_p1_d4, launch_trace_p1_d4},
    },
};

} // namespace

const Launchers& ffr::launchers(int precision, int dims)
{
    return kLaunchers[precision][dims - 1];
}

struct ffr_ctx
{
    ffr_opts opts{};
    HostFlame flame;
    std::vector<uint8_t> prog_host;
    int device = 0;
    int sm_count = 1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_done = nullptr;
    unsigned char* d_prog = nullptr;
    unsigned int* d_counts = nullptr;
    unsigned int* d_hi = nullptr;
    double* d_colors = nullptr;
    DevStats* d_stats = nullptr;
    unsigned long long* d_scratch = nullptr;   // file staging / reductions
    size_t scratch_bytes = 0;
    unsigned int* h_cancel = nullptr;          // mapped pinned flag
    unsigned int* d_cancel = nullptr;
    unsigned long long isaac_init[16] = {};
    // upper bound of any cell's count (decides when high words are needed)
    unsigned long long count_bound = 0;
    // autotuner decision (kernel, warp aggregation), valid for spill mode
    bool tuned = false;
    bool tuned_spill = false;
    int tuned_kernel = FFR_KERNEL_PLAIN;
    int tuned_agg = 0;
    bool tuned_hot = false;
    // resident CTAs per SM the tuned launch uses at most (0: all that fit);
    // a lower cap runs each thread's streams one after another and never
    // changes which streams run, so the buffer does not depend on it
    int tuned_cap = 0;
    bool tuned_jit = true;          // TuneChoice::jit_considered, ms_per_sample
    double tuned_ms_per_sample = 0.0;
    int probe_cap = 0;              // the cap an autotuner probe is planned with
    bool hot_searched = false;      // a hot-cell search ran (probe or autotuner)
    // shape of the last plan(): CTAs per SM allowed, threads per CTA, streams
    // each thread runs (reported in ffr_stats)
    int plan_cap = 0, plan_block = 0;
    uint64_t plan_spt = 0;
    // hot-cell table of the plain kernel (kHotSlots keys), installed by the
    // autotuner; hot_mult 0 = none
    unsigned int* d_hot = nullptr;
    unsigned int hot_mult = 0;
    int hot_cells = 0;
    // the per-flame kernel (jit.h), once compiled and loaded for this
    // context's flame structure; jit_source is empty for programs that have
    // none (the FP32 merged form)
    const JitKernel* jit = nullptr;
    std::string jit_source;
    const JitKernel* jit_sorted = nullptr;      // the xform-sorted per-flame kernel
    std::string jit_sorted_source;
    // kernels launched by the current call besides the render kernel
    unsigned int aux_launches = 0;
    std::string err = "no error";

    const Launchers& L() const { return kLaunchers[opts.precision][flame.dims - 1]; }
    size_t buffer_bytes() const
    {
        return (size_t)flame.cells * (1 + (size_t)flame.color_dims) * 8;
    }
};

namespace {

ffr_status fail(ffr_ctx* c, ffr_status s, const std::string& m)
{
    if (c)
        c->err = m;
    else
        g_create_error = m;
    return s;
}

ffr_status cuda_fail(ffr_ctx* c, cudaError_t e, const char* where)
{
    return fail(c, FFR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CU(ctx, call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess)                          \
            return cuda_fail((ctx), e_, #call);         \
    } while (0)

// wait for the context stream with the context's time limit; on timeout the
// running kernel is asked to stop through the mapped cancel flag, then
// waited for once more (its poll interval is 4096 samples).
ffr_status wait_stream(ffr_ctx* c)
{
    CU(c, cudaEventRecord(c->ev_done, c->stream));
    const uint64_t limit = c->opts.timeout_ms;
    if (limit == 0)
    {
        CU(c, cudaEventSynchronize(c->ev_done));
        return FFR_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;)
    {
        cudaError_t q = cudaEventQuery(c->ev_done);
        if (q == cudaSuccess)
            return FFR_OK;
        if (q != cudaErrorNotReady)
            return cuda_fail(c, q, "cudaEventQuery");
        const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
            std::chrono::steady_clock::now() - t0).count();
        if ((uint64_t)ms >= limit)
            break;
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    *(volatile unsigned int*)c->h_cancel = 1u;
    const auto t1 = std::chrono::steady_clock::now();
    for (;;)
    {
        cudaError_t q = cudaEventQuery(c->ev_done);
        if (q == cudaSuccess)
            break;
        if (q != cudaErrorNotReady)
            return cuda_fail(c, q, "cudaEventQuery");
        const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
            std::chrono::steady_clock::now() - t1).count();
        if ((uint64_t)ms >= std::max<uint64_t>(limit, 1000))
            return fail(c, FFR_ERR_TIMEOUT, "device work did not stop after cancel");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    *(volatile unsigned int*)c->h_cancel = 0u;
    return fail(c, FFR_ERR_TIMEOUT, "render exceeded timeout_ms ("
        + std::to_string(limit) + " ms) and was cancelled");
}

// Context buffers come from a per-device stream-ordered pool that keeps up
// to kPoolKeepBytes of the memory of destroyed contexts for the next ones
// (allocated and freed in order on the context's stream): creating and
// destroying a context per render, as a caller of ffr_create / ffr_render /
// ffr_destroy does, then costs no device-wide synchronisation and no driver
// allocation, while memory beyond that returns to the device.
constexpr unsigned long long kPoolKeepBytes = 4ull << 30;
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;

cudaError_t ctx_pool(int device, cudaMemPool_t* out)
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pools.find(device);
    if (it != g_pools.end())
    {
        *out = it->second;
        return cudaSuccess;
    }
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess)
        return e;
    unsigned long long keep = kPoolKeepBytes;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess)
    {
        cudaMemPoolDestroy(pool);
        return e;
    }
    g_pools[device] = pool;
    *out = pool;
    return cudaSuccess;
}

// bytes the device's context pool holds without an allocation using them
// (free for a new context, although cudaMemGetInfo counts them as used)
size_t pool_cached(int device)
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pools.find(device);
    if (it == g_pools.end())
        return 0;
    unsigned long long reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(it->second, cudaMemPoolAttrReservedMemCurrent, &reserved)
            != cudaSuccess
        || cudaMemPoolGetAttribute(it->second, cudaMemPoolAttrUsedMemCurrent, &used)
            != cudaSuccess)
        return 0;
    return reserved > used ? (size_t)(reserved - used) : 0;
}

// free device memory for a context: the device's free memory plus its
// context pool's unused bytes
cudaError_t ctx_free_bytes(int device, size_t* fr)
{
    size_t tot = 0;
    cudaError_t e = cudaMemGetInfo(fr, &tot);
    if (e == cudaSuccess)
        *fr += pool_cached(device);
    return e;
}

template <typename T>
cudaError_t ctx_alloc(ffr_ctx* c, T** p, size_t bytes)
{
    cudaMemPool_t pool = nullptr;
    cudaError_t e = ctx_pool(c->device, &pool);
    if (e != cudaSuccess)
        return e;
    void* v = nullptr;
    e = cudaMallocFromPoolAsync(&v, bytes, pool, c->stream);
    *p = static_cast<T*>(v);
    return e;
}

void ctx_release(ffr_ctx* c, void* p)
{
    if (p)
        cudaFreeAsync(p, c->stream);
}

ffr_status ensure_scratch(ffr_ctx* c, size_t bytes)
{
    if (c->scratch_bytes >= bytes)
        return FFR_OK;
    ctx_release(c, c->d_scratch);
    c->d_scratch = nullptr;
    c->scratch_bytes = 0;
    size_t fr = 0;
    CU(c, ctx_free_bytes(c->device, &fr));
    if (bytes + (64u << 20) > fr)
        return fail(c, FFR_ERR_OOM, "not enough free device memory for a "
            + std::to_string(bytes) + "-byte staging buffer");
    CU(c, ctx_alloc(c, &c->d_scratch, bytes));
    c->scratch_bytes = bytes;
    return FFR_OK;
}

// The high-word buffer, zeroed; the wait makes it ready for any stream (a
// batch renders on its own stream; pool memory and the memset are ordered
// on the context's)
ffr_status ensure_hi(ffr_ctx* c)
{
    if (c->d_hi)
        return FFR_OK;
    CU(c, ctx_alloc(c, &c->d_hi, c->flame.cells * sizeof(unsigned int)));
    CU(c, cudaMemsetAsync(c->d_hi, 0, c->flame.cells * sizeof(unsigned int), c->stream));
    CU(c, cudaStreamSynchronize(c->stream));
    return FFR_OK;
}

// Cancel flags: mapped pinned words handed out from per-device blocks of
// kFlagBlock (pinning a page per context cost more than the rest of
// ffr_create); a flag returns to its device's free list with its context.
constexpr int kFlagBlock = 1024;
std::mutex g_flag_mu;
std::map<int, std::vector<std::pair<unsigned int*, unsigned int*>>> g_flag_free;

cudaError_t take_flag(int device, unsigned int** h, unsigned int** d)
{
    std::lock_guard<std::mutex> lk(g_flag_mu);
    auto& fl = g_flag_free[device];
    if (fl.empty())
    {
        unsigned int* blk = nullptr;
        unsigned int* dblk = nullptr;
        cudaError_t e = cudaHostAlloc(&blk, kFlagBlock * sizeof(unsigned int),
                                      cudaHostAllocMapped | cudaHostAllocPortable);
        if (e != cudaSuccess)
            return e;
        if ((e = cudaHostGetDevicePointer(&dblk, blk, 0)) != cudaSuccess)
        {
            cudaFreeHost(blk);
            return e;
        }
        for (int i = kFlagBlock - 1; i >= 0; --i)
            fl.emplace_back(blk + i, dblk + i);
    }
    *h = fl.back().first;
    *d = fl.back().second;
    fl.pop_back();
    *(volatile unsigned int*)*h = 0u;
    return cudaSuccess;
}

void give_flag(int device, unsigned int* h, unsigned int* d)
{
    std::lock_guard<std::mutex> lk(g_flag_mu);
    g_flag_free[device].emplace_back(h, d);
}

void destroy(ffr_ctx* c)
{
    if (!c)
        return;
    cudaSetDevice(c->device);
    if (c->stream)
    {
        // back to the pool in stream order, then wait for the stream
        ctx_release(c, c->d_prog);
        ctx_release(c, c->d_counts);
        ctx_release(c, c->d_hi);
        ctx_release(c, c->d_colors);
        ctx_release(c, c->d_stats);
        ctx_release(c, c->d_scratch);
        ctx_release(c, c->d_hot);
        cudaStreamSynchronize(c->stream);
    }
    if (c->h_cancel)
        give_flag(c->device, c->h_cancel, c->d_cancel);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    delete c;
}

static_assert(offsetof(ProgHeader<double>, rng_words_max)
              == offsetof(ProgHeader<float>, rng_words_max), "program header layout");

// words one selectable xform application draws at most (ProgHeader)
int program_words(const ffr_ctx* c)
{
    const ProgHeader<double>* h = reinterpret_cast<const ProgHeader<double>*>(c->prog_host.data());
    return (int)h->rng_words_max;       // same offset in the float header
}

// A per-flame kernel of the context's program (the plain one, or with
// sorted the xform-sorted one), compiled on first use (or found in the
// caches); ready_only: only if no compile is needed
ffr_status ensure_jit(ffr_ctx* c, bool sorted, bool ready_only = false)
{
    const JitKernel*& k = sorted ? c->jit_sorted : c->jit;
    if (k)
        return FFR_OK;
    std::string& src = sorted ? c->jit_sorted_source : c->jit_source;
    if (src.empty())
        src = jit_source(c->prog_host, c->opts.precision, c->flame.color_dims > 0, sorted);
    std::string err;
    k = jit_kernel(src, c->opts.precision, &err, !ready_only);
    if (!k)
        return ready_only ? FFR_ERR_ARG : fail(c, FFR_ERR_CUDA, err);
    return FFR_OK;
}

// Estimated render time above which the autotuner compiles a flame's
// per-flame kernels itself: FFR_JIT_AUTO_SECONDS, default 8 (negative: never)
double jit_auto_seconds()
{
    const char* v = std::getenv("FFR_JIT_AUTO_SECONDS");
    if (!v || !*v)
        return 8.0;
    char* end = nullptr;
    const double s = std::strtod(v, &end);
    if (end == v)
        return 8.0;
    return s < 0 ? 1e300 : s;
}

// Compile the context's per-flame plain and/or sorted kernels with NVRTC,
// the two in parallel (failures leave them uncompiled: the autotuner then
// keeps to the precompiled kernels)
void compile_jit(ffr_ctx* c, bool plain, bool sorted)
{
    const bool color = c->flame.color_dims > 0;
    if (plain && c->jit_source.empty())
        c->jit_source = jit_source(c->prog_host, c->opts.precision, color, false);
    if (sorted && c->jit_sorted_source.empty())
        c->jit_sorted_source = jit_source(c->prog_host, c->opts.precision, color, true);
    const int prec = c->opts.precision;
    auto one = [prec](const std::string* src) {
        std::string err;
        if (!src->empty())
            jit_compile_only(*src, prec, &err);
    };
    std::thread t;
    if (plain && sorted)
        t = std::thread(one, &c->jit_sorted_source);
    if (plain)
        one(&c->jit_source);
    else if (sorted)
        one(&c->jit_sorted_source);
    if (t.joinable())
        t.join();
}

// Launch plan: kernel, streams, trajectory length and grid.  The hot-cell
// table's shared memory is planned for FFR_KERNEL_HOT and when *hot is set
// on entry, for the plain kernel with fewer than 2^30 cells and fewer than
// 2^32 samples per CTA (the table's counts are u32); *hot on return: the
// launch uses the context's table (planned and present).
ffr_status plan(ffr_ctx* c, uint64_t samples, int kreq, uint64_t* streams, uint64_t* L,
                int* grid, int* kernel, bool* hot = nullptr)
{
    const bool want_hot = (kreq == FFR_KERNEL_HOT || (hot && *hot))
        && c->flame.cells < (1ull << 30);
    if (kreq == FFR_KERNEL_HOT)
        kreq = FFR_KERNEL_PLAIN;
    if (hot)
        *hot = false;
    int bps = 0, block = 0;
    size_t smem = 0;
    const int color = c->flame.color_dims > 0, spill = c->d_hi != nullptr;
    const unsigned int pb = prog_smem_for(c->prog_host.data());
    const int nxf = (int)c->flame.xforms.size();
    int k = kreq;
    // programs in the FP32 merged form have no per-flame kernel: their
    // precompiled instantiation already runs without type dispatch
    if ((k == FFR_KERNEL_JIT || k == FFR_KERNEL_JIT_SORTED) && merged_for(c->prog_host.data()))
        k = FFR_KERNEL_PLAIN;
    if (k == FFR_KERNEL_JIT_SORTED && (c->flame.dims > 3 || nxf > kSortedMaxXforms))
        return fail(c, FFR_ERR_ARG, "per-flame xform-sorted kernel cannot run this flame "
            "(more than 3 dims or 16 xforms)");
    if (k == FFR_KERNEL_JIT || k == FFR_KERNEL_JIT_SORTED)
    {
        ffr_status js = ensure_jit(c, k == FFR_KERNEL_JIT_SORTED);
        if (js != FFR_OK)
            return js;
    }
    const bool jit_k = k == FFR_KERNEL_JIT || k == FFR_KERNEL_JIT_SORTED;
    if (k != FFR_KERNEL_PLAIN && !jit_k && !c->L().occ_sorted)
    {
        // no xform-sorted instantiation for this dimension count
        if (k == FFR_KERNEL_SORTED)
            return fail(c, FFR_ERR_ARG, "xform-sorted kernel cannot run this flame "
                "(dims " + std::to_string(c->flame.dims) + ": plain kernel only)");
        k = FFR_KERNEL_PLAIN;
    }
    if (k != FFR_KERNEL_PLAIN && !jit_k)
    {
        CU(c, c->L().occ_sorted(color, spill, &bps, &block, pb, nxf, program_words(c), &smem));
        if (bps >= 1)
            k = FFR_KERNEL_SORTED;
        else if (k == FFR_KERNEL_SORTED)
            return fail(c, FFR_ERR_ARG, "xform-sorted kernel cannot run this flame (more than "
                "16 xforms or not enough shared memory)");
        else
            k = FFR_KERNEL_PLAIN;
    }
    const bool use_hot = want_hot && (k == FFR_KERNEL_PLAIN || k == FFR_KERNEL_JIT);
    if (k == FFR_KERNEL_PLAIN)
        CU(c, c->L().occ(color, merged_for(c->prog_host.data()),
                         rsl_words_for(c->prog_host.data()), use_hot ? 1 : 0, &bps,
                         &block, pb, nxf, &smem));
    else if (k == FFR_KERNEL_JIT)
    {
        block = kJitBlock;
        smem = chaos_smem_bytes<kJitBlock>(pb, nxf, rsl_words_for(c->prog_host.data()), use_hot);
        CU(c, jit_occupancy(c->jit, smem, &bps));
    }
    else if (k == FFR_KERNEL_JIT_SORTED)
    {
        block = kSortedBlock;
        smem = sorted_smem_bytes<kSortedBlock>(pb, nxf, program_words(c), c->flame.dims,
                                               c->opts.precision == FFR_FP64 ? 8 : 4);
        CU(c, jit_occupancy(c->jit_sorted, smem, &bps));
        if (bps < 1)
            return fail(c, FFR_ERR_ARG, "per-flame xform-sorted kernel cannot run this flame "
                "(not enough shared memory)");
    }
    *kernel = k;
    if (bps < 1)
        return fail(c, FFR_ERR_ARG, "render kernel does not fit on an SM "
            "(program " + std::to_string(c->prog_host.size()) + " bytes)");
    const uint64_t resident = (uint64_t)c->sm_count * bps * block;
    uint64_t S = c->opts.streams ? c->opts.streams : resident;
    // the autotuner's cap on resident CTAs per SM (streams stay as above)
    int cap = c->probe_cap ? c->probe_cap : (c->tuned ? c->tuned_cap : 0);
    cap = cap > 0 && cap < bps ? cap : bps;
    uint64_t len = c->opts.traj_len;
    if (len == 0)
        len = samples ? std::max<uint64_t>(1, (samples + S - 1) / S) : 1;
    const uint64_t ntraj = samples ? (samples + len - 1) / len : 0;
    const uint64_t active = std::min<uint64_t>(S, ntraj);
    uint64_t blocks = (active + block - 1) / block;
    blocks = std::min<uint64_t>(blocks, (uint64_t)c->sm_count * cap);
    if (blocks < 1)
        blocks = 1;
    // per-thread xform counters are u32: bound one thread's samples
    const uint64_t threads = blocks * block;
    const uint64_t streams_per_thread = (active + threads - 1) / threads;
    const uint64_t traj_per_stream = S ? (ntraj + S - 1) / S : 0;
    const long double per_thread = (long double)streams_per_thread * traj_per_stream * len;
    if (per_thread >= 4294967296.0L)
        return fail(c, FFR_ERR_ARG, "too many samples per GPU thread (raise streams)");
    if (use_hot && per_thread * block >= 4294967296.0L)
        return plan(c, samples, kreq, streams, L, grid, kernel, nullptr);
    *streams = S;
    *L = len;
    *grid = (int)blocks;
    c->plan_cap = cap;
    c->plan_block = block;
    c->plan_spt = streams_per_thread;
    if (hot)
        *hot = use_hot && c->hot_mult != 0;
    return FFR_OK;
}

// zero a DevStats block on the context stream (+inf/-inf extreme keys)
ffr_status reset_stats(ffr_ctx* c, DevStats* d)
{
    DevStats* head = reinterpret_cast<DevStats*>(new (std::nothrow) unsigned char[sizeof(DevStats)]);
    if (!head)
        return fail(c, FFR_ERR_OOM, "out of host memory");
    std::memset(head, 0, offsetof(DevStats, xf_dist));
    for (int i = 0; i < kMaxDims; ++i)
    {
        head->ext_lo[i] = order_key(INFINITY);
        head->ext_hi[i] = order_key(-INFINITY);
    }
    cudaError_t e = cudaMemcpyAsync(d, head, offsetof(DevStats, xf_dist),
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d->xf_dist, 0,
                            sizeof(unsigned long long) * c->flame.xforms.size(), c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);    // head is a host temporary
    delete[] reinterpret_cast<unsigned char*>(head);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "reset stats");
    return FFR_OK;
}

void fill_args(ffr_ctx* c, RenderArgs& a, uint64_t samples, uint64_t seed, uint64_t bad_limit,
               uint64_t S, uint64_t L, unsigned int* counts, unsigned int* hi, double* colors,
               DevStats* stats, int agg)
{
    std::memset(&a, 0, sizeof a);
    a.prog = c->d_prog;
    a.prog_bytes = prog_smem_for(c->prog_host.data());
    a.nxf = (int)c->flame.xforms.size();
    a.color_dims = c->flame.color_dims;
    a.spill = hi != nullptr;
    a.seed = seed;
    a.streams = S;
    a.samples = samples;
    a.traj_len = L;
    a.settle = c->opts.settle;
    a.bad_limit = bad_limit;
    a.counts = counts;
    a.hi = hi;
    a.colors = colors;
    a.stats = stats;
    a.cancel = c->d_cancel;
    a.rng_words = program_words(c);
    a.agg = agg;
    a.rsl_words = rsl_words_for(c->prog_host.data());
    a.merged = merged_for(c->prog_host.data());
    std::memcpy(a.isaac_init, c->isaac_init, sizeof a.isaac_init);
    set_geometry(a, c->prog_host.data(), c->opts.precision);
}

// one render launch of the planned kernel on the context stream
cudaError_t launch_render_kernel(ffr_ctx* c, int kernel, const RenderArgs& a, int grid)
{
    if (kernel == FFR_KERNEL_SORTED)
        return c->L().sorted(a, grid, c->stream);
    if (kernel == FFR_KERNEL_JIT)
        return jit_launch(c->jit, a, grid,
                          chaos_smem_bytes<kJitBlock>(a.prog_bytes, a.nxf, a.rsl_words,
                                                      a.hot_keys != nullptr),
                          c->stream);
    if (kernel == FFR_KERNEL_JIT_SORTED)
        return jit_launch(c->jit_sorted, a, grid,
                          sorted_smem_bytes<kSortedBlock>(a.prog_bytes, a.nxf, a.rng_words,
                                                          c->flame.dims,
                                                          c->opts.precision == FFR_FP64 ? 8 : 4),
                          c->stream);
    return c->L().render(a, grid, c->stream);
}

// the leading fields of DevStats (everything before xf_dist)
struct StatsHeadCopy
{
    unsigned long long s_iter, s_plot, bad_total, dropped, bad_claim;
    unsigned int stop, cancelled;
    unsigned long long ext_lo[kMaxDims], ext_hi[kMaxDims];
};
static_assert(sizeof(StatsHeadCopy) == offsetof(DevStats, xf_dist), "DevStats head layout");
static_assert(offsetof(StatsHeadCopy, ext_lo) == offsetof(DevStats, ext_lo), "DevStats head layout");

// per-xform counts (sorted order -> JSON ids) and bad-value records of the
// last render of c into *st (the reference's stats getters)
ffr_status read_stats(ffr_ctx* c, const StatsHeadCopy& hs, ffr_stats* st)
{
    std::memset(st, 0, sizeof *st);
    for (int i = 0; i < FFR_MAX_DIMS; ++i)
    {
        st->ext_lo[i] = INFINITY;
        st->ext_hi[i] = -INFINITY;
    }
    st->xform_ids = c->flame.xform_ids;
    st->settle = c->opts.settle;
    st->samples_iterated = hs.s_iter;
    st->samples_plotted = hs.s_plot;
    st->bad_values = hs.bad_total;
    st->dropped = hs.dropped;
    for (int i = 0; i < c->flame.dims; ++i)
    {
        st->ext_lo[i] = key_to_double(hs.ext_lo[i]);
        st->ext_hi[i] = key_to_double(hs.ext_hi[i]);
    }
    const size_t nxf = c->flame.xforms.size();
    std::vector<unsigned long long> dist(nxf);
    CU(c, cudaMemcpy(dist.data(), c->d_stats->xf_dist, sizeof(unsigned long long) * nxf,
                     cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nxf; ++k)
    {
        const uint64_t id = c->flame.xforms[k].id;
        if (id < FFR_MAX_XFORM_IDS)
            st->xf_dist[id] += dist[k];
    }
    const unsigned long long nrec = std::min<unsigned long long>(hs.bad_claim, kMaxBadRecords);
    if (nrec)
    {
        CU(c, cudaMemcpy(st->bad_xf, c->d_stats->bad_xf, sizeof(unsigned long long) * nrec,
                         cudaMemcpyDeviceToHost));
        std::vector<double> pts(kMaxDims * nrec);
        CU(c, cudaMemcpy(pts.data(), c->d_stats->bad_pts, sizeof(double) * kMaxDims * nrec,
                         cudaMemcpyDeviceToHost));
        for (unsigned long long k = 0; k < nrec; ++k)
            for (int i = 0; i < c->flame.dims; ++i)
                st->bad_pts[k][i] = pts[k * kMaxDims + i];
    }
    st->bad_recorded = nrec;
    return FFR_OK;
}

// Renders this large are autotuned; smaller ones use the static choice.
constexpr uint64_t kTuneMinSamples = 1ull << 25;

// Process-wide memory of tuning decisions, keyed by everything the choice
// depends on: the program bytes (flame + precision), settle, streams and
// trajectory options, spill mode and device.
struct TuneKey
{
    std::string prog;
    uint64_t settle, streams, traj_len;
    int spill, device;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(prog, settle, streams, traj_len, spill, device)
            < std::tie(o.prog, o.settle, o.streams, o.traj_len, o.spill, o.device);
    }
};
struct TuneChoice
{
    int kernel = FFR_KERNEL_PLAIN;
    int agg = 0;
    int cap = 0;                            // resident CTAs per SM (0: all that fit)
    unsigned int hot_mult = 0;              // 0: no hot-cell table
    std::vector<unsigned int> hot_keys;     // kHotSlots keys when hot_mult != 0
    // the per-flame kernels were candidates (or do not apply); else the
    // precompiled candidates' best probe time per sample, by which a longer
    // render reconsiders them
    bool jit_considered = true;
    double ms_per_sample = 0.0;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune_cache;

TuneKey tune_key(const ffr_ctx* c)
{
    return TuneKey{std::string(c->prog_host.begin(), c->prog_host.end()), c->opts.settle,
                   c->opts.streams, c->opts.traj_len, c->d_hi != nullptr, c->device};
}

// Hot-cell table from a probe's counts (u32, cells < 2^30): candidates
// holding at least 1/4096 of the probe's samples each, placed by
// hot_place; *mult = 0 when the flame has no such cells.  out: 1 +
// kHotCollectCap device words.
ffr_status hot_table(ffr_ctx* c, const unsigned int* counts, unsigned long long* out,
                     unsigned int* mult, std::vector<unsigned int>& keys)
{
    *mult = 0;
    const uint64_t cells = c->flame.cells;
    if (cells >= (1ull << 30))
        return FFR_OK;
    unsigned long long init[3] = {0ull, ~0ull, 0ull}, red[3];
    CU(c, cudaMemcpyAsync(out, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
    CU(c, launch_hist_reduce(counts, nullptr, cells, out, c->stream));
    ++c->aux_launches;
    CU(c, cudaMemcpyAsync(red, out, sizeof red, cudaMemcpyDeviceToHost, c->stream));
    CU(c, cudaStreamSynchronize(c->stream));
    const uint64_t sum = red[0];
    if (sum < 4096)
        return FFR_OK;
    std::vector<unsigned long long> found;
    bool got = false;
    CU(c, collect_hot_candidates(counts, (unsigned int)cells, sum >> 12, red[2], out, c->stream,
                                 found, &got, &c->aux_launches));
    if (!got || !hot_place(found, sum, mult, keys))
        *mult = 0;
    return FFR_OK;
}

// install a hot-cell table (mult 0: none) on the context
ffr_status set_hot(ffr_ctx* c, unsigned int mult, const std::vector<unsigned int>& keys)
{
    c->hot_mult = 0;
    if (mult == 0)
        return FFR_OK;
    if (!c->d_hot)
        CU(c, ctx_alloc(c, &c->d_hot, kHotSlots * sizeof(unsigned int)));
    CU(c, cudaMemcpyAsync(c->d_hot, keys.data(), kHotSlots * sizeof(unsigned int),
                          cudaMemcpyHostToDevice, c->stream));
    CU(c, cudaStreamSynchronize(c->stream));
    c->hot_mult = mult;
    c->hot_cells = (int)std::count_if(keys.begin(), keys.end(),
                                      [](unsigned int k) { return k != kHotEmpty; });
    return FFR_OK;
}

// The context's hot-cell table from one probe render of the plain kernel
// (samples, at most 2^24 and 2^22 in FP64) into scratch buffers, searched
// once per context (FFR_KERNEL_HOT renders, batch members).
ffr_status ensure_hot_table(ffr_ctx* c, uint64_t samples)
{
    if (c->hot_searched)
        return FFR_OK;
    c->hot_searched = true;
    if (c->flame.cells >= (1ull << 30))
        return FFR_OK;
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t off_st = up(c->flame.cells * 4);
    const size_t off_col = off_st + up(sizeof(DevStats));
    const size_t r = (size_t)c->flame.color_dims;
    const size_t off_hs = off_col + up(c->flame.cells * r * 8);
    const size_t need = off_hs + (1 + kHotCollectCap) * sizeof(unsigned long long);
    unsigned char* buf = nullptr;
    CU(c, cudaMalloc(&buf, need));
    unsigned int* pc = reinterpret_cast<unsigned int*>(buf);
    DevStats* pst = reinterpret_cast<DevStats*>(buf + off_st);
    double* pcol = r ? reinterpret_cast<double*>(buf + off_col) : nullptr;
    unsigned long long* phs = reinterpret_cast<unsigned long long*>(buf + off_hs);
    const uint64_t P = std::max<uint64_t>(1, std::min<uint64_t>(
        samples, c->opts.precision == FFR_FP64 ? (1u << 22) : (1u << 24)));
    uint64_t S = 0, L = 0;
    int grid = 0, kk = 0;
    ffr_status st = FFR_OK;
    {
        cudaError_t e = cudaMemsetAsync(buf, 0, c->flame.cells * 4, c->stream);
        if (e != cudaSuccess)
            st = cuda_fail(c, e, "hot-cell probe");
    }
    if (st == FFR_OK)
        st = plan(c, P, FFR_KERNEL_PLAIN, &S, &L, &grid, &kk);
    if (st == FFR_OK)
        st = reset_stats(c, pst);
    if (st == FFR_OK)
    {
        RenderArgs a;
        fill_args(c, a, P, 0x5eedull, ~0ull, S, L, pc, nullptr, pcol, pst, 1);
        cudaError_t e = c->L().render(a, grid, c->stream);
        if (e != cudaSuccess)
            st = cuda_fail(c, e, "hot-cell probe");
        else
            ++c->aux_launches;
    }
    unsigned int mult = 0;
    std::vector<unsigned int> keys;
    if (st == FFR_OK)
        st = hot_table(c, pc, phs, &mult, keys);
    if (st == FFR_OK)
        st = set_hot(c, mult, keys);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(buf);
    if (st == FFR_OK && e != cudaSuccess)
        st = cuda_fail(c, e, "hot-cell probe");
    return st;
}

// Autotuner: times a probe render of each (kernel, warp aggregation)
// candidate into scratch buffers of the same geometry, then, if the probe
// counts show hot cells, the plain kernel with a hot-cell table, and keeps
// the fastest for this context.  The probe never touches the context's
// buffer, so results do not depend on whether tuning ran.  *hot: use the
// context's hot-cell table.
ffr_status autotune(ffr_ctx* c, uint64_t samples, int* kernel, int* agg, bool* hot)
{
    const bool spill = c->d_hi != nullptr;
    *hot = false;
    // a decision made without the per-flame kernels stands unless this
    // render is long enough for them to be compiled
    auto stands = [&](bool jit_considered, double ms_per_sample) {
        return jit_considered
            || ms_per_sample * 1e-3 * (double)samples <= jit_auto_seconds();
    };
    if (c->tuned && c->tuned_spill == spill && stands(c->tuned_jit, c->tuned_ms_per_sample))
    {
        *kernel = c->tuned_kernel;
        *agg = c->tuned_agg;
        *hot = c->tuned_hot;
        return FFR_OK;
    }
    {
        TuneChoice ch;
        bool have = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(tune_key(c));
            if (it != g_tune_cache.end()
                    && stands(it->second.jit_considered, it->second.ms_per_sample))
            {
                ch = it->second;
                have = true;
            }
        }
        if (have)
        {
            ffr_status s = set_hot(c, ch.hot_mult, ch.hot_keys);
            if (s != FFR_OK)
                return s;
            c->tuned = true;
            c->tuned_spill = spill;
            c->tuned_kernel = *kernel = ch.kernel;
            c->tuned_agg = *agg = ch.agg;
            c->tuned_cap = ch.cap;
            c->tuned_jit = ch.jit_considered;
            c->tuned_ms_per_sample = ch.ms_per_sample;
            c->tuned_hot = *hot = ch.hot_mult != 0;
            c->hot_searched = true;
            return FFR_OK;
        }
    }
    // static choice: FP32 plain, FP64 sorted where it fits (FP64 pays more
    // for divergent lanes)
    *kernel = c->opts.precision == FFR_FP64 ? FFR_KERNEL_AUTO : FFR_KERNEL_PLAIN;
    *agg = kDefaultAgg;
    if (samples < kTuneMinSamples)
        return FFR_OK;
    const size_t cells = c->flame.cells;
    const size_t r = (size_t)c->flame.color_dims;
    // scratch: counts | high words | colours | statistics | hot-cell
    // search, each 256-byte aligned (an odd cell count would otherwise
    // leave the u64 fields of the statistics on a 4-byte boundary)
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t off_hi = up(cells * 4);
    const size_t off_col = off_hi + (spill ? up(cells * 4) : 0);
    const size_t off_st = off_col + up(cells * r * 8);
    const size_t off_hs = off_st + up(sizeof(DevStats));
    const size_t need = off_hs + (1 + kHotCollectCap) * sizeof(unsigned long long);
    size_t fr = 0, tot = 0;
    CU(c, cudaMemGetInfo(&fr, &tot));
    if (need > fr / 4)
        return FFR_OK;
    unsigned char* buf = nullptr;
    CU(c, cudaMalloc(&buf, need));
    unsigned int* pc = reinterpret_cast<unsigned int*>(buf);
    unsigned int* ph = spill ? reinterpret_cast<unsigned int*>(buf + off_hi) : nullptr;
    double* pcol = r ? reinterpret_cast<double*>(buf + off_col) : nullptr;
    DevStats* pst = reinterpret_cast<DevStats*>(buf + off_st);
    unsigned long long* phs = reinterpret_cast<unsigned long long*>(buf + off_hs);
    uint64_t P = std::min<uint64_t>(samples, c->opts.precision == FFR_FP64 ? (1u << 22)
                                                                           : (1u << 24));
    float best = 1e30f;
    int best_k = *kernel, best_a = 0;
    bool best_h = false;
    ffr_status st = FFR_OK;
    {
        // the probes' counts locate the hot cells: start them from zero
        cudaError_t e = cudaMemsetAsync(pc, 0, cells * 4, c->stream);
        if (e != cudaSuccess)
            st = cuda_fail(c, e, "autotune scratch");
    }
    // The probes run as many streams at once as the render will (with
    // proportionally shorter trajectories), whatever streams and trajectory
    // length the context fixes: contention on hot cells, which decides
    // between the candidates, grows with the threads binning at once, and a
    // probe of P samples in the context's own long trajectories could run on
    // a few thousand threads.  The probes render into scratch buffers, so
    // their streams never reach the context's buffer.
    uint64_t probe_streams = 0, probe_len = 0;
    {
        uint64_t S0 = 0, L0 = 0;
        int g0 = 0, k0 = 0;
        if (plan(c, samples, FFR_KERNEL_PLAIN, &S0, &L0, &g0, &k0) == FFR_OK && L0 > 0)
        {
            const uint64_t ntraj = (samples + L0 - 1) / L0;
            probe_streams = std::max<uint64_t>(1, std::min<uint64_t>(S0, ntraj));
            // a render on few streams: probes of about 2048 samples per
            // stream (at least 2^20), not 2^24 samples on a few threads
            P = std::min<uint64_t>(P, std::max<uint64_t>(1u << 20, probe_streams * 2048));
            probe_len = std::max<uint64_t>(1, P / probe_streams);
        }
    }
    // one candidate: time two probe launches, keep the faster candidate
    auto probe = [&](int k, int g, bool h) -> ffr_status {
        uint64_t S = 0, L = 0;
        int grid = 0, kk = 0;
        bool hh = h;
        ffr_status ps;
        {
            const uint64_t saved_s = c->opts.streams, saved_l = c->opts.traj_len;
            if (probe_streams)
            {
                c->opts.streams = probe_streams;
                c->opts.traj_len = probe_len;
            }
            ps = plan(c, P, k, &S, &L, &grid, &kk, &hh);
            c->opts.streams = saved_s;
            c->opts.traj_len = saved_l;
        }
        if (ps != FFR_OK || hh != h)
            return FFR_OK;      // candidate does not apply to this flame
        RenderArgs a;
        fill_args(c, a, P, 0x5eedull + (uint64_t)k * 2 + g, ~0ull, S, L, pc, ph, pcol, pst, g);
        if (h)
        {
            a.hot_keys = c->d_hot;
            a.hot_mult = c->hot_mult;
        }
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep)
        {
            ffr_status st = reset_stats(c, pst);
            if (st != FFR_OK)
                return st;
            CU(c, cudaEventRecord(c->ev0, c->stream));
            CU(c, launch_render_kernel(c, kk, a, grid));
            ++c->aux_launches;
            CU(c, cudaEventRecord(c->ev1, c->stream));
            CU(c, cudaEventSynchronize(c->ev1));
            CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        }
        if (ms < best)
        {
            best = ms;
            best_k = kk;
            best_a = g;
            best_h = h;
        }
        return FFR_OK;
    };
    // the per-flame kernels are candidates when compiled already (an
    // earlier FFR_KERNEL_JIT* render or ffr_jit_prepare, in this process or
    // in the FFR_JIT_CACHE directory), or when this render would run longer
    // than jit_auto_seconds() at the best precompiled candidate's probe rate:
    // the compile (about a second per kernel, the two in parallel) is then
    // small against the render
    const bool merged = merged_for(c->prog_host.data()) != 0;
    const bool sortable = !merged && c->flame.dims <= 3
        && c->flame.xforms.size() <= (size_t)kSortedMaxXforms;
    bool jit_ready = !merged && ensure_jit(c, false, true) == FFR_OK;
    bool jit_sorted_ready = sortable && ensure_jit(c, true, true) == FFR_OK;
    for (int k : {FFR_KERNEL_PLAIN, FFR_KERNEL_SORTED})
        for (int g : {0, 1})
            if (st == FFR_OK)
                st = probe(k, g, false);
    const double ms_per_sample = best < 1e30f ? (double)best / (double)P : 0.0;
    bool jit_considered = merged || (jit_ready && (jit_sorted_ready || !sortable));
    if (st == FFR_OK && !jit_considered
            && ms_per_sample * 1e-3 * (double)samples > jit_auto_seconds())
    {
        compile_jit(c, !jit_ready, sortable && !jit_sorted_ready);
        jit_ready = ensure_jit(c, false, true) == FFR_OK;
        jit_sorted_ready = sortable && ensure_jit(c, true, true) == FFR_OK;
        jit_considered = true;      // also when NVRTC failed: not retried
    }
    auto ready = [&](int k) {
        return k == FFR_KERNEL_JIT ? jit_ready : k == FFR_KERNEL_JIT_SORTED ? jit_sorted_ready
                                                                           : true;
    };
    for (int k : {FFR_KERNEL_JIT, FFR_KERNEL_JIT_SORTED})
        for (int g : {0, 1})
            if (st == FFR_OK && ready(k))
                st = probe(k, g, false);
    // the probes' counts (u32: far below 2^32 per cell) locate hot cells
    unsigned int mult = 0;
    std::vector<unsigned int> keys;
    if (st == FFR_OK)
        st = hot_table(c, pc, phs, &mult, keys);
    if (st == FFR_OK)
        st = set_hot(c, mult, keys);
    if (st == FFR_OK && mult)
        for (int k : {FFR_KERNEL_PLAIN, FFR_KERNEL_JIT})
            for (int g : {0, 1})
                if (st == FFR_OK && ready(k))
                    st = probe(k, g, true);
    // launch shape for the best candidate: fewer resident CTAs per SM, each
    // thread then running more streams one after another (the streams, and
    // so the buffer, stay the same); kept only when 3% faster
    int best_cap = 0;
    if (st == FFR_OK)
    {
        uint64_t S0 = 0, L0 = 0;
        int g0 = 0, k0 = 0;
        bool h0 = best_h;
        c->probe_cap = 0;
        if (plan(c, P, best_k, &S0, &L0, &g0, &k0, &h0) == FFR_OK)
        {
            const int full = c->plan_cap;
            for (int cap : {full - 1, (full + 1) / 2})
            {
                if (cap < 1 || cap >= full || st != FFR_OK)
                    continue;
                c->probe_cap = cap;
                const float prev = best;
                st = probe(best_k, best_a, best_h);
                if (best < 0.97f * prev)
                    best_cap = cap;
                else
                    best = prev;
            }
        }
        c->probe_cap = 0;
    }
    cudaFree(buf);
    if (st != FFR_OK)
        return st;
    if (!best_h)
    {
        c->hot_mult = 0;
        mult = 0;
        keys.clear();
    }
    c->tuned = true;
    c->tuned_spill = spill;
    c->tuned_kernel = *kernel = best_k;
    c->tuned_agg = *agg = best_a;
    c->tuned_hot = *hot = best_h;
    c->tuned_cap = best_cap;
    c->tuned_jit = jit_considered;
    c->tuned_ms_per_sample = ms_per_sample;
    // the table (or its absence) is the autotuner's decision: batches reuse it
    c->hot_searched = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (g_tune_cache.size() > 4096)
        g_tune_cache.clear();
    TuneChoice ch;
    ch.kernel = best_k;
    ch.agg = best_a;
    ch.cap = best_cap;
    ch.hot_mult = mult;
    ch.hot_keys = std::move(keys);
    ch.jit_considered = jit_considered;
    ch.ms_per_sample = ms_per_sample;
    g_tune_cache[tune_key(c)] = std::move(ch);
    return FFR_OK;
}

} // namespace

extern "C" {

void ffr_default_opts(ffr_opts* o)
{
    if (!o)
        return;
    std::memset(o, 0, sizeof *o);
    o->abi_version = FFR_ABI_VERSION;
    o->device = 0;
    o->precision = FFR_FP64;
    o->settle = 53;
    o->streams = 0;
    o->traj_len = 0;
    o->timeout_ms = 0;
    o->kernel = FFR_KERNEL_AUTO;
}

ffr_status ffr_create(const char* json, size_t len, const ffr_opts* opts, ffr_ctx** out)
{
    if (!out)
        return fail(nullptr, FFR_ERR_ARG, "ffr_create: out is NULL");
    *out = nullptr;
    if (!json)
        return fail(nullptr, FFR_ERR_ARG, "ffr_create: json is NULL");
    ffr_opts o;
    if (opts)
        o = *opts;
    else
        ffr_default_opts(&o);
    if (o.abi_version != FFR_ABI_VERSION)
        return fail(nullptr, FFR_ERR_ARG, "ffr_create: ABI version mismatch");
    if (o.precision != FFR_FP64 && o.precision != FFR_FP32)
        return fail(nullptr, FFR_ERR_ARG, "ffr_create: unknown precision");
    if (o.kernel < FFR_KERNEL_AUTO || o.kernel > FFR_KERNEL_JIT_SORTED)
        return fail(nullptr, FFR_ERR_ARG, "ffr_create: unknown kernel");
    ffr_ctx* c = new (std::nothrow) ffr_ctx;
    if (!c)
        return fail(nullptr, FFR_ERR_OOM, "ffr_create: out of host memory");
    c->opts = o;
    try
    {
        c->flame = parse_flame(std::string(json, len));
        c->prog_host = o.precision == FFR_FP64 ? build_program<double>(c->flame)
                                               : build_program<float>(c->flame);
    }
    catch (const FlameError& e)
    {
        delete c;
        return fail(nullptr, FFR_ERR_PARSE, e.what());
    }
    catch (const std::exception& e)
    {
        delete c;
        return fail(nullptr, FFR_ERR_PARSE, e.what());
    }
    if (c->flame.xforms.size() > (size_t)kMaxXformIds)
    {
        delete c;
        return fail(nullptr, FFR_ERR_ARG, "too many xforms");
    }
    c->device = o.device;
    auto cfail = [&](cudaError_t e, const char* what) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(e);
        destroy(c);
        return fail(nullptr, FFR_ERR_CUDA, m);
    };
    cudaError_t e;
    if ((e = cudaSetDevice(c->device)) != cudaSuccess)
        return cfail(e, "cudaSetDevice");
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cfail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess
            || (e = cudaEventCreate(&c->ev1)) != cudaSuccess
            || (e = cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming)) != cudaSuccess)
        return cfail(e, "cudaEventCreate");
    if ((e = take_flag(c->device, &c->h_cancel, &c->d_cancel)) != cudaSuccess)
        return cfail(e, "cudaHostAlloc(cancel flag)");
    // admission by free device memory
    const size_t need = c->flame.cells * sizeof(unsigned int)
        + c->flame.cells * (size_t)c->flame.color_dims * sizeof(double)
        + sizeof(DevStats) + c->prog_host.size();
    size_t fr = 0;
    if ((e = ctx_free_bytes(c->device, &fr)) != cudaSuccess)
        return cfail(e, "cudaMemGetInfo");
    if (need + (256u << 20) > fr)
    {
        destroy(c);
        return fail(nullptr, FFR_ERR_OOM, "buffer needs " + std::to_string(need)
            + " bytes of device memory, " + std::to_string(fr) + " free");
    }
    if ((e = ctx_alloc(c, &c->d_prog, c->prog_host.size())) != cudaSuccess)
        return cfail(e, "cudaMalloc(program)");
    if ((e = ctx_alloc(c, &c->d_counts, c->flame.cells * sizeof(unsigned int))) != cudaSuccess)
        return cfail(e, "cudaMalloc(counts)");
    if (c->flame.color_dims
            && (e = ctx_alloc(c, &c->d_colors,
                              c->flame.cells * c->flame.color_dims * sizeof(double))) != cudaSuccess)
        return cfail(e, "cudaMalloc(colors)");
    if ((e = ctx_alloc(c, &c->d_stats, sizeof(DevStats))) != cudaSuccess)
        return cfail(e, "cudaMalloc(stats)");
    if ((e = cudaMemcpyAsync(c->d_prog, c->prog_host.data(), c->prog_host.size(),
                             cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
        return cfail(e, "cudaMemcpy(program)");
    if ((e = cudaMemsetAsync(c->d_counts, 0, c->flame.cells * sizeof(unsigned int), c->stream)) != cudaSuccess)
        return cfail(e, "cudaMemset(counts)");
    if (c->d_colors
            && (e = cudaMemsetAsync(c->d_colors, 0, c->flame.cells * c->flame.color_dims * sizeof(double), c->stream)) != cudaSuccess)
        return cfail(e, "cudaMemset(colors)");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return cfail(e, "cudaStreamSynchronize");
    isaac_init_table(c->isaac_init);
    *out = c;
    return FFR_OK;
}

void ffr_destroy(ffr_ctx* c)
{
    destroy(c);
}

ffr_status ffr_jit_prepare(const char* json, size_t len, const ffr_opts* opts)
{
    if (!json)
        return fail(nullptr, FFR_ERR_ARG, "ffr_jit_prepare: json is NULL");
    ffr_opts o;
    if (opts)
        o = *opts;
    else
        ffr_default_opts(&o);
    if (o.abi_version != FFR_ABI_VERSION)
        return fail(nullptr, FFR_ERR_ARG, "ffr_jit_prepare: ABI version mismatch");
    if (o.precision != FFR_FP64 && o.precision != FFR_FP32)
        return fail(nullptr, FFR_ERR_ARG, "ffr_jit_prepare: unknown precision");
    // the per-flame kernels asked for: plain (FFR_KERNEL_JIT), xform-sorted
    // (FFR_KERNEL_JIT_SORTED), or both (any other kernel value)
    std::vector<std::string> srcs;
    try
    {
        const HostFlame f = parse_flame(std::string(json, len));
        const std::vector<uint8_t> prog = o.precision == FFR_FP64 ? build_program<double>(f)
                                                                  : build_program<float>(f);
        for (bool sorted : {false, true})
            if (o.kernel != (sorted ? FFR_KERNEL_JIT : FFR_KERNEL_JIT_SORTED))
                srcs.push_back(jit_source(prog, o.precision, f.color_dims > 0, sorted));
    }
    catch (const std::exception& e)
    {
        return fail(nullptr, FFR_ERR_PARSE, e.what());
    }
    // the kernels compile in parallel (an empty source: FP32 merged form, or
    // no sorted kernel for the flame)
    std::vector<std::string> errs(srcs.size());
    std::vector<char> ok(srcs.size(), 1);
    std::vector<std::thread> threads;
    for (size_t i = 0; i < srcs.size(); ++i)
        if (!srcs[i].empty())
            threads.emplace_back([&, i] {
                ok[i] = jit_compile_only(srcs[i], o.precision, &errs[i]) ? 1 : 0;
            });
    for (std::thread& t : threads)
        t.join();
    for (size_t i = 0; i < srcs.size(); ++i)
        if (!ok[i])
            return fail(nullptr, FFR_ERR_CUDA, errs[i]);
    return FFR_OK;
}

const char* ffr_last_error(const ffr_ctx* c)
{
    return c ? c->err.c_str() : g_create_error.c_str();
}

ffr_status ffr_info(const ffr_ctx* c, uint32_t* dims, uint64_t* cells,
                    uint32_t* color_dims, size_t* buffer_bytes)
{
    if (!c)
        return FFR_ERR_ARG;
    if (dims) *dims = (uint32_t)c->flame.dims;
    if (cells) *cells = c->flame.cells;
    if (color_dims) *color_dims = (uint32_t)c->flame.color_dims;
    if (buffer_bytes) *buffer_bytes = c->buffer_bytes();
    return FFR_OK;
}

ffr_status ffr_size(const ffr_ctx* c, uint64_t* size)
{
    if (!c || !size)
        return FFR_ERR_ARG;
    for (int i = 0; i < c->flame.dims; ++i)
        size[i] = c->flame.size[i];
    return FFR_OK;
}

const char* ffr_flame_json(const ffr_ctx* c)
{
    return c ? c->flame.echo.c_str() : "";
}

static ffr_status import_file(ffr_ctx* c, const void* cells, size_t bytes, int overwrite)
{
    if (!c)
        return FFR_ERR_ARG;
    if (!cells && bytes)
        return fail(c, FFR_ERR_ARG, "buffer pointer is NULL");
    const size_t need = c->buffer_bytes();
    if (bytes < need)
        return fail(c, FFR_ERR_IO, "error reading file: buffer has " + std::to_string(bytes)
            + " bytes, flame needs " + std::to_string(need));
    CU(c, cudaSetDevice(c->device));
    ffr_status s = ensure_scratch(c, need + 64);
    if (s != FFR_OK)
        return s;
    unsigned long long* dmax = c->d_scratch + need / 8;
    CU(c, cudaMemcpyAsync(c->d_scratch, cells, need, cudaMemcpyHostToDevice, c->stream));
    // counts reaching 2^32 need the high-word plane
    CU(c, cudaMemsetAsync(dmax, 0, 8, c->stream));
    CU(c, launch_file_max(c->d_scratch, c->flame.cells, c->flame.color_dims, dmax, c->stream));
    unsigned long long file_max = 0;
    CU(c, cudaMemcpyAsync(&file_max, dmax, 8, cudaMemcpyDeviceToHost, c->stream));
    CU(c, cudaStreamSynchronize(c->stream));
    const long double bound = overwrite ? (long double)file_max
                                        : (long double)c->count_bound + file_max;
    if (bound >= 4294967295.0L)
    {
        s = ensure_hi(c);
        if (s != FFR_OK)
            return s;
    }
    CU(c, launch_accumulate(c->d_scratch, c->flame.cells, c->flame.color_dims, c->d_counts,
                            c->d_hi, c->d_colors, overwrite, c->stream));
    s = wait_stream(c);
    if (s != FFR_OK)
        return s;
    // tighten the bound from the actual maximum
    uint64_t sum = 0, mn = 0, mx = 0;
    s = ffr_histogram(c, &sum, &mn, &mx);
    if (s != FFR_OK)
        return s;
    c->count_bound = mx;
    return FFR_OK;
}

ffr_status ffr_add_buffer(ffr_ctx* c, const void* cells, size_t bytes)
{
    return import_file(c, cells, bytes, 0);
}

ffr_status ffr_load_buffer(ffr_ctx* c, const void* cells, size_t bytes)
{
    return import_file(c, cells, bytes, 1);
}

ffr_status ffr_plan(ffr_ctx* c, uint64_t samples, uint64_t* streams, uint64_t* traj_len)
{
    if (!c)
        return FFR_ERR_ARG;
    CU(c, cudaSetDevice(c->device));
    uint64_t S = 0, L = 0;
    int grid = 0, kernel = 0;
    ffr_status s = plan(c, samples, c->opts.kernel, &S, &L, &grid, &kernel);
    if (s != FFR_OK)
        return s;
    if (streams) *streams = S;
    if (traj_len) *traj_len = L;
    return FFR_OK;
}

namespace {

// Before a render that could carry some count past 2^32 by the running bound
// (every sample so far plus this render's), replace the bound by the exact
// largest count, so that high words (and the slower returning atomics of
// spill mode) are used only when a cell really can overflow.
ffr_status tighten_bound(ffr_ctx* c, uint64_t samples)
{
    if (c->d_hi || c->count_bound + samples < 0xFFFFFFFFULL)
        return FFR_OK;
    uint64_t sum = 0, mn = 0, mx = 0;
    ffr_status s = ffr_histogram(c, &sum, &mn, &mx);
    if (s != FFR_OK)
        return s;
    c->count_bound = mx;
    return FFR_OK;
}

} // namespace

ffr_status ffr_render(ffr_ctx* c, uint64_t samples, uint64_t seed, uint64_t bad_limit,
                      ffr_stats* st)
{
    if (!c)
        return FFR_ERR_ARG;
    if (st)
    {
        std::memset(st, 0, sizeof *st);
        for (int i = 0; i < FFR_MAX_DIMS; ++i)
        {
            st->ext_lo[i] = INFINITY;
            st->ext_hi[i] = -INFINITY;
        }
        st->xform_ids = c->flame.xform_ids;
        st->settle = c->opts.settle;
    }
    c->aux_launches = 0;
    if (samples == 0)
        return FFR_OK;      // render(0) returns true (buffer_renderer.hpp:276-277)
    CU(c, cudaSetDevice(c->device));
    {
        ffr_status s = tighten_bound(c, samples);
        if (s != FFR_OK)
            return s;
    }
    if (c->count_bound + samples >= 0xFFFFFFFFULL)
    {
        ffr_status s = ensure_hi(c);
        if (s != FFR_OK)
            return s;
    }
    int kreq = c->opts.kernel, agg = kDefaultAgg;
    bool hot = false;
    if (kreq == FFR_KERNEL_AUTO)
    {
        ffr_status ts = autotune(c, samples, &kreq, &agg, &hot);
        if (ts != FFR_OK)
            return ts;
    }
    else if (kreq == FFR_KERNEL_HOT)
    {
        ffr_status ts = ensure_hot_table(c, samples);
        if (ts != FFR_OK)
            return ts;
        agg = agg_after_search(true);
    }
    uint64_t S = 0, L = 0;
    int grid = 0, kernel = 0;
    ffr_status s = plan(c, samples, kreq, &S, &L, &grid, &kernel, &hot);
    if (s != FFR_OK)
        return s;
    if ((s = reset_stats(c, c->d_stats)) != FFR_OK)
        return s;
    RenderArgs a;
    fill_args(c, a, samples, seed, bad_limit, S, L, c->d_counts, c->d_hi, c->d_colors,
              c->d_stats, agg);
    if (hot)
    {
        a.hot_keys = c->d_hot;
        a.hot_mult = c->hot_mult;
    }
    *c->h_cancel = 0u;
    CU(c, cudaEventRecord(c->ev0, c->stream));
    CU(c, launch_render_kernel(c, kernel, a, grid));
    CU(c, cudaEventRecord(c->ev1, c->stream));
    s = wait_stream(c);
    c->count_bound += samples;
    if (s != FFR_OK)
        return s;
    StatsHeadCopy hs;
    CU(c, cudaMemcpy(&hs, c->d_stats, sizeof hs, cudaMemcpyDeviceToHost));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (st)
    {
        if ((s = read_stats(c, hs, st)) != FFR_OK)
            return s;
        st->streams = S;
        st->traj_len = L;
        st->kernel_ms = ms;
        st->kernel = kernel;
        st->agg = agg;
        st->hot_cells = hot ? c->hot_cells : 0;
        st->aux_launches = (int32_t)c->aux_launches;
        st->ctas = (uint64_t)grid;
        st->streams_per_thread = c->plan_spt;
        st->ctas_per_sm = c->plan_cap;
        st->threads_per_cta = c->plan_block;
    }
    if (hs.cancelled)
        return fail(c, FFR_ERR_TIMEOUT, "render cancelled");
    if (hs.stop)
        return fail(c, FFR_BAD_VALUES, "render failure (flame may not be sufficiently contractive)");
    return FFR_OK;
}

ffr_status ffr_read_buffer(ffr_ctx* c, void* cells, size_t bytes)
{
    if (!c)
        return FFR_ERR_ARG;
    const size_t need = c->buffer_bytes();
    if (!cells || bytes < need)
        return fail(c, FFR_ERR_IO, "error writing output: destination too small");
    CU(c, cudaSetDevice(c->device));
    ffr_status s = ensure_scratch(c, need + 64);
    if (s != FFR_OK)
        return s;
    CU(c, launch_export(c->d_scratch, c->flame.cells, c->flame.color_dims, c->d_counts,
                        c->d_hi, c->d_colors, c->stream));
    CU(c, cudaMemcpyAsync(cells, c->d_scratch, need, cudaMemcpyDeviceToHost, c->stream));
    return wait_stream(c);
}

ffr_status ffr_histogram(ffr_ctx* c, uint64_t* sum, uint64_t* mn, uint64_t* mx)
{
    if (!c)
        return FFR_ERR_ARG;
    CU(c, cudaSetDevice(c->device));
    ffr_status s = ensure_scratch(c, 64);
    if (s != FFR_OK)
        return s;
    unsigned long long init[3] = {0ull, ~0ull, 0ull}, out[3];
    unsigned long long* d = c->d_scratch + (c->scratch_bytes / 8 - 4);
    CU(c, cudaMemcpyAsync(d, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
    CU(c, launch_hist_reduce(c->d_counts, c->d_hi, c->flame.cells, d, c->stream));
    ++c->aux_launches;
    CU(c, cudaMemcpyAsync(out, d, sizeof out, cudaMemcpyDeviceToHost, c->stream));
    s = wait_stream(c);
    if (s != FFR_OK)
        return s;
    if (sum) *sum = out[0];
    if (mn) *mn = out[1];
    if (mx) *mx = out[2];
    return FFR_OK;
}

ffr_status ffr_render_image(ffr_ctx* c, int mode, double gamma, uint32_t bits, void* pixels,
                            size_t bytes, ffr_image_info* info)
{
    if (!c)
        return FFR_ERR_ARG;
    if (c->flame.dims != 2)
        return fail(c, FFR_ERR_ARG, "only 2D flames supported");
    if (mode < FFR_IMAGE_MONO || mode > FFR_IMAGE_RGB)
        return fail(c, FFR_ERR_ARG, "no coloring flag");
    // ffr_img.cpp:89-95
    if (!(gamma >= 1e-20))
        return fail(c, FFR_ERR_ARG, "gamma too small");
    if (bits != 8 && bits != 16)
        return fail(c, FFR_ERR_ARG, "bits per channel must be 8 or 16");
    if (mode == FFR_IMAGE_MONO)
        bits = 8;       // the reference writes monochrome as an 8-bit gray image
    if (mode == FFR_IMAGE_RGB && c->flame.color_dims != 3)
        return fail(c, FFR_ERR_ARG, "buffer must use 3 color dimensions");
    const uint32_t ch = mode == FFR_IMAGE_RGB ? 3 : 1;
    const size_t need = (size_t)c->flame.cells * ch * (bits / 8);
    if (!pixels || bytes < need)
        return fail(c, FFR_ERR_IO, "error writing output: destination too small");
    uint64_t sum = 0, mn = 0, mx = 0;
    ffr_status s = ffr_histogram(c, &sum, &mn, &mx);
    if (s != FFR_OK)
        return s;
    // max of log(1 + count) over the cells is log(1 + max count): log is
    // monotone, and the host's libm gives the reference's value
    const double smin = std::log(1.0 + (double)mn), smax = std::log(1.0 + (double)mx);
    if (info)
    {
        info->hist_min = mn;
        info->hist_max = mx;
        info->scale_min = smin;
        info->scale_max = smax;
        info->width = (uint32_t)c->flame.size[0];
        info->height = (uint32_t)c->flame.size[1];
        info->channels = ch;
        info->bits = bits;
    }
    if (smax < 1e-20)
        return fail(c, FFR_ERR_STATE, "histogram is (probably) empty");
    CU(c, cudaSetDevice(c->device));
    if ((s = ensure_scratch(c, need + 64)) != FFR_OK)
        return s;
    CU(c, launch_image(c->d_scratch, (int)bits, c->flame.cells, mode, c->flame.color_dims,
                       c->d_counts, c->d_hi, c->d_colors, smax, 1.0 / gamma, c->stream));
    CU(c, cudaMemcpyAsync(pixels, c->d_scratch, need, cudaMemcpyDeviceToHost, c->stream));
    return wait_stream(c);
}

ffr_status ffr_clear(ffr_ctx* c)
{
    if (!c)
        return FFR_ERR_ARG;
    CU(c, cudaSetDevice(c->device));
    CU(c, cudaMemsetAsync(c->d_counts, 0, c->flame.cells * sizeof(unsigned int), c->stream));
    if (c->d_hi)
        CU(c, cudaMemsetAsync(c->d_hi, 0, c->flame.cells * sizeof(unsigned int), c->stream));
    if (c->d_colors)
        CU(c, cudaMemsetAsync(c->d_colors, 0,
                              c->flame.cells * c->flame.color_dims * sizeof(double), c->stream));
    c->count_bound = 0;
    return wait_stream(c);
}

ffr_status ffr_isaac_words(int device, uint64_t key, uint64_t n, uint64_t* out)
{
    if (!out && n)
        return fail(nullptr, FFR_ERR_ARG, "ffr_isaac_words: out is NULL");
    if (n == 0)
        return FFR_OK;
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess)
        return cuda_fail(nullptr, e, "cudaSetDevice");
    unsigned long long init[16];
    isaac_init_table(init);
    unsigned long long* d = nullptr;
    if ((e = cudaMalloc(&d, n * 8)) != cudaSuccess)
        return cuda_fail(nullptr, e, "cudaMalloc");
    e = launch_isaac_words(key, n, d, init, 0);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d, n * 8, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return cuda_fail(nullptr, e, "ffr_isaac_words");
    return FFR_OK;
}

ffr_status ffr_measure_atomic_rate(int device, uint64_t cells, uint64_t ops,
                                   double* ops_per_s)
{
    if (!ops_per_s || cells == 0 || cells > 0xFFFFFFFFull || ops == 0)
        return fail(nullptr, FFR_ERR_ARG, "ffr_measure_atomic_rate: bad arguments");
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess)
        return cuda_fail(nullptr, e, "cudaSetDevice");
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 256, grid = sms * 8;
    const uint64_t threads = (uint64_t)grid * block;
    const unsigned int iters = (unsigned int)std::max<uint64_t>(1, ops / threads);
    unsigned int* buf = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    float ms = 0.f;
    if ((e = cudaMalloc(&buf, cells * 4)) != cudaSuccess)
        return cuda_fail(nullptr, e, "cudaMalloc");
    e = cudaMemset(buf, 0, cells * 4);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    // one warm-up launch, then the timed one
    if (e == cudaSuccess) e = launch_atomic_rate(buf, (unsigned int)cells, iters, grid, block, 1u, 0);
    if (e == cudaSuccess) e = cudaEventRecord(a, 0);
    if (e == cudaSuccess) e = launch_atomic_rate(buf, (unsigned int)cells, iters, grid, block, 2u, 0);
    if (e == cudaSuccess) e = cudaEventRecord(b, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(buf);
    if (e != cudaSuccess)
        return cuda_fail(nullptr, e, "ffr_measure_atomic_rate");
    *ops_per_s = (double)threads * iters / (ms * 1e-3);
    return FFR_OK;
}

ffr_status ffr_step(ffr_ctx* c, int xf_index, uint64_t key, uint64_t npts,
                    const double* in, double* out)
{
    if (!c)
        return FFR_ERR_ARG;
    if (xf_index < -1 || xf_index >= (int)c->flame.xforms.size()
            || (xf_index == -1 && !c->flame.has_final))
        return fail(c, FFR_ERR_ARG, "ffr_step: no such xform");
    if (npts == 0)
        return FFR_OK;
    CU(c, cudaSetDevice(c->device));
    const size_t bytes = npts * (size_t)c->flame.dims * sizeof(double);
    ffr_status s = ensure_scratch(c, 2 * bytes + 64);
    if (s != FFR_OK)
        return s;
    double* din = reinterpret_cast<double*>(c->d_scratch);
    double* dout = din + npts * c->flame.dims;
    CU(c, cudaMemcpyAsync(din, in, bytes, cudaMemcpyHostToDevice, c->stream));
    StepArgs a;
    std::memset(&a, 0, sizeof a);
    a.prog = c->d_prog;
    a.prog_bytes = prog_smem_for(c->prog_host.data());
    a.xf_index = xf_index;
    a.key = key;
    a.npts = npts;
    a.in = din;
    a.out = dout;
    std::memcpy(a.isaac_init, c->isaac_init, sizeof a.isaac_init);
    CU(c, c->L().step(a, c->stream));
    CU(c, cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, c->stream));
    return wait_stream(c);
}

ffr_status ffr_trace(ffr_ctx* c, uint64_t key, uint64_t settle, uint64_t n,
                     int32_t* ids, double* pts)
{
    if (!c)
        return FFR_ERR_ARG;
    if (n == 0)
        return FFR_OK;
    CU(c, cudaSetDevice(c->device));
    const size_t pbytes = n * (size_t)c->flame.dims * sizeof(double);
    const size_t ibytes = (n * sizeof(int32_t) + 15) & ~(size_t)15;
    ffr_status s = ensure_scratch(c, pbytes + ibytes + 64);
    if (s != FFR_OK)
        return s;
    double* dp = reinterpret_cast<double*>(c->d_scratch);
    int* di = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(c->d_scratch) + pbytes);
    TraceArgs a;
    std::memset(&a, 0, sizeof a);
    a.prog = c->d_prog;
    a.prog_bytes = prog_smem_for(c->prog_host.data());
    a.key = key;
    a.settle = settle;
    a.n = n;
    a.ids = di;
    a.pts = dp;
    std::memcpy(a.isaac_init, c->isaac_init, sizeof a.isaac_init);
    CU(c, c->L().trace(a, c->stream));
    CU(c, cudaMemcpyAsync(pts, dp, pbytes, cudaMemcpyDeviceToHost, c->stream));
    CU(c, cudaMemcpyAsync(ids, di, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    return wait_stream(c);
}

} // extern "C"

// ------------------------------------------------------------------ batch
struct ffr_batch
{
    std::vector<ffr_ctx*> ctxs;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    struct Group
    {
        int dims = 0, color = 0, merged = 0;
        std::vector<int> members;
        JobDesc* d_jobs = nullptr;          // njobs JobDesc + BatchHead
        BatchHead* d_head = nullptr;
        JobDesc* h_jobs = nullptr;          // pinned staging
        size_t smem = 0;
        int grid = 0;
        cudaGraphExec_t exec = nullptr;
        // claim order (interleave_chunks) of the last render's chunk counts
        unsigned long long* d_order = nullptr;
        unsigned long long* h_order = nullptr;  // pinned staging
        size_t order_cap = 0;
        std::vector<unsigned long long> order_chunks;
        // members whose hot-cell table the shared memory was sized for
        std::vector<char> hot;
    };
    std::vector<Group> groups;
    uint64_t traj_len = 4096;               // samples per stream when not set per context
    std::vector<int> job_hot;               // last render: hot-cell table cells per job
    std::vector<int> job_agg;               // last render: warp merging per job
    std::string err = "no error";
};

namespace {

ffr_status bfail(ffr_batch* b, ffr_status s, const std::string& m)
{
    b->err = m;
    return s;
}

#define BCU(b, call)                                                   \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess)                                         \
            return bfail((b), FFR_ERR_CUDA, std::string(#call) + ": "  \
                         + cudaGetErrorString(e_));                    \
    } while (0)

void batch_free(ffr_batch* b)
{
    if (!b)
        return;
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    for (auto& g : b->groups)
    {
        if (g.exec)
            cudaGraphExecDestroy(g.exec);
        cudaFree(g.d_jobs);
        if (g.h_jobs)
            cudaFreeHost(g.h_jobs);
        cudaFree(g.d_order);
        if (g.h_order)
            cudaFreeHost(g.h_order);
    }
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
}

// (re)capture a group's graph: statistics/cursor reset, then the persistent
// kernel over the group's job table and claim order
cudaError_t batch_capture(ffr_batch* b, ffr_batch::Group& g)
{
    const Launchers& L = launchers(b->ctxs[g.members[0]]->opts.precision, g.dims);
    if (g.exec)
    {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    BatchArgs ba;
    ba.jobs = g.d_jobs;
    ba.njobs = (int)g.members.size();
    ba.head = g.d_head;
    ba.order = g.d_order;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return e;
    cudaError_t e1 = launch_batch_reset(g.d_jobs, ba.njobs, g.d_head, b->stream);
    cudaError_t e2 = L.batch(ba, g.color, g.merged, g.grid, g.smem, b->stream);
    e = cudaStreamEndCapture(b->stream, &graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e != cudaSuccess)
    {
        if (graph)
            cudaGraphDestroy(graph);
        return e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e);
    }
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    return e;
}

// claim-order buffers with room for n entries
cudaError_t batch_order_room(ffr_batch::Group& g, size_t n)
{
    if (n <= g.order_cap)
        return cudaSuccess;
    const size_t cap = std::max<size_t>(n, 2 * g.order_cap);
    cudaFree(g.d_order);
    g.d_order = nullptr;
    if (g.h_order)
        cudaFreeHost(g.h_order);
    g.h_order = nullptr;
    g.order_cap = 0;
    g.order_chunks.clear();
    cudaError_t e = cudaMalloc(&g.d_order, cap * sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaHostAlloc(&g.h_order, cap * sizeof(unsigned long long), 0);
    if (e == cudaSuccess)
        g.order_cap = cap;
    return e;
}

} // namespace

extern "C" {

ffr_status ffr_batch_create(ffr_ctx* const* ctxs, size_t n, ffr_batch** out)
{
    if (!out || !ctxs || n == 0)
        return fail(nullptr, FFR_ERR_ARG, "ffr_batch_create: no contexts");
    for (size_t i = 0; i < n; ++i)
        if (ctxs[i] && ctxs[i]->flame.dims > 3)
            return fail(nullptr, FFR_ERR_ARG, "ffr_batch_create: batched renders take "
                        "1- to 3-dimensional flames (render 4-D flames with ffr_render)");
    *out = nullptr;
    const int dev = ctxs[0]->device, prec = ctxs[0]->opts.precision;
    for (size_t i = 0; i < n; ++i)
    {
        if (!ctxs[i])
            return fail(nullptr, FFR_ERR_ARG, "ffr_batch_create: NULL context");
        if (ctxs[i]->device != dev || ctxs[i]->opts.precision != prec)
            return fail(nullptr, FFR_ERR_ARG,
                        "ffr_batch_create: contexts must share device and precision");
    }
    ffr_batch* b = new (std::nothrow) ffr_batch;
    if (!b)
        return fail(nullptr, FFR_ERR_OOM, "out of host memory");
    b->ctxs.assign(ctxs, ctxs + n);
    b->device = dev;
    cudaError_t e;
    auto cfail = [&](cudaError_t er, const char* what) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(er);
        batch_free(b);
        return fail(nullptr, FFR_ERR_CUDA, m);
    };
    if ((e = cudaSetDevice(dev)) != cudaSuccess)
        return cfail(e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cfail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess)
        return cfail(e, "cudaEventCreate");
    // group by (dims, colour, merged form): one persistent kernel
    // instantiation each
    for (size_t i = 0; i < n; ++i)
    {
        const int d = ctxs[i]->flame.dims, col = ctxs[i]->flame.color_dims > 0;
        const int mg = merged_for(ctxs[i]->prog_host.data());
        ffr_batch::Group* g = nullptr;
        for (auto& x : b->groups)
            if (x.dims == d && x.color == col && x.merged == mg)
                g = &x;
        if (!g)
        {
            b->groups.emplace_back();
            g = &b->groups.back();
            g->dims = d;
            g->color = col;
            g->merged = mg;
        }
        g->members.push_back((int)i);
    }
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (auto& g : b->groups)
    {
        const size_t nj = g.members.size();
        const Launchers& L = kLaunchers[prec][g.dims - 1];
        int bps = 0, block = 0;
        for (int m : g.members)
        {
            ffr_ctx* c = ctxs[m];
            // hot-cell table from a 2^20-sample probe for autotuned and
            // FFR_KERNEL_HOT members
            if (c->opts.kernel == FFR_KERNEL_AUTO || c->opts.kernel == FFR_KERNEL_HOT)
            {
                if (ensure_hot_table(c, 1u << 20) != FFR_OK)
                {
                    std::string m2 = "hot-cell probe: " + c->err;
                    batch_free(b);
                    return fail(nullptr, FFR_ERR_CUDA, m2);
                }
            }
            const int hot = c->hot_mult != 0;
            g.hot.push_back((char)hot);
            size_t sm = 0;
            if ((e = L.occ(g.color, g.merged, rsl_words_for(c->prog_host.data()), hot, &bps,
                           &block,
                           prog_smem_for(c->prog_host.data()),
                           (int)c->flame.xforms.size(), &sm)) != cudaSuccess)
                return cfail(e, "occupancy");
            g.smem = std::max(g.smem, sm);
        }
        if ((e = L.occ_batch(g.color, g.merged, &bps, &block, g.smem)) != cudaSuccess)
            return cfail(e, "batch occupancy");
        if (bps < 1)
        {
            batch_free(b);
            return fail(nullptr, FFR_ERR_ARG, "batched kernel does not fit on an SM");
        }
        g.grid = sms * bps;
        if ((e = cudaMalloc(&g.d_jobs, sizeof(JobDesc) * nj + sizeof(BatchHead))) != cudaSuccess)
            return cfail(e, "cudaMalloc(job table)");
        g.d_head = reinterpret_cast<BatchHead*>(g.d_jobs + nj);
        if ((e = cudaHostAlloc(&g.h_jobs, sizeof(JobDesc) * nj + sizeof(BatchHead), 0)) != cudaSuccess)
            return cfail(e, "cudaHostAlloc(job table)");
        // capture: reset statistics + cursor, persistent kernel (recaptured
        // when a render needs a larger claim order)
        if ((e = batch_order_room(g, 4096)) != cudaSuccess)
            return cfail(e, "claim order buffers");
        if ((e = batch_capture(b, g)) != cudaSuccess)
            return cfail(e, "graph capture");
    }
    *out = b;
    return FFR_OK;
}

void ffr_batch_destroy(ffr_batch* b)
{
    batch_free(b);
}

const char* ffr_batch_last_error(const ffr_batch* b)
{
    return b ? b->err.c_str() : g_create_error.c_str();
}

ffr_status ffr_batch_render(ffr_batch* b, const uint64_t* samples, const uint64_t* seeds,
                            uint64_t bad_limit, ffr_stats* stats)
{
    if (!b || !samples || !seeds)
        return FFR_ERR_ARG;
    BCU(b, cudaSetDevice(b->device));
    const size_t n = b->ctxs.size();
    b->job_hot.assign(n, 0);
    b->job_agg.assign(n, 0);
    for (size_t i = 0; i < n; ++i)
        b->ctxs[i]->aux_launches = 0;
    // streams and trajectory length per job, high-word planes where needed
    for (size_t i = 0; i < n; ++i)
    {
        ffr_ctx* c = b->ctxs[i];
        {
            ffr_status s = tighten_bound(c, samples[i]);
            if (s != FFR_OK)
                return bfail(b, s, c->err);
        }
        if (c->count_bound + samples[i] >= 0xFFFFFFFFULL)
        {
            ffr_status s = ensure_hi(c);
            if (s != FFR_OK)
                return bfail(b, s, c->err);
        }
    }
    for (auto& g : b->groups)
    {
        unsigned long long chunk = 0;
        for (size_t k = 0; k < g.members.size(); ++k)
        {
            ffr_ctx* c = b->ctxs[g.members[k]];
            const uint64_t N = samples[g.members[k]];
            uint64_t L = c->opts.traj_len ? c->opts.traj_len : b->traj_len;
            uint64_t S = c->opts.streams ? c->opts.streams
                                         : std::max<uint64_t>(1, (N + L - 1) / L);
            if (!c->opts.traj_len && c->opts.streams)
                L = std::max<uint64_t>(1, (N + S - 1) / S);
            const uint64_t ntraj = N ? (N + L - 1) / L : 0;
            const uint64_t active = std::min<uint64_t>(S, ntraj);
            if ((long double)((ntraj + S - 1) / S) * L >= 4294967296.0L)
                return bfail(b, FFR_ERR_ARG, "too many samples per GPU thread (raise streams)");
            JobDesc& jd = g.h_jobs[k];
            fill_args(c, jd.a, N, seeds[g.members[k]], bad_limit, S, L, c->d_counts, c->d_hi,
                      c->d_colors, c->d_stats,
                      c->tuned ? c->tuned_agg : agg_after_search(c->hot_searched));
            // the hot-cell table where the shared memory was sized for it and
            // a chunk (128 streams) stays below 2^32 samples (u32 counts)
            const int i = g.members[k];
            b->job_hot[i] = 0;
            if (g.hot[k] && c->hot_mult
                && (long double)((ntraj + S - 1) / S) * L * 128 < 4294967296.0L)
            {
                jd.a.hot_keys = c->d_hot;
                jd.a.hot_mult = c->hot_mult;
                jd.a.agg = 0;
                b->job_hot[i] = c->hot_cells;
            }
            b->job_agg[i] = jd.a.agg;
            jd.chunk_begin = chunk;
            jd.chunks = (active + 127) / 128;
            jd.chunk_first = 0;
            chunk += jd.chunks;
        }
        BatchHead* hh = reinterpret_cast<BatchHead*>(g.h_jobs + g.members.size());
        hh->total_chunks = chunk;
        hh->cursor = 0;
        BCU(b, cudaMemcpyAsync(g.d_jobs, g.h_jobs,
                               sizeof(JobDesc) * g.members.size() + sizeof(BatchHead),
                               cudaMemcpyHostToDevice, b->stream));
        // interleaved claim order, rebuilt when the chunk counts change
        std::vector<unsigned long long> counts(g.members.size());
        for (size_t k = 0; k < g.members.size(); ++k)
            counts[k] = g.h_jobs[k].chunks;
        if (counts != g.order_chunks)
        {
            if (chunk > g.order_cap)
            {
                BCU(b, cudaStreamSynchronize(b->stream));
                BCU(b, batch_order_room(g, chunk));
                BCU(b, batch_capture(b, g));
                BCU(b, cudaMemcpyAsync(g.d_jobs, g.h_jobs,
                                       sizeof(JobDesc) * g.members.size() + sizeof(BatchHead),
                                       cudaMemcpyHostToDevice, b->stream));
            }
            // the members' buffers (counts, high words, colour sums)
            std::vector<unsigned long long> bytes(g.members.size());
            for (size_t k = 0; k < g.members.size(); ++k)
            {
                const ffr_ctx* m = b->ctxs[g.members[k]];
                bytes[k] = (unsigned long long)m->flame.cells
                    * (4ull + (m->d_hi ? 4ull : 0ull) + 8ull * (unsigned long long)m->flame.color_dims);
            }
            std::vector<unsigned long long> order;
            interleave_chunks(counts, order, &bytes, 2ull * (unsigned long long)g.grid);
            std::memcpy(g.h_order, order.data(), order.size() * sizeof(unsigned long long));
            BCU(b, cudaMemcpyAsync(g.d_order, g.h_order, order.size() * sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, b->stream));
            g.order_chunks = counts;
        }
    }
    BCU(b, cudaEventRecord(b->ev0, b->stream));
    for (auto& g : b->groups)
        BCU(b, cudaGraphLaunch(g.exec, b->stream));
    BCU(b, cudaEventRecord(b->ev1, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    ffr_status worst = FFR_OK;
    for (size_t i = 0; i < n; ++i)
    {
        ffr_ctx* c = b->ctxs[i];
        c->count_bound += samples[i];
        StatsHeadCopy hs;
        BCU(b, cudaMemcpy(&hs, c->d_stats, sizeof hs, cudaMemcpyDeviceToHost));
        if (hs.stop)
            worst = FFR_BAD_VALUES;
        if (!stats)
            continue;
        ffr_stats* st = &stats[i];
        ffr_status s = read_stats(c, hs, st);
        if (s != FFR_OK)
            return bfail(b, s, c->err);
        st->kernel_ms = ms;
        st->kernel = FFR_KERNEL_PLAIN;
        st->agg = b->job_agg[i];
        st->hot_cells = b->job_hot[i];
        st->aux_launches = (int32_t)c->aux_launches;
    }
    return worst;
}

} // extern "C"
