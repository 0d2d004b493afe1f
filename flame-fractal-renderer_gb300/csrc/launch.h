// Interface between the host runtime (api.cpp) and the kernel translation
// units.  Plain structs shared by host and device code; the run-time
// compiled kernels (NVRTC, jit.cpp) see only those and the device helpers
// (the host-only parts are left out under __CUDACC_RTC__).
#pragma once

#include "std_types.h"
#ifndef __CUDACC_RTC__
#include <functional>
#include <queue>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#endif

#include "flame_program.h"

namespace ffr {

// Device-side statistics of one render call (the reference's `stats`
// struct, buffer_renderer.hpp:85-106).  Extremes are stored as order-keys
// (monotone u64 encodings of doubles) so atomicMin/atomicMax merge them.
struct DevStats
{
    unsigned long long s_iter;
    unsigned long long s_plot;
    unsigned long long bad_total;
    unsigned long long dropped;
    unsigned long long bad_claim;
    unsigned int stop;          // bad-value limit exceeded
    unsigned int cancelled;     // host cancel flag seen
    unsigned long long ext_lo[kMaxDims];
    unsigned long long ext_hi[kMaxDims];
    unsigned long long xf_dist[kMaxXformIds];   // by sorted xform index
    unsigned long long bad_xf[kMaxBadRecords];  // xform id of each bad value
    double bad_pts[kMaxBadRecords][kMaxDims];
};

struct RenderArgs
{
    const unsigned char* prog;      // device copy of the program blob
    unsigned int prog_bytes;        // its shared-memory part (prog_smem_for)
    int nxf;
    int color_dims;
    int spill;                      // counts may pass 2^32: keep high words
    unsigned long long seed;
    unsigned long long streams;     // total streams of the job
    unsigned long long samples;
    unsigned long long traj_len;
    unsigned long long settle;
    unsigned long long bad_limit;
    unsigned int* counts;           // u32 low words, one per cell
    unsigned int* hi;               // u32 high words (spill), or null
    double* colors;                 // cells * color_dims, or null
    DevStats* stats;
    const volatile unsigned int* cancel;   // host-mapped cancel flag, or null
    int rng_words;                  // largest RNG draw of one xform (sorted kernel)
    int agg;                        // warp-aggregate increments of equal cells
    int rsl_words;                  // ISAAC result array words (16 or kIsaacRslMax)
    // the program is in the FP32 merged form (ProgHeader::merged): the
    // launch runs the instantiation without the other 91 variations
    int merged;
    // hot-cell table of the plain kernel (kHotSlots keys), or null; needs
    // fewer than 2^30 cells and fewer than 2^32 samples per CTA
    const unsigned int* hot_keys;
    unsigned int hot_mult;
    unsigned long long isaac_init[16];
    // the program header's geometry, copied here so the render loop reads
    // it from kernel parameters instead of shared memory each sample
    // (set_geometry); the bounds and scales in the kernel's precision
    double lo_d[kMaxDims], hi_d[kMaxDims], mult_d_d[kMaxDims];
    float lo_f[kMaxDims], hi_f[kMaxDims], mult_d_f[kMaxDims];
    unsigned int size32[kMaxDims];          // buffer size per axis
    unsigned long long mult_i[kMaxDims];    // cell stride per axis
    unsigned long long cells;
    // FP64 bounds as ord_key values (the FP64 kernels test bounds on them)
    unsigned long long lo_key[kMaxDims], hi_key[kMaxDims];
};

// Monotone 64-bit key of a double with -0 taken as +0: for doubles a, b
// that are not NaN, a < b exactly when ord_key(a) < ord_key(b), and a == b
// exactly when the keys are equal.  The FP64 kernels compare and order
// points on these keys on the integer pipes instead of the FP64 pipe.  A
// NaN with the sign bit clear keys above +inf, one with it set below -inf.
__host__ __device__ inline unsigned long long ord_key(double d)
{
    unsigned long long u;
    memcpy(&u, &d, 8);
    if (u == 0x8000000000000000ULL)
        u = 0;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

#ifndef __CUDACC_RTC__
// copy the geometry of a program blob (precision 0 FP64, 1 FP32) into a
inline void set_geometry(RenderArgs& a, const void* prog, int precision)
{
    if (precision == 0)
    {
        ProgHeader<double> h;
        memcpy(&h, prog, sizeof h);
        for (int i = 0; i < kMaxDims; ++i)
        {
            a.lo_d[i] = h.lo[i];
            a.hi_d[i] = h.hi[i];
            a.mult_d_d[i] = h.mult_d[i];
            a.size32[i] = (unsigned int)h.size[i];
            a.mult_i[i] = h.mult_i[i];
            a.lo_key[i] = ord_key(h.lo[i]);
            a.hi_key[i] = ord_key(h.hi[i]);
        }
        a.cells = h.cells;
    }
    else
    {
        ProgHeader<float> h;
        memcpy(&h, prog, sizeof h);
        for (int i = 0; i < kMaxDims; ++i)
        {
            a.lo_f[i] = h.lo[i];
            a.hi_f[i] = h.hi[i];
            a.mult_d_f[i] = h.mult_d[i];
            a.size32[i] = (unsigned int)h.size[i];
            a.mult_i[i] = h.mult_i[i];
        }
        a.cells = h.cells;
    }
}
#endif

// xform counting in the render kernels: flames of up to kPackedXfCounters
// xforms count in eight 8-bit fields of one register per thread (flushed
// into per-CTA totals every 255 samples); up to kLocalXfCounters in per-thread
// u32 counters in shared memory; beyond that in per-CTA u64 totals directly
constexpr int kPackedXfCounters = 8;
constexpr int kLocalXfCounters = 16;
// ISAAC result array per render thread: one 16-word block, plus up to 8
// words carried across a refill ahead (isaac64.cuh) when the flame's xforms
// draw different numbers of words (ProgHeader::draws_vary).  A carry of 8
// (not 16) keeps such flames at 5 CTAs of 128 threads per SM.
constexpr int kIsaacRslMax = 24;

#ifndef __CUDACC_RTC__
// result-array words for a program blob (16 or kIsaacRslMax)
inline int rsl_words_for(const void* prog)
{
    static_assert(offsetof(ProgHeader<double>, draws_vary)
                  == offsetof(ProgHeader<float>, draws_vary), "program header layout");
    uint32_t v = 0;
    memcpy(&v, static_cast<const unsigned char*>(prog) + offsetof(ProgHeader<double>, draws_vary),
           sizeof v);
    return v ? kIsaacRslMax : 16;
}
#endif

__host__ __device__ inline unsigned int align16u(unsigned int x) { return (x + 15u) & ~15u; }

#ifndef __CUDACC_RTC__
// ProgHeader::smem_bytes of a program blob: the part the kernels copy into
// shared memory (RenderArgs::prog_bytes)
inline unsigned int prog_smem_for(const void* prog)
{
    static_assert(offsetof(ProgHeader<double>, smem_bytes)
                  == offsetof(ProgHeader<float>, smem_bytes), "program header layout");
    uint32_t v = 0;
    memcpy(&v, static_cast<const unsigned char*>(prog) + offsetof(ProgHeader<double>, smem_bytes),
           sizeof v);
    return v;
}

// The kernel variation set for a program blob (RenderArgs::merged): 0 =
// general (FP64 programs, and FP32 ones outside the merged form); 1 = the
// merged-form instantiation with a branch per type the flame uses; 2 = the
// merged-form instantiation evaluating all seven types without branches, for
// 2-D flames that use at least five of them
inline int merged_for(const void* prog)
{
    static_assert(offsetof(ProgHeader<double>, merged) == offsetof(ProgHeader<float>, merged),
                  "program header layout");
    static_assert(offsetof(ProgHeader<double>, tier_a_present)
                  == offsetof(ProgHeader<float>, tier_a_present), "program header layout");
    uint32_t v = 0, present = 0;
    int32_t dims = 0;
    const unsigned char* b = static_cast<const unsigned char*>(prog);
    memcpy(&v, b + offsetof(ProgHeader<double>, merged), sizeof v);
    memcpy(&present, b + offsetof(ProgHeader<double>, tier_a_present), sizeof present);
    memcpy(&dims, b + offsetof(ProgHeader<double>, dims), sizeof dims);
    if (!v)
        return 0;
    int types = 0;
    for (int k = 0; k < 7; ++k)
        types += (present >> k) & 1u;
    return dims == 2 && types >= 5 ? 2 : 1;
}
#endif

// Hot cells: a flame's density can sit largely in a few cells (fixed
// points, attractor cores; the 1920x1080 benchmark flame puts 18% of its
// samples in 64 cells and 5.5% in one 128-byte line), and atomic adds on
// those few L2 lines then cap the binning rate.  The plain render kernel can
// count up to kHotCells such cells per CTA in shared memory: a direct-mapped
// table of kHotSlots keys (slot = (cell * hot_mult) >> (32 - kHotSlotBits),
// the multiplier chosen so that the keys do not collide; empty slots hold
// kHotEmpty) and their u32 counts, added to the buffer once when the CTA
// ends.
constexpr int kHotSlotBits = 8;
constexpr int kHotSlots = 1 << kHotSlotBits;
constexpr int kHotCells = 64;
constexpr unsigned int kHotEmpty = 0xFFFFFFFFu;
// candidates a hot-cell search collects at most per threshold
constexpr unsigned int kHotCollectCap = 1024;

#ifndef __CUDACC_RTC__
// Hot-cell table from candidate cells (count << 32 | cell, any order, from
// launch_hot_collect) of a buffer holding about sum samples: the up to
// kHotCells hottest, if together they hold at least 1/50 of sum, placed by
// an odd multiplier under which no two share a slot.  On success *mult is
// that multiplier, keys holds kHotSlots entries (kHotEmpty where unused)
// and the result is true; found is sorted hottest first.
bool hot_place(std::vector<unsigned long long>& found, unsigned long long sum,
               unsigned int* mult, std::vector<unsigned int>& keys);
#endif

// Dynamic shared memory of the plain and batch render kernels: the program,
// ISAAC state (randmem [16][BLOCK], results [rsl_words][BLOCK]), the
// xform counters (per-thread u32 when kPackedXfCounters < nxf <=
// kLocalXfCounters, else one u64 total per xform for the CTA), and with hot
// the hot-cell table (kHotSlots keys, then kHotSlots counts).
template <int BLOCK>
__host__ __device__ inline size_t chaos_smem_bytes(unsigned int prog_bytes, int nxf,
                                                   int rsl_words, bool hot = false)
{
    size_t s = align16u(prog_bytes);
    s += (16 + (size_t)rsl_words) * (size_t)BLOCK * sizeof(uint64_t);
    if (nxf > kPackedXfCounters && nxf <= kLocalXfCounters)
        s += (size_t)nxf * BLOCK * sizeof(uint32_t);
    else
        s += (size_t)nxf * sizeof(unsigned long long);
    if (hot)
        s += 2 * (size_t)kHotSlots * sizeof(uint32_t);
    return s;
}

// The xform-sorted render kernel (chaos_sorted.cuh): threads per CTA, the
// xforms a CTA handles (per-xform lists and counters in shared memory), its
// ISAAC result array and dynamic shared memory
constexpr int kSortedBlock = 256;
constexpr int kSortedMaxXforms = 16;
constexpr int kRslWords = 24;          // 16 fresh words + carried tail
constexpr int kMaxRefillLow = kRslWords - 16;

template <int T>
__host__ __device__ inline size_t sorted_smem_bytes(unsigned int prog_bytes, int nxf,
                                                    int words, int dims, int real_bytes)
{
    size_t s = align16u(prog_bytes);
    s += (16 + kRslWords + 3) * (size_t)T * 8;            // ISAAC state
    s += (size_t)words * T * 8;                           // pre-drawn words [W][T]
    s += (((size_t)dims * T * real_bytes) + 15) & ~(size_t)15;   // staged points [D][T]
    s += (((size_t)nxf * T * 4) + 15) & ~(size_t)15;      // per-thread xform counts
    s += (((size_t)nxf * T * 2) + 15) & ~(size_t)15;      // per-xform lists (u16)
    s += (((size_t)T * 2) + 15) & ~(size_t)15;            // refill list (u16)
    s += (((size_t)T) + 15) & ~(size_t)15;                // words left at refill (u8)
    s += (2 * kSortedMaxXforms + 2) * 4;                  // list counters x2
    return s;
}

// One job of a batched launch: the arguments ffr_render would use for the
// context alone, and its range of chunks (BLOCK streams each) in the
// batch's chunk order.  The launch runs the job's chunks chunk_first ..
// chunk_first + chunks - 1 (chunk k = streams k*BLOCK .. k*BLOCK+BLOCK-1), so
// a job can be split over several launches (the serving loop's rounds).
struct JobDesc
{
    RenderArgs a;
    unsigned long long chunk_begin;
    unsigned long long chunks;
    unsigned long long chunk_first;
};

// Device-side header of a batch: chunk count and the claim cursor (reset
// by batch_reset_kernel before each launch).
struct BatchHead
{
    unsigned long long total_chunks;
    unsigned long long cursor;
};

struct BatchArgs
{
    const JobDesc* jobs;
    int njobs;
    BatchHead* head;
    // claim order: entry c = (job << 32) | chunk within the job's range,
    // interleaved (interleave_chunks) so the CTAs running at any moment
    // work on many jobs' buffers instead of one job's at a time
    const unsigned long long* order;
};

#ifndef __CUDACC_RTC__
// Claim order for jobs of chunks[k] chunks: chunk r of job k gets the key
// (r + 1/2) / chunks[k] and claims run in ascending key order (ties by job),
// so every job advances at the same relative pace and concurrent CTAs spread
// over the jobs in proportion to their size.  (Binning every CTA into one
// job's buffer at a time concentrates the L2 atomics: the 256-flame batch
// ran 27% slower in job order.)  With bytes (each job's buffer size), the
// jobs are taken in windows of consecutive jobs -- at least kMinWindowJobs
// jobs and min_chunks chunks (enough to keep every resident CTA busy), and
// more while their buffers add up to at most kWindowBytes -- interleaved
// within a window, one window after another, so that the buffers the running
// CTAs bin into stay within L2 instead of every buffer of a large batch
// being in flight at once.  Any order gives the same buffers.
constexpr size_t kMinWindowJobs = 16;
constexpr unsigned long long kWindowBytes = 64ull << 20;

inline void interleave_chunks(const std::vector<unsigned long long>& chunks,
                              std::vector<unsigned long long>& order,
                              const std::vector<unsigned long long>* bytes = nullptr,
                              unsigned long long min_chunks = 0)
{
    order.clear();
    struct Item
    {
        double key;
        unsigned long long job, r;
        bool operator>(const Item& o) const
        {
            return key > o.key || (key == o.key && job > o.job);
        }
    };
    size_t k0 = 0;
    while (k0 < chunks.size())
    {
        size_t k1 = chunks.size();
        if (bytes)
        {
            unsigned long long sum = 0, n = 0;
            k1 = k0;
            while (k1 < chunks.size()
                   && (k1 - k0 < kMinWindowJobs || n < min_chunks
                       || sum + (*bytes)[k1] <= kWindowBytes))
            {
                sum += (*bytes)[k1];
                n += chunks[k1++];
            }
        }
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
        for (size_t k = k0; k < k1; ++k)
            if (chunks[k])
                heap.push({0.5 / (double)chunks[k], k, 0});
        while (!heap.empty())
        {
            Item it = heap.top();
            heap.pop();
            order.push_back((it.job << 32) | it.r);
            if (++it.r < chunks[it.job])
            {
                it.key = ((double)it.r + 0.5) / (double)chunks[it.job];
                heap.push(it);
            }
        }
        k0 = k1;
    }
}
#endif

// Single xform application on a batch of points (one stream per point).
struct StepArgs
{
    const unsigned char* prog;
    unsigned int prog_bytes;
    int xf_index;                   // sorted xform index, -1 = final
    unsigned long long key;
    unsigned long long npts;
    const double* in;               // npts * dims
    double* out;
    unsigned long long isaac_init[16];
};

// First n samples of one trajectory (xform ids and points).
struct TraceArgs
{
    const unsigned char* prog;
    unsigned int prog_bytes;
    unsigned long long key;
    unsigned long long settle;
    unsigned long long n;
    int* ids;
    double* pts;                    // n * dims
    unsigned long long isaac_init[16];
};

#ifndef __CUDACC_RTC__
// Isaac::init with flag = false: the 16-word randmem every stream starts from
void isaac_init_table(unsigned long long out[16]);

// set the message ffr_last_error(NULL) returns on this thread
void set_global_error(const std::string& m);
#endif

// the 16-word randmem table every stream starts from (isaac64.cuh)
struct IsaacInit
{
    unsigned long long w[16];
};

// Warp-merged binning (RenderArgs::agg) where neither an autotuner decision
// nor a hot-cell search exists: lanes of a warp that hit the same cell make
// one atomic add.  Flames with hot cells (fixed points, dense cores) gain
// much more (the 1920x1080 benchmark flame: 30 G binned/s merged, 22
// unmerged) than flames without collisions lose (a match per sample).  Once
// a search has run, flames with a hot-cell table count their hot cells in
// shared memory and flames without one have no collisions worth merging
// (a uniform Sierpinski triangle: 1.9 ms merged, 1.1 ms unmerged per 1e8
// samples), so both bin unmerged (agg_after_search).
constexpr int kDefaultAgg = 1;
#ifndef __CUDACC_RTC__
inline int agg_after_search(bool searched) { return searched ? 0 : kDefaultAgg; }
#endif

#ifndef __CUDACC_RTC__
// precision: 0 = FP64 mirror, 1 = FP32
#define FFR_DECLARE_LAUNCHERS(P, D)                                              \
    cudaError_t launch_render_p##P##_d##D(const RenderArgs&, int grid,          \
                                          cudaStream_t);                        \
    cudaError_t occupancy_p##P##_d##D(int color, int merged, int rsl_words,     \
                                      int hot, int* blocks_per_sm, int* block,  \
                                      unsigned int prog_bytes, int nxf,         \
                                      size_t* smem);                            \
    cudaError_t launch_sorted_p##P##_d##D(const RenderArgs&, int grid,          \
                                          cudaStream_t);                        \
    cudaError_t occupancy_sorted_p##P##_d##D(int color, int spill,              \
                                             int* blocks_per_sm, int* block,    \
                                             unsigned int prog_bytes, int nxf,  \
                                             int words, size_t* smem);          \
    cudaError_t launch_batch_p##P##_d##D(const BatchArgs&, int color,           \
                                         int merged, int grid, size_t smem,     \
                                         cudaStream_t);                         \
    cudaError_t occupancy_batch_p##P##_d##D(int color, int merged,              \
                                            int* blocks_per_sm, int* block,     \
                                            size_t smem);                       \
    cudaError_t launch_step_p##P##_d##D(const StepArgs&, cudaStream_t);         \
    cudaError_t launch_trace_p##P##_d##D(const TraceArgs&, cudaStream_t);

FFR_DECLARE_LAUNCHERS(0, 1)
FFR_DECLARE_LAUNCHERS(0, 2)
FFR_DECLARE_LAUNCHERS(0, 3)
FFR_DECLARE_LAUNCHERS(1, 1)
FFR_DECLARE_LAUNCHERS(1, 2)
FFR_DECLARE_LAUNCHERS(1, 3)
// four dimensions: plain render, step and trace kernels only (no sorted or
// batch instantiation; the Launchers entries for those are null)
FFR_DECLARE_LAUNCHERS(0, 4)
FFR_DECLARE_LAUNCHERS(1, 4)

typedef cudaError_t (*RenderFn)(const RenderArgs&, int, cudaStream_t);
typedef cudaError_t (*OccFn)(int, int, int, int, int*, int*, unsigned int, int, size_t*);
typedef cudaError_t (*StepFn)(const StepArgs&, cudaStream_t);
typedef cudaError_t (*TraceFn)(const TraceArgs&, cudaStream_t);
typedef cudaError_t (*OccSortedFn)(int, int, int*, int*, unsigned int, int, int, size_t*);
typedef cudaError_t (*BatchFn)(const BatchArgs&, int, int, int, size_t, cudaStream_t);
typedef cudaError_t (*OccBatchFn)(int, int, int*, int*, size_t);

// the launch functions of one (precision, dims) kernel instantiation
struct Launchers
{
    RenderFn render;
    OccFn occ;
    RenderFn sorted;
    OccSortedFn occ_sorted;
    BatchFn batch;
    OccBatchFn occ_batch;
    StepFn step;
    TraceFn trace;
};

// precision 0 (FP64) or 1 (FP32), dims 1..3 (api.cpp)
const Launchers& launchers(int precision, int dims);

// buffer_kernels.cu
cudaError_t launch_isaac_words(unsigned long long key, unsigned long long n,
                               unsigned long long* out,
                               const unsigned long long* init16, cudaStream_t);
cudaError_t launch_accumulate(const unsigned long long* file, unsigned long long cells,
                              int color_dims, unsigned int* counts, unsigned int* hi,
                              double* colors, int overwrite, cudaStream_t);
cudaError_t launch_export(unsigned long long* file, unsigned long long cells,
                          int color_dims, const unsigned int* counts,
                          const unsigned int* hi, const double* colors, cudaStream_t);
cudaError_t launch_file_max(const unsigned long long* file, unsigned long long cells,
                            int color_dims, unsigned long long* out, cudaStream_t);
// histogram sum/min/max over counts (+ hi); out[0]=sum, out[1]=min, out[2]=max
cudaError_t launch_hist_reduce(const unsigned int* counts, const unsigned int* hi,
                               unsigned long long cells, unsigned long long* out,
                               cudaStream_t);

// cells with count >= thr: out[0] = how many, out[1 ..] = (count << 32 |
// cell) for the first cap of them (out holds 1 + cap words).  Counts are
// read with volatile (relaxed) loads, so a render may still be adding to
// the buffer.
cudaError_t launch_hot_collect(const unsigned int* counts, unsigned int cells, unsigned int thr,
                               unsigned long long* out, unsigned int cap, cudaStream_t);
// Hot-cell candidates into found (host): cells with count >= thr, the
// threshold raised fourfold while more than kHotCollectCap qualify (up to
// thr_max); *got is false when no threshold left few enough.  out: 1 +
// kHotCollectCap device words; waits for the stream.  *launches (or null)
// grows by the kernels launched.
cudaError_t collect_hot_candidates(const unsigned int* counts, unsigned int cells,
                                   unsigned long long thr, unsigned long long thr_max,
                                   unsigned long long* out, cudaStream_t st,
                                   std::vector<unsigned long long>& found, bool* got,
                                   unsigned int* launches);

cudaError_t launch_atomic_rate(unsigned int* buf, unsigned int cells, unsigned int iters,
                               int grid, int block, unsigned int salt, cudaStream_t);

// zero the statistics of every job (one CTA per job) and the batch cursor
cudaError_t launch_batch_reset(const JobDesc* jobs, int njobs, BatchHead* head,
                               cudaStream_t);

// image_kernels.cu: ffr-img's pixel mapping (mode 0 mono, 1 gray, 2 RGB)
cudaError_t launch_image(void* out, int bits, unsigned long long cells, int mode,
                         int color_dims, const unsigned int* counts, const unsigned int* hi,
                         const double* colors, double max_l, double gp, cudaStream_t st);

// zero one statistics block (nxf per-xform counters), extremes to +/-inf
cudaError_t launch_stats_reset(DevStats* st, int nxf, cudaStream_t);

#endif

// monotone u64 key of a double (NaN never stored)
__host__ __device__ inline unsigned long long order_key(double d)
{
    unsigned long long u;
    memcpy(&u, &d, 8);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

__host__ __device__ inline double key_to_double(unsigned long long k)
{
    unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    double d;
    memcpy(&d, &u, 8);
    return d;
}

} // namespace ffr
