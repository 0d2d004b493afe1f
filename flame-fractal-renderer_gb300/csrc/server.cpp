// Serving loop of libffr_gpu.so (ffr_server_* in include/ffr_gpu.h):
// continuous batching of render jobs over the persistent batch kernel, with
// device-resident buffers and admission by a device-memory budget.
//
// Data flow.  Submission parses the flame on the caller's thread and queues
// the job.  The scheduler thread admits queued jobs in arrival order
// (stream-ordered pool allocations on the aux stream: buffer, statistics),
// then issues rounds.  A round takes a slice of every running job's chunks
// (chunk = 128 consecutive streams of the job), evenly shared, builds one
// job table per (dims, colour) group and launches the persistent batch
// kernel once per group on the round's stream.  Two round slots alternate,
// so while the host waits for round r, round r+1 is already queued on the
// other stream and its CTAs fill the SMs that round r's tail leaves idle.
// When a round's event completes, every job whose chunks are all done reads
// back its statistics and is finished.
//
// Each job's streams and trajectories are the ones ffr_render runs for the
// same flame with streams = ceil(samples / traj_len) and that traj_len, so
// results do not depend on the mix; only the order of the integer adds (and
// of colour sums) differs.
#include "ffr_gpu.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "flame.hpp"
#include "launch.h"

using namespace ffr;

namespace {

constexpr int kChunkStreams = 128;          // BLOCK of the batch kernel
constexpr int kRoundSlots = 2;
// dims 1..3 x kernel variation set (merged_for: 0 general, 1 and 2 the
// merged-form instantiations) x colour off/on:
// group g = ((dims - 1) * 3 + variation set) * 2 + colour
constexpr int kGroups = 18;
constexpr size_t kStagingBytes = 16u << 20; // device staging of one read slot
constexpr int kReadSlots = 4;               // concurrent buffer reads

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Server;

// A resident count buffer (one flame); shared by the job that created it
// and the jobs continuing it.  Device memory comes from the server's pool.
struct SrvBuffer
{
    Server* srv = nullptr;
    HostFlame flame;
    std::vector<uint8_t> prog;
    int rng_words = 0;
    size_t smem = 0;                    // batch kernel shared memory for this program
    unsigned char* d_prog = nullptr;
    unsigned int* d_counts = nullptr;
    unsigned int* d_hi = nullptr;
    double* d_colors = nullptr;
    size_t dev_bytes = 0;               // held in the pool (counted in used)
    uint64_t count_bound = 0;           // upper bound of any cell's count
    int running = 0;                    // admitted, unfinished jobs on it
    bool allocated = false;
    bool alloc_failed = false;
    std::vector<unsigned long long> init;   // -i data, added at admission
    // hot-cell table of the render kernel (kHotSlots keys), searched once in
    // the buffer's counts after its first finished round; hot_mult 0 = none
    unsigned int* d_hot = nullptr;
    unsigned int hot_mult = 0;
    int hot_cells = 0;
    bool hot_searched = false;
    size_t smem_hot = 0;                // batch kernel shared memory with the table
    ~SrvBuffer();
    size_t file_bytes() const { return (size_t)flame.cells * (1 + (size_t)flame.color_dims) * 8; }
    size_t counts_bytes() const { return (size_t)flame.cells * 4; }
    size_t colors_bytes() const { return (size_t)flame.cells * flame.color_dims * 8; }
};

struct SrvJob
{
    uint64_t id = 0, parent = 0;
    std::shared_ptr<SrvBuffer> buf;
    uint64_t samples = 0, seed = 0, bad_limit = 0;
    uint64_t S = 0, L = 0;
    uint64_t chunks_total = 0, chunks_issued = 0, chunks_done = 0;
    DevStats* d_stats = nullptr;
    int slot = -1;                      // cancel flag index while admitted
    int spill = 0;
    int hot_cells = 0;                  // hot-cell table cells of its last round
    int last_agg = kDefaultAgg;         // warp merging of its last round
    int state = FFR_JOB_QUEUED;
    ffr_status status = FFR_OK;
    bool cancel_req = false;
    uint64_t t_submit = 0, t_admit = 0, t_done = 0;
    // statistics, read back at completion
    uint64_t s_iter = 0, s_plot = 0, bad_total = 0, dropped = 0;
    double ext_lo[kMaxDims], ext_hi[kMaxDims];
    std::vector<uint64_t> xf_dist;      // by JSON xform id
    std::vector<uint64_t> bad_xf;
    std::vector<double> bad_pts;        // kMaxDims per record
};

struct RoundPart
{
    SrvJob* job;
    uint64_t chunks;
};

struct RoundSlot
{
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    JobDesc* d_jobs = nullptr;          // capacity max_active
    BatchHead* d_heads = nullptr;       // kGroups
    JobDesc* h_jobs = nullptr;          // pinned mirror: jobs then heads
    unsigned long long* d_order = nullptr;  // claim order of the round's chunks
    unsigned long long* h_order = nullptr;  // pinned mirror
    size_t order_cap = 0;
    bool busy = false;
    uint64_t started_ns = 0;
    std::vector<RoundPart> parts;
};

struct Server
{
    ffr_server_opts o{};
    int sms = 1;
    uint64_t budget = 0;
    unsigned long long isaac_init[16] = {};
    cudaMemPool_t pool = nullptr;
    cudaStream_t aux = nullptr;         // allocations, resets, statistics
    // Buffer reads.  Each slot exports a slice of cells into its device
    // staging, copies it into one of two pinned host buffers (a true async
    // DMA: a copy into the caller's pageable memory would be a synchronous
    // driver call that holds up the scheduler's launches) and the host then
    // copies the previous slice out while the next one is in flight.
    struct ReadSlot
    {
        cudaStream_t stream = nullptr;
        unsigned long long* d_stage = nullptr;
        unsigned char* h_stage[2] = {nullptr, nullptr};
        cudaEvent_t ev[2] = {nullptr, nullptr};
        bool busy = false;
    };
    ReadSlot readers[kReadSlots];
    std::mutex rd_mu;
    std::condition_variable rd_cv;
    cudaEvent_t ev_alloc = nullptr;     // after the latest admission work
    unsigned long long* d_red = nullptr;    // 3 words: histogram sum, min, max
    unsigned long long* d_hotc = nullptr;   // 1 + kHotCollectCap words: hot-cell search
    unsigned int* h_cancel = nullptr;   // mapped pinned flags, one per slot
    unsigned int* d_cancel = nullptr;
    std::vector<int> free_slots;
    RoundSlot rounds[kRoundSlots];
    int next_round = 0;

    std::mutex mu;
    std::condition_variable cv_work;    // scheduler wake-up
    std::condition_variable cv_done;    // job completions
    std::map<uint64_t, std::unique_ptr<SrvJob>> jobs;
    std::deque<SrvJob*> queue;
    std::vector<SrvJob*> active;        // admitted, unfinished, admission order
    uint64_t next_id = 1;
    bool stop = false;
    bool broken = false;
    std::string err = "no error";
    std::thread thread;

    std::atomic<uint64_t> used{0}, peak{0};

    void add_used(size_t b)
    {
        const uint64_t u = used.fetch_add(b) + b;
        uint64_t p = peak.load();
        while (u > p && !peak.compare_exchange_weak(p, u))
        {
        }
    }
    void loop();
    void admit_locked();
    bool launch_round_locked();
    void finish_round_locked(RoundSlot& r, cudaError_t e, const std::string& why);
    void hot_search_locked(SrvBuffer& b, uint64_t sum);
    void finish_job_locked(SrvJob* j);
    void fail_job_locked(SrvJob* j, ffr_status st);
};

SrvBuffer::~SrvBuffer()
{
    if (!srv)
        return;
    cudaSetDevice(srv->o.device);
    if (d_prog) cudaFreeAsync(d_prog, srv->aux);
    if (d_counts) cudaFreeAsync(d_counts, srv->aux);
    if (d_hi) cudaFreeAsync(d_hi, srv->aux);
    if (d_colors) cudaFreeAsync(d_colors, srv->aux);
    if (d_hot) cudaFreeAsync(d_hot, srv->aux);
    srv->used.fetch_sub(dev_bytes);
}

thread_local std::string g_server_error = "no error";

ffr_status sfail(Server* s, ffr_status st, const std::string& m)
{
    if (s)
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = m;
    }
    else
        g_server_error = m;
    set_global_error(m);
    return st;
}

template <typename T>
cudaError_t pool_alloc(Server* s, T** p, size_t bytes)
{
    return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, s->pool, s->aux);
}

void Server::fail_job_locked(SrvJob* j, ffr_status st)
{
    j->state = FFR_JOB_FAILED;
    j->status = st;
    j->t_done = now_ns();
    cv_done.notify_all();
}

// Admit queued jobs in arrival order while slots and the budget allow.
void Server::admit_locked()
{
    while (!queue.empty() && !free_slots.empty() && !broken)
    {
        SrvJob* j = queue.front();
        SrvBuffer& b = *j->buf;
        if (j->cancel_req)
        {
            queue.pop_front();
            j->state = FFR_JOB_CANCELLED;
            j->status = FFR_ERR_TIMEOUT;
            j->t_done = now_ns();
            cv_done.notify_all();
            continue;
        }
        if (b.alloc_failed)
        {
            queue.pop_front();
            fail_job_locked(j, FFR_ERR_OOM);
            continue;
        }
        if (!b.d_hi && b.allocated && b.running == 0 && b.count_bound + j->samples >= 0xFFFFFFFFULL)
        {
            // the bound counts every sample rendered so far; replace it by
            // the exact largest count before deciding on high words
            unsigned long long init[3] = {0ull, ~0ull, 0ull}, out[3] = {0ull, 0ull, 0ull};
            cudaError_t er = cudaMemcpyAsync(d_red, init, sizeof init, cudaMemcpyHostToDevice, aux);
            if (er == cudaSuccess)
                er = launch_hist_reduce(b.d_counts, nullptr, b.flame.cells, d_red, aux);
            if (er == cudaSuccess)
                er = cudaMemcpyAsync(out, d_red, sizeof out, cudaMemcpyDeviceToHost, aux);
            if (er == cudaSuccess)
                er = cudaStreamSynchronize(aux);
            if (er == cudaSuccess)
                b.count_bound = out[2];
            else
                cudaGetLastError();
        }
        const bool need_hi = b.count_bound + j->samples >= 0xFFFFFFFFULL && !b.d_hi;
        // counts of jobs already running on this buffer carry no high words
        if (need_hi && b.running > 0)
            break;
        size_t need = sizeof(DevStats);
        if (!b.allocated)
            need += b.prog.size() + b.counts_bytes() + b.colors_bytes() + b.file_bytes() * (!b.init.empty());
        if (need_hi)
            need += b.counts_bytes();
        if (used.load() + need > budget)
            break;
        queue.pop_front();
        cudaError_t e = cudaSuccess;
        if (!b.allocated)
        {
            e = pool_alloc(this, &b.d_prog, b.prog.size());
            if (e == cudaSuccess)
                e = pool_alloc(this, &b.d_counts, b.counts_bytes());
            if (e == cudaSuccess && b.flame.color_dims)
                e = pool_alloc(this, &b.d_colors, b.colors_bytes());
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(b.d_prog, b.prog.data(), b.prog.size(),
                                    cudaMemcpyHostToDevice, aux);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(b.d_counts, 0, b.counts_bytes(), aux);
            if (e == cudaSuccess && b.d_colors)
                e = cudaMemsetAsync(b.d_colors, 0, b.colors_bytes(), aux);
            b.dev_bytes = b.prog.size() + b.counts_bytes() + b.colors_bytes();
            add_used(b.dev_bytes);
            if (e == cudaSuccess && !b.init.empty())
            {
                unsigned long long* tmp = nullptr;
                e = pool_alloc(this, &tmp, b.file_bytes());
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(tmp, b.init.data(), b.file_bytes(),
                                        cudaMemcpyHostToDevice, aux);
                if (e == cudaSuccess)
                    e = launch_accumulate(tmp, b.flame.cells, b.flame.color_dims, b.d_counts,
                                          nullptr, b.d_colors, 0, aux);
                if (tmp)
                    cudaFreeAsync(tmp, aux);
                // the pageable source is consumed once the copy has been staged
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(aux);
                std::vector<unsigned long long>().swap(b.init);
            }
            b.allocated = e == cudaSuccess;
            b.alloc_failed = !b.allocated;
        }
        if (e == cudaSuccess && need_hi)
        {
            e = pool_alloc(this, &b.d_hi, b.counts_bytes());
            if (e == cudaSuccess)
                e = cudaMemsetAsync(b.d_hi, 0, b.counts_bytes(), aux);
            if (e == cudaSuccess)
            {
                b.dev_bytes += b.counts_bytes();
                add_used(b.counts_bytes());
            }
        }
        if (e == cudaSuccess)
            e = pool_alloc(this, &j->d_stats, sizeof(DevStats));
        if (e == cudaSuccess)
        {
            add_used(sizeof(DevStats));
            e = launch_stats_reset(j->d_stats, (int)b.flame.xforms.size(), aux);
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(ev_alloc, aux);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            err = std::string("admission: ") + cudaGetErrorString(e);
            fail_job_locked(j, e == cudaErrorMemoryAllocation ? FFR_ERR_OOM : FFR_ERR_CUDA);
            continue;
        }
        b.count_bound += j->samples;
        b.running += 1;
        j->spill = b.d_hi != nullptr;
        j->slot = free_slots.back();
        free_slots.pop_back();
        h_cancel[j->slot] = 0u;
        j->state = FFR_JOB_RUNNING;
        j->t_admit = now_ns();
        active.push_back(j);
        if (j->chunks_total == 0)
            finish_job_locked(j);
    }
}

// jobs with at most this many chunks (128 streams each) left join every
// round (they finish in it)
constexpr uint64_t kSmallJobChunks = 32;

// Build and launch one round on a free round slot; false if there is no
// free slot or no chunk left to issue.
bool Server::launch_round_locked()
{
    RoundSlot* r = nullptr;
    for (int k = 0; k < kRoundSlots && !r; ++k)
    {
        RoundSlot& c = rounds[(next_round + k) % kRoundSlots];
        if (!c.busy)
            r = &c;
    }
    if (!r || broken)
        return false;
    // The round's jobs: the oldest ones while their buffers add up to at
    // most kWindowBytes (at least kMinWindowJobs of them, launch.h), so that
    // the buffers a round bins into stay within L2, plus every job that this
    // round can finish outright (at most kSmallJobChunks chunks left), so
    // that small jobs never wait behind large ones.  (Rounds over every
    // running job kept hundreds of buffers, gigabytes, in flight at once.)
    std::vector<SrvJob*> cand;
    {
        size_t in_window = 0;
        unsigned long long window_bytes = 0;
        for (SrvJob* j : active)
        {
            if (j->cancel_req || j->chunks_issued >= j->chunks_total)
                continue;
            const SrvBuffer& b = *j->buf;
            const unsigned long long bytes = (unsigned long long)b.flame.cells
                * (4ull + 8ull * (unsigned long long)b.flame.color_dims);
            if (in_window < kMinWindowJobs || window_bytes + bytes <= kWindowBytes)
            {
                ++in_window;
                window_bytes += bytes;
                cand.push_back(j);
            }
            else if (j->chunks_total - j->chunks_issued <= kSmallJobChunks)
                cand.push_back(j);
        }
    }
    if (cand.empty())
        return false;
    uint64_t budget_chunks = o.round_chunks;
    if (!budget_chunks)
    {
        int bps = 0, block = 0;
        const SrvBuffer& b0 = *cand.front()->buf;
        launchers(o.precision, b0.flame.dims).occ_batch(b0.flame.color_dims > 0,
                                                        merged_for(b0.prog.data()), &bps,
                                                        &block, b0.smem);
        budget_chunks = 4ull * (uint64_t)sms * (uint64_t)std::max(1, bps);
    }
    budget_chunks = std::min<uint64_t>(budget_chunks, r->order_cap);
    // even share, then what is left to the oldest jobs
    std::vector<uint64_t> take(cand.size(), 0);
    const uint64_t share = std::max<uint64_t>(1, budget_chunks / cand.size());
    uint64_t left = budget_chunks;
    for (size_t i = 0; i < cand.size() && left; ++i)
    {
        const uint64_t t = std::min({share, cand[i]->chunks_total - cand[i]->chunks_issued, left});
        take[i] = t;
        left -= t;
    }
    for (size_t i = 0; i < cand.size() && left; ++i)
    {
        const uint64_t t = std::min(cand[i]->chunks_total - cand[i]->chunks_issued - take[i], left);
        take[i] += t;
        left -= t;
    }
    // job tables by group
    r->parts.clear();
    int nj = 0;
    struct G { int off = 0, n = 0; uint64_t chunks = 0; size_t smem = 0; };
    G groups[kGroups];
    std::vector<int> order;
    for (int g = 0; g < kGroups; ++g)
    {
        groups[g].off = nj;
        for (size_t i = 0; i < cand.size(); ++i)
        {
            if (!take[i])
                continue;
            SrvJob* j = cand[i];
            const SrvBuffer& b = *j->buf;
            const int gi = ((b.flame.dims - 1) * 3 + merged_for(b.prog.data())) * 2
                + (b.flame.color_dims > 0);
            if (gi != g)
                continue;
            JobDesc& jd = r->h_jobs[nj++];
            RenderArgs& a = jd.a;
            std::memset(&jd, 0, sizeof jd);
            a.prog = b.d_prog;
            a.prog_bytes = prog_smem_for(b.prog.data());
            a.nxf = (int)b.flame.xforms.size();
            a.color_dims = b.flame.color_dims;
            a.spill = j->spill;
            a.seed = j->seed;
            a.streams = j->S;
            a.samples = j->samples;
            a.traj_len = j->L;
            a.settle = o.settle;
            a.bad_limit = j->bad_limit;
            a.counts = b.d_counts;
            a.hi = j->spill ? b.d_hi : nullptr;
            a.colors = b.d_colors;
            a.stats = j->d_stats;
            a.cancel = d_cancel + j->slot;
            a.rng_words = b.rng_words;
            a.agg = agg_after_search(b.hot_searched);
            a.rsl_words = rsl_words_for(b.prog.data());
            a.merged = merged_for(b.prog.data());
            std::memcpy(a.isaac_init, isaac_init, sizeof a.isaac_init);
            set_geometry(a, b.prog.data(), o.precision);
            jd.chunk_begin = groups[g].chunks;
            jd.chunks = take[i];
            jd.chunk_first = j->chunks_issued;
            groups[g].chunks += take[i];
            groups[g].smem = std::max(groups[g].smem, b.smem);
            // the buffer's hot-cell table, while a chunk (kChunkStreams
            // streams) stays below 2^32 samples (the table's u32 counts)
            const uint64_t ntraj = (j->samples + j->L - 1) / j->L;
            if (b.hot_mult && (long double)((ntraj + j->S - 1) / j->S) * j->L * kChunkStreams
                                  < 4294967296.0L)
            {
                a.hot_keys = b.d_hot;
                a.hot_mult = b.hot_mult;
                a.agg = 0;
                groups[g].smem = std::max(groups[g].smem, b.smem_hot);
                j->hot_cells = b.hot_cells;
            }
            j->last_agg = a.agg;
            groups[g].n += 1;
            j->chunks_issued += take[i];
            r->parts.push_back({j, take[i]});
        }
    }
    BatchHead* hh = reinterpret_cast<BatchHead*>(r->h_jobs + o.max_active);
    for (int g = 0; g < kGroups; ++g)
    {
        hh[g].total_chunks = groups[g].chunks;
        hh[g].cursor = 0;
    }
    // interleaved claim order per group (the round's chunks of many jobs)
    size_t order_off[kGroups] = {};
    size_t order_len = 0;
    {
        std::vector<unsigned long long> counts, ord;
        for (int g = 0; g < kGroups; ++g)
        {
            order_off[g] = order_len;
            if (!groups[g].n)
                continue;
            counts.assign(groups[g].n, 0);
            for (int k = 0; k < groups[g].n; ++k)
                counts[k] = r->h_jobs[groups[g].off + k].chunks;
            interleave_chunks(counts, ord);
            std::memcpy(r->h_order + order_len, ord.data(), ord.size() * sizeof(unsigned long long));
            order_len += ord.size();
        }
    }
    cudaError_t e = cudaStreamWaitEvent(r->stream, ev_alloc, 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(r->d_jobs, r->h_jobs, sizeof(JobDesc) * nj, cudaMemcpyHostToDevice,
                            r->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(r->d_heads, hh, sizeof(BatchHead) * kGroups, cudaMemcpyHostToDevice,
                            r->stream);
    if (e == cudaSuccess && order_len)
        e = cudaMemcpyAsync(r->d_order, r->h_order, order_len * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, r->stream);
    for (int g = 0; g < kGroups && e == cudaSuccess; ++g)
    {
        if (!groups[g].n)
            continue;
        const int dims = g / 6 + 1, merged = (g / 2) % 3, color = g & 1;
        const Launchers& L = launchers(o.precision, dims);
        int bps = 0, block = 0;
        e = L.occ_batch(color, merged, &bps, &block, groups[g].smem);
        if (e != cudaSuccess)
            break;
        if (bps < 1)
        {
            e = cudaErrorInvalidConfiguration;
            break;
        }
        const uint64_t grid = std::min<uint64_t>((uint64_t)sms * bps, groups[g].chunks);
        BatchArgs ba;
        ba.jobs = r->d_jobs + groups[g].off;
        ba.njobs = groups[g].n;
        ba.head = r->d_heads + g;
        ba.order = r->d_order + order_off[g];
        e = L.batch(ba, color, merged, (int)grid, groups[g].smem, r->stream);
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(r->done, r->stream);
    r->busy = true;
    r->started_ns = now_ns();
    next_round = (int)((r - rounds) + 1) % kRoundSlots;
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        finish_round_locked(*r, e, "round launch");
    }
    return true;
}

// Read back a finished job's statistics and mark it done.
void Server::finish_job_locked(SrvJob* j)
{
    SrvBuffer& b = *j->buf;
    struct Head
    {
        unsigned long long s_iter, s_plot, bad_total, dropped, bad_claim;
        unsigned int stop, cancelled;
        unsigned long long ext_lo[kMaxDims], ext_hi[kMaxDims];
    } hs;
    static_assert(sizeof(Head) == offsetof(DevStats, xf_dist), "DevStats head layout");
    const size_t nxf = b.flame.xforms.size();
    std::vector<unsigned long long> dist(nxf);
    cudaError_t e = cudaSuccess;
    std::memset(&hs, 0, sizeof hs);
    if (j->d_stats)
    {
        e = cudaMemcpyAsync(&hs, j->d_stats, sizeof hs, cudaMemcpyDeviceToHost, aux);
        if (e == cudaSuccess && nxf)
            e = cudaMemcpyAsync(dist.data(), j->d_stats->xf_dist, nxf * 8,
                                cudaMemcpyDeviceToHost, aux);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(aux);
        const unsigned long long nrec = std::min<unsigned long long>(hs.bad_claim, kMaxBadRecords);
        if (e == cudaSuccess && nrec)
        {
            j->bad_xf.resize(nrec);
            j->bad_pts.resize(nrec * kMaxDims);
            e = cudaMemcpyAsync(j->bad_xf.data(), j->d_stats->bad_xf, nrec * 8,
                                cudaMemcpyDeviceToHost, aux);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(j->bad_pts.data(), j->d_stats->bad_pts,
                                    nrec * kMaxDims * 8, cudaMemcpyDeviceToHost, aux);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(aux);
        }
        cudaFreeAsync(j->d_stats, aux);
        used.fetch_sub(sizeof(DevStats));
        j->d_stats = nullptr;
    }
    j->s_iter = hs.s_iter;
    j->s_plot = hs.s_plot;
    j->bad_total = hs.bad_total;
    j->dropped = hs.dropped;
    for (int i = 0; i < kMaxDims; ++i)
    {
        j->ext_lo[i] = i < b.flame.dims ? key_to_double(hs.ext_lo[i]) : INFINITY;
        j->ext_hi[i] = i < b.flame.dims ? key_to_double(hs.ext_hi[i]) : -INFINITY;
    }
    j->xf_dist.assign(b.flame.xform_ids, 0);
    for (size_t k = 0; k < nxf; ++k)
        if (b.flame.xforms[k].id < j->xf_dist.size())
            j->xf_dist[b.flame.xforms[k].id] += dist[k];
    if (e != cudaSuccess)
    {
        err = std::string("statistics: ") + cudaGetErrorString(e);
        j->state = FFR_JOB_FAILED;
        j->status = FFR_ERR_CUDA;
    }
    else if (j->cancel_req || hs.cancelled)
    {
        j->state = FFR_JOB_CANCELLED;
        j->status = FFR_ERR_TIMEOUT;
    }
    else
    {
        j->state = FFR_JOB_DONE;
        j->status = hs.stop ? FFR_BAD_VALUES : FFR_OK;
    }
    j->t_done = now_ns();
    b.running -= 1;
    if (j->slot >= 0)
        free_slots.push_back(j->slot);
    j->slot = -1;
    active.erase(std::remove(active.begin(), active.end(), j), active.end());
    cv_done.notify_all();
}

// Account a completed (or failed) round: chunks done, finished jobs.
// Hot-cell table from a buffer holding about sum samples: candidates with at
// least sum/4096 counts each (raising the threshold while more than
// kHotCollectCap qualify), placed by hot_place.  Another round may still be
// adding to the buffer; the collect kernel's relaxed loads see some of its
// counts, which only moves the estimate.  Failures leave the buffer without
// a table (renders do not need one).
void Server::hot_search_locked(SrvBuffer& b, uint64_t sum)
{
    std::vector<unsigned long long> found;
    bool got = false;
    cudaError_t e = collect_hot_candidates(b.d_counts, (unsigned int)b.flame.cells, sum >> 12,
                                           0xFFFFFFFFull, d_hotc, aux, found, &got, nullptr);
    unsigned int mult = 0;
    std::vector<unsigned int> keys;
    if (e != cudaSuccess)
        cudaGetLastError();
    if (!got || !hot_place(found, sum, &mult, keys))
        return;
    const size_t bytes = kHotSlots * sizeof(unsigned int);
    e = pool_alloc(this, &b.d_hot, bytes);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.d_hot, keys.data(), bytes, cudaMemcpyHostToDevice, aux);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(aux);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        if (b.d_hot)
            cudaFreeAsync(b.d_hot, aux);
        b.d_hot = nullptr;
        return;
    }
    b.dev_bytes += bytes;
    add_used(bytes);
    b.hot_mult = mult;
    b.hot_cells = (int)std::count_if(keys.begin(), keys.end(),
                                     [](unsigned int k) { return k != kHotEmpty; });
    b.smem_hot = chaos_smem_bytes<kChunkStreams>(prog_smem_for(b.prog.data()),
                                                 (int)b.flame.xforms.size(),
                                                 rsl_words_for(b.prog.data()), true);
}

void Server::finish_round_locked(RoundSlot& r, cudaError_t e, const std::string& why)
{
    if (e != cudaSuccess)
    {
        err = why + ": " + cudaGetErrorString(e);
        broken = true;
    }
    for (const RoundPart& p : r.parts)
        p.job->chunks_done += p.chunks;
    // a buffer whose job has rounds to go gets its hot-cell table from the
    // counts so far (once per buffer)
    if (e == cudaSuccess)
        for (const RoundPart& p : r.parts)
        {
            SrvJob* j = p.job;
            SrvBuffer& b = *j->buf;
            if (b.hot_searched || !b.allocated || j->state != FFR_JOB_RUNNING
                || j->chunks_issued >= j->chunks_total || b.flame.cells >= (1ull << 30))
                continue;
            b.hot_searched = true;
            const uint64_t sum = (uint64_t)((long double)j->samples * j->chunks_done
                                            / j->chunks_total);
            if (sum >= (1u << 16))
                hot_search_locked(b, sum);
        }
    for (const RoundPart& p : r.parts)
    {
        SrvJob* j = p.job;
        if (j->state != FFR_JOB_RUNNING)
            continue;
        if (e != cudaSuccess)
        {
            j->buf->running -= 1;
            if (j->slot >= 0)
                free_slots.push_back(j->slot);
            j->slot = -1;
            active.erase(std::remove(active.begin(), active.end(), j), active.end());
            fail_job_locked(j, e == cudaErrorNotReady ? FFR_ERR_TIMEOUT : FFR_ERR_CUDA);
            continue;
        }
        const bool all_issued = j->chunks_issued == j->chunks_total || j->cancel_req;
        if (all_issued && j->chunks_done == j->chunks_issued)
            finish_job_locked(j);
    }
    r.parts.clear();
    r.busy = false;
}

void Server::loop()
{
    cudaSetDevice(o.device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;)
    {
        if (!stop)
            admit_locked();
        // cancelled running jobs with nothing in flight finish here
        for (size_t i = 0; i < active.size();)
        {
            SrvJob* j = active[i];
            if (j->cancel_req && j->chunks_done == j->chunks_issued)
                finish_job_locked(j);
            else
                ++i;
        }
        while (!stop && launch_round_locked())
        {
        }
        RoundSlot* oldest = nullptr;
        for (RoundSlot& r : rounds)
            if (r.busy && (!oldest || r.started_ns < oldest->started_ns))
                oldest = &r;
        if (!oldest)
        {
            if (stop)
                break;
            cv_work.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        // wait for the oldest round without holding the lock
        const uint64_t limit = o.timeout_ms;
        const uint64_t t0 = now_ns();
        cudaError_t q;
        bool cancelled = false;
        lk.unlock();
        for (;;)
        {
            q = cudaEventQuery(oldest->done);
            if (q != cudaErrorNotReady)
                break;
            const uint64_t ms = (now_ns() - t0) / 1000000ull;
            if (limit && !cancelled && ms >= limit)
            {
                // ask the round's kernels to stop (they poll every 4096 samples)
                for (const RoundPart& p : oldest->parts)
                    if (p.job->slot >= 0)
                        ((volatile unsigned int*)h_cancel)[p.job->slot] = 1u;
                cancelled = true;
            }
            if (limit && ms >= 2 * limit + 1000)
                break;
            std::this_thread::sleep_for(std::chrono::microseconds(100));
        }
        lk.lock();
        if (q == cudaErrorNotReady)
        {
            // the device did not stop: nothing of this round can be reused
            err = "round did not finish after cancel";
            broken = true;
            for (const RoundPart& p : oldest->parts)
                if (p.job->state == FFR_JOB_RUNNING)
                {
                    p.job->state = FFR_JOB_FAILED;
                    p.job->status = FFR_ERR_TIMEOUT;
                    p.job->t_done = now_ns();
                }
            cv_done.notify_all();
            break;
        }
        if (cancelled && q == cudaSuccess)
            for (const RoundPart& p : oldest->parts)
                p.job->cancel_req = true;
        finish_round_locked(*oldest, q, "round");
        if (broken)
        {
            // nothing more is launched: let the other round drain (bounded),
            // then fail every job still waiting or running
            for (RoundSlot& r : rounds)
            {
                if (!r.busy)
                    continue;
                const uint64_t t1 = now_ns();
                lk.unlock();
                while (cudaEventQuery(r.done) == cudaErrorNotReady
                       && now_ns() - t1 < 5000000000ull)
                    std::this_thread::sleep_for(std::chrono::microseconds(200));
                lk.lock();
                r.parts.clear();
                r.busy = false;
            }
            for (SrvJob* j : queue)
                fail_job_locked(j, FFR_ERR_CUDA);
            queue.clear();
            for (SrvJob* j : active)
                if (j->state == FFR_JOB_RUNNING)
                    fail_job_locked(j, FFR_ERR_CUDA);
            active.clear();
            break;
        }
    }
}

Server* as_server(ffr_server* s) { return reinterpret_cast<Server*>(s); }

void server_free(Server* s)
{
    if (!s)
        return;
    cudaSetDevice(s->o.device);
    s->jobs.clear();        // drops buffer references (frees on aux)
    for (RoundSlot& r : s->rounds)
    {
        if (r.stream)
            cudaStreamSynchronize(r.stream);
        cudaFree(r.d_jobs);
        if (r.h_jobs)
            cudaFreeHost(r.h_jobs);
        cudaFree(r.d_order);
        if (r.h_order)
            cudaFreeHost(r.h_order);
        if (r.done)
            cudaEventDestroy(r.done);
        if (r.stream)
            cudaStreamDestroy(r.stream);
    }
    for (auto& r : s->readers)
    {
        if (r.stream)
        {
            cudaStreamSynchronize(r.stream);
            cudaStreamDestroy(r.stream);
        }
        cudaFree(r.d_stage);
        for (int k = 0; k < 2; ++k)
        {
            if (r.h_stage[k])
                cudaFreeHost(r.h_stage[k]);
            if (r.ev[k])
                cudaEventDestroy(r.ev[k]);
        }
    }
    if (s->aux)
    {
        cudaStreamSynchronize(s->aux);
        cudaStreamDestroy(s->aux);
    }
    if (s->ev_alloc)
        cudaEventDestroy(s->ev_alloc);
    cudaFree(s->d_red);
    if (s->h_cancel)
        cudaFreeHost(s->h_cancel);
    if (s->pool)
        cudaMemPoolDestroy(s->pool);
    delete s;
}

SrvJob* find_job(Server* s, uint64_t id)
{
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second.get();
}

bool terminal(int state)
{
    return state == FFR_JOB_DONE || state == FFR_JOB_FAILED || state == FFR_JOB_CANCELLED;
}

void fill_info(const SrvJob* j, ffr_job_info* info)
{
    if (!info)
        return;
    std::memset(info, 0, sizeof *info);
    info->state = j->state;
    info->status = j->status;
    info->samples = j->samples;
    info->buffer_bytes = j->buf->file_bytes();
    info->parent = j->parent;
    info->submit_ns = j->t_submit;
    info->admit_ns = j->t_admit;
    info->done_ns = j->t_done;
}

// queue a job on buffer b (new or continued); called with the lock held
ffr_status enqueue_locked(Server* s, std::shared_ptr<SrvBuffer> b, uint64_t parent,
                          uint64_t samples, uint64_t seed, uint64_t bad_limit, uint64_t* id)
{
    std::unique_ptr<SrvJob> j(new (std::nothrow) SrvJob);
    if (!j)
    {
        s->err = "out of host memory";
        return FFR_ERR_OOM;
    }
    j->id = s->next_id++;
    j->parent = parent;
    j->buf = std::move(b);
    j->samples = samples;
    j->seed = seed;
    j->bad_limit = bad_limit;
    j->L = s->o.traj_len;
    j->S = samples ? (samples + j->L - 1) / j->L : 0;
    j->chunks_total = (j->S + kChunkStreams - 1) / kChunkStreams;
    j->t_submit = now_ns();
    for (int i = 0; i < kMaxDims; ++i)
    {
        j->ext_lo[i] = INFINITY;
        j->ext_hi[i] = -INFINITY;
    }
    *id = j->id;
    s->queue.push_back(j.get());
    s->jobs.emplace(j->id, std::move(j));
    s->cv_work.notify_all();
    return FFR_OK;
}

} // namespace

extern "C" {

void ffr_server_default_opts(ffr_server_opts* o)
{
    if (!o)
        return;
    std::memset(o, 0, sizeof *o);
    o->abi_version = FFR_ABI_VERSION;
    o->device = 0;
    o->precision = FFR_FP32;
    o->settle = 53;
    o->traj_len = 4096;
    o->max_active = 256;
}

ffr_status ffr_server_create(const ffr_server_opts* opts, ffr_server** out)
{
    if (!out)
        return sfail(nullptr, FFR_ERR_ARG, "ffr_server_create: out is NULL");
    *out = nullptr;
    ffr_server_opts o;
    if (opts)
        o = *opts;
    else
        ffr_server_default_opts(&o);
    if (o.abi_version != FFR_ABI_VERSION)
        return sfail(nullptr, FFR_ERR_ARG, "ffr_server_create: ABI version mismatch");
    if (o.precision != FFR_FP64 && o.precision != FFR_FP32)
        return sfail(nullptr, FFR_ERR_ARG, "ffr_server_create: unknown precision");
    if (!o.traj_len)
        o.traj_len = 4096;
    if (o.traj_len >= (1ull << 31))
        return sfail(nullptr, FFR_ERR_ARG, "ffr_server_create: traj_len must be below 2^31");
    if (!o.max_active)
        o.max_active = 256;
    if (o.max_active > 65536)
        return sfail(nullptr, FFR_ERR_ARG, "ffr_server_create: max_active above 65536");
    Server* s = new (std::nothrow) Server;
    if (!s)
        return sfail(nullptr, FFR_ERR_OOM, "out of host memory");
    s->o = o;
    auto cfail = [&](cudaError_t e, const char* what) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(e);
        server_free(s);
        return sfail(nullptr, FFR_ERR_CUDA, m);
    };
    cudaError_t e;
    if ((e = cudaSetDevice(o.device)) != cudaSuccess)
        return cfail(e, "cudaSetDevice");
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, o.device);
    isaac_init_table(s->isaac_init);
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof pp);
    pp.allocType = cudaMemAllocationTypePinned;
    pp.handleTypes = cudaMemHandleTypeNone;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = o.device;
    if ((e = cudaMemPoolCreate(&s->pool, &pp)) != cudaSuccess)
        return cfail(e, "cudaMemPoolCreate");
    uint64_t keep = ~0ull;      // keep freed blocks for reuse
    if ((e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
        return cfail(e, "cudaMemPoolSetAttribute");
    if ((e = cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking)) != cudaSuccess
            )
        return cfail(e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&s->ev_alloc, cudaEventDisableTiming)) != cudaSuccess)
        return cfail(e, "cudaEventCreate");
    if ((e = cudaEventRecord(s->ev_alloc, s->aux)) != cudaSuccess)
        return cfail(e, "cudaEventRecord");
    if ((e = cudaMalloc(&s->d_red, (4 + 1 + kHotCollectCap) * sizeof(unsigned long long)))
            != cudaSuccess)
        return cfail(e, "cudaMalloc(reduction)");
    s->d_hotc = s->d_red + 4;
    if ((e = cudaHostAlloc(&s->h_cancel, sizeof(unsigned int) * o.max_active,
                           cudaHostAllocMapped)) != cudaSuccess)
        return cfail(e, "cudaHostAlloc(cancel flags)");
    std::memset(s->h_cancel, 0, sizeof(unsigned int) * o.max_active);
    if ((e = cudaHostGetDevicePointer(&s->d_cancel, s->h_cancel, 0)) != cudaSuccess)
        return cfail(e, "cudaHostGetDevicePointer");
    for (int k = (int)o.max_active - 1; k >= 0; --k)
        s->free_slots.push_back(k);
    const size_t table = sizeof(JobDesc) * o.max_active + sizeof(BatchHead) * kGroups;
    for (RoundSlot& r : s->rounds)
    {
        if ((e = cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return cfail(e, "cudaStreamCreate");
        if ((e = cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming)) != cudaSuccess)
            return cfail(e, "cudaEventCreate");
        if ((e = cudaMalloc(&r.d_jobs, table)) != cudaSuccess)
            return cfail(e, "cudaMalloc(job table)");
        r.d_heads = reinterpret_cast<BatchHead*>(r.d_jobs + o.max_active);
        if ((e = cudaHostAlloc(&r.h_jobs, table, 0)) != cudaSuccess)
            return cfail(e, "cudaHostAlloc(job table)");
        // the largest round: round_chunks, or two chunks for each of up to 16
        // resident CTAs per SM
        r.order_cap = std::max<size_t>(o.round_chunks, 2 * (size_t)s->sms * 16);
        if ((e = cudaMalloc(&r.d_order, r.order_cap * sizeof(unsigned long long))) != cudaSuccess)
            return cfail(e, "cudaMalloc(claim order)");
        if ((e = cudaHostAlloc(&r.h_order, r.order_cap * sizeof(unsigned long long), 0)) != cudaSuccess)
            return cfail(e, "cudaHostAlloc(claim order)");
    }
    size_t fr = 0, tot = 0;
    if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess)
        return cfail(e, "cudaMemGetInfo");
    const uint64_t reserve = 2ull << 30;
    const uint64_t avail = fr > reserve ? fr - reserve : 0;
    s->budget = o.hbm_budget ? std::min<uint64_t>(o.hbm_budget, avail) : avail;
    if (s->budget < kStagingBytes * kReadSlots)
        return cfail(cudaErrorMemoryAllocation, "device-memory budget below the read staging");
    for (auto& r : s->readers)
    {
        if ((e = cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return cfail(e, "cudaStreamCreate");
        if ((e = cudaMalloc(&r.d_stage, kStagingBytes)) != cudaSuccess)
            return cfail(e, "cudaMalloc(read staging)");
        for (int k = 0; k < 2; ++k)
        {
            if ((e = cudaHostAlloc(&r.h_stage[k], kStagingBytes, 0)) != cudaSuccess)
                return cfail(e, "cudaHostAlloc(read staging)");
            if ((e = cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming)) != cudaSuccess)
                return cfail(e, "cudaEventCreate");
        }
        s->add_used(kStagingBytes);
    }
    try
    {
        s->thread = std::thread([s] { s->loop(); });
    }
    catch (const std::exception& ex)
    {
        server_free(s);
        return sfail(nullptr, FFR_ERR_ARG, std::string("scheduler thread: ") + ex.what());
    }
    *out = reinterpret_cast<ffr_server*>(s);
    return FFR_OK;
}

void ffr_server_destroy(ffr_server* srv)
{
    Server* s = as_server(srv);
    if (!s)
        return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (SrvJob* j : s->queue)
        {
            j->state = FFR_JOB_CANCELLED;
            j->status = FFR_ERR_TIMEOUT;
        }
        s->queue.clear();
        s->cv_done.notify_all();
        for (SrvJob* j : s->active)
        {
            j->cancel_req = true;
            if (j->slot >= 0)
                ((volatile unsigned int*)s->h_cancel)[j->slot] = 1u;
        }
        s->cv_work.notify_all();
    }
    if (s->thread.joinable())
        s->thread.join();
    server_free(s);
}

const char* ffr_server_last_error(const ffr_server* srv)
{
    Server* s = reinterpret_cast<Server*>(const_cast<ffr_server*>(srv));
    if (!s)
        return g_server_error.c_str();
    // a copy per calling thread: other threads may set the message meanwhile
    thread_local std::string copy;
    std::lock_guard<std::mutex> lk(s->mu);
    copy = s->err;
    return copy.c_str();
}

ffr_status ffr_server_submit(ffr_server* srv, const char* json, size_t len, const void* init,
                             size_t init_bytes, uint64_t samples, uint64_t seed,
                             uint64_t bad_limit, uint64_t* job)
{
    Server* s = as_server(srv);
    if (!s || !json || !job)
        return sfail(s, FFR_ERR_ARG, "ffr_server_submit: NULL argument");
    *job = 0;
    auto b = std::make_shared<SrvBuffer>();
    try
    {
        b->flame = parse_flame(std::string(json, len));
        b->prog = s->o.precision == FFR_FP64 ? build_program<double>(b->flame)
                                             : build_program<float>(b->flame);
    }
    catch (const std::exception& ex)
    {
        return sfail(s, FFR_ERR_PARSE, ex.what());
    }
    if (b->flame.xforms.size() > (size_t)kMaxXformIds)
        return sfail(s, FFR_ERR_ARG, "too many xforms");
    if (b->flame.dims > 3)
        return sfail(s, FFR_ERR_ARG, "the serving loop renders 1- to 3-dimensional flames "
                                     "(render 4-D flames with ffr_render)");
    {
        const ProgHeader<double>* h = reinterpret_cast<const ProgHeader<double>*>(b->prog.data());
        b->rng_words = (int)h->rng_words_max;   // same offset in the float header
    }
    if (init)
    {
        if (init_bytes < b->file_bytes())
            return sfail(s, FFR_ERR_IO, "error reading file");
        b->init.resize(b->file_bytes() / 8);
        std::memcpy(b->init.data(), init, b->file_bytes());
    }
    b->smem = chaos_smem_bytes<kChunkStreams>(prog_smem_for(b->prog.data()),
                                              (int)b->flame.xforms.size(),
                                              rsl_words_for(b->prog.data()));
    const uint64_t need = kStagingBytes * kReadSlots + b->prog.size() + b->counts_bytes()
        + b->colors_bytes()
        + sizeof(DevStats) + (init ? b->file_bytes() : 0);
    if (need > s->budget)
        return sfail(s, FFR_ERR_OOM, "buffer needs " + std::to_string(need)
            + " bytes of device memory, server budget " + std::to_string(s->budget));
    b->srv = s;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->broken || s->stop)
    {
        b->srv = nullptr;
        s->err = "server stopped: " + s->err;
        return FFR_ERR_STATE;
    }
    return enqueue_locked(s, std::move(b), 0, samples, seed, bad_limit, job);
}

ffr_status ffr_server_continue(ffr_server* srv, uint64_t parent, uint64_t samples,
                               uint64_t seed, uint64_t bad_limit, uint64_t* job)
{
    Server* s = as_server(srv);
    if (!s || !job)
        return sfail(s, FFR_ERR_ARG, "ffr_server_continue: NULL argument");
    *job = 0;
    std::lock_guard<std::mutex> lk(s->mu);
    SrvJob* p = find_job(s, parent);
    if (!p)
    {
        s->err = "no job " + std::to_string(parent);
        return FFR_ERR_ARG;
    }
    if (s->broken || s->stop)
    {
        s->err = "server stopped: " + s->err;
        return FFR_ERR_STATE;
    }
    return enqueue_locked(s, p->buf, parent, samples, seed, bad_limit, job);
}

ffr_status ffr_server_poll(ffr_server* srv, uint64_t job, ffr_job_info* info)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    SrvJob* j = find_job(s, job);
    if (!j)
    {
        s->err = "no job " + std::to_string(job);
        return FFR_ERR_ARG;
    }
    fill_info(j, info);
    return FFR_OK;
}

ffr_status ffr_server_wait(ffr_server* srv, uint64_t job, uint64_t timeout_ms,
                           ffr_job_info* info)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto until = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;)
    {
        SrvJob* j = find_job(s, job);
        if (!j)
        {
            s->err = "no job " + std::to_string(job);
            return FFR_ERR_ARG;
        }
        if (terminal(j->state))
        {
            fill_info(j, info);
            return FFR_OK;
        }
        if (timeout_ms)
        {
            if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout)
            {
                j = find_job(s, job);
                if (j && terminal(j->state))
                    continue;
                if (j)
                    fill_info(j, info);
                s->err = "job " + std::to_string(job) + " not finished within timeout";
                return FFR_ERR_TIMEOUT;
            }
        }
        else
            s->cv_done.wait(lk);
    }
}

ffr_status ffr_server_job_stats(ffr_server* srv, uint64_t job, ffr_stats* st)
{
    Server* s = as_server(srv);
    if (!s || !st)
        return FFR_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    SrvJob* j = find_job(s, job);
    if (!j)
    {
        s->err = "no job " + std::to_string(job);
        return FFR_ERR_ARG;
    }
    if (!terminal(j->state))
    {
        s->err = "job " + std::to_string(job) + " has not finished";
        return FFR_ERR_STATE;
    }
    std::memset(st, 0, sizeof *st);
    st->samples_iterated = j->s_iter;
    st->samples_plotted = j->s_plot;
    st->bad_values = j->bad_total;
    st->dropped = j->dropped;
    for (int i = 0; i < FFR_MAX_DIMS; ++i)
    {
        st->ext_lo[i] = j->ext_lo[i];
        st->ext_hi[i] = j->ext_hi[i];
    }
    st->xform_ids = j->buf->flame.xform_ids;
    for (size_t k = 0; k < j->xf_dist.size() && k < FFR_MAX_XFORM_IDS; ++k)
        st->xf_dist[k] = j->xf_dist[k];
    st->bad_recorded = j->bad_xf.size();
    for (size_t k = 0; k < j->bad_xf.size(); ++k)
    {
        st->bad_xf[k] = j->bad_xf[k];
        for (int i = 0; i < FFR_MAX_DIMS; ++i)
            st->bad_pts[k][i] = j->bad_pts[k * kMaxDims + i];
    }
    st->streams = j->S;
    st->traj_len = j->L;
    st->settle = s->o.settle;
    st->kernel_ms = j->t_done > j->t_submit ? (j->t_done - j->t_submit) * 1e-6 : 0.0;
    st->kernel = FFR_KERNEL_PLAIN;
    st->agg = j->last_agg;
    st->hot_cells = j->hot_cells;
    return j->status;
}

ffr_status ffr_server_read(ffr_server* srv, uint64_t job, void* cells, size_t bytes)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::shared_ptr<SrvBuffer> b;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        SrvJob* j = find_job(s, job);
        if (!j)
        {
            s->err = "no job " + std::to_string(job);
            return FFR_ERR_ARG;
        }
        b = j->buf;
        if (!b->allocated)
        {
            s->err = "job " + std::to_string(job) + " has no buffer on the device yet";
            return FFR_ERR_STATE;
        }
    }
    const size_t need = b->file_bytes();
    if (!cells || bytes < need)
        return sfail(s, FFR_ERR_IO, "error writing output: destination too small");
    // a free read slot
    Server::ReadSlot* r = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->rd_mu);
        for (;;)
        {
            for (auto& x : s->readers)
                if (!x.busy)
                {
                    r = &x;
                    break;
                }
            if (r)
                break;
            s->rd_cv.wait(lk);
        }
        r->busy = true;
    }
    cudaSetDevice(s->o.device);
    const size_t words = 1 + (size_t)b->flame.color_dims;
    const uint64_t step = std::max<uint64_t>(1, kStagingBytes / 8 / words);
    const uint64_t nslices = (b->flame.cells + step - 1) / step;
    unsigned char* dst = static_cast<unsigned char*>(cells);
    auto slice_cells = [&](uint64_t k) { return std::min<uint64_t>(step, b->flame.cells - k * step); };
    cudaError_t e = cudaStreamWaitEvent(r->stream, s->ev_alloc, 0);
    for (uint64_t k = 0; k <= nslices && e == cudaSuccess; ++k)
    {
        if (k < nslices)
        {
            // slice k: export, DMA into pinned buffer k % 2 (its previous
            // slice, k - 2, was copied out in the previous iteration)
            const uint64_t c0 = k * step, n = slice_cells(k);
            e = launch_export(r->d_stage, n, b->flame.color_dims, b->d_counts + c0,
                              b->d_hi ? b->d_hi + c0 : nullptr,
                              b->d_colors ? b->d_colors + c0 * b->flame.color_dims : nullptr,
                              r->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(r->h_stage[k & 1], r->d_stage, n * words * 8,
                                    cudaMemcpyDeviceToHost, r->stream);
            if (e == cudaSuccess)
                e = cudaEventRecord(r->ev[k & 1], r->stream);
        }
        if (k >= 1 && e == cudaSuccess)
        {
            // slice k - 1 to the caller while slice k is in flight
            const uint64_t j = k - 1;
            e = cudaEventSynchronize(r->ev[j & 1]);
            if (e == cudaSuccess)
                std::memcpy(dst + j * step * words * 8, r->h_stage[j & 1],
                            slice_cells(j) * words * 8);
        }
    }
    if (e != cudaSuccess)
        cudaStreamSynchronize(r->stream);
    {
        std::lock_guard<std::mutex> lk(s->rd_mu);
        r->busy = false;
    }
    s->rd_cv.notify_one();
    if (e != cudaSuccess)
        return sfail(s, FFR_ERR_CUDA, std::string("read: ") + cudaGetErrorString(e));
    return FFR_OK;
}

ffr_status ffr_server_cancel(ffr_server* srv, uint64_t job)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    SrvJob* j = find_job(s, job);
    if (!j)
    {
        s->err = "no job " + std::to_string(job);
        return FFR_ERR_ARG;
    }
    if (terminal(j->state))
        return FFR_OK;
    j->cancel_req = true;
    if (j->state == FFR_JOB_QUEUED)
    {
        s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), j), s->queue.end());
        j->state = FFR_JOB_CANCELLED;
        j->status = FFR_ERR_TIMEOUT;
        j->t_done = now_ns();
        s->cv_done.notify_all();
        return FFR_OK;
    }
    if (j->slot >= 0)
        ((volatile unsigned int*)s->h_cancel)[j->slot] = 1u;
    s->cv_work.notify_all();
    return FFR_OK;
}

ffr_status ffr_server_release(ffr_server* srv, uint64_t job)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::unique_ptr<SrvJob> gone;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job);
        if (it == s->jobs.end())
        {
            s->err = "no job " + std::to_string(job);
            return FFR_ERR_ARG;
        }
        if (!terminal(it->second->state))
        {
            s->err = "job " + std::to_string(job) + " is still queued or running";
            return FFR_ERR_STATE;
        }
        gone = std::move(it->second);
        s->jobs.erase(it);
    }
    cudaSetDevice(s->o.device);
    gone.reset();           // frees the buffer when this was its last job
    std::lock_guard<std::mutex> lk(s->mu);
    s->cv_work.notify_all();    // memory may have been freed for the queue head
    return FFR_OK;
}

ffr_status ffr_server_load(ffr_server* srv, uint64_t* queued, uint64_t* running,
                           uint64_t* bytes_used, uint64_t* bytes_peak)
{
    Server* s = as_server(srv);
    if (!s)
        return FFR_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (queued) *queued = s->queue.size();
    if (running) *running = s->active.size();
    if (bytes_used) *bytes_used = s->used.load();
    if (bytes_peak) *bytes_peak = s->peak.load();
    return s->broken ? FFR_ERR_CUDA : FFR_OK;
}

} // extern "C"
