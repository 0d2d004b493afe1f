// ffr_render_noalloc: a render that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc themselves or let a
// library do so -- for example a host application whose device memory is
// owned by another allocator (a framework's caching pool, a pre-sized arena
// on an embedded deployment) and that must not have a second allocator
// competing for the same GPU memory or fragmenting it.  They hand in a count
// buffer they already own; this entry point renders into it.
//
// How: the two pieces of device scratch the render kernel needs besides the
// caller's buffers -- the copy of the flame program it reads every sample and
// the statistics/coordination block it updates (sample counters, bad-value
// counter and stop flag, extremes, per-xform counts, bad-value records) --
// live in one file-scope __device__ array, kNoAllocScratchBytes long.  Every
// GPU that loads this library holds that array until the process exits.
// The kernel is the same render kernel ffr_render launches.
#include "ffr_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "flame.hpp"
#include "launch.h"

namespace ffr {

namespace {

// largest flame program this entry point accepts (ffr_create takes up to
// kMaxProgramBytes); a 2-D flame of about 40 xforms with one variation each
constexpr size_t kNoAllocProgramBytes = 16 * 1024;
constexpr size_t kStatsOffset = kNoAllocProgramBytes;
constexpr size_t kNoAllocScratchBytes =
    kStatsOffset + ((sizeof(DevStats) + 255) / 256) * 256;
constexpr int kMaxDevices = 64;

// Device scratch shared by every call on a device: [program | DevStats].
// In host code this name is only a stand-in for the symbol; the device
// address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// the leading fields of DevStats (everything before xf_dist), copied on
// their own so no 160 KB host copy of the whole block is needed
struct StatsHead
{
    unsigned long long s_iter, s_plot, bad_total, dropped, bad_claim;
    unsigned int stop, cancelled;
    unsigned long long ext_lo[kMaxDims], ext_hi[kMaxDims];
};
static_assert(sizeof(StatsHead) == offsetof(DevStats, xf_dist), "DevStats head layout");
static_assert(offsetof(StatsHead, ext_lo) == offsetof(DevStats, ext_lo), "DevStats head layout");
static_assert(offsetof(StatsHead, stop) == offsetof(DevStats, stop), "DevStats head layout");

// errors are reported through ffr_last_error(NULL), like ffr_create's
ffr_status nofail(ffr_status s, const std::string& m)
{
    set_global_error(m);
    return s;
}

ffr_status nocuda(cudaError_t e, const char* where)
{
    return nofail(FFR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// once per device, with that device current
ffr_status scratch_for(int device, unsigned char** out)
{
    if (device < 0 || device >= kMaxDevices)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[device])
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return nocuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_ptr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
    return FFR_OK;
}

// a caller buffer must be device (or managed) memory of the render's device:
// the kernel dereferences it there
ffr_status device_buffer(const void* p, int device, const char* name)
{
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return nocuda(e, (std::string("ffr_render_noalloc: ") + name).c_str());
    }
    if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
            || (at.type == cudaMemoryTypeDevice && at.device != device))
        return nofail(FFR_ERR_ARG, std::string("ffr_render_noalloc: ") + name
            + " is not device memory of device " + std::to_string(device));
    return FFR_OK;
}

void pick_launchers(int precision, int dims, RenderFn* r, OccFn* o)
{
    static const RenderFn rf[2][4] = {
        {launch_render_p0_d1, launch_render_p0_d2, launch_render_p0_d3, launch_render_p0_d4},
        {launch_render_p1_d1, launch_render_p1_d2, launch_render_p1_d3, launch_render_p1_d4}};
    static const OccFn of[2][4] = {
        {occupancy_p0_d1, occupancy_p0_d2, occupancy_p0_d3, occupancy_p0_d4},
        {occupancy_p1_d1, occupancy_p1_d2, occupancy_p1_d3, occupancy_p1_d4}};
    *r = rf[precision][dims - 1];
    *o = of[precision][dims - 1];
}

} // namespace

} // namespace ffr

using namespace ffr;

extern "C" ffr_status ffr_render_noalloc(const char* json, size_t len, const ffr_opts* opts,
                                         uint32_t* d_counts, double* d_colors,
                                         uint64_t cells, uint64_t samples, uint64_t seed,
                                         uint64_t bad_limit, ffr_stats* stats)
{
    if (!json || !d_counts)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: json and d_counts are required");
    ffr_opts o;
    if (opts)
        o = *opts;
    else
        ffr_default_opts(&o);
    if (o.abi_version != FFR_ABI_VERSION
            || (o.precision != FFR_FP64 && o.precision != FFR_FP32))
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: bad options");
    // the autotuner, the xform-sorted kernel and the hot-cell search all need
    // device memory of their own, and a bounded wait needs a mapped cancel
    // flag: this entry point runs the plain kernel and waits until it ends
    if (o.kernel != FFR_KERNEL_AUTO && o.kernel != FFR_KERNEL_PLAIN)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: only the plain kernel runs here "
                                   "(opts.kernel must be FFR_KERNEL_AUTO or FFR_KERNEL_PLAIN)");
    if (o.timeout_ms != 0)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: no bounded wait here "
                                   "(opts.timeout_ms must be 0)");
    if (samples > 0xFFFFFFFFull)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: at most 2^32-1 samples per call "
                                   "(u32 cells, no high-word buffer)");
    HostFlame f;
    std::vector<uint8_t> prog;
    try
    {
        f = parse_flame(std::string(json, len));
        prog = o.precision == FFR_FP64 ? build_program<double>(f) : build_program<float>(f);
    }
    catch (const std::exception& e)
    {
        return nofail(FFR_ERR_PARSE, e.what());
    }
    if (prog.size() > kNoAllocProgramBytes)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: flame program is "
            + std::to_string(prog.size()) + " bytes; this entry point's device scratch holds "
            + std::to_string(kNoAllocProgramBytes) + " (use ffr_create/ffr_render)");
    if (cells != f.cells)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: cells " + std::to_string(cells)
            + " does not match the flame's buffer (" + std::to_string(f.cells) + ")");
    if (f.color_dims > 0 && !d_colors)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: colour flame needs d_colors");
    if (stats)
    {
        std::memset(stats, 0, sizeof *stats);
        for (int i = 0; i < FFR_MAX_DIMS; ++i)
        {
            stats->ext_lo[i] = INFINITY;
            stats->ext_hi[i] = -INFINITY;
        }
        stats->xform_ids = f.xform_ids;
        stats->settle = o.settle;
    }
    if (samples == 0)
        return FFR_OK;
    cudaError_t e;
    ffr_status s0;
    if ((e = cudaSetDevice(o.device)) != cudaSuccess)
        return nocuda(e, "cudaSetDevice");
    if ((s0 = device_buffer(d_counts, o.device, "d_counts")) != FFR_OK)
        return s0;
    if (f.color_dims > 0 && (s0 = device_buffer(d_colors, o.device, "d_colors")) != FFR_OK)
        return s0;
    unsigned char* scratch = nullptr;
    ffr_status s = scratch_for(o.device, &scratch);
    if (s != FFR_OK)
        return s;
    DevStats* dstats = reinterpret_cast<DevStats*>(scratch + kStatsOffset);
    RenderFn render;
    OccFn occ;
    pick_launchers(o.precision, f.dims, &render, &occ);
    const int nxf = (int)f.xforms.size();
    int bps = 0, block = 0, sms = 1;
    size_t smem = 0;
    if ((e = occ(f.color_dims > 0, merged_for(prog.data()), rsl_words_for(prog.data()), 0,
                 &bps, &block,
                 prog_smem_for(prog.data()), nxf, &smem))
            != cudaSuccess)
        return nocuda(e, "occupancy");
    if (bps < 1)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: render kernel does not fit on an SM");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device);
    const uint64_t S = o.streams ? o.streams : (uint64_t)sms * bps * block;
    const uint64_t L = o.traj_len ? o.traj_len : std::max<uint64_t>(1, (samples + S - 1) / S);
    const uint64_t ntraj = (samples + L - 1) / L;
    const uint64_t active = S < ntraj ? S : ntraj;
    uint64_t blocks = (active + block - 1) / block;
    if (blocks > (uint64_t)sms * bps)
        blocks = (uint64_t)sms * bps;
    if (blocks < 1)
        blocks = 1;
    const uint64_t per_thread = ((active + blocks * block - 1) / (blocks * block))
        * ((ntraj + S - 1) / S) * L;
    if (per_thread >= 0xFFFFFFFFull)
        return nofail(FFR_ERR_ARG, "ffr_render_noalloc: too many samples per GPU thread");
    // every call reuses the scratch: copy the program, zero the statistics
    StatsHead head;
    std::memset(&head, 0, sizeof head);
    for (int i = 0; i < kMaxDims; ++i)
    {
        head.ext_lo[i] = order_key(INFINITY);
        head.ext_hi[i] = order_key(-INFINITY);
    }
    cudaStream_t st = 0;
    if ((e = cudaMemcpyAsync(scratch, prog.data(), prog.size(), cudaMemcpyHostToDevice, st))
            != cudaSuccess)
        return nocuda(e, "cudaMemcpy(program)");
    if ((e = cudaMemcpyAsync(dstats, &head, sizeof head, cudaMemcpyHostToDevice, st))
            != cudaSuccess)
        return nocuda(e, "cudaMemcpy(stats)");
    if ((e = cudaMemsetAsync(dstats->xf_dist, 0, sizeof(unsigned long long) * nxf, st))
            != cudaSuccess)
        return nocuda(e, "cudaMemset(stats)");
    RenderArgs a;
    std::memset(&a, 0, sizeof a);
    a.prog = scratch;
    a.prog_bytes = prog_smem_for(prog.data());
    a.nxf = nxf;
    a.color_dims = f.color_dims;
    a.spill = 0;
    a.seed = seed;
    a.streams = S;
    a.samples = samples;
    a.traj_len = L;
    a.settle = o.settle;
    a.bad_limit = bad_limit;
    a.counts = d_counts;
    a.hi = nullptr;
    a.colors = d_colors;
    a.stats = dstats;
    a.cancel = nullptr;
    a.rsl_words = rsl_words_for(prog.data());
    a.merged = merged_for(prog.data());
    isaac_init_table(a.isaac_init);
    set_geometry(a, prog.data(), o.precision);
    const auto t0 = std::chrono::steady_clock::now();
    if ((e = render(a, (int)blocks, st)) != cudaSuccess)
        return nocuda(e, "render launch");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
        return nocuda(e, "render");
    const double wall_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if ((e = cudaMemcpy(&head, dstats, sizeof head, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return nocuda(e, "cudaMemcpy(stats)");
    if (stats)
    {
        std::vector<unsigned long long> dist(nxf);
        if ((e = cudaMemcpy(dist.data(), dstats->xf_dist, sizeof(unsigned long long) * nxf,
                            cudaMemcpyDeviceToHost)) != cudaSuccess)
            return nocuda(e, "cudaMemcpy(stats)");
        const unsigned long long nrec =
            head.bad_claim < (unsigned long long)kMaxBadRecords ? head.bad_claim : kMaxBadRecords;
        // the kernel writes a record's first dims coordinates only: the
        // others hold whatever an earlier call on this device left there
        std::vector<double> pts(kMaxDims * nrec);
        if (nrec && ((e = cudaMemcpy(stats->bad_xf, dstats->bad_xf, 8 * nrec,
                                     cudaMemcpyDeviceToHost)) != cudaSuccess
                     || (e = cudaMemcpy(pts.data(), dstats->bad_pts, 8 * kMaxDims * nrec,
                                        cudaMemcpyDeviceToHost)) != cudaSuccess))
            return nocuda(e, "cudaMemcpy(stats)");
        for (unsigned long long k = 0; k < nrec; ++k)
            for (int i = 0; i < f.dims; ++i)
                stats->bad_pts[k][i] = pts[k * kMaxDims + i];
        stats->samples_iterated = head.s_iter;
        stats->samples_plotted = head.s_plot;
        stats->bad_values = head.bad_total;
        stats->dropped = head.dropped;
        for (int i = 0; i < f.dims; ++i)
        {
            stats->ext_lo[i] = key_to_double(head.ext_lo[i]);
            stats->ext_hi[i] = key_to_double(head.ext_hi[i]);
        }
        for (int k = 0; k < nxf; ++k)
            if (f.xforms[k].id < FFR_MAX_XFORM_IDS)
                stats->xf_dist[f.xforms[k].id] += dist[k];
        stats->bad_recorded = nrec;
        stats->streams = S;
        stats->traj_len = L;
        stats->kernel = FFR_KERNEL_PLAIN;
        stats->kernel_ms = wall_ms;
    }
    if (head.stop)
        return nofail(FFR_BAD_VALUES, "render failure (flame may not be sufficiently contractive)");
    return FFR_OK;
}
