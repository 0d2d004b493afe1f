/*
 * ffr_gpu.h -- C ABI of the GB300 chaos-game buffer generator
 * (libffr_gpu.so).  Plain pointers, sizes and status codes; no C++ types and
 * no exceptions cross this boundary.
 *
 * It replaces the reference's in-process C++ interface of the ffr-buf path:
 *   BufferRenderer<dims>(Flame(Json))      src/renderers/buffer_renderer.hpp:254-256
 *   BufferRenderer::addBuffer(istream&)    src/renderers/buffer_renderer.hpp:419-452
 *   BufferRenderer::render(...)            src/renderers/buffer_renderer.hpp:269-338
 *   BufferRenderer::renderSeeded(...)      src/renderers/buffer_renderer.hpp:349-372
 *   BufferRenderer::writeBuffer(ostream&)  src/renderers/buffer_renderer.hpp:476-480
 *   BufferRenderer::histogramSum/Min/Max   src/renderers/buffer_renderer.hpp:483-507
 *   stats getters                          src/renderers/buffer_renderer.hpp:509-584
 * and its caller, run_renderer<dims>() in src/ffr_buf.cpp:146-274.
 *
 * Buffer bytes are the reference file layout: for each cell (x fastest, then
 * y rows, then z planes) one u64 count followed by color_dims f64 colour
 * sums, native (little) endian, no header.
 *
 * Threading: one context per host thread, or external locking.  Device work
 * runs on a stream owned by the context; every call returns after its work
 * has finished (or reports FFR_ERR_TIMEOUT) unless stated otherwise.
 */
#ifndef FFR_GPU_H
#define FFR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFR_ABI_VERSION 4

typedef enum ffr_status {
    FFR_OK = 0,
    /* bad-value limit exceeded; buffer and stats are still valid and the
       reference CLI still writes its output and exits 0 (ffr_buf.cpp:228-230) */
    FFR_BAD_VALUES = 1,
    FFR_ERR_PARSE = 2,    /* JSON or flame validation error (JsonError) */
    FFR_ERR_ARG = 3,      /* invalid argument (runtime_error in render()) */
    FFR_ERR_IO = 4,       /* short or mismatched buffer ("error reading file") */
    FFR_ERR_OOM = 5,      /* device memory admission failed */
    FFR_ERR_TIMEOUT = 6,  /* a bounded wait ran out */
    FFR_ERR_CUDA = 7,     /* CUDA runtime error */
    FFR_ERR_STATE = 8     /* call not valid in the context's current state */
} ffr_status;

typedef enum ffr_precision {
    /* mirror of the reference's double arithmetic (num_t = double,
       src/types/types.hpp:29), no FMA contraction */
    FFR_FP64 = 0,
    /* FP32 iteration; xform choices and RNG draws still exact per stream */
    FFR_FP32 = 1
} ffr_precision;

typedef struct ffr_opts {
    uint32_t abi_version;      /* FFR_ABI_VERSION */
    int32_t device;            /* CUDA device ordinal */
    int32_t precision;         /* ffr_precision */
    /* render kernel: 0 = automatic (renders of 2^25 samples or more are
       autotuned once per context over kernel x warp-merged binning on a
       scratch buffer), 1 = plain (one thread runs its trajectory's xforms,
       lanes diverge), 2 = xform-sorted (a CTA groups its threads' points by
       chosen xform each step); every choice gives the same buffer */
    int32_t kernel;
    /* iterations discarded at each trajectory start; the reference uses
       settle_iters<double> = 53 (src/types/constants.hpp:41-47) */
    uint64_t settle;
    /* independent ISAAC streams run concurrently (one per GPU thread);
       0 = choose from the device (SMs x resident threads) */
    uint64_t streams;
    /* samples per trajectory (the reference's batch size, one
       RenderIterator per batch, buffer_renderer.hpp:155); 0 = N / streams */
    uint64_t traj_len;
    /* wall-clock limit in ms for any single device wait; 0 = none */
    uint64_t timeout_ms;
} ffr_opts;

/* dimensions 1..4: ffr-buf's 1..3 (ffr_buf.cpp:134-141) and 4, which the
   reference's BufferRenderer<dims> template also renders; 4-D flames run
   through ffr_render / ffr_render_noalloc (plain kernel), not batches or the
   serving loop */
#define FFR_MAX_DIMS 4
#define FFR_MAX_XFORM_IDS 4096
#define FFR_MAX_BAD_RECORDS 4096

/* Render kernel (ffr_opts.kernel).  AUTO: autotuned for renders of 2^25
   samples and more (plain or xform-sorted, warp-merged binning or not, hot-
   cell table or not), else plain (FP32) or sorted where it fits (FP64).
   HOT: the plain kernel counting the flame's hottest cells (found by one
   probe render) in per-CTA shared memory, without warp merging; streams
   are planned with that memory reserved.  JIT: the plain kernel compiled
   for this flame's structure at run time (NVRTC; each xform's variation
   types fixed in the code instead of dispatched per variation, as the
   reference's XForm::applyIteration, src/types/xform.hpp:211-227,
   dispatches through virtual calls), compiled on the first render that
   needs it unless ffr_jit_prepare compiled it, cached per process and, with
   FFR_JIT_CACHE naming a directory (writable by this user alone: its cubins
   are loaded and run), on disk; FP32 programs of the seven
   benchmark variations run their precompiled merged instantiation instead
   (stats.kernel PLAIN).  JIT_SORTED: the xform-sorted kernel compiled the
   same way, its warps running each xform's own code (flames of 1..3 dims and
   at most 16 xforms).  AUTO also times the per-flame kernels when they are
   already compiled, and compiles them itself (about a second each, the two
   in parallel) when the render would take longer than FFR_JIT_AUTO_SECONDS
   (environment, default 8; negative: never) with the best precompiled
   kernel.  All choices give identical buffers for equal streams and
   trajectory lengths. */
enum { FFR_KERNEL_AUTO = 0, FFR_KERNEL_PLAIN = 1, FFR_KERNEL_SORTED = 2, FFR_KERNEL_HOT = 3,
       FFR_KERNEL_JIT = 4, FFR_KERNEL_JIT_SORTED = 5 };

typedef struct ffr_stats {
    uint64_t samples_iterated;   /* getSamplesIterated */
    uint64_t samples_plotted;    /* getSamplesPlotted */
    uint64_t bad_values;         /* getBadValueXForms().size() */
    uint64_t dropped;            /* in-bounds points whose index fell past the
                                    last cell (undefined in the reference) */
    double ext_lo[FFR_MAX_DIMS]; /* getPointExtremes */
    double ext_hi[FFR_MAX_DIMS];
    uint64_t xform_ids;          /* getXFormIDCount */
    uint64_t xf_dist[FFR_MAX_XFORM_IDS];   /* getXFormDistribution */
    uint64_t bad_recorded;       /* entries filled in bad_xf / bad_pts */
    uint64_t bad_xf[FFR_MAX_BAD_RECORDS];  /* getBadValueXForms (first ones) */
    double bad_pts[FFR_MAX_BAD_RECORDS][FFR_MAX_DIMS];  /* getBadValuePoints */
    /* launch parameters actually used */
    uint64_t streams;
    uint64_t traj_len;
    uint64_t settle;
    double kernel_ms;            /* device time of the render kernel(s) */
    int32_t kernel;              /* FFR_KERNEL_PLAIN, _SORTED, _JIT or _JIT_SORTED */
    int32_t agg;                 /* 1: equal-cell increments were warp-merged */
    int32_t hot_cells;           /* cells counted in per-CTA shared memory
                                    (the autotuner's hot-cell table), or 0 */
    int32_t aux_launches;        /* kernels this call launched besides the
                                    render kernel: count-bound reductions,
                                    autotuner probes, hot-cell search */
    /* launch shape: CTAs of threads_per_cta threads, at most ctas_per_sm
       resident per SM (the autotuner may cap it below what fits), each
       thread running streams_per_thread streams one after the other (the
       reference's trajectories per thread, buffer_renderer.hpp:296-334) */
    uint64_t ctas;
    uint64_t streams_per_thread;
    int32_t ctas_per_sm;
    int32_t threads_per_cta;
} ffr_stats;

typedef struct ffr_ctx ffr_ctx;

/* Fill *opts with defaults (device 0, FP64, settle 53, auto streams). */
void ffr_default_opts(ffr_opts *opts);

/* Parse and validate a flame (JSON text, comments allowed), allocate the
   zeroed count/colour buffer on the device.  Replaces Flame<dims>(Json) +
   BufferRenderer<dims>(flame).  On failure *out is NULL and
   ffr_last_error(NULL) holds the message. */
ffr_status ffr_create(const char *json, size_t len, const ffr_opts *opts,
                      ffr_ctx **out);

void ffr_destroy(ffr_ctx *ctx);

/* Compile the per-flame kernels of a flame for these options (their
   precision; the flame's dimensions and colour) ahead of its renders:
   opts->kernel FFR_KERNEL_JIT or FFR_KERNEL_JIT_SORTED compiles that one,
   any other value both (the sorted one where the flame allows it).  Uses
   NVRTC only: no device is touched, so it can run before a device is
   chosen, and later contexts of flames with the same structure (the same
   variation types per xform, whatever their weights, parameters and
   affines) find the kernel compiled.  FFR_OK also for flames that have no
   per-flame kernel (FP32, benchmark variations only).  FFR_ERR_PARSE: the
   flame; FFR_ERR_CUDA: NVRTC missing or the compile failed (message in
   ffr_last_error(NULL)). */
ffr_status ffr_jit_prepare(const char *json, size_t len, const ffr_opts *opts);

/* Message of the last failing call on ctx (or of the last failing
   ffr_create on this thread when ctx is NULL).  Never NULL. */
const char *ffr_last_error(const ffr_ctx *ctx);

/* Geometry of the context's buffer. */
ffr_status ffr_info(const ffr_ctx *ctx, uint32_t *dims, uint64_t *cells,
                    uint32_t *color_dims, size_t *buffer_bytes);

/* Buffer size per dimension (Flame::getSize, src/types/flame.hpp:221-224);
   size must hold `dims` entries. */
ffr_status ffr_size(const ffr_ctx *ctx, uint64_t *size);

/* The parsed flame as compact JSON (the CLI's "flame:" echo,
   src/ffr_buf.cpp:130).  Owned by ctx. */
const char *ffr_flame_json(const ffr_ctx *ctx);

/* Add a buffer in the file layout (addBuffer, buffer_renderer.hpp:419-452):
   u64 counts add as integers, f64 colours add as doubles.  bytes must be at
   least the buffer size (extra trailing bytes are ignored, as a stream with
   more data is); a shorter input is FFR_ERR_IO and leaves the buffer
   unchanged. */
ffr_status ffr_add_buffer(ffr_ctx *ctx, const void *cells, size_t bytes);

/* Render `samples` post-settle samples (render()/renderSeeded()).  Stream s
   of `seed` is Isaac<u64,4> seeded with setSeed(seed + fmix64(s)).
   bad_limit is the reference's -z (default 256).  stats may be NULL. */
ffr_status ffr_render(ffr_ctx *ctx, uint64_t samples, uint64_t seed,
                      uint64_t bad_limit, ffr_stats *stats);

/* Copy the buffer out in the file layout (writeBuffer).  bytes must be at
   least the buffer size. */
ffr_status ffr_read_buffer(ffr_ctx *ctx, void *cells, size_t bytes);

/* Overwrite the buffer from the file layout (readBuffer). */
ffr_status ffr_load_buffer(ffr_ctx *ctx, const void *cells, size_t bytes);

/* histogramSum / histogramMin / histogramMax over the count channel. */
ffr_status ffr_histogram(ffr_ctx *ctx, uint64_t *sum, uint64_t *min,
                         uint64_t *max);

/* Zero the buffer (a fresh BufferRenderer). */
ffr_status ffr_clear(ffr_ctx *ctx);

/* ---------------------------------------------------------------------
 * Image output (the ffr-img side of the reference): buffer -> pixels on the
 * device, pixels -> PNG on the host.
 * ------------------------------------------------------------------- */
enum { FFR_IMAGE_MONO = 0, FFR_IMAGE_GRAY = 1, FFR_IMAGE_RGB = 2 };

typedef struct ffr_image_info {
    uint64_t hist_min, hist_max;    /* "histogram bounds" (ffr_img.cpp:212-218) */
    double scale_min, scale_max;    /* "scaler bounds": log(1 + count) */
    uint32_t width, height;         /* flame size x, y */
    uint32_t channels;              /* 1 (mono, gray) or 3 (RGB) */
    uint32_t bits;                  /* 8 or 16 per channel */
} ffr_image_info;

/* ffr-img's pixel mapping of the context's 2-D buffer (render_image,
   src/ffr_img.cpp:199-309; ImageRenderer::renderGrayImage /
   renderColorImageRGB, src/renderers/image_renderer.hpp:139-191):
   mode FFR_IMAGE_MONO (count != 0, always 8 bits), FFR_IMAGE_GRAY
   (pow(log(1 + count) / max, 1/gamma)) or FFR_IMAGE_RGB (the gray level
   times the mean of the 3 colour dimensions).  pixels receives width x height
   pixels of `channels` native-endian u8/u16 samples, row y at offset y*width
   (the buffer's order).  Errors as the reference: non-2-D flame, gamma below
   1e-20, bits other than 8/16, RGB without 3 colour dimensions (FFR_ERR_ARG);
   an empty histogram (FFR_ERR_STATE). */
ffr_status ffr_render_image(ffr_ctx *ctx, int mode, double gamma, uint32_t bits,
                            void *pixels, size_t bytes, ffr_image_info *info);

/* PNG file bytes of 8- or 16-bit gray (channels 1) or RGB (channels 3)
   pixels (writePng, src/utils/image.cpp:9-16; uncompressed deflate blocks).
   *len receives the file size; when cap is smaller (or out is NULL) nothing
   is written and the call returns FFR_ERR_IO. */
ffr_status ffr_encode_png(const void *pixels, uint32_t width, uint32_t height,
                          uint32_t channels, uint32_t bits, void *out, size_t cap,
                          size_t *len);

/* ---------------------------------------------------------------------
 * Batched render: many flames (contexts on one device, one precision) in
 * one persistent launch per (dims, colour) group, replayed from a captured
 * CUDA graph.  No single reference counterpart: it runs, for every context,
 * exactly what ffr_render would run for it alone (same streams, same
 * trajectories), so each buffer is identical to a solo render of the same
 * samples and seed.  Work is split into chunks of one CTA's worth of
 * streams claimed from a global cursor, so flames of very different sizes
 * and sample counts share the GPU without stragglers.
 * ------------------------------------------------------------------- */
typedef struct ffr_batch ffr_batch;

/* Group n contexts (not owned; they must outlive the batch). */
ffr_status ffr_batch_create(ffr_ctx *const *ctxs, size_t n, ffr_batch **out);
void ffr_batch_destroy(ffr_batch *b);

/* Render samples[i] samples with seeds[i] into context i, for all i at
   once.  stats may be NULL or an array of n (each filled as ffr_render
   would); returns the first non-OK status (FFR_BAD_VALUES if any job hit
   its bad-value limit). */
ffr_status ffr_batch_render(ffr_batch *b, const uint64_t *samples,
                            const uint64_t *seeds, uint64_t bad_limit,
                            ffr_stats *stats);

/* Message of the last failing call on b. */
const char *ffr_batch_last_error(const ffr_batch *b);

/* ---------------------------------------------------------------------
 * Serving loop: render jobs submitted while others run (continuous
 * batching), buffers resident on the device.  No reference counterpart: the
 * reference renders one flame per ffr-buf process (src/ffr_buf.cpp:146-274)
 * and its -i accumulation reads buffer files back from the host
 * (src/ffr_buf.cpp:167-183, buffer_renderer.hpp:419-452).
 *
 * A job of N samples runs ceil(N / traj_len) streams with one trajectory of
 * traj_len samples each (the last one shorter), exactly what ffr_render runs
 * for a context with opts.streams = ceil(N / traj_len) and opts.traj_len =
 * traj_len, so its counts are identical alone and in any mix of jobs.
 *
 * One scheduler thread admits queued jobs in arrival order while the
 * server's device-memory budget and job slots allow, then runs the admitted
 * jobs in rounds: one persistent launch per (dims, colour) group over a
 * slice of every running job's chunks (128 streams each), the slice shared
 * evenly between running jobs.  Two rounds are in flight at once, so a job
 * that arrives while others run joins the next round and its work overlaps
 * theirs on the device.  A job's buffer stays resident after it completes
 * until every job on it is released; ffr_server_continue adds samples to a
 * resident buffer (-i accumulation without a host round trip).
 *
 * All functions are thread-safe.  Job ids start at 1.
 * ------------------------------------------------------------------- */
typedef struct ffr_server ffr_server;

typedef struct ffr_server_opts {
    uint32_t abi_version;      /* FFR_ABI_VERSION */
    int32_t device;
    int32_t precision;         /* ffr_precision, shared by all jobs */
    int32_t reserved;
    uint64_t settle;           /* default 53 */
    uint64_t traj_len;         /* samples per stream; default 4096 */
    /* device bytes the server may hold: buffers, per-job statistics
       (about 170 KB each) and a fixed 64 MiB of read staging (4 slots);
       0 = free device memory at creation minus 2 GiB */
    uint64_t hbm_budget;
    uint64_t max_active;       /* jobs admitted at once; default 256 */
    uint64_t round_chunks;     /* chunks per round; 0 = four times the resident CTAs */
    uint64_t timeout_ms;       /* limit of one round's device work; 0 = none */
} ffr_server_opts;

enum {
    FFR_JOB_QUEUED = 0,        /* waiting for memory or a slot */
    FFR_JOB_RUNNING = 1,       /* admitted: buffer resident, chunks running */
    FFR_JOB_DONE = 2,          /* finished; status FFR_OK or FFR_BAD_VALUES */
    FFR_JOB_FAILED = 3,        /* status says why */
    FFR_JOB_CANCELLED = 4
};

typedef struct ffr_job_info {
    int32_t state;             /* FFR_JOB_* */
    int32_t status;            /* ffr_status once finished */
    uint64_t samples;
    uint64_t buffer_bytes;     /* size of the buffer in the file layout */
    uint64_t parent;           /* job whose buffer this one continues, or 0 */
    uint64_t submit_ns;        /* steady-clock times of submission, */
    uint64_t admit_ns;         /* admission (0 while queued) */
    uint64_t done_ns;          /* and completion (0 while unfinished) */
} ffr_job_info;

void ffr_server_default_opts(ffr_server_opts *opts);

/* Start the scheduler thread on opts->device.  Errors: ffr_last_error(NULL). */
ffr_status ffr_server_create(const ffr_server_opts *opts, ffr_server **out);

/* Cancel outstanding jobs, wait for in-flight rounds, free everything. */
void ffr_server_destroy(ffr_server *s);

const char *ffr_server_last_error(const ffr_server *s);

/* Queue a render of `samples` samples of the flame `json` into a new
   buffer, first adding `init` (the file layout, init_bytes >= the buffer
   size, or NULL for a zero buffer) as ffr_add_buffer does.  The flame is
   parsed here (FFR_ERR_PARSE / FFR_ERR_IO come back at once); a buffer
   larger than the whole budget is FFR_ERR_OOM. */
ffr_status ffr_server_submit(ffr_server *s, const char *json, size_t len,
                             const void *init, size_t init_bytes,
                             uint64_t samples, uint64_t seed, uint64_t bad_limit,
                             uint64_t *job);

/* Queue `samples` more samples into the buffer of job `parent` (queued,
   running or finished, not released). */
ffr_status ffr_server_continue(ffr_server *s, uint64_t parent, uint64_t samples,
                               uint64_t seed, uint64_t bad_limit, uint64_t *job);

ffr_status ffr_server_poll(ffr_server *s, uint64_t job, ffr_job_info *info);

/* Wait until the job has finished (any terminal state) or timeout_ms has
   passed (FFR_ERR_TIMEOUT; 0 = no limit).  info may be NULL. */
ffr_status ffr_server_wait(ffr_server *s, uint64_t job, uint64_t timeout_ms,
                           ffr_job_info *info);

/* Statistics of a finished job, as ffr_render reports them (kernel_ms is the
   job's submission-to-completion time). */
ffr_status ffr_server_job_stats(ffr_server *s, uint64_t job, ffr_stats *st);

/* Copy the job's buffer out in the file layout (its current contents; the
   final ones once the job and every job continuing it have finished). */
ffr_status ffr_server_read(ffr_server *s, uint64_t job, void *cells, size_t bytes);

/* Stop a queued or running job (running chunks stop within 4096 samples). */
ffr_status ffr_server_cancel(ffr_server *s, uint64_t job);

/* Forget a finished job; its buffer is freed once no job refers to it.
   FFR_ERR_STATE while the job is queued or running. */
ffr_status ffr_server_release(ffr_server *s, uint64_t job);

/* Current load: queued and running jobs, device bytes held now and at most
   since creation.  Any pointer may be NULL. */
ffr_status ffr_server_load(ffr_server *s, uint64_t *queued, uint64_t *running,
                           uint64_t *bytes_used, uint64_t *bytes_peak);

/* ---------------------------------------------------------------------
 * Verification entry points: the same device code as ffr_render, exposed
 * one function at a time so each can be checked against the reference.
 * ------------------------------------------------------------------- */

/* n words of Isaac<u64,4> after setSeed(key): Isaac::next()
   (src/rng/isaac.hpp:321-329, seeding 267-282), generated on the device of
   `device`. */
ffr_status ffr_isaac_words(int device, uint64_t key, uint64_t n, uint64_t *out);

/* XForm::applyIteration (src/types/xform.hpp:211-227) of sorted xform
   `xf_index` (0 = largest weight; -1 = final xform) applied to npts points
   (dims doubles each); point k draws from stream key + fmix64(k).  Runs in
   the context's precision; results are returned as doubles. */
ffr_status ffr_step(ffr_ctx *ctx, int xf_index, uint64_t key, uint64_t npts,
                    const double *in, double *out);

/* One trajectory (RenderIterator, src/renderers/render_iterator.hpp:52-139)
   from setSeed(key): random start, `settle` discarded iterations, then n
   iterations; ids[k] = chosen xform id, pts[k*dims..] = point after it. */
ffr_status ffr_trace(ffr_ctx *ctx, uint64_t key, uint64_t settle, uint64_t n,
                     int32_t *ids, double *pts);

/* Launch configuration ffr_render would use for `samples` (streams and
   trajectory length after defaults are applied). */
ffr_status ffr_plan(ffr_ctx *ctx, uint64_t samples, uint64_t *streams,
                    uint64_t *traj_len);

/* ---------------------------------------------------------------------
 * Measurement (no counterpart in the reference): the roofline denominator
 * of the binning step.  Issues `ops` relaxed 4-byte atomic adds at uniformly
 * random cells of a zeroed `cells`-cell u32 buffer on `device` and reports
 * the achieved rate (one warm-up launch, one timed launch, CUDA events).
 * ------------------------------------------------------------------- */
ffr_status ffr_measure_atomic_rate(int device, uint64_t cells, uint64_t ops,
                                   double *ops_per_s);

/* ---------------------------------------------------------------------
 * Render without device allocation.  No counterpart in the reference: the
 * reference renders into a std::vector it allocates itself.
 *
 * For callers that cannot call cudaMalloc (their device memory belongs to
 * another allocator -- a framework's caching pool, a fixed arena -- and a
 * second allocator must not compete for it): they pass a count buffer they
 * already own and the same render kernel as ffr_render accumulates into it.
 * This call makes no device allocation (no cudaMalloc, cudaFree or
 * allocating library routine); the flame JSON is parsed on the host as in
 * ffr_create.
 *
 * d_counts: device array of `cells` u32 counts (the flame's buffer size,
 *   x fastest), added to, never cleared.  Counts are 32-bit here: a cell must
 *   have room for this call's hits; at most 2^32-1 samples per call.
 * d_colors: device array of cells * color_dims f64 colour sums, required when
 *   the flame has colour_dimensions > 0, else ignored.
 * The kernel's scratch (flame program + statistics) is one fixed device
 * array per GPU (about 180 KB, held until the process exits); flames whose
 * program exceeds its 16 KB program part are rejected with FFR_ERR_ARG.
 * The first call on a device looks up that array's device address (with
 * that device current); make that first call before any stream capture.
 * Calls share the array: calls that overlap on the GPU (from several host
 * threads) race, so serialise them.  Work runs on the legacy default stream
 * and the call returns when it is done.
 * Options: precision, device, settle, streams and traj_len as in
 * ffr_render; kernel must be FFR_KERNEL_AUTO or FFR_KERNEL_PLAIN (the plain
 * kernel always runs: the tuner, the xform-sorted kernel and the hot-cell
 * search would need device memory) and timeout_ms must be 0 (the call waits
 * for the kernel to end), else FFR_ERR_ARG.  d_counts (and d_colors for a
 * colour flame) must be memory of opts->device, else FFR_ERR_ARG.
 * stats->kernel_ms is the host wall time from launch to completion.
 * Errors: ffr_last_error(NULL).
 * ------------------------------------------------------------------- */
ffr_status ffr_render_noalloc(const char *json, size_t len, const ffr_opts *opts,
                              uint32_t *d_counts, double *d_colors, uint64_t cells,
                              uint64_t samples, uint64_t seed, uint64_t bad_limit,
                              ffr_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* FFR_GPU_H */
