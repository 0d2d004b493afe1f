// Xform-sorted ("wavefront") render kernel.
//
// Same per-stream semantics as chaos_body (chaos_kernel.cuh): stream s runs
// its trajectories in order, drawing the reference's RNG words in the
// reference's order (RenderIterator::_init / iterate,
// src/renderers/render_iterator.hpp:52-139; BufferRenderer::_render_batch,
// src/renderers/buffer_renderer.hpp:151-250), so FP64 buffers are identical
// to the plain kernel's.  What changes is who does which part of a step:
//
//   phase A  (owner thread, one per stream)  draw the xform-choice word and
//            the words that xform's variations will draw, stage the point,
//            enter the CTA's per-xform list (one __match_any_sync warp
//            aggregation + one shared atomic per (warp, xform)), and when
//            fewer than `low` words are left, queue an ISAAC refill;
//   phase B  (every warp)  first the queued refills, 32 streams per warp at
//            a time, then 32-entry chunks of one xform's list: every lane of
//            a chunk runs the same xform body, instead of a warp running the
//            union of the xforms (and refills) its lanes happen to need;
//   phase C  (owner)  final xform, colour, statistics, bad values, binning.
//
// ISAAC state of each stream lives in shared memory as [word][thread]:
// randmem (16 words), randa/b/c, and a 24-word result array.  Words are
// consumed from rsl[cnt-1] downwards (Isaac::next, src/rng/isaac.hpp:
// 321-329).  A refill moves the cnt unconsumed words up to rsl[16..16+cnt)
// and generates the next 16 into rsl[0..16), so consumption simply continues
// downwards: the word sequence is the reference's, only its timing moves.
//
// Two barriers per iteration; list counters are double-buffered and the next
// iteration's are zeroed during phase B.  A stream whose trajectory hits a
// bad value re-settles through the same sorted path and finishes the bad
// sample (extremes, stale final point) when its settle iterations are done,
// as the reference does after iter.init().
#pragma once

#include "chaos_kernel.cuh"

namespace ffr {

// ISAAC state of one stream in shared memory, stride T
template <int T>
struct SmemIsaac
{
    uint64_t* mem;      // [16]
    uint64_t* rsl;      // [kRslWords]
    uint64_t* abc;      // [3]: randa, randb, randc

    __device__ __forceinline__ uint64_t& M(int i) { return mem[i * T]; }

    __device__ __forceinline__ void step(int i, uint64_t mx, uint64_t& aa, uint64_t& bb)
    {
        const uint64_t x = M(i);
        aa = mx + M((i + 8) & 15);
        const uint64_t y = M((int)((x >> 3) & 15)) + aa + bb;
        M(i) = y;
        bb = M((int)((y >> 7) & 15)) + x;
        rsl[i * T] = bb;
    }

    // Isaac::gen (isaac.hpp:77-90) into rsl[0..16)
    __device__ __forceinline__ void gen()
    {
        uint64_t aa = abc[0];
        const uint64_t cc = abc[2 * T] + 1;
        uint64_t bb = abc[T] + cc;
#pragma unroll 1
        for (int i = 0; i < 16; i += 4)
        {
            step(i + 0, ~(aa ^ (aa << 21)), aa, bb);
            step(i + 1, aa ^ (aa >> 5), aa, bb);
            step(i + 2, aa ^ (aa << 12), aa, bb);
            step(i + 3, aa ^ (aa >> 33), aa, bb);
        }
        abc[0] = aa;
        abc[T] = bb;
        abc[2 * T] = cc;
    }

    // keep the `left` unconsumed words (rsl[0..left)) above the new block
    __device__ __forceinline__ void refill(int left)
    {
        for (int k = left - 1; k >= 0; --k)
            rsl[(16 + k) * T] = rsl[k * T];
        gen();
    }

    template <typename W>
    __device__ __forceinline__ void seed(uint64_t key, const W* init16)
    {
#pragma unroll
        for (int i = 0; i < 16; ++i)
            M(i) = init16[i];
        abc[0] = key;
        abc[T] = ~key;
        abc[2 * T] = key ^ kIsaacSeedXor;
        gen();
    }
};

// the owner's view: Isaac::next over the shared state
template <int T>
struct OwnerRng
{
    SmemIsaac<T> st;
    int cnt;
    __device__ __forceinline__ uint64_t next()
    {
        if (cnt == 0)
        {
            // rare: more words than the queued refills provided
            st.gen();
            cnt = 16;
        }
        --cnt;
        return st.rsl[cnt * T];
    }
};

// pre-drawn words of one owner, consumed in draw order by the worker
template <int T>
struct PreDrawn
{
    const uint64_t* w;
    int k;
    __device__ __forceinline__ uint64_t next() { return w[(k++) * T]; }
};

// One xform application by a warp that applies xform xi on every lane (a
// chunk of phase B, the final xform): the flame's per-xform code (SP, a
// per-flame kernel), or apply_xform
template <int D, typename R, typename SP, typename Rng>
__device__ __forceinline__ void sorted_xform(const Prog<R>& pg, int xi, const R* p, R* out,
                                             Rng& rng)
{
    if constexpr (SP::on)
        SP::template xform<D, R>(pg, xi, p, out, rng);
    else
        apply_xform<D, R>(pg, pg.xf[xi], p, out, rng);
}

template <int D, typename R, bool COLOR, int T, typename SP = NoSpec>
__device__ __forceinline__ void sorted_body(const RenderArgs& a, unsigned char* smem)
{
    using Tr = RealTraits<R>;
    Prog<R> pg;
    pg.bind(smem, a.prog);
    const ProgHeader<R>& h = *pg.h;
    const int nxf = a.nxf;
    const int W = (int)h.rng_words_max;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    constexpr int kWarps = T / 32;

    unsigned char* q = smem + align16u(a.prog_bytes);
    uint64_t* imem = reinterpret_cast<uint64_t*>(q);
    q += 16 * T * 8;
    uint64_t* irsl = reinterpret_cast<uint64_t*>(q);
    q += kRslWords * T * 8;
    uint64_t* iabc = reinterpret_cast<uint64_t*>(q);
    q += 3 * T * 8;
    uint64_t* words = reinterpret_cast<uint64_t*>(q);
    q += (size_t)W * T * 8;
    R* stage = reinterpret_cast<R*>(q);
    q += ((size_t)D * T * sizeof(R) + 15) & ~(size_t)15;
    uint32_t* xfc = reinterpret_cast<uint32_t*>(q);
    q += ((size_t)nxf * T * 4 + 15) & ~(size_t)15;
    uint16_t* list = reinterpret_cast<uint16_t*>(q);
    q += ((size_t)nxf * T * 2 + 15) & ~(size_t)15;
    uint16_t* glist = reinterpret_cast<uint16_t*>(q);
    q += ((size_t)T * 2 + 15) & ~(size_t)15;
    uint8_t* gleft = q;
    q += ((size_t)T + 15) & ~(size_t)15;
    uint32_t* cnt = reinterpret_cast<uint32_t*>(q);         // [2][kSortedMaxXforms]
    uint32_t* gcnt = cnt + 2 * kSortedMaxXforms;            // [2]

    for (int i = 0; i < nxf; ++i)
        xfc[i * T + tid] = 0u;
    if (tid < 2 * kSortedMaxXforms + 2)
        cnt[tid] = 0u;

    OwnerRng<T> rng;
    rng.st.mem = imem + tid;
    rng.st.rsl = irsl + tid;
    rng.st.abc = iabc + tid;
    rng.cnt = 0;

    // words needed between two refill points: the final xform's draws, then
    // the next choice word and that xform's draws
    int low = 1 + W;
    if (h.has_final)
        low += pg.xf[nxf].rng_words;
    if (low > kMaxRefillLow)
        low = kMaxRefillLow;

    unsigned long long s_iter = 0, s_plot = 0, dropped = 0;
    Extremes<D, R> ext;
    ext.init();
    const int r = COLOR ? a.color_dims : 0;
    R c[COLOR ? kMaxColorDims : 1], cf[COLOR ? kMaxColorDims : 1];
    (void)c; (void)cf;

    const unsigned long long L = a.traj_len;
    const unsigned long long ntraj = (a.samples + L - 1) / L;
    const unsigned long long nstreams = a.streams < ntraj ? a.streams : ntraj;
    const unsigned long long gstride = (unsigned long long)gridDim.x * T;
    volatile unsigned int* vstop = &a.stats->stop;

    unsigned long long s = (unsigned long long)blockIdx.x * T + tid;
    unsigned long long tj = s;
    unsigned long long len = 0;
    unsigned long long settle_left = 0;
    bool pending = false;          // bad sample waiting for its re-settle
    bool active = false;
    R p[D], pf[D];
#pragma unroll
    for (int i = 0; i < D; ++i)
        p[i] = pf[i] = R(0);
    unsigned int poll = 0;

    auto colour_init = [&]() {
        if (COLOR)
            for (int i = 0; i < r; ++i)
                c[i] = Tr::unit(rng.next());
    };
    // RenderIterator::_init up to the settle loop (render_iterator.hpp:54)
    auto start_point = [&]() {
#pragma unroll
        for (int i = 0; i < D; ++i)
            p[i] = R(2) * Tr::unit(rng.next()) - R(1);
        settle_left = a.settle;
        if (settle_left == 0)
            colour_init();
    };
    // next trajectory of this stream, or of the next stream of this thread
    auto next_trajectory = [&](bool first) -> bool {
        if (!first)
            tj += a.streams;
        for (;;)
        {
            if (s >= nstreams)
                return false;
            if (tj < ntraj)
                break;
            s += gstride;
            tj = s;
            first = true;
        }
        if (first && tj == s)
        {
            rng.st.seed(stream_key(a.seed, s), a.isaac_init);
            rng.cnt = 16;
        }
        if (*vstop)
            return false;
        len = a.samples - tj * L;
        if (len > L)
            len = L;
        start_point();
        return true;
    };
    // extremes, bounds, index and binning of a finished sample
    auto tail = [&]() {
        ext.update(p);
        if (!in_bounds<D, R>(a, pf))
            return;
        ++s_plot;
        uint64_t bi;
        if (sizeof(R) == sizeof(double))
        {
            bi = to_index<R>((pf[0] - h.lo[0]) * h.mult_d[0]);
#pragma unroll
            for (int i = 1; i < D; ++i)
                bi += to_index<R>((pf[i] - h.lo[i]) * h.mult_d[i]) * h.mult_i[i];
        }
        else
        {
            bi = 0;
#pragma unroll
            for (int i = 0; i < D; ++i)
            {
                uint64_t di = to_index<R>((pf[i] - h.lo[i]) * h.mult_d[i]);
                di = di < h.size[i] ? di : h.size[i] - 1;
                bi += di * h.mult_i[i];
            }
        }
        if (bi >= h.cells)
        {
            ++dropped;
            return;
        }
        bin_count(a, bi, nullptr);
        if (COLOR)
            for (int i = 0; i < r; ++i)
                atomicAdd(&a.colors[bi * r + i], as_double(cf[i]));
    };
    auto sample_done = [&]() {
        if (--len == 0)
            active = next_trajectory(false);
    };

    __syncthreads();
    active = next_trajectory(true);
    int parity = 0;
    for (;;)
    {
        // ---- phase A: choose, pre-draw, stage, list, queue refills
        int x = -1;
        bool want_refill = false;
        if (active)
        {
            x = pick_branchless(pg.thresh, nxf, rng.next() >> 11);
            const int nw = pg.xf[x].rng_words;
            for (int j = 0; j < nw; ++j)
                words[j * T + tid] = rng.next();
#pragma unroll
            for (int i = 0; i < D; ++i)
                stage[i * T + tid] = p[i];
            want_refill = rng.cnt < low;
        }
        uint32_t* cc = cnt + parity * kSortedMaxXforms;
        uint32_t* gc = gcnt + parity;
        {
            const unsigned int same = __match_any_sync(0xffffffffu, x);
            const int leader = __ffs(same) - 1;
            unsigned int base = 0;
            if (lane == leader && x >= 0)
                base = atomicAdd(&cc[x], (unsigned int)__popc(same));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (x >= 0)
                list[x * T + base + __popc(same & ((1u << lane) - 1u))] = (uint16_t)tid;
        }
        {
            const unsigned int rq = __ballot_sync(0xffffffffu, want_refill);
            unsigned int base = 0;
            if (lane == 0 && rq)
                base = atomicAdd(gc, (unsigned int)__popc(rq));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (want_refill)
            {
                glist[base + __popc(rq & ((1u << lane) - 1u))] = (uint16_t)tid;
                gleft[tid] = (uint8_t)rng.cnt;
            }
        }
        if (!__syncthreads_or(active))
            break;

        // ---- phase B: refills, then uniform-xform chunks
        if (tid < kSortedMaxXforms)
            cnt[(parity ^ 1) * kSortedMaxXforms + tid] = 0u;
        if (tid == 0)
            gcnt[parity ^ 1] = 0u;
        const int ng = (int)*gc;
        const int gch = (ng + 31) >> 5;
        int total = gch;
        for (int i = 0; i < nxf; ++i)
            total += (int)((cc[i] + 31u) >> 5);
        for (int ch = warp; ch < total; ch += kWarps)
        {
            if (ch < gch)
            {
                const int k = ch * 32 + lane;
                if (k < ng)
                {
                    const int o = glist[k];
                    SmemIsaac<T> other{imem + o, irsl + o, iabc + o};
                    other.refill(gleft[o]);
                }
                continue;
            }
            int i = 0, acc = gch;
            for (;;)
            {
                const int n = (int)((cc[i] + 31u) >> 5);
                if (ch < acc + n)
                    break;
                acc += n;
                ++i;
            }
            const unsigned int k = (unsigned int)(ch - acc) * 32u + lane;
            if (k < cc[i])
            {
                const int o = list[i * T + k];
                R pin[D], pout[D];
#pragma unroll
                for (int d = 0; d < D; ++d)
                    pin[d] = stage[d * T + o];
                PreDrawn<T> pw{words + o, 0};
                sorted_xform<D, R, SP>(pg, i, pin, pout, pw);
#pragma unroll
                for (int d = 0; d < D; ++d)
                    stage[d * T + o] = pout[d];
            }
        }
        __syncthreads();
        parity ^= 1;
        if (want_refill)
            rng.cnt += 16;

        // ---- phase C: owner finishes its sample
        if (!active)
            continue;
#pragma unroll
        for (int i = 0; i < D; ++i)
            p[i] = stage[i * T + tid];
        if (settle_left > 0)
        {
            // settle iteration (render_iterator.hpp:55-56): no final xform,
            // no colour, no statistics
            if (--settle_left == 0)
            {
                colour_init();
                if (pending)
                {
                    pending = false;
                    tail();
                    sample_done();
                }
            }
        }
        else
        {
            const XformT<R>& xf = pg.xf[x];
            if (COLOR && xf.has_color)
            {
                const R sp = xf.color_speed;
                const R* col = pg.color + (size_t)x * r;
                for (int i = 0; i < r; ++i)
                    c[i] = (R(1) - sp) * c[i] + sp * col[i];
            }
            if (h.has_final)
            {
                const XformT<R>& ff = pg.xf[nxf];
                sorted_xform<D, R, SP>(pg, nxf, p, pf, rng);
                if (COLOR)
                {
                    if (ff.has_color)
                    {
                        const R sp = ff.color_speed;
                        const R* col = pg.color + (size_t)nxf * r;
                        for (int i = 0; i < r; ++i)
                            cf[i] = (R(1) - sp) * c[i] + sp * col[i];
                    }
                    else
                        for (int i = 0; i < r; ++i)
                            cf[i] = c[i];
                }
            }
            else
            {
#pragma unroll
                for (int i = 0; i < D; ++i)
                    pf[i] = p[i];
                if (COLOR)
                    for (int i = 0; i < r; ++i)
                        cf[i] = c[i];
            }
            ++s_iter;
            ++xfc[x * T + tid];
            if (bad_point<D, R>(p))
            {
                const unsigned long long tot = atomicAdd(&a.stats->bad_total, 1ull) + 1;
                const unsigned long long slot = atomicAdd(&a.stats->bad_claim, 1ull);
                if (slot < (unsigned long long)kMaxBadRecords)
                {
                    a.stats->bad_xf[slot] = xf.id;
#pragma unroll
                    for (int i = 0; i < D; ++i)
                        a.stats->bad_pts[slot][i] = as_double(p[i]);
                }
                if (tot > a.bad_limit)
                {
                    atomicExch(&a.stats->stop, 1u);
                    active = false;
                    continue;
                }
                // iter.init(): new start, re-settle, then finish this sample
                start_point();
                if (settle_left == 0)
                {
                    tail();
                    sample_done();
                }
                else
                    pending = true;
            }
            else
            {
                tail();
                sample_done();
            }
        }
        if (active && ((++poll) & kStopPollMask) == 0)
        {
            if (*vstop || (a.cancel && *a.cancel))
            {
                if (a.cancel && *a.cancel)
                    atomicExch(&a.stats->cancelled, 1u);
                active = false;
            }
        }
    }

    // statistics: warp reduce, one atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
        s_iter += __shfl_down_sync(0xffffffffu, s_iter, off);
        s_plot += __shfl_down_sync(0xffffffffu, s_plot, off);
        dropped += __shfl_down_sync(0xffffffffu, dropped, off);
    }
    ext.warp_reduce();
    if (lane == 0)
    {
        if (s_iter)
            atomicAdd(&a.stats->s_iter, s_iter);
        if (s_plot)
            atomicAdd(&a.stats->s_plot, s_plot);
        if (dropped)
            atomicAdd(&a.stats->dropped, dropped);
        ext.merge(a.stats);
    }
    for (int i = 0; i < nxf; ++i)
    {
        unsigned long long v = xfc[i * T + tid];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0 && v)
            atomicAdd(&a.stats->xf_dist[i], v);
    }
}

template <int D, typename R, bool COLOR, int T>
__global__ void __launch_bounds__(T, 2) chaos_sorted_kernel(const RenderArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    load_program<T>(smem, a.prog, a.prog_bytes);
    __syncthreads();
    sorted_body<D, R, COLOR, T>(a, smem);
}

} // namespace ffr
