// Chaos-game kernels: one GPU thread = one ISAAC stream running its
// trajectories in order.  Replaces, per stream, the reference's
//   BufferRenderer::_render_batch   src/renderers/buffer_renderer.hpp:151-250
//   RenderIterator::_init/iterate   src/renderers/render_iterator.hpp:52-139
//   Flame::getRandomXForm           src/types/flame.hpp:212-219
//   XForm::applyIteration           src/types/xform.hpp:211-227
//   Affine::apply_to                src/types/affine.hpp:104-110
// and, across the grid, BufferRenderer::render's thread pool
// (buffer_renderer.hpp:269-338): trajectory j of the job runs on stream
// j mod streams, stream s seeded with setSeed(seed + fmix64(s)).
//
// Shared memory per CTA: the flame program (copied once), the ISAAC state
// [16][BLOCK] x2, and per-thread xform counters [nxf][BLOCK] (u32) when
// nxf <= kLocalXfCounters, else one u64 counter per xform for the CTA.
// Binning: one relaxed atomic add per in-bounds sample into the u32 count
// buffer (fire-and-forget RED unless counts can pass 2^32, in which case the
// returned old value carries into the u32 high-word buffer).
#pragma once

#include "std_types.h"

#include "flame_program.h"
#include "isaac64.cuh"
#include "launch.h"
#include "variations.cuh"

namespace ffr {

constexpr int kStopPollMask = 4095;     // poll stop/cancel every 4096 samples

// Program view over the shared-memory copy
template <typename R>
struct Prog
{
    const ProgHeader<R>* h;
    const uint64_t* thresh;
    const XformT<R>* xf;
    const VarT<R>* var;
    const R* color;
    uint32_t present;       // ProgHeader::tier_a_present
    uint32_t merged;        // ProgHeader::merged
    const float* fast;      // the compact merged 2-D table, or null

    // sbase: the shared-memory copy of the blob's first h->smem_bytes;
    // gbase: the whole blob in global memory, for the sections beyond
    __device__ __forceinline__ void bind(const unsigned char* sbase, const unsigned char* gbase)
    {
        h = reinterpret_cast<const ProgHeader<R>*>(sbase);
        present = h->tier_a_present;
        merged = h->merged;
        const unsigned int lim = h->smem_bytes;
        auto at = [&](unsigned int off) { return (off < lim ? sbase : gbase) + off; };
        thresh = reinterpret_cast<const uint64_t*>(at(h->off_thresh));
        xf = reinterpret_cast<const XformT<R>*>(at(h->off_xf));
        var = reinterpret_cast<const VarT<R>*>(at(h->off_var));
        color = reinterpret_cast<const R*>(at(h->off_color));
        fast = h->off_fast ? reinterpret_cast<const float*>(at(h->off_fast)) : nullptr;
    }
};

// cooperative 16-byte copy of the program into shared memory
template <int BLOCK>
__device__ __forceinline__ void load_program(unsigned char* dst, const unsigned char* src,
                                             unsigned int bytes)
{
    for (unsigned int k = threadIdx.x * 16u; k < bytes; k += BLOCK * 16u)
        *reinterpret_cast<uint4*>(dst + k) = *reinterpret_cast<const uint4*>(src + k);
}

// 0 + y: the first step of the reference's sums that start from zero
// (Affine::apply_to's dot products, applyIteration's variation sum), which
// is y itself except that -0 becomes +0 (and a NaN stays a NaN).  In FP64
// the sign-bit test and the select run on the integer pipes instead of an
// FP64 add on the FP64 pipe, which bounds the FP64 kernels on this part; in
// FP32 the add stays (it is the same fused multiply-add as before).
template <typename R>
__device__ __forceinline__ R zero_plus(R y)
{
    if constexpr (sizeof(R) == sizeof(double))
        return __double_as_longlong(y) == (long long)0x8000000000000000ull ? R(0) : y;
    else
        return R(0) + y;
}

// Affine::apply_to: ret = b; ret[i] += (0 + A[i][0] x[0] + ...).  The
// coefficients (A row-major kMaxDims x kMaxDims, then b; XformT keeps both
// affines on 16-byte boundaries) come in 16-byte loads, the ones a
// dimension does not use are never loaded.
template <int D, typename R>
__device__ __forceinline__ void affine(const R* aff, const R* x, R* out)
{
    constexpr int kN = kMaxDims * kMaxDims + kMaxDims;
    constexpr int kPer = 16 / (int)sizeof(R);
    static_assert(kN % kPer == 0, "affine coefficients fill whole 16-byte words");
    R c[kN];
#pragma unroll
    for (int k = 0; k < kN; k += kPer)
    {
        const uint4 w = *reinterpret_cast<const uint4*>(aff + k);
        memcpy(&c[k], &w, sizeof w);
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
    {
        R d = zero_plus(c[i * kMaxDims] * x[0]);
#pragma unroll
        for (int j = 1; j < D; ++j)
            d += c[i * kMaxDims + j] * x[j];
        out[i] = c[kMaxDims * kMaxDims + i] + d;
    }
}

// Affine::apply_to of an absent affine of a 1-D or 2-D xform (the identity,
// A = I and b = 0, which the reference applies all the same): row i is
// 0 + ((0 + 1 x_i) + 0 x_j ...), which is x_i with -0 as +0, or NaN when x_i
// is NaN or another coordinate is infinite or NaN (0 times those is NaN).
// FP64: the same values from the bit patterns on the integer pipes; FP32:
// the arithmetic (affine).
template <int D, typename R>
__device__ __forceinline__ void identity_affine(const R* aff, const R* x, R* out)
{
    if constexpr (sizeof(R) == sizeof(double))
    {
        (void)aff;
        constexpr unsigned long long kAbs = 0x7fffffffffffffffULL;
        constexpr unsigned long long kInf = 0x7ff0000000000000ULL;
        bool nonfinite[D];
#pragma unroll
        for (int j = 0; j < D; ++j)
            nonfinite[j] = ((unsigned long long)__double_as_longlong(x[j]) & kAbs) >= kInf;
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            const unsigned long long u = (unsigned long long)__double_as_longlong(x[i]);
            bool nan = (u & kAbs) > kInf;
#pragma unroll
            for (int j = 0; j < D; ++j)
                if (j != i)
                    nan |= nonfinite[j];
            out[i] = nan ? __longlong_as_double(0x7fffffffffffffffLL) : zero_plus(x[i]);
        }
    }
    else
        affine<D>(aff, x, out);
}

// The merged 2-D application from the compact table (flame_program.h): the
// same operations in the same order as affine<2> + merged_variations +
// affine<2> on XformT, from five 16-byte loads instead of eight, so the
// result is the one the general instantiation computes.  False (nothing
// written, nothing drawn) when merged_variations declines the point.
template <bool ALL, typename Rng>
__device__ __forceinline__ bool apply_fast2(const float* f, const float* p, float* out,
                                            Rng& rng, uint32_t present, bool carry)
{
    const float4 r0 = *reinterpret_cast<const float4*>(f);
    const float4 r1 = *reinterpret_cast<const float4*>(f + 4);
    const float4 r2 = *reinterpret_cast<const float4*>(f + 8);
    float t[2], v[2];
    {
        float d = 0.0f;
        d += r0.x * p[0];
        d += r0.y * p[1];
        t[0] = r0.z + d;
        d = 0.0f;
        d += r0.w * p[0];
        d += r1.x * p[1];
        t[1] = r1.y + d;
    }
    if (!merged_variations<2, ALL>(f + 12, t, v, rng, present, carry))
        return false;
    float d = 0.0f;
    d += r1.z * v[0];
    d += r1.w * v[1];
    out[0] = r2.x + d;
    d = 0.0f;
    d += r2.y * v[0];
    d += r2.z * v[1];
    out[1] = r2.w + d;
    return true;
}

// XForm::applyIteration (xform.hpp:211-227).  For dims < 3 both affines are
// always applied (identity when absent), for dims >= 3 only when present.
// VS (variation set): 0 = the general instantiation; 1 and 2 = the
// instantiations for FP32 programs in the merged form (ProgHeader::merged),
// which contain only the seven benchmark types: they carry no code for the
// other 91 (smaller kernels, no stack frame) and compute exactly what the
// general instantiation computes for them; 2 evaluates all seven types
// without per-type branches (merged_variations ALL).  carry: julia's word
// is taken without a branch (the ISAAC carry area is in use).
template <int D, typename R, int VS = 0, typename Rng>
__device__ __forceinline__ void apply_xform(const Prog<R>& pg, const XformT<R>& x,
                                            const R* p, R* out, Rng& rng, int xi = -1,
                                            bool carry = false)
{
    constexpr bool MERGED = VS != 0;
    if constexpr (MERGED && D == 2 && sizeof(R) == sizeof(float))
    {
        if (pg.fast && xi >= 0 && apply_fast2<VS == 2>(pg.fast + xi * kFast2Floats,
                                                       reinterpret_cast<const float*>(p),
                                                       reinterpret_cast<float*>(out), rng,
                                                       pg.present, carry))
            return;
    }
    R t[D], v[D];
    if (x.has_pre)
        affine<D>(x.pre, p, t);
    else if (D < 3)
        identity_affine<D>(x.pre, p, t);
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            t[i] = p[i];
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
        v[i] = R(0);
    const int vb = x.var_begin, ve = x.var_begin + x.var_count;
    // FP32 programs in the merged form: each type once, weighted (falls
    // through to the per-slot loop for points too large for it)
    const bool merged = sizeof(R) == sizeof(float) && (MERGED || pg.merged)
        && merged_variations<D>(reinterpret_cast<const float*>(x.coef),
                                reinterpret_cast<const float*>(t),
                                reinterpret_cast<float*>(v), rng, pg.present, carry, x.plane);
    if (!merged && pg.present == kTaLinear)
    {
        // every variation of the flame is linear (IFS fractals): v = sum of
        // w_j * t in the reference's accumulation order, no dispatch
        if (vb < ve)
        {
            const R w0 = pg.var[vb].weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] = zero_plus(t[i] * w0);
        }
        for (int k = vb + 1; k < ve; ++k)
        {
            const R w = pg.var[k].weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] += t[i] * w;
        }
    }
    else if (!merged)
    {
        // 2-D flames: the plane primitives of the benchmark variations, once
        // per application (the same values every variation would compute)
        PlanePrims<R> pp;
        pp.valid = false;
        pp.q = pp.rt = pp.ang = R(0);
        if (D == 2 && (pg.present & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
        {
            using T = RealTraits<R>;
            const R px = t[0], py = t[D - 1];
            pp.valid = true;
            pp.q = px * px + py * py;
            if (pg.present & (kTaHorseshoe | kTaPolar | kTaJulia))
                pp.rt = T::sqrt_(pp.q);
            if (pg.present & (kTaPolar | kTaJulia))
                pp.ang = T::atan2_(py, px);
        }
        for (int k = vb; k < ve; ++k)
        {
            const VarT<R>& var = pg.var[k];
            R o[D];
            if (MERGED)
                variation_tier_a<D, R>(var, t, o, rng, pg.present, pp);
            else
                variation<D, R>(var, t, o, rng, pg.present, pp);
            const R w = var.weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] += o[i] * w;
        }
    }
    if (x.has_post)
        affine<D>(x.post, v, out);
    else if (D < 3)
        identity_affine<D>(x.post, v, out);
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            out[i] = v[i];
    }
}

// Per-flame kernels (compiled at run time for one flame, jit.cpp).  A spec
// type SP fixes at compile time, for each variation slot k (the k-th
// variation of an xform), the types that slot holds in the flame's xforms,
// and the flame's kTa* bits (SP::present) and largest variation count
// (SP::slots).  apply_xform_spec is apply_xform's general path with the
// 98-way type switch of each slot narrowed to those types and the
// benchmark types' shared body to the ones the slot holds.  Everything
// else -- affines, plane primitives, the slot loop -- stays common to all
// lanes of a warp, as in apply_xform (code specialised per xform instead
// would run each xform's affines and primitives one xform after another
// in a warp whose lanes chose different xforms).  The arithmetic is
// apply_xform's on the same program data, so the buffers are the general
// kernel's.
struct NoSpec
{
    static constexpr bool on = false;
};

// o = V(t) for a variation of one of the types TYPES... or, when TA is not
// 0, of a benchmark type in TA (kTa* bits)
template <int D, typename R, uint32_t TA, int... TYPES>
struct SlotTypes
{
    template <typename Rng>
    __device__ static __forceinline__ void eval(const VarT<R>& var, const R* t, R* o, Rng& rng,
                                                const PlanePrims<R>& pp)
    {
        variation_tier_a<D, R>(var, t, o, rng, TA, pp);
    }
};

template <int D, typename R, uint32_t TA, int T0, int... REST>
struct SlotTypes<D, R, TA, T0, REST...>
{
    template <typename Rng>
    __device__ static __forceinline__ void eval(const VarT<R>& var, const R* t, R* o, Rng& rng,
                                                const PlanePrims<R>& pp)
    {
        if constexpr (TA == 0 && sizeof...(REST) == 0)
            variation<D, R, T0>(var, t, o, rng, 0u, pp);    // the slot's only type
        else
        {
            if (var.type == T0)
                variation<D, R, T0>(var, t, o, rng, TA, pp);
            else
                SlotTypes<D, R, TA, REST...>::eval(var, t, o, rng, pp);
        }
    }
};

// slots S..SP::slots-1 of an xform of n variations from pg.var[vb] on
template <typename SP, int S, int D, typename R, typename Rng>
__device__ __forceinline__ void spec_slots(const Prog<R>& pg, int vb, int n, const R* t, R* v,
                                           Rng& rng, const PlanePrims<R>& pp)
{
    if constexpr (S < SP::slots)
    {
        if (S < n)
        {
            const VarT<R>& var = pg.var[vb + S];
            R o[D];
            SP::template slot<S, D, R>(var, t, o, rng, pp);
            const R w = var.weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] = S == 0 ? zero_plus(o[i] * w) : v[i] + o[i] * w;
            spec_slots<SP, S + 1, D, R>(pg, vb, n, t, v, rng, pp);
        }
    }
}

// XForm::applyIteration through the flame's spec (apply_xform's general path)
template <int D, typename R, typename SP, typename Rng>
__device__ __forceinline__ void apply_xform_spec(const Prog<R>& pg, const XformT<R>& x,
                                                 const R* p, R* out, Rng& rng)
{
    R t[D], v[D];
    if (x.has_pre)
        affine<D>(x.pre, p, t);
    else if (D < 3)
        identity_affine<D>(x.pre, p, t);
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            t[i] = p[i];
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
        v[i] = R(0);
    const int vb = x.var_begin, n = x.var_count;
    if constexpr (SP::present == kTaLinear)
    {
        // every variation of the flame is linear (apply_xform's IFS loop)
        if (n > 0)
        {
            const R w0 = pg.var[vb].weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] = zero_plus(t[i] * w0);
        }
        for (int k = vb + 1; k < vb + n; ++k)
        {
            const R w = pg.var[k].weight;
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] += t[i] * w;
        }
    }
    else
    {
        PlanePrims<R> pp;
        pp.valid = false;
        pp.q = pp.rt = pp.ang = R(0);
        if constexpr (D == 2 && (SP::present & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
        {
            using T = RealTraits<R>;
            const R px = t[0], py = t[D - 1];
            pp.valid = true;
            pp.q = px * px + py * py;
            if (SP::present & (kTaHorseshoe | kTaPolar | kTaJulia))
                pp.rt = T::sqrt_(pp.q);
            if (SP::present & (kTaPolar | kTaJulia))
                pp.ang = T::atan2_(py, px);
        }
        spec_slots<SP, 0, D, R>(pg, vb, n, t, v, rng, pp);
    }
    if (x.has_post)
        affine<D>(x.post, v, out);
    else if (D < 3)
        identity_affine<D>(x.post, v, out);
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            out[i] = v[i];
    }
}

// Per-xform code for kernels whose warps apply one xform at a time (the
// xform-sorted kernel's chunks, the final xform): XForm::applyIteration for
// an xform known at compile time, its variations from pg.var[K] on with
// types TYPES... in order; PRESENT = the kTa* bits of its own types (the
// plane primitives it needs; the variation results do not depend on which
// other types share them); PRE / POST: it has the affine (used above 2
// dims only, as in apply_xform).  The arithmetic is apply_xform's general
// path on the same program data.
template <int D, typename R, uint32_t PRESENT, bool FIRST, int K, int... TYPES>
struct FixedVars
{
    template <typename Rng>
    __device__ static __forceinline__ void run(const Prog<R>&, const R*, R*, Rng&,
                                               const PlanePrims<R>&)
    {
    }
};

template <int D, typename R, uint32_t PRESENT, bool FIRST, int K, int T0, int... REST>
struct FixedVars<D, R, PRESENT, FIRST, K, T0, REST...>
{
    template <typename Rng>
    __device__ static __forceinline__ void run(const Prog<R>& pg, const R* t, R* v, Rng& rng,
                                               const PlanePrims<R>& pp)
    {
        const VarT<R>& var = pg.var[K];
        R o[D];
        variation<D, R, T0>(var, t, o, rng, PRESENT, pp);
        const R w = var.weight;
#pragma unroll
        for (int i = 0; i < D; ++i)
            v[i] = FIRST ? zero_plus(o[i] * w) : v[i] + o[i] * w;
        FixedVars<D, R, PRESENT, false, K + 1, REST...>::run(pg, t, v, rng, pp);
    }
};

template <int D, typename R, uint32_t PRESENT, bool PRE, bool POST, int K, int... TYPES>
struct FixedXform
{
    template <typename Rng>
    __device__ static __forceinline__ void apply(const Prog<R>& pg, const XformT<R>& x,
                                                 const R* p, R* out, Rng& rng)
    {
        R t[D], v[D];
        if constexpr (PRE)
            affine<D>(x.pre, p, t);
        else if constexpr (D < 3)
            identity_affine<D>(x.pre, p, t);
        else
        {
#pragma unroll
            for (int i = 0; i < D; ++i)
                t[i] = p[i];
        }
#pragma unroll
        for (int i = 0; i < D; ++i)
            v[i] = R(0);
        PlanePrims<R> pp;
        pp.valid = false;
        pp.q = pp.rt = pp.ang = R(0);
        if constexpr (D == 2 && (PRESENT & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
        {
            using T = RealTraits<R>;
            const R px = t[0], py = t[D - 1];
            pp.valid = true;
            pp.q = px * px + py * py;
            if (PRESENT & (kTaHorseshoe | kTaPolar | kTaJulia))
                pp.rt = T::sqrt_(pp.q);
            if (PRESENT & (kTaPolar | kTaJulia))
                pp.ang = T::atan2_(py, px);
        }
        FixedVars<D, R, PRESENT, true, K, TYPES...>::run(pg, t, v, rng, pp);
        if constexpr (POST)
            affine<D>(x.post, v, out);
        else if constexpr (D < 3)
            identity_affine<D>(x.post, v, out);
        else
        {
#pragma unroll
            for (int i = 0; i < D; ++i)
                out[i] = v[i];
        }
    }
};

// one xform application in the render loop: the flame's own code (SP), or
// apply_xform
template <int D, typename R, int VS, typename SP, typename Rng>
__device__ __forceinline__ void xform_step(const Prog<R>& pg, const XformT<R>& x, int xi,
                                           const R* p, R* out, Rng& rng, bool carry)
{
    if constexpr (SP::on)
        apply_xform_spec<D, R, SP>(pg, x, p, out, rng);
    else
        apply_xform<D, R, VS>(pg, x, p, out, rng, xi, carry);
}

// first i with m <= thresh[i]: the thresholds of the first nxf-1 xforms are
// non-decreasing (prefix sums of non-negative weights) and the last is 2^53,
// so the index is the number of leading thresholds below m.  A fixed-trip
// count instead of a search loop: lanes do not diverge on it.
__device__ __forceinline__ int pick_branchless(const uint64_t* thresh, int nxf, uint64_t m)
{
    // thresholds in pairs (16-byte loads; the array is 16-byte aligned and
    // holds nxf entries, so the pair of the last tested one is in bounds)
    int x = 0;
#pragma unroll 2
    for (int i = 0; i < nxf - 1; i += 2)
    {
        const ulonglong2 t = *reinterpret_cast<const ulonglong2*>(thresh + i);
        x += m > t.x ? 1 : 0;
        x += (i + 1 < nxf - 1 && m > t.y) ? 1 : 0;
    }
    return x;
}

// Flame::getRandomXForm via exact integer thresholds (flame_program.h)
template <typename R, typename Rng>
__device__ __forceinline__ int pick_xform(const Prog<R>& pg, int nxf, Rng& rng)
{
    return pick_branchless(pg.thresh, nxf, rng.next() >> 11);
}

// The thresholds of a flame of up to kRegThresholds + 1 xforms held in
// registers for a whole render (unused ones 2^64 - 1, never below m), so a
// choice costs compares only, no shared loads: the merged-form kernels,
// whose register budget allows it.  Same choice as pick_branchless.
constexpr int kRegThresholds = 7;
struct RegThresh
{
    uint64_t t[kRegThresholds];
    __device__ __forceinline__ void load(const uint64_t* th, int nxf)
    {
#pragma unroll
        for (int i = 0; i < kRegThresholds; ++i)
            t[i] = i < nxf - 1 ? th[i] : ~0ull;
    }
    __device__ __forceinline__ int pick(uint64_t m) const
    {
        int x = 0;
#pragma unroll
        for (int i = 0; i < kRegThresholds; ++i)
            x += m > t[i] ? 1 : 0;
        return x;
    }
};

template <int D, typename R>
__device__ __forceinline__ bool bad_point(const R* p)
{
    // |x| > threshold or NaN (utils/flame.hpp:26-29), as one unordered test;
    // FP64 on the bit patterns (for |x| the IEEE order is the unsigned
    // order of the bits, and a NaN's bits lie above every finite value's)
    bool b = false;
    if constexpr (sizeof(R) == sizeof(double))
    {
        constexpr unsigned long long kAbs = 0x7fffffffffffffffULL;
        const unsigned long long thr =
            (unsigned long long)__double_as_longlong(RealTraits<double>::bad);
#pragma unroll
        for (int i = 0; i < D; ++i)
            b |= ((unsigned long long)__double_as_longlong(p[i]) & kAbs) > thr;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            b |= !(RealTraits<R>::fabs_(p[i]) <= RealTraits<R>::bad);
    }
    return b;
}

// the final point inside the bounds: inclusive [lo, hi] per axis
// (render_iterator.hpp:72-79); NaN is out (documented deviation).  FP64 on
// ord_key values (launch.h), FP32 as float compares.
template <int D, typename R>
__device__ __forceinline__ bool in_bounds(const RenderArgs& a, const R* pf)
{
    bool inb = true;
    if constexpr (sizeof(R) == sizeof(double))
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            const unsigned long long k = ord_key(pf[i]);
            inb &= (k >= a.lo_key[i]) && (k <= a.hi_key[i]);
        }
    }
    else
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
            inb &= (pf[i] >= a.lo_f[i]) && (pf[i] <= a.hi_f[i]);
    }
    return inb;
}

// One thread's running point extremes (buffer_renderer.hpp:188-194: a
// coordinate below the minimum replaces it, one above the maximum replaces
// that; a NaN replaces neither), merged over the warp and then into the
// statistics' order keys.  FP32: min/max instructions.  FP64: ord_key
// values, min/max on the integer pipes (the order key is the statistics'
// own encoding; -0 and +0 share a key, within the documented deviation on
// the sign of a zero extreme).
template <int D, typename R>
struct Extremes
{
    R lo[D], hi[D];
    __device__ __forceinline__ void init()
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            lo[i] = R(1) / R(0);
            hi[i] = -R(1) / R(0);
        }
    }
    __device__ __forceinline__ void update(const R* p)
    {
        // one min/max instruction each: the running extreme is never NaN,
        // and a NaN p keeps it, as the compare does
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            lo[i] = fminf(p[i], lo[i]);
            hi[i] = fmaxf(p[i], hi[i]);
        }
    }
    __device__ __forceinline__ void warp_reduce()
    {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < D; ++i)
            {
                const R l = __shfl_down_sync(0xffffffffu, lo[i], off);
                const R h = __shfl_down_sync(0xffffffffu, hi[i], off);
                lo[i] = l < lo[i] ? l : lo[i];
                hi[i] = h > hi[i] ? h : hi[i];
            }
    }
    __device__ __forceinline__ void merge(DevStats* st) const
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            if (lo[i] == lo[i] && lo[i] != R(1) / R(0))
                atomicMin(&st->ext_lo[i], order_key((double)lo[i]));
            if (hi[i] == hi[i] && hi[i] != -R(1) / R(0))
                atomicMax(&st->ext_hi[i], order_key((double)hi[i]));
        }
    }
};

template <int D>
struct Extremes<D, double>
{
    static constexpr unsigned long long kPosInf = 0xfff0000000000000ULL;   // ord_key(+inf)
    static constexpr unsigned long long kNegInf = 0x000fffffffffffffULL;   // ord_key(-inf)
    unsigned long long lo[D], hi[D];
    __device__ __forceinline__ void init()
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            lo[i] = kPosInf;
            hi[i] = kNegInf;
        }
    }
    __device__ __forceinline__ void update(const double* p)
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            const unsigned long long u = (unsigned long long)__double_as_longlong(p[i]);
            if ((u & 0x7fffffffffffffffULL) <= 0x7ff0000000000000ULL)   // not NaN
            {
                const unsigned long long k = ord_key(p[i]);
                lo[i] = k < lo[i] ? k : lo[i];
                hi[i] = k > hi[i] ? k : hi[i];
            }
        }
    }
    __device__ __forceinline__ void warp_reduce()
    {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < D; ++i)
            {
                const unsigned long long l = __shfl_down_sync(0xffffffffu, lo[i], off);
                const unsigned long long h = __shfl_down_sync(0xffffffffu, hi[i], off);
                lo[i] = l < lo[i] ? l : lo[i];
                hi[i] = h > hi[i] ? h : hi[i];
            }
    }
    __device__ __forceinline__ void merge(DevStats* st) const
    {
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            if (lo[i] != kPosInf)
                atomicMin(&st->ext_lo[i], lo[i]);
            if (hi[i] != kNegInf)
                atomicMax(&st->ext_hi[i], hi[i]);
        }
    }
};

template <typename R> __device__ __forceinline__ uint64_t to_index(R x);
template <> __device__ __forceinline__ uint64_t to_index<double>(double x)
{
    return (uint64_t)x;     // size_t conversion truncates (buffer_renderer.hpp:202)
}
template <> __device__ __forceinline__ uint64_t to_index<float>(float x)
{
    return (uint64_t)x;
}

// The same truncation to 32 bits.  An in-bounds coordinate gives a value in
// [0, size] with size <= 65535 (Flame validation), where the 32-bit and the
// 64-bit conversions agree.
template <typename R> __device__ __forceinline__ uint32_t to_index32(R x);
template <> __device__ __forceinline__ uint32_t to_index32<double>(double x)
{
    return (uint32_t)x;
}
template <> __device__ __forceinline__ uint32_t to_index32<float>(float x)
{
    return (uint32_t)x;
}

// geometry of RenderArgs in the kernel's precision
template <typename R> struct Geo;
template <> struct Geo<double>
{
    __device__ static __forceinline__ double lo(const RenderArgs& a, int i) { return a.lo_d[i]; }
    __device__ static __forceinline__ double hi(const RenderArgs& a, int i) { return a.hi_d[i]; }
    __device__ static __forceinline__ double mult(const RenderArgs& a, int i) { return a.mult_d_d[i]; }
};
template <> struct Geo<float>
{
    __device__ static __forceinline__ float lo(const RenderArgs& a, int i) { return a.lo_f[i]; }
    __device__ static __forceinline__ float hi(const RenderArgs& a, int i) { return a.hi_f[i]; }
    __device__ static __forceinline__ float mult(const RenderArgs& a, int i) { return a.mult_d_f[i]; }
};

template <typename R>
__device__ __forceinline__ double as_double(R x) { return (double)x; }

// n more counts for cell bi; with a.spill the returned old value detects
// the u32 wrap and carries into the high word
__device__ __forceinline__ void add_count(const RenderArgs& a, uint64_t bi, unsigned int n)
{
    if (a.spill)
    {
        const unsigned int old = atomicAdd(&a.counts[bi], n);
        if (old + n < old)
            atomicAdd(&a.hi[bi], 1u);
    }
    else
        atomicAdd(&a.counts[bi], n);
}

// One count for cell bi.  A cell of the hot-cell table (hot: the CTA's
// keys, then its counts, or null) counts in shared memory.  With a.agg,
// lanes of the warp that bin the same cell in this step are merged by
// __match_any_sync into one atomic add of their number (hot cells: fixed
// points, dense attractor cores); otherwise every lane issues its own
// fire-and-forget add.  With a.spill the returned old value detects the u32
// wrap and carries into the high word.
__device__ __forceinline__ void bin_count(const RenderArgs& a, uint64_t bi, unsigned int* hot)
{
    if (hot)
    {
        // the table needs fewer than 2^30 cells: bi fits 32 bits
        const unsigned int k = (unsigned int)bi;
        const unsigned int slot = (k * a.hot_mult) >> (32 - kHotSlotBits);
        if (hot[slot] == k)
        {
            atomicAdd(&hot[kHotSlots + slot], 1u);
            return;
        }
    }
    if (a.agg)
    {
        const unsigned int same = __match_any_sync(__activemask(), (unsigned long long)bi);
        if ((int)(threadIdx.x & 31u) != __ffs(same) - 1)
            return;
        add_count(a, bi, (unsigned int)__popc(same));
        return;
    }
    add_count(a, bi, 1u);
}

// Runs streams s_first, s_first + s_stride, ... (below the job's active
// stream count), then merges this CTA's statistics into a.stats.
template <int D, typename R, bool COLOR, int BLOCK, int VS = 0, typename SP = NoSpec>
__device__ __forceinline__ void chaos_body(const RenderArgs& a, unsigned char* smem,
                                           unsigned long long s_first,
                                           unsigned long long s_stride)
{
    using T = RealTraits<R>;
    Prog<R> pg;
    pg.bind(smem, a.prog);
    const ProgHeader<R>& h = *pg.h;
    const int nxf = a.nxf;
    uint64_t* ismem = reinterpret_cast<uint64_t*>(smem + align16u(a.prog_bytes));
    const int rsl_words = a.rsl_words;
    // refill ahead keeps every word of a step in the result array
    const bool carry = rsl_words > 16;
    uint32_t* xfc_local = reinterpret_cast<uint32_t*>(ismem + (16 + rsl_words) * BLOCK);
    unsigned long long* xfc_shared = reinterpret_cast<unsigned long long*>(xfc_local);
    const bool packed_xfc = nxf <= kPackedXfCounters;
    const bool local_xfc = !packed_xfc && nxf <= kLocalXfCounters;
    // packed: 8-bit per-xform fields of xpk, flushed every 255 samples
    unsigned long long xpk = 0;
    unsigned int xsince = 0;
    auto xflush = [&]() __attribute__((always_inline)) {
        for (int i = 0; i < nxf; ++i)
        {
            const unsigned int n = (unsigned int)(xpk >> (8 * i)) & 255u;
            if (n)
                atomicAdd(&xfc_shared[i], (unsigned long long)n);
        }
        xpk = 0;
        xsince = 0;
    };
    if (local_xfc)
    {
        for (int i = 0; i < nxf; ++i)
            xfc_local[i * BLOCK + threadIdx.x] = 0u;
    }
    else
    {
        for (int i = threadIdx.x; i < nxf; i += BLOCK)
            xfc_shared[i] = 0ull;
        __syncthreads();
    }

    DevIsaac<BLOCK, kIsaacRslMax> rng;
    rng.mem = ismem + threadIdx.x;
    rng.rsl = ismem + 16 * BLOCK + threadIdx.x;
    // words one sample step can draw: the choice, the chosen xform's
    // variations, the final xform's
    const unsigned int low = 1u + h.rng_words_max + (h.has_final ? pg.xf[nxf].rng_words : 0u);
    // refill ahead, warp-uniformly, once some lane could run dry this step
    // (only with a carry area: when every xform draws the same number of
    // words the lanes stay in phase and run dry together anyway)
    auto refill_ahead = [&]() __attribute__((always_inline)) {
        if (rsl_words > 16 && __any_sync(__activemask(), rng.cnt < low)
                && (int)rng.cnt <= rsl_words - 16)
            rng.refill();
    };

    // the xform choice: thresholds in registers for the all-seven merged kernels
    // of up to kRegThresholds + 1 xforms, else shared-memory loads
    RegThresh rth;
    const bool reg_pick = VS == 2 && nxf <= kRegThresholds + 1;
    if (reg_pick)
        rth.load(pg.thresh, nxf);
    auto choose = [&]() __attribute__((always_inline)) {
        if (VS == 2 && reg_pick)
            return rth.pick(rng.next() >> 11);
        return pick_xform<R>(pg, nxf, rng);
    };

    // hot-cell table: keys from a.hot_keys, counts zeroed
    unsigned int* hot = nullptr;
    if (a.hot_keys)
    {
        hot = reinterpret_cast<unsigned int*>(smem + chaos_smem_bytes<BLOCK>(a.prog_bytes, nxf,
                                                                             rsl_words));
        for (int i = threadIdx.x; i < kHotSlots; i += BLOCK)
        {
            hot[i] = a.hot_keys[i];
            hot[kHotSlots + i] = 0u;
        }
        __syncthreads();
    }

    // per-thread counters fit 32 bits: a thread runs fewer than 2^32
    // samples (checked by the launch planners)
    unsigned int s_iter = 0, s_plot = 0, dropped = 0;
    using G = Geo<R>;
    // below 2^30 cells the index sum (per-axis indices can reach the axis
    // size in FP64, as in the reference) stays under 2^32
    const bool idx32 = a.cells < (1ull << 30);
    Extremes<D, R> ext;
    ext.init();
    const int r = COLOR ? a.color_dims : 0;
    R c[COLOR ? kMaxColorDims : 1], cf[COLOR ? kMaxColorDims : 1];
    (void)c; (void)cf;

    const unsigned long long L = a.traj_len;
    const unsigned long long ntraj = (a.samples + L - 1) / L;
    const unsigned long long nstreams = a.streams < ntraj ? a.streams : ntraj;
    bool stop = false;
    volatile unsigned int* vstop = &a.stats->stop;

    for (unsigned long long s = s_first; s < nstreams && !stop; s += s_stride)
    {
        rng.seed(stream_key(a.seed, s), a.isaac_init);
        for (unsigned long long tj = s; tj < ntraj && !stop; tj += a.streams)
        {
            unsigned long long len64 = a.samples - tj * L;
            if (len64 > L)
                len64 = L;
            unsigned int len = (unsigned int)len64;
            // _render_batch entry check (buffer_renderer.hpp:153)
            if (*vstop)
            {
                stop = true;
                break;
            }
            R p[D], pf[D];
            // RenderIterator::_init (render_iterator.hpp:52-60); inlined so
            // the trajectory state stays in registers
            auto init = [&]() __attribute__((always_inline)) {
#pragma unroll
                for (int i = 0; i < D; ++i)
                    p[i] = R(2) * T::unit(rng.next()) - R(1);
                for (unsigned long long k = 0; k < a.settle; ++k)
                {
                    refill_ahead();
                    const int xi = choose();
                    R q[D];
                    xform_step<D, R, VS, SP>(pg, pg.xf[xi], xi, p, q, rng, carry);
#pragma unroll
                    for (int i = 0; i < D; ++i)
                        p[i] = q[i];
                }
                if (COLOR)
                    for (int i = 0; i < r; ++i)
                        c[i] = T::unit(rng.next());
            };
            init();
            unsigned int poll = 0;
            for (; len > 0; --len)
            {
                refill_ahead();
                const int xi = choose();
                const XformT<R>& xf = pg.xf[xi];
                {
                    R q[D];
                    xform_step<D, R, VS, SP>(pg, xf, xi, p, q, rng, carry);
#pragma unroll
                    for (int i = 0; i < D; ++i)
                        p[i] = q[i];
                }
                if (COLOR && xf.has_color)
                {
                    const R sp = xf.color_speed;
                    const R* col = pg.color + (size_t)xi * r;
                    for (int i = 0; i < r; ++i)
                        c[i] = (R(1) - sp) * c[i] + sp * col[i];
                }
                if (h.has_final)
                {
                    const XformT<R>& ff = pg.xf[nxf];
                    xform_step<D, R, VS, SP>(pg, ff, nxf, p, pf, rng, carry);
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
                if (packed_xfc)
                {
                    xpk += 1ull << (8 * xi);
                    if (++xsince == 255u)
                        xflush();
                }
                else if (local_xfc)
                    ++xfc_local[xi * BLOCK + threadIdx.x];
                else
                    atomicAdd(&xfc_shared[xi], 1ull);
                // bad value (buffer_renderer.hpp:175-186)
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
                        stop = true;
                        break;
                    }
                    init();
                }
                // extreme coordinates (buffer_renderer.hpp:188-194)
                ext.update(p);
                if (in_bounds<D, R>(a, pf))
                {
                    ++s_plot;
                    uint64_t bi;
                    if (idx32)
                    {
                        // fewer than 2^30 cells: the index sum fits 32 bits
                        uint32_t b = 0;
#pragma unroll
                        for (int i = 0; i < D; ++i)
                        {
                            uint32_t di = to_index32<R>((pf[i] - G::lo(a, i)) * G::mult(a, i));
                            // FP32: per-axis index clamped to the axis
                            if (sizeof(R) == sizeof(float))
                                di = di < a.size32[i] ? di : a.size32[i] - 1u;
                            b += di * (uint32_t)a.mult_i[i];
                        }
                        bi = b;
                    }
                    else if (sizeof(R) == sizeof(double))
                    {
                        // buffer_renderer.hpp:200-209
                        bi = to_index<R>((pf[0] - G::lo(a, 0)) * G::mult(a, 0));
#pragma unroll
                        for (int i = 1; i < D; ++i)
                            bi += to_index<R>((pf[i] - G::lo(a, i)) * G::mult(a, i)) * a.mult_i[i];
                    }
                    else
                    {
                        bi = 0;
#pragma unroll
                        for (int i = 0; i < D; ++i)
                        {
                            uint64_t di = to_index<R>((pf[i] - G::lo(a, i)) * G::mult(a, i));
                            di = di < a.size32[i] ? di : a.size32[i] - 1u;
                            bi += di * a.mult_i[i];
                        }
                    }
                    // FP32 clamps each axis index to the axis, so the cell
                    // is always inside the buffer
                    if (sizeof(R) == sizeof(float) || bi < a.cells)
                    {
                        bin_count(a, bi, hot);
                        if (COLOR)
                            for (int i = 0; i < r; ++i)
                                atomicAdd(&a.colors[bi * r + i], as_double(cf[i]));
                    }
                    else
                        ++dropped;
                }
                if (((++poll) & kStopPollMask) == 0)
                {
                    if (*vstop || (a.cancel && *a.cancel))
                    {
                        if (a.cancel && *a.cancel)
                            atomicExch(&a.stats->cancelled, 1u);
                        stop = true;
                        break;
                    }
                }
            }
        }
    }

    // merge statistics: warp reduce (in 64 bits), then one atomic per warp
    const unsigned int lane = threadIdx.x & 31u;
    unsigned long long w_iter = s_iter, w_plot = s_plot, w_dropped = dropped;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
        w_iter += __shfl_down_sync(0xffffffffu, w_iter, off);
        w_plot += __shfl_down_sync(0xffffffffu, w_plot, off);
        w_dropped += __shfl_down_sync(0xffffffffu, w_dropped, off);
    }
    ext.warp_reduce();
    if (lane == 0)
    {
        if (w_iter)
            atomicAdd(&a.stats->s_iter, w_iter);
        if (w_plot)
            atomicAdd(&a.stats->s_plot, w_plot);
        if (w_dropped)
            atomicAdd(&a.stats->dropped, w_dropped);
        ext.merge(a.stats);
    }
    if (packed_xfc)
        xflush();
    __syncthreads();
    // the CTA's hot-cell counts (below 2^32: the planner bounds a CTA's
    // samples) into the buffer
    if (hot)
    {
        for (int i = threadIdx.x; i < kHotSlots; i += BLOCK)
        {
            const unsigned int n = hot[kHotSlots + i];
            if (n)
                add_count(a, hot[i], n);
        }
    }
    if (local_xfc)
    {
        for (int i = 0; i < nxf; ++i)
        {
            unsigned long long v = xfc_local[i * BLOCK + threadIdx.x];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
                v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0 && v)
                atomicAdd(&a.stats->xf_dist[i], v);
        }
    }
    else
    {
        for (int i = threadIdx.x; i < nxf; i += BLOCK)
            if (xfc_shared[i])
                atomicAdd(&a.stats->xf_dist[i], xfc_shared[i]);
    }
}

// Resident CTAs of 128 threads the register budget must allow.  FP32: 6,
// so that flames whose xforms draw equal numbers of words (16-word ISAAC
// result arrays, about 37 KB of shared memory per CTA) run 6 CTAs per SM;
// the FP32 body fits in 80 registers without spilling.  FP64: 4 (its body
// needs about 120 registers; at 80 it spills).  Variation set 2 (2-D
// merged flames of five or more types, which in practice include julia and
// so keep the 8-word ISAAC carry: 5 CTAs per SM by shared memory): 5, which
// leaves room for the thresholds in registers (RegThresh).
template <typename R>
__host__ __device__ constexpr int render_min_blocks(int vs = 0)
{
    return sizeof(R) == 4 ? (vs == 2 ? 5 : 6) : 4;
}

template <int D, typename R, bool COLOR, int BLOCK, int VS = 0>
__global__ void __launch_bounds__(BLOCK, render_min_blocks<R>(VS)) chaos_kernel(const RenderArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    load_program<BLOCK>(smem, a.prog, a.prog_bytes);
    __syncthreads();
    chaos_body<D, R, COLOR, BLOCK, VS>(a, smem,
                                           (unsigned long long)blockIdx.x * BLOCK + threadIdx.x,
                                           (unsigned long long)gridDim.x * BLOCK);
}

// Persistent multi-flame render: each CTA claims (job, chunk of BLOCK
// streams) pairs from a global cursor, in the claim order of b.order, until
// the job table is exhausted.  A
// job's streams are the ones ffr_render would run for that context alone,
// so every job's buffer is the same alone and in the batch.  The claimed
// job's arguments are copied to shared memory and its program is reloaded
// only when the CTA moves to another job.
template <int D, typename R, bool COLOR, int BLOCK, int VS = 0>
__global__ void __launch_bounds__(BLOCK, render_min_blocks<R>(VS)) chaos_batch_kernel(const BatchArgs b)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(16) RenderArgs s_args;
    __shared__ unsigned long long s_chunk;
    __shared__ int s_job;
    int cur = -1;
    const unsigned long long total = b.head->total_chunks;
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            const unsigned long long c = atomicAdd(&b.head->cursor, 1ull);
            int j = -1;
            if (c < total)
            {
                const unsigned long long e = b.order[c];
                j = (int)(e >> 32);
                s_chunk = (e & 0xffffffffull) + b.jobs[j].chunk_first;
            }
            s_job = j;
        }
        __syncthreads();
        const int j = s_job;
        if (j < 0)
            break;
        if (j != cur)
        {
            const unsigned int* src = reinterpret_cast<const unsigned int*>(&b.jobs[j].a);
            unsigned int* dst = reinterpret_cast<unsigned int*>(&s_args);
            for (unsigned int k = threadIdx.x; k < sizeof(RenderArgs) / 4; k += BLOCK)
                dst[k] = src[k];
            __syncthreads();
            load_program<BLOCK>(smem, s_args.prog, s_args.prog_bytes);
            __syncthreads();
            cur = j;
        }
        chaos_body<D, R, COLOR, BLOCK, VS>(s_args, smem, s_chunk * BLOCK + threadIdx.x,
                                               ~0ull >> 1);
        __syncthreads();
    }
}

// XForm::applyIteration on a batch of points; point k uses stream
// key(KEY, k), as the reference driver seeds before each point.
template <int D, typename R>
__global__ void __launch_bounds__(128) step_kernel(const StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    load_program<128>(smem, a.prog, a.prog_bytes);
    __syncthreads();
    Prog<R> pg;
    pg.bind(smem, a.prog);
    uint64_t* ismem = reinterpret_cast<uint64_t*>(smem + align16u(a.prog_bytes));
    DevIsaac<128> rng;
    rng.mem = ismem + threadIdx.x;
    rng.rsl = ismem + 16 * 128 + threadIdx.x;
    const int xi = a.xf_index < 0 ? pg.h->nxf : a.xf_index;
    for (unsigned long long k = (unsigned long long)blockIdx.x * 128 + threadIdx.x;
         k < a.npts; k += (unsigned long long)gridDim.x * 128)
    {
        rng.seed(stream_key(a.key, k), a.isaac_init);
        R p[D], q[D];
#pragma unroll
        for (int i = 0; i < D; ++i)
            p[i] = (R)a.in[k * D + i];
        apply_xform<D, R>(pg, pg.xf[xi], p, q, rng);
#pragma unroll
        for (int i = 0; i < D; ++i)
            a.out[k * D + i] = (double)q[i];
    }
}

// One trajectory from stream key KEY: start, settle, then n samples
// (xform id and point after each), single thread.
template <int D, typename R>
__global__ void trace_kernel(const TraceArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    load_program<1>(smem, a.prog, a.prog_bytes);
    __syncthreads();
    Prog<R> pg;
    pg.bind(smem, a.prog);
    uint64_t* ismem = reinterpret_cast<uint64_t*>(smem + align16u(a.prog_bytes));
    DevIsaac<1> rng;
    rng.mem = ismem;
    rng.rsl = ismem + 16;
    rng.seed(a.key, a.isaac_init);
    using T = RealTraits<R>;
    R p[D];
#pragma unroll
    for (int i = 0; i < D; ++i)
        p[i] = R(2) * T::unit(rng.next()) - R(1);
    for (unsigned long long k = 0; k < a.settle; ++k)
    {
        R q[D];
        apply_xform<D, R>(pg, pg.xf[pick_xform<R>(pg, pg.h->nxf, rng)], p, q, rng);
#pragma unroll
        for (int i = 0; i < D; ++i)
            p[i] = q[i];
    }
    for (unsigned long long k = 0; k < a.n; ++k)
    {
        const int xi = pick_xform<R>(pg, pg.h->nxf, rng);
        R q[D];
        apply_xform<D, R>(pg, pg.xf[xi], p, q, rng);
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            p[i] = q[i];
            a.pts[k * D + i] = (double)q[i];
        }
        a.ids[k] = (int)pg.xf[xi].id;
    }
}

} // namespace ffr
