// Device variation functors, one case per reference class in
// src/variations/variations.hpp.  Each case states the reference lines it
// follows; the floating-point operation order is the reference's, so the FP64
// instantiation (compiled without FMA contraction) rounds exactly like the
// reference wherever only + - * / sqrt are involved.
//
// Calling convention: t = pre-affine point (D coordinates); o = V(t) with all
// D coordinates written (2-D variations write zero off their plane, as
// VariationFrom2D::calc_h does, variations.hpp:98-105).
#pragma once

#include "std_types.h"

#include "flame_program.h"
#include "isaac64.cuh"

namespace ffr {

template <typename R> struct RealTraits;

template <> struct RealTraits<double>
{
    // constants.hpp: eps<double> = 1e-20, bad_value_threshold<double> = 1e20
    static constexpr double eps = 1e-20;
    static constexpr double bad = 1e20;
    static constexpr double pi = 3.14159265358979323846;
    static constexpr double inv_pi = 0.31830988618379067154;   // M_1_PI
    // FlameRNG::randNum for double and u64 words: (w >> 11) / 2^53
    __device__ static __forceinline__ double unit(uint64_t w)
    {
        return (double)(w >> 11) * 0x1p-53;
    }
    __device__ static __forceinline__ double sin_(double x) { return sin(x); }
    __device__ static __forceinline__ double cos_(double x) { return cos(x); }
    __device__ static __forceinline__ void sincos_(double x, double* s, double* c) { sincos(x, s, c); }
    __device__ static __forceinline__ double atan2_(double y, double x) { return atan2(y, x); }
    __device__ static __forceinline__ double sqrt_(double x) { return sqrt(x); }
    __device__ static __forceinline__ double fabs_(double x) { return fabs(x); }
    __device__ static __forceinline__ double recip_(double x) { return 1.0 / x; }
    static constexpr double pi_4 = 0.78539816339744830962;      // M_PI_4
    __device__ static __forceinline__ double tan_(double x) { return tan(x); }
    __device__ static __forceinline__ double log_(double x) { return log(x); }
    __device__ static __forceinline__ double log10_(double x) { return log10(x); }
    __device__ static __forceinline__ double exp_(double x) { return exp(x); }
    __device__ static __forceinline__ double pow_(double x, double y) { return pow(x, y); }
    __device__ static __forceinline__ double sinh_(double x) { return sinh(x); }
    __device__ static __forceinline__ double cosh_(double x) { return cosh(x); }
    __device__ static __forceinline__ double acos_(double x) { return acos(x); }
    __device__ static __forceinline__ double floor_(double x) { return floor(x); }
    __device__ static __forceinline__ double fmod_(double x, double y) { return fmod(x, y); }
    __device__ static __forceinline__ double rint_(double x) { return rint(x); }
    __device__ static __forceinline__ double copysign_(double x, double y) { return copysign(x, y); }
    __device__ static __forceinline__ double hypot_(double x, double y) { return hypot(x, y); }
    __device__ static __forceinline__ double trunc_(double x) { return trunc(x); }
};

template <> struct RealTraits<float>
{
    // constants.hpp: eps<float> = 1e-10, bad_value_threshold<float> = 1e10
    static constexpr float eps = 1e-10f;
    static constexpr float bad = 1e10f;
    static constexpr float pi = 3.14159265358979323846f;
    static constexpr float inv_pi = 0.31830988618379067154f;
    // FlameRNG::randNum for float and u64 words: (w >> 40) / 2^24
    __device__ static __forceinline__ float unit(uint64_t w)
    {
        return (float)(uint32_t)(w >> 40) * 0x1p-24f;
    }
    // FP32 mode: SFU approximations (sin, cos, reciprocal); accepted by the
    // histogram total-variation check against the FP64 oracle
    __device__ static __forceinline__ float sin_(float x) { return __sinf(x); }
    __device__ static __forceinline__ float cos_(float x) { return __cosf(x); }
    __device__ static __forceinline__ void sincos_(float x, float* s, float* c) { __sincosf(x, s, c); }
    // atan2 from atan(t) ~ t * P(t^2) on [0, 1] (degree-6 P fitted for this
    // project by weighted least squares toward equal relative error; max
    // error 6e-7 rad) with the usual octant reduction
    __device__ static __forceinline__ float atan2_(float y, float x)
    {
        const float ax = fabsf(x), ay = fabsf(y);
        const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
        const float t = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
        const float s = t * t;
        float p = 0.007864936254918575f;
        p = fmaf(p, s, -0.03701813146471977f);
        p = fmaf(p, s, 0.08387769013643265f);
        p = fmaf(p, s, -0.13487586379051208f);
        p = fmaf(p, s, 0.1988159865140915f);
        p = fmaf(p, s, -0.3332653045654297f);
        p = fmaf(p, s, 0.9999993443489075f);
        float r = p * t;
        r = ay > ax ? 1.57079632679489662f - r : r;
        r = x < 0.0f ? 3.14159265358979324f - r : r;
        r = copysignf(r, y);
        return (x != x || y != y) ? x + y : r;
    }
    __device__ static __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    __device__ static __forceinline__ float fabs_(float x) { return fabsf(x); }
    __device__ static __forceinline__ float recip_(float x) { return __fdividef(1.0f, x); }
    static constexpr float pi_4 = 0.78539816339744830962f;
    __device__ static __forceinline__ float tan_(float x) { return tanf(x); }
    __device__ static __forceinline__ float log_(float x) { return logf(x); }
    __device__ static __forceinline__ float log10_(float x) { return log10f(x); }
    __device__ static __forceinline__ float exp_(float x) { return expf(x); }
    __device__ static __forceinline__ float pow_(float x, float y) { return powf(x, y); }
    __device__ static __forceinline__ float sinh_(float x) { return sinhf(x); }
    __device__ static __forceinline__ float cosh_(float x) { return coshf(x); }
    __device__ static __forceinline__ float acos_(float x) { return acosf(x); }
    __device__ static __forceinline__ float floor_(float x) { return floorf(x); }
    __device__ static __forceinline__ float fmod_(float x, float y) { return fmodf(x, y); }
    __device__ static __forceinline__ float rint_(float x) { return rintf(x); }
    __device__ static __forceinline__ float copysign_(float x, float y) { return copysignf(x, y); }
    __device__ static __forceinline__ float hypot_(float x, float y) { return hypotf(x, y); }
    __device__ static __forceinline__ float trunc_(float x) { return truncf(x); }
};

// t[i] for a run-time i without dynamic register indexing
template <int D, typename R>
__device__ __forceinline__ R coord(const R* t, int i)
{
    if (D == 1)
        return t[0];
    if (D == 2)
        return t[(i & 1) & (D - 1)];
    R r = t[0];
#pragma unroll
    for (int k = 1; k < D; ++k)
        r = i == k ? t[k] : r;
    return r;
}

// Point::normsum<2> (point.hpp:300-307): squares summed in coordinate order
template <int D, typename R>
__device__ __forceinline__ R nsq(const R* t)
{
    R r = t[0] * t[0];
#pragma unroll
    for (int i = 1; i < D; ++i)
        r += t[i] * t[i];
    return r;
}

// Point::norm<2> (point.hpp:270-290): |x| in 1-D, else sqrt(normsum<2>)
template <int D, typename R>
__device__ __forceinline__ R n2(const R* t)
{
    if (D == 1)
        return RealTraits<R>::fabs_(t[0]);
    return RealTraits<R>::sqrt_(nsq<D>(t));
}

// Point::normsum(p) (point.hpp:325-331)
template <int D, typename R>
__device__ __forceinline__ R normsum_p(const R* t, R p)
{
    using T = RealTraits<R>;
    R r = T::pow_(T::fabs_(t[0]), p);
#pragma unroll
    for (int i = 1; i < D; ++i)
        r += T::pow_(T::fabs_(t[i]), p);
    return r;
}

// FlameRNG::randGaussianPair (flame_rng.hpp:115-140), first value
template <typename R, typename Rng>
__device__ __forceinline__ R rand_gauss(Rng& rng)
{
    using T = RealTraits<R>;
    const R u1 = T::unit(rng.next());
    const R u2 = (R(2) * T::pi) * T::unit(rng.next());
    const R r = T::sqrt_(R(-2) * T::log_(u1));
    R s, c;
    T::sincos_(u2, &s, &c);
    return r * c;
}

// FlameRNG::randDirection<dims> (flame_rng.hpp:171-217); above 3 dims a
// vector of gaussian pairs (randGaussianPair, the last pair's second value
// unused for odd dims) divided by its norm, Point / k being multiplication
// by 1 / k (point.hpp:135-139)
template <int D, typename R, typename Rng>
__device__ __forceinline__ void rand_dir(Rng& rng, R* d)
{
    using T = RealTraits<R>;
    if (D > 3)
    {
#pragma unroll
        for (int i = 0; i < D; i += 2)
        {
            const R u1 = T::unit(rng.next());
            const R u2 = (R(2) * T::pi) * T::unit(rng.next());
            const R r = T::sqrt_(R(-2) * T::log_(u1));
            R s, c;
            T::sincos_(u2, &s, &c);
            d[i] = r * c;
            if (i + 1 < D)
                d[i + 1] = r * s;
        }
        const R k = R(1) / n2<D>(d);
#pragma unroll
        for (int i = 0; i < D; ++i)
            d[i] *= k;
        return;
    }
    if (D == 1)
    {
        d[0] = T::copysign_(R(1), T::unit(rng.next()) - R(0.5));
    }
    else if (D == 2)
    {
        const R a = (R(2) * T::pi) * T::unit(rng.next());
        R sa, ca;
        T::sincos_(a, &sa, &ca);
        d[0] = ca;
        d[D > 1 ? 1 : 0] = sa;
    }
    else
    {
        const R u = R(2) * T::unit(rng.next()) - R(1);
        const R tt = (R(2) * T::pi) * T::unit(rng.next());
        const R r = T::sqrt_(R(1) - u * u);
        R st, ct;
        T::sincos_(tt, &st, &ct);
        d[0] = r * ct;
        d[D > 1 ? 1 : 0] = r * st;
        d[D > 2 ? 2 : 0] = u;
    }
}

// The seven variations of the benchmark flames (linear, sinusoidal,
// spherical, swirl, horseshoe, polar, julia).
constexpr uint64_t kTierAMask = (1ull << V_LINEAR) | (1ull << V_SINUSOIDAL)
    | (1ull << V_SPHERICAL) | (1ull << V_SWIRL) | (1ull << V_HORSESHOE) | (1ull << V_POLAR)
    | (1ull << V_JULIA);

__host__ __device__ inline bool tier_a(int type)
{
    return type >= 0 && type < 64 && ((kTierAMask >> type) & 1ull);
}

// bits of ProgHeader::tier_a_present
enum : uint32_t
{
    kTaLinear = 1u << 0, kTaSinusoidal = 1u << 1, kTaSpherical = 1u << 2, kTaSwirl = 1u << 3,
    kTaHorseshoe = 1u << 4, kTaPolar = 1u << 5, kTaJulia = 1u << 6, kTaOther = 1u << 7
};

// Primitives of the pre-affine point shared by the 2-D benchmark variations
// of one xform application.  In a 2-D flame every 2-D variation acts on the
// plane (0, 1), so they are computed once per application, not once per
// variation (valid = false: the variation computes its own).
template <typename R>
struct PlanePrims
{
    bool valid;
    R q, rt, ang;       // x^2 + y^2, sqrt of it, atan2(y, x)
};

// The seven benchmark variations in one body.  In a warp whose lanes apply
// different variations, the 98-way switch runs one body per distinct type,
// each behind a divergent branch.  Here every shared primitive (sqrt of r^2
// for horseshoe/polar/julia, atan2 for polar/julia, one sincos for swirl and
// julia, one reciprocal for spherical and horseshoe) is computed by every
// lane, once, guarded only by `present` (the flame's set of types, uniform
// across the grid), and each lane selects its own result; the only per-lane
// branch left is julia's random word.  Every type still evaluates exactly
// its reference expression in the reference's operation order (the FP64
// results are bit-identical to the switch), and julia draws its word at the
// same point of the RNG sequence.
template <int D, typename R, int FIXED = -1, typename Rng>
__device__ __forceinline__ void variation_tier_a(const VarT<R>& v, const R* t, R* out, Rng& rng,
                                                 uint32_t present, const PlanePrims<R>& pp)
{
    using T = RealTraits<R>;
    const int ty = FIXED >= 0 ? FIXED : v.type;
    const bool is_sin = ty == V_SINUSOIDAL, is_sph = ty == V_SPHERICAL;
    if (!(present & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
    {
        // only N-D types in the flame: no plane coordinates needed
        R k = R(0);
        if (present & kTaSpherical)
            k = T::recip_(nsq<D>(t) + T::eps);          /* spherical 197-208 */
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            R o = t[i];                                 /* linear 169-177 */
            if (present & kTaSinusoidal)                /* sinusoidal 183-191 */
            {
                const R sn = T::sin_(t[i]);
                o = is_sin ? sn : o;
            }
            if (present & kTaSpherical)
            {
                const R sp = t[i] * k;
                o = is_sph ? sp : o;
            }
            out[i] = o;
        }
        return;
    }
    const bool is_nd = ty < kFirst2D;
    const bool is_sw = ty == V_SWIRL, is_hs = ty == V_HORSESHOE, is_po = ty == V_POLAR,
               is_ju = ty == V_JULIA;
    const int ax = v.axis_x, ay = v.axis_y;
    const R x = coord<D>(t, ax), y = coord<D>(t, ay);
    R q, rt = R(0), ang = R(0), s = R(0), c = R(0), k = R(0);
    if (pp.valid)
    {
        q = pp.q;
        rt = pp.rt;
        ang = pp.ang;
    }
    else
    {
        q = x * x + y * y;                              /* R2SQ */
        if (present & (kTaHorseshoe | kTaPolar | kTaJulia))
            rt = T::sqrt_(q);                           /* R2 */
        if (present & (kTaPolar | kTaJulia))
            ang = T::atan2_(y, x);
    }
    if (present & (kTaSwirl | kTaJulia))
    {
        R arg = q;                                      /* swirl 509-522: sincos(r^2) */
        if (present & kTaJulia)
        {
            R bit = R(0);
            if (is_ju)                                  /* julia 807-819: randBool */
                bit = (rng.next() & 1u) ? R(1) : R(0);
            const R ja = R(0.5) * ang + bit * T::pi;
            arg = is_ju ? ja : arg;
        }
        T::sincos_(arg, &s, &c);
    }
    if (present & (kTaSpherical | kTaHorseshoe))
    {
        R den = rt + T::eps;                            /* horseshoe 527-540 */
        if (present & kTaSpherical)
        {
            const R ds = nsq<D>(t) + T::eps;            /* spherical 197-208 */
            den = is_sph ? ds : den;
        }
        k = T::recip_(den);
    }
    R X = R(0), Y = R(0);
    if (present & kTaSwirl)
    {
        const R a0 = x * s - y * c, a1 = x * c + y * s;
        X = is_sw ? a0 : X;
        Y = is_sw ? a1 : Y;
    }
    if (present & kTaHorseshoe)
    {
        const R a0 = ((x - y) * (x + y)) * k, a1 = (R(2.0) * x * y) * k;
        X = is_hs ? a0 : X;
        Y = is_hs ? a1 : Y;
    }
    if (present & kTaPolar)                             /* polar 545-555 */
    {
        const R a0 = ang * T::inv_pi, a1 = rt - R(1.0);
        X = is_po ? a0 : X;
        Y = is_po ? a1 : Y;
    }
    if (present & kTaJulia)
    {
        const R a0 = c * rt, a1 = s * rt;
        X = is_ju ? a0 : X;
        Y = is_ju ? a1 : Y;
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
    {
        R o = t[i];                                     /* linear 169-177 */
        if (present & kTaSinusoidal)                    /* sinusoidal 183-191 */
        {
            const R sn = T::sin_(t[i]);
            o = is_sin ? sn : o;
        }
        if (present & kTaSpherical)
        {
            const R sp = t[i] * k;
            o = is_sph ? sp : o;
        }
        const R p2 = i == ax ? X : (i == ay ? Y : R(0));
        out[i] = is_nd ? o : p2;
    }
}

// julia's random bit (FlameRNG::randBool, w & 1) in lanes whose xform has
// julia, nothing drawn in the others
template <typename Rng>
__device__ __forceinline__ uint32_t julia_bit(Rng& rng, bool has, bool)
{
    return has ? (uint32_t)(rng.next() & 1u) : 0u;
}
// the render kernels' generator: with the carry area in use the word is
// known to be in the result array, so it is taken without a branch (the
// same word next() would return)
template <int B, int C>
__device__ __forceinline__ uint32_t julia_bit(DevIsaac<B, C>& rng, bool has, bool carry)
{
    if (!carry)
        return has ? (uint32_t)(rng.next() & 1u) : 0u;
    const uint32_t hj = has ? 1u : 0u;
    rng.cnt -= hj;
    const uint64_t w = rng.Rs((int)min(rng.cnt, (uint32_t)(C - 1)));
    return hj & (uint32_t)w;
}

// The merged form of an FP32 xform application (ProgHeader::merged):
// v = sum over the flame's types T of coef[T] * V_T(t), each type evaluated
// once whatever the number of variation slots, instead of one evaluation
// (of every type present, then a select) per slot.  The types' formulas are
// those of variation_tier_a; only the order of the weighted sum differs
// from the reference's slot order, which FP32 rounding already departs
// from.  A type the xform lacks has coef 0 and contributes 0 * V_T(t) = 0
// because every V_T is finite while sum t_i^2 < 1e36; beyond that (and for
// NaN) the function returns false and the caller evaluates the slots one by
// one, so an infinite or NaN point propagates exactly as per-slot
// evaluation propagates it.  Julia draws its word only in lanes whose xform
// has julia (coef[7], even at weight 0), at the same point of the sequence
// as the per-slot loop (the xform's only drawing variation, so its place
// among the slots does not matter).
//
// ALL: every one of the seven types is evaluated, without a branch per type
// (a type absent from the flame has coef 0 in every xform): one block of
// straight-line code the compiler schedules across types, for flames that
// use most of them.  carry: the render kernels' refill ahead guarantees
// julia's word is in the result array (ISAAC carry area), so the draw is a
// conditional take instead of a branch.  Neither changes which words are
// drawn or what is added.
//
// Above 2 dims each of swirl, horseshoe, polar and julia acts on its own
// plane (XformT::plane, per lane): its coordinates are read from that plane
// and its result added back to it (VariationFrom2D::calc_h,
// variations.hpp:98-105), its primitives computed on that plane.
template <int D, bool ALL = false, typename Rng>
__device__ __forceinline__ bool merged_variations(const float* coef, const float* t, float* v,
                                                  Rng& rng, uint32_t present, bool carry = false,
                                                  const uint8_t* planes = nullptr)
{
    using T = RealTraits<float>;
    if (ALL)
        present = kTaLinear | kTaSinusoidal | kTaSpherical | kTaSwirl | kTaHorseshoe
            | kTaPolar | kTaJulia;
    const float4 c0 = *reinterpret_cast<const float4*>(coef);
    const float4 c1 = *reinterpret_cast<const float4*>(coef + 4);
    const float q = nsq<D>(t);
    if (!(q < 1e36f))
        return false;
#pragma unroll
    for (int i = 0; i < D; ++i)
        v[i] = 0.0f;
    if (present & kTaLinear)                                     /* linear 169-177 */
#pragma unroll
        for (int i = 0; i < D; ++i)
            v[i] = c0.x * t[i];
    if (present & kTaSinusoidal)                                 /* sinusoidal 183-191 */
#pragma unroll
        for (int i = 0; i < D; ++i)
            v[i] = fmaf(c0.y, T::sin_(t[i]), v[i]);
    if (present & kTaSpherical)                                  /* spherical 197-208 */
    {
        const float k = c0.z * T::recip_(q + T::eps);
#pragma unroll
        for (int i = 0; i < D; ++i)
            v[i] = fmaf(k, t[i], v[i]);
    }
    if (D == 2 && (present & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
    {
        const float x = t[0], y = t[D - 1];
        float rt = 0.0f, ang = 0.0f;
        // sqrt(q) as q / sqrt(q) from the reciprocal square root (two
        // instructions instead of the correctly rounded sequence; a few ulp)
        if (present & (kTaHorseshoe | kTaPolar | kTaJulia))
            rt = q > 0.0f ? q * rsqrtf(q) : 0.0f;
        if (present & (kTaPolar | kTaJulia))
            ang = T::atan2_(y, x);
        float X = v[0], Y = v[D - 1];
        if (present & kTaSwirl)                                  /* swirl 509-522 */
        {
            float s, c;
            T::sincos_(q, &s, &c);
            X = fmaf(c0.w, x * s - y * c, X);
            Y = fmaf(c0.w, x * c + y * s, Y);
        }
        if (present & kTaHorseshoe)                              /* horseshoe 527-540 */
        {
            const float k = c1.x * T::recip_(rt + T::eps);
            X = fmaf(k, (x - y) * (x + y), X);
            Y = fmaf(k, 2.0f * x * y, Y);
        }
        if (present & kTaPolar)                                  /* polar 545-555 */
        {
            X = fmaf(c1.y, ang * T::inv_pi, X);
            Y = fmaf(c1.y, rt - 1.0f, Y);
        }
        if (present & kTaJulia)                                  /* julia 807-819 */
        {
            const float bit = julia_bit(rng, c1.w != 0.0f, carry) ? 1.0f : 0.0f;
            float s, c;
            T::sincos_(0.5f * ang + bit * T::pi, &s, &c);
            const float k = c1.z * rt;
            X = fmaf(k, c, X);
            Y = fmaf(k, s, Y);
        }
        v[0] = X;
        v[D - 1] = Y;
    }
    if (D > 2 && (present & (kTaSwirl | kTaHorseshoe | kTaPolar | kTaJulia)))
    {
        const uint2 pl = *reinterpret_cast<const uint2*>(planes);
        // plane k of (swirl, horseshoe, polar, julia): its x, y and a way to
        // add (X, Y) back onto those coordinates
        auto on_plane = [&](int k, float& x, float& y, int& ax, int& ay) {
            const uint32_t w = k < 2 ? pl.x : pl.y;
            ax = (int)((w >> (16 * (k & 1))) & 0xffu);
            ay = (int)((w >> (16 * (k & 1) + 8)) & 0xffu);
            x = coord<D>(t, ax);
            y = coord<D>(t, ay);
        };
        auto add = [&](int ax, int ay, float X, float Y) {
#pragma unroll
            for (int i = 0; i < D; ++i)
                v[i] += i == ax ? X : (i == ay ? Y : 0.0f);
        };
        float x, y;
        int ax, ay;
        if (present & kTaSwirl)                                  /* swirl 509-522 */
        {
            on_plane(0, x, y, ax, ay);
            float s, c;
            T::sincos_(x * x + y * y, &s, &c);
            add(ax, ay, c0.w * (x * s - y * c), c0.w * (x * c + y * s));
        }
        if (present & kTaHorseshoe)                              /* horseshoe 527-540 */
        {
            on_plane(1, x, y, ax, ay);
            const float q2 = x * x + y * y;
            const float rt = q2 > 0.0f ? q2 * rsqrtf(q2) : 0.0f;
            const float k = c1.x * T::recip_(rt + T::eps);
            add(ax, ay, k * ((x - y) * (x + y)), k * (2.0f * x * y));
        }
        if (present & kTaPolar)                                  /* polar 545-555 */
        {
            on_plane(2, x, y, ax, ay);
            const float q2 = x * x + y * y;
            const float rt = q2 > 0.0f ? q2 * rsqrtf(q2) : 0.0f;
            add(ax, ay, c1.y * (T::atan2_(y, x) * T::inv_pi), c1.y * (rt - 1.0f));
        }
        if (present & kTaJulia)                                  /* julia 807-819 */
        {
            on_plane(3, x, y, ax, ay);
            const float bit = julia_bit(rng, c1.w != 0.0f, carry) ? 1.0f : 0.0f;
            const float q2 = x * x + y * y;
            const float rt = q2 > 0.0f ? q2 * rsqrtf(q2) : 0.0f;
            float s, c;
            T::sincos_(0.5f * T::atan2_(y, x) + bit * T::pi, &s, &c);
            const float k = c1.z * rt;
            add(ax, ay, k * c, k * s);
        }
    }
    return true;
}

// one variation: o = V(t).  Restates each class of
// src/variations/variations.hpp (line numbers in the case comments) in the
// reference's operation order; Point / k is multiplication by (1/k), as
// Point::operator/= does (src/types/point.hpp:127-131).  RNG draws go
// through rng.next() in the reference's order (FlameRNG,
// src/rng/flame_rng.hpp).
//
// FIXED >= 0: the variation's type is FIXED, known when the kernel is
// compiled (the per-flame kernels, jit.cpp); the same expressions as for a
// type read from v, with the other types' code left out.
template <int D, typename R, int FIXED = -1, typename Rng>
__device__ __forceinline__ void variation(const VarT<R>& v, const R* t, R* o, Rng& rng,
                                          uint32_t present, const PlanePrims<R>& pp)
{
    using T = RealTraits<R>;
    const int vtype = FIXED >= 0 ? FIXED : v.type;
    if (tier_a(vtype))
    {
        variation_tier_a<D, R, FIXED>(v, t, o, rng, present, pp);
        return;
    }
    const int ax = v.axis_x, ay = v.axis_y;
    R* out = o;

    const R* P = v.p;
    R x, y, r, a, s, c, X = R(0), Y = R(0), d;
        if (vtype < kFirst2D) {
        switch (vtype) {
        case V_LINEAR: /* 169-177 */
            for (int i = 0; i < D; ++i) out[i] = t[i];
            return;
        case V_SINUSOIDAL: /* 183-191 */
            for (int i = 0; i < D; ++i) out[i] = T::sin_(t[i]);
            return;
        case V_SPHERICAL: /* 197-208 */
            r = T::recip_(nsq<D>(t) + T::eps);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_BENT: /* 216-240: p = neg[dims], pos[dims] */
            for (int i = 0; i < D; ++i)
                out[i] = t[i] < R(0.0) ? t[i] * P[i] : t[i] * P[D + i];
            return;
        case V_RECTANGLES: /* 245-270 */
            for (int i = 0; i < D; ++i)
                out[i] = P[i] == R(0.0) ? t[i]
                    : (R(2.0) * T::floor_(t[i] / P[i]) + R(1.0)) * P[i] - t[i];
            return;
        case V_FISHEYE: /* 275-292: p = addval */
            r = T::recip_(n2<D>(t) + P[0]);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_BUBBLE: /* 297-314 */
            r = T::recip_(nsq<D>(t) + P[0]);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_NOISE: { /* 319-330 */
            R dir[D];
            r = T::unit(rng.next());
            rand_dir<D, R>(rng, dir);
            for (int i = 0; i < D; ++i) out[i] = (t[i] * dir[i]) * r;
            return;
        }
        case V_BLUR: { /* 335-347 */
            R dir[D];
            r = T::unit(rng.next());
            rand_dir<D, R>(rng, dir);
            for (int i = 0; i < D; ++i) out[i] = dir[i] * r;
            return;
        }
        case V_GAUSSIAN_BLUR: /* 352-364 */
        case V_PRE_BLUR: { /* 434-446 */
            R dir[D];
            r = rand_gauss<R>(rng);
            rand_dir<D, R>(rng, dir);
            for (int i = 0; i < D; ++i) out[i] = dir[i] * r;
            return;
        }
        case V_SQUARE_NOISE: /* 369-378, randPoint2 */
            for (int i = 0; i < D; ++i) out[i] = T::unit(rng.next()) - R(0.5);
            return;
        case V_SEPARATION: /* 383-405: p = sep^2[dims], inside[dims] */
            for (int i = 0; i < D; ++i) {
                s = T::copysign_(R(1.0), t[i]);
                out[i] = s * (T::sqrt_(t[i] * t[i] + P[i]) - s * P[D + i]);
            }
            return;
        case V_SPLITS: /* 410-429 */
            for (int i = 0; i < D; ++i) {
                s = T::copysign_(R(1.0), t[i]);
                out[i] = t[i] + s * P[i];
            }
            return;
        case V_MODULUS: /* 451-471: p = 2*params, 1/(2*params) */
            for (int i = 0; i < D; ++i)
                out[i] = t[i] - P[i] * T::floor_(t[i] * P[D + i] + R(0.5));
            return;
        case V_CELLN: /* 476-505: p = sizes, 1/sizes */
            for (int i = 0; i < D; ++i) {
                R fx = T::floor_(t[i] * P[D + i]);
                R dx = t[i] - fx * P[i];
                R xs = T::copysign_(R(2.0), fx);
                R x2 = fx * xs;
                x2 -= (R)(fx < 0);
                out[i] = dx + x2 * P[i];
            }
            return;
        case V_SPHERICAL_P: /* 2312-2328 */
            r = T::recip_(normsum_p<D>(t, P[0]) + T::eps);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_UNIT_SPHERE: /* 2333-2342 */
            r = T::recip_(n2<D>(t) + T::eps);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_UNIT_SPHERE_P: /* 2347-2363: norm(p) = T::pow_(normsum, 1/p) */
            r = T::recip_(T::pow_(normsum_p<D>(t, P[0]), R(1.0) / P[0]) + T::eps);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        case V_UNIT_CUBE: { /* 2368-2376: norm<0> */
            R m = T::fabs_(t[0]);
            if (D > 1)
                for (int i = 1; i < D; ++i) {
                    R q = T::fabs_(t[i]);
                    m = (m < q) ? q : m;
                }
            r = T::recip_(m + T::eps);
            for (int i = 0; i < D; ++i) out[i] = t[i] * r;
            return;
        }
        default:
            for (int i = 0; i < D; ++i) out[i] = (R(0) / R(0));
            return;
        }
    }
    x = coord<D>(t, ax);
    y = coord<D>(t, ay);
#define R2SQ (x * x + y * y)
#define R2 T::sqrt_(x * x + y * y)
#define ANG T::atan2_(y, x)
    switch (vtype) {
    case V_SWIRL: /* 509-522 */
        r = R2SQ; T::sincos_(r, &s, &c);
        X = x * s - y * c; Y = x * c + y * s; break;
    case V_HORSESHOE: /* 527-540 */
        r = T::recip_(R2 + T::eps);
        X = ((x - y) * (x + y)) * r; Y = (R(2.0) * x * y) * r; break;
    case V_POLAR: /* 545-555 */
        a = ANG; r = R2; X = a * T::inv_pi; Y = r - R(1.0); break;
    case V_POLAR2: /* 561-570 */
        X = ANG; Y = T::log_(R2SQ); break;
    case V_HANDKERCHIEF: /* 575-585 */
        a = ANG; r = R2; X = T::sin_(a + r) * r; Y = T::cos_(a - r) * r; break;
    case V_HEART: /* 590-602 */
        a = ANG; r = R2; T::sincos_(r * a, &s, &c); X = s * r; Y = (-c) * r; break;
    case V_DISC: /* 607-619 */
        a = ANG; r = R2; T::sincos_(T::pi * r, &s, &c); X = s * a; Y = c * a; break;
    case V_DISC2: /* 624-655: p = rotpi, cosadd, sinadd */
        d = P[0] * (x + y); T::sincos_(d, &s, &c); a = ANG;
        X = (c + P[1]) * a; Y = (s + P[2]) * a; break;
    case V_WAVES: /* 660-680: p = xf, xs, yf, ys */
        X = x + P[1] * T::sin_(y * P[0]); Y = y + P[3] * T::sin_(x * P[2]); break;
    case V_FAN: { /* 685-709: p = dx, dy */
        R dx2 = P[0] * R(0.5);
        a = ANG;
        R m = T::copysign_(R(1.0), dx2 - T::fmod_(a + P[1], P[0]));
        a += m * dx2;
        T::sincos_(a, &s, &c);
        r = R2;
        X = c * r; Y = s * r; break;
    }
    case V_RINGS: /* 714-733: p = dx */
        r = R2; s = y / r; c = x / r;
        r = T::fmod_(r + P[0], R(2.0) * P[0]) - P[0] + r * (R(1.0) - P[0]);
        X = c * r; Y = s * r; break;
    case V_SPIRAL: { /* 738-752 */
        R sa, ca, sr, cr;
        r = R2; sa = y / r; ca = x / r;
        T::sincos_(r, &sr, &cr);
        R r1 = T::recip_(r + T::eps);
        X = (ca + sr) * r1; Y = (sa - cr) * r1; break;
    }
    case V_HYPERBOLIC: /* 757-767 */
        r = R2; s = y / r; c = x / r;
        X = s / (r + T::eps); Y = c * r; break;
    case V_DIAMOND: { /* 772-784 */
        R sr, cr;
        r = R2; s = y / r; c = x / r;
        T::sincos_(r, &sr, &cr);
        X = s * cr; Y = c * sr; break;
    }
    case V_EX: { /* 789-803 */
        a = ANG; r = R2;
        R n0 = T::sin_(a + r), n1 = T::cos_(a - r);
        R m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
        X = m0 + m1; Y = m0 - m1; break;
    }
    case V_JULIA: /* 807-819 */
        a = R(0.5) * T::atan2_(y, x) + ((rng.next() & 1u) ? R(1) : R(0)) * T::pi;
        T::sincos_(a, &s, &c);
        r = R2;
        X = c * r; Y = s * r; break;
    case V_EXPONENTIAL: /* 825-838 */
        d = T::exp_(x - R(1.0)); T::sincos_(T::pi * y, &s, &c);
        X = c * d; Y = s * d; break;
    case V_POWER: /* 843-853 */
        r = R2; s = y / r; c = x / r; d = T::pow_(r, s);
        X = c * d; Y = s * d; break;
    case V_COSINE: /* 858-870 */
        T::sincos_(x * T::pi, &s, &c);
        X = c * T::cosh_(y); Y = (-s) * T::sinh_(y); break;
    case V_BLOB: /* 875-896: p = mid, amp, waves */
        r = R2; s = y / r; c = x / r; a = ANG;
        r *= P[0] + P[1] * T::sin_(P[2] * a);
        X = c * r; Y = s * r; break;
    case V_PDJ: /* 901-925: p = a, b, c, d */
        X = T::sin_(P[0] * y) - T::cos_(P[1] * x); Y = T::sin_(P[2] * x) - T::cos_(P[3] * y); break;
    case V_CYLINDER: /* 930-938 */
        X = T::sin_(x); Y = y; break;
    case V_PERSPECTIVE: /* 943-962: p = dist, vsin, vfcos */
        d = T::recip_(P[0] - y * P[1]);
        X = (P[0] * x) * d; Y = (P[2] * y) * d; break;
    case V_JULIAN: { /* 967-989: p = abspower, invpower, cn */
        int32_t tt = (int32_t)T::trunc_(P[0] * T::unit(rng.next()));
        a = (T::atan2_(y, x) + (R(2.0) * T::pi) * tt) * P[1];
        r = T::pow_(R2SQ, P[2]);
        T::sincos_(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case V_JULIASCOPE: { /* 994-1018 */
        int32_t tt = (int32_t)T::trunc_(P[0] * T::unit(rng.next()));
        R dir = T::copysign_(R(1.0), T::unit(rng.next()) - R(0.5));
        a = ((R(2.0) * T::pi) * tt + dir * T::atan2_(y, x)) * P[1];
        r = T::pow_(R2SQ, P[2]);
        T::sincos_(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case V_RADIAL_BLUR: { /* 1023-1045: p = spin, zoom, flam3weight */
        R g = P[2] * rand_gauss<R>(rng);
        R ra = R2;
        a = T::atan2_(y, x) + P[0] * g;
        T::sincos_(a, &s, &c);
        R rz = P[1] * g - R(1.0);
        X = c * ra + x * rz; Y = s * ra + y * rz; break;
    }
    case V_PIE: { /* 1050-1072: p = slices, rotation, thickness, invslices2pi */
        int32_t sl = (int32_t)(T::unit(rng.next()) * P[0] + R(0.5));
        a = P[1] + (sl + T::unit(rng.next()) * P[2]) * P[3];
        r = T::unit(rng.next());
        T::sincos_(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case V_NGON: { /* 1077-1102: p = powerval, angle, corners, circle, invangle */
        r = T::pow_(R2SQ, P[0]);
        R theta = T::atan2_(y, x);
        R phi = theta - P[1] * T::floor_(theta * P[4]);
        phi -= (phi > P[1] * R(0.5) ? R(1.0) : R(0.0)) * P[1];
        R amp = P[2] * (T::recip_(T::cos_(phi) + T::eps) - R(1.0)) + P[3];
        amp /= r + T::eps;
        X = x * amp; Y = y * amp; break;
    }
    case V_CURL: { /* 1107-1129: p = c1, c2 */
        R re = R(1.0) + P[0] * x + P[1] * (x * x - y * y);
        R im = P[0] * y + R(2.0) * P[1] * x * y;
        r = T::recip_(re * re + im * im + T::eps);
        X = (x * re + y * im) * r; Y = (y * re - x * im) * r; break;
    }
    case V_ARCH: /* 1134-1151: p = flam3weight */
        a = P[0] * T::unit(rng.next()) * T::pi;
        T::sincos_(a, &s, &c);
        X = s; Y = s * s / c; break;
    case V_TANGENT: /* 1156-1166 */
        X = T::sin_(x) / T::cos_(y); Y = T::tan_(y); break;
    case V_RAYS: /* 1172-1191 */
        a = P[0] * T::unit(rng.next()) * T::pi;
        r = P[0] / (R2SQ + T::eps);
        d = T::tan_(a) * r;
        X = T::cos_(x) * d; Y = T::sin_(y) * d; break;
    case V_BLADE: { /* 1196-1213 */
        R sr, cr;
        r = T::unit(rng.next()) * P[0] * R2;
        T::sincos_(r, &sr, &cr);
        X = (cr + sr) * x; Y = (cr - sr) * x; break;
    }
    case V_SECANT: { /* 1218-1235 */
        R cr = T::cos_(P[0] * R2);
        R icr = R(1.0) / cr;
        R sg = T::copysign_(R(1.0), -cr);
        X = x; Y = icr + sg; break;
    }
    case V_TWINTRIAN: { /* 1240-1260 */
        R sr, cr;
        r = T::unit(rng.next()) * P[0] * R2;
        T::sincos_(r, &sr, &cr);
        R diff = T::log10_(sr * sr) + cr;
        if (T::fabs_(diff) > T::bad || (diff != diff))
            diff = -R(30.0);
        X = diff * x; Y = (diff - sr * T::pi) * x; break;
    }
    case V_CROSS: /* 1265-1277 */
        s = x * x - y * y;
        r = T::sqrt_(T::recip_(s * s + T::eps));
        X = x * r; Y = y * r; break;
    case V_EXP: /* 1282-1295 */
        d = T::exp_(x); T::sincos_(y, &s, &c);
        X = c * d; Y = s * d; break;
    case V_LOG: /* 1300-1308 */
        X = T::log_(R2SQ); Y = T::atan2_(y, x); break;
    case V_SIN: /* 1313-1327 */
        T::sincos_(x, &s, &c);
        X = s * T::cosh_(y); Y = c * T::sinh_(y); break;
    case V_COS: /* 1332-1346 */
        T::sincos_(x, &s, &c);
        { R ch = T::cosh_(y), sh = T::sinh_(y); X = c * ch; Y = (-s) * sh; }
        break;
    case V_TAN: { /* 1351-1366 */
        T::sincos_(R(2.0) * x, &s, &c);
        R sh = T::sinh_(R(2.0) * y), ch = T::cosh_(R(2.0) * y);
        d = T::recip_(c + ch);
        X = s * d; Y = sh * d; break;
    }
    case V_SEC: { /* 1371-1386 */
        T::sincos_(x, &s, &c);
        R sh = T::sinh_(y), ch = T::cosh_(y);
        d = T::recip_(T::cos_(R(2.0) * x) + T::cosh_(R(2.0) * y));
        X = (c * ch) * d; Y = (s * sh) * d; break;
    }
    case V_CSC: { /* 1391-1406 */
        T::sincos_(x, &s, &c);
        R sh = T::sinh_(y), ch = T::cosh_(y);
        d = T::recip_(T::cosh_(R(2.0) * y) - T::cos_(R(2.0) * x));
        X = (s * ch) * d; Y = ((-c) * sh) * d; break;
    }
    case V_COT: { /* 1411-1426 */
        T::sincos_(R(2.0) * x, &s, &c);
        R sh = T::sinh_(R(2.0) * y), ch = T::cosh_(R(2.0) * y);
        d = T::recip_(ch - c);
        X = s * d; Y = (-sh) * d; break;
    }
    case V_SINH: { /* 1431-1445 */
        T::sincos_(y, &s, &c);
        R sh = T::sinh_(x), ch = T::cosh_(x);
        X = sh * c; Y = ch * s; break;
    }
    case V_COSH: { /* 1450-1464 */
        T::sincos_(y, &s, &c);
        R sh = T::sinh_(x), ch = T::cosh_(x);
        X = ch * c; Y = sh * s; break;
    }
    case V_TANH: { /* 1469-1484 */
        T::sincos_(R(2.0) * y, &s, &c);
        R sh = T::sinh_(R(2.0) * x), ch = T::cosh_(R(2.0) * x);
        d = T::recip_(c + ch);
        X = sh * d; Y = s * d; break;
    }
    case V_SECH: { /* 1489-1504 */
        T::sincos_(y, &s, &c);
        R sh = T::sinh_(x), ch = T::cosh_(x);
        d = T::recip_(T::cos_(R(2.0) * y) + T::cosh_(R(2.0) * x));
        X = (c * ch) * d; Y = ((-s) * sh) * d; break;
    }
    case V_CSCH: { /* 1509-1524 */
        T::sincos_(y, &s, &c);
        R sh = T::sinh_(x), ch = T::cosh_(x);
        d = T::recip_(T::cosh_(R(2.0) * x) - T::cos_(R(2.0) * y));
        X = (sh * c) * d; Y = ((-ch) * s) * d; break;
    }
    case V_COTH: { /* 1529-1544 */
        T::sincos_(R(2.0) * y, &s, &c);
        R sh = T::sinh_(R(2.0) * x), ch = T::cosh_(R(2.0) * x);
        d = T::recip_(ch - c);
        X = sh * d; Y = s * d; break;
    }
    case V_AUGER: { /* 1549-1571: p = freq, weight, scale/2, sym */
        R ss = T::sin_(P[0] * x), tt = T::sin_(P[0] * y);
        R dy = y + P[1] * (P[2] + T::fabs_(y)) * ss;
        R dx = x + P[1] * (P[2] + T::fabs_(x)) * tt;
        X = x + P[3] * (dx - x); Y = dy; break;
    }
    case V_FLUX: { /* 1576-1600: p = 2 + spread, weight */
        R xpw = x + P[1], xmw = x - P[1], y2 = y * y;
        R avgr = P[0] * T::sqrt_(T::sqrt_(y2 + xpw * xpw) / T::sqrt_(y2 + xmw * xmw));
        R avga = (T::atan2_(y, xmw) - T::atan2_(y, xpw)) * R(0.5);
        /* sincosg(avga, c, s) stores the sine in c (variations.hpp:1597) */
        T::sincos_(avga, &c, &s);
        X = c * avgr; Y = s * avgr; break;
    }
    case V_MOBIUS: { /* 1605-1630: p = a0 a1 b0 b1 c0 c1 d0 d1 */
        R re_u = P[0] * x - P[1] * y + P[2];
        R im_u = P[0] * y + P[1] * x + P[3];
        R re_v = P[4] * x - P[5] * y + P[6];
        R im_v = P[4] * y + P[5] * x + P[7];
        R rad = T::recip_(re_v * re_v + im_v * im_v + T::eps);
        X = (re_u * re_v + im_u * im_v) * rad;
        Y = (im_u * re_v - re_u * im_v) * rad; break;
    }
    case V_SCRY: { /* 1635-1650 */
        R tt = R2SQ;
        r = T::recip_(T::sqrt_(tt) * (tt + T::recip_(P[0] + T::eps)));
        X = x * r; Y = y * r; break;
    }
    case V_SPLIT: { /* 1655-1673: p = xsize*pi, ysize*pi */
        R xs = T::copysign_(R(1.0), T::cos_(x * P[0]));
        R ys = T::copysign_(R(1.0), T::cos_(y * P[1]));
        X = x * ys; Y = y * xs; break;
    }
    case V_STRIPES: { /* 1678-1696: p = 1 - space, warp */
        R rx = T::floor_(x + R(0.5)), ox = x - rx;
        X = ox * P[0] + rx; Y = y + ox * ox * P[1]; break;
    }
    case V_WEDGE: { /* 1701-1724: p = swirl, count, angle, hole, cf */
        r = R2;
        a = T::atan2_(y, x) + P[0] * r;
        R cc = T::floor_((P[1] * a + T::pi) * (T::inv_pi * R(0.5)));
        a = a * P[4] + cc * P[2];
        T::sincos_(a, &s, &c);
        X = c * (r + P[3]); Y = s * (r + P[3]); break;
    }
    case V_WEDGE_JULIA: { /* 1729-1756: p = angle, count, invpower, cn, abspower, cf */
        r = T::pow_(R2SQ, P[3]);
        int32_t tr = (int32_t)(P[4] * T::unit(rng.next()));
        a = (T::atan2_(y, x) + (R(2.0) * T::pi) * tr) * P[2];
        R cc = T::floor_((P[1] * a + T::pi) * (T::inv_pi * R(0.5)));
        a = a * P[5] + cc * P[0];
        T::sincos_(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case V_WEDGE_SPH: { /* 1761-1785: p = angle, count, swirl, hole, cf */
        r = T::recip_(R2 + T::eps);
        a = T::atan2_(y, x) + P[2] * r;
        R cc = T::floor_((P[1] * a + T::pi) * (T::inv_pi * R(0.5)));
        a = a * P[4] + cc * P[0];
        T::sincos_(a, &s, &c);
        X = c * (r + P[3]); Y = s * (r + P[3]); break;
    }
    case V_WHORL: /* 1790-1810: p = inside, outside, weight */
        r = R2;
        a = T::atan2_(y, x);
        a += (r >= P[2] ? P[1] : P[0]) / (P[2] - r);
        T::sincos_(a, &s, &c);
        X = c * r; Y = s * r; break;
    case V_SUPERSHAPE: { /* 1815-1842: p = m/4, -1/n1, n2, n3, rnd, holes */
        R theta = P[0] * T::atan2_(y, x) + T::pi_4;
        R st, ct;
        T::sincos_(theta, &st, &ct);
        R t1 = T::pow_(T::fabs_(ct), P[2]), t2 = T::pow_(T::fabs_(st), P[3]);
        R tr = R2;
        r = (P[4] * T::unit(rng.next()) + (R(1.0) - P[4]) * tr) - P[5];
        r *= T::pow_(t1 + t2, P[1]) / tr;
        X = x * r; Y = y * r; break;
    }
    case V_FLOWER: /* 1847-1864: p = petals, holes */
        r = (T::unit(rng.next()) - P[1]) * T::cos_(P[0] * T::atan2_(y, x));
        r /= R2 + T::eps;
        X = x * r; Y = y * r; break;
    case V_CONIC: { /* 1869-1886: p = eccen, holes */
        R tr = R2;
        R ct = x / (tr + T::eps);
        r = (T::unit(rng.next()) - P[1]) * P[0] / (tr + tr * P[0] * ct);
        X = x * r; Y = y * r; break;
    }
    case V_PARABOLA: { /* 1891-1909: p = height, width */
        R sr, cr;
        T::sincos_(R2, &sr, &cr);
        X = P[0] * sr * sr * T::unit(rng.next());
        Y = P[1] * cr * T::unit(rng.next()); break;
    }
    case V_BIPOLAR: { /* 1914-1935: p = -pi/2 * shift */
        R x2y2 = R2SQ, tt = x2y2 + R(1.0), x2 = R(2.0) * x;
        R yy = R(0.5) * T::atan2_(R(2.0) * y, x2y2 - R(1.0)) + P[0];
        yy -= T::pi * T::floor_(yy * T::inv_pi + R(0.5));
        X = T::log_((tt + x2) / (tt - x2)); Y = yy; break;
    }
    case V_BOARDERS: { /* 1940-1983: p = prob */
        R rx = T::rint_(x), ry = T::rint_(y), ox = x - rx, oy = y - ry;
        if (T::unit(rng.next()) >= P[0]) {
            X = ox * R(0.5) + rx; Y = oy * R(0.5) + ry;
        } else {
            R mag = R(1.0) - P[0];
            if (T::fabs_(ox) >= T::fabs_(oy)) {
                R sg = T::copysign_(mag, ox);
                X = ox * R(0.5) + rx + sg; Y = oy * R(0.5) + ry + sg * oy / ox;
            } else {
                R sg = T::copysign_(mag, oy);
                X = ox * R(0.5) + rx + sg * ox / oy; Y = oy * R(0.5) + ry + sg;
            }
        }
        break;
    }
    case V_BUTTERFLY: { /* 1988-2003 */
        R y2 = R(2.0) * y;
        r = T::sqrt_(T::fabs_(x * y) / (x * x + y2 * y2 + T::eps));
        X = x * r; Y = y2 * r; break;
    }
    case V_CELL: { /* 2008-2033: p = size, 1/size */
        R fx = T::floor_(x * P[1]), fy = T::floor_(y * P[1]);
        R dx = x - fx * P[0], dy = y - fy * P[0];
        R xs = T::copysign_(R(2.0), fx), ys = T::copysign_(R(2.0), fy);
        R x2 = fx * xs, y2 = fy * ys;
        x2 -= (R)(fx < 0);
        y2 -= (R)(fy < 0);
        X = dx + x2 * P[0]; Y = -dy - y2 * P[0]; break;
    }
    case V_CPOW: { /* 2038-2061: p = va, vc, vd, power */
        a = T::atan2_(y, x);
        R lnr = R(0.5) * T::log_(R2SQ);
        R ang = P[1] * a + P[2] * lnr + P[0] * T::floor_(P[3] * T::unit(rng.next()));
        T::sincos_(ang, &s, &c);
        d = T::exp_(P[1] * lnr - P[2] * a);
        X = c * d; Y = s * d; break;
    }
    case V_CURVE: /* 2066-2091: p = xamp, yamp, 1/xlen^2, 1/ylen^2 */
        X = x + P[0] * T::exp_(-y * y * P[2]);
        Y = y + P[1] * T::exp_(-x * x * P[3]); break;
    case V_EDISC: { /* 2096-2120 */
        R tmp = R2SQ + R(1.0), tmp2 = R(2.0) * x;
        R xmax = R(0.5) * (T::sqrt_(tmp + tmp2) + T::sqrt_(tmp - tmp2));
        R a1 = T::log_(xmax + T::sqrt_(xmax - R(1.0)));
        R a2 = -T::acos_(x / xmax);
        R s1, c1;
        T::sincos_(a1, &s1, &c1);
        R s2 = T::sinh_(a2), c2 = T::cosh_(a2);
        s1 *= T::copysign_(R(1.0), -y);
        X = c2 * c1; Y = s2 * s1; break;
    }
    case V_ELLIPTIC: { /* 2125-2144 */
        R tmp = R2SQ + R(1.0), x2 = R(2.0) * x;
        R xmax = R(0.5) * (T::sqrt_(tmp + x2) + T::sqrt_(tmp - x2));
        R aa = x / xmax, bb = R(1.0) - aa * aa, ssx = xmax - R(1.0);
        bb = bb < R(0.0) ? R(0.0) : T::sqrt_(bb);
        ssx = ssx < R(0.0) ? R(0.0) : T::sqrt_(ssx);
        X = T::atan2_(aa, bb); Y = T::copysign_(R(1.0), y) * T::log_(xmax + ssx); break;
    }
    case V_ESCHER: { /* 2149-2171: p = vc, vd */
        a = T::atan2_(y, x);
        R lnr = R(0.5) * T::log_(R2SQ);
        R n = P[0] * a + P[1] * lnr;
        T::sincos_(n, &s, &c);
        d = T::exp_(P[0] * lnr - P[1] * a);
        X = c * d; Y = s * d; break;
    }
    case V_FOCI: { /* 2176-2192 */
        R expx = R(0.5) * T::exp_(x), expnx = R(0.25) / expx;
        T::sincos_(y, &s, &c);
        d = T::recip_(expx + expnx - c);
        X = (expx - expnx) * d; Y = s * d; break;
    }
    case V_LAZYSUSAN: { /* 2197-2230: p = x, y, spin, twist, space, weight */
        R xx = x - P[0], yy = y + P[1];
        r = T::hypot_(xx, yy);
        if (r < P[5]) {
            a = T::atan2_(yy, xx) + P[2] + P[3] * (P[5] - r);
            T::sincos_(a, &s, &c);
            X = r * c + P[0]; Y = r * s - P[1];
        } else {
            r = R(1.0) + P[4] / (r + T::eps);
            X = r * xx + P[0]; Y = r * yy - P[1];
        }
        break;
    }
    case V_LOONIE: { /* 2235-2254: p = weight, weight^2 */
        R r2 = R2SQ;
        r = P[0];
        if (r2 < P[1])
            r *= T::sqrt_(P[1] / (r2 + T::eps) - R(1.0));
        X = x * r; Y = y * r; break;
    }
    case V_OSCOPE: { /* 2259-2281: p = 2 pi freq, amp, damp, sep */
        R damp = T::exp_(-T::fabs_(x) * P[2]);
        R tt = P[1] * damp * T::cos_(P[0] * x) + P[3];
        X = x; Y = T::copysign_(R(1.0), T::fabs_(y) - tt) * y; break;
    }
    case V_POPCORN: /* 2286-2305: p = x, y, c */
        X = x + P[0] * T::sin_(T::tan_(y * P[2]));
        Y = y + P[1] * T::sin_(T::tan_(x * P[2])); break;
    default:
        X = Y = (R(0) / R(0)); break;
    }
#undef R2SQ
#undef R2
#undef ANG
    for (int i = 0; i < D; ++i)
        out[i] = i == ax ? X : (i == ay ? Y : R(0));
}

} // namespace ffr
