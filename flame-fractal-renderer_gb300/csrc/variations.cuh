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

#include <cstdint>

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
};

// t[i] for a run-time i without dynamic register indexing
template <int D, typename R>
__device__ __forceinline__ R coord(const R* t, int i)
{
    if (D <= 2)
        return t[i & 1];
    R r = t[0];
#pragma unroll
    for (int k = 1; k < D; ++k)
        r = i == k ? t[k] : r;
    return r;
}

// one variation: o = V(t)
template <int D, typename R, typename Rng>
__device__ __forceinline__ void variation(const VarT<R>& v, const R* t, R* o, Rng& rng)
{
    using T = RealTraits<R>;
    const int ax = v.axis_x, ay = v.axis_y;
    R x2 = R(0), y2 = R(0);
    switch (v.type)
    {
    case V_LINEAR:                       // variations.hpp:169-177
#pragma unroll
        for (int i = 0; i < D; ++i)
            o[i] = t[i];
        return;
    case V_SINUSOIDAL:                   // variations.hpp:183-191
#pragma unroll
        for (int i = 0; i < D; ++i)
            o[i] = T::sin_(t[i]);
        return;
    case V_SPHERICAL:                    // variations.hpp:197-208
    {
        R r2 = t[0] * t[0];
#pragma unroll
        for (int i = 1; i < D; ++i)
            r2 += t[i] * t[i];
        const R r = T::recip_(r2 + T::eps);
#pragma unroll
        for (int i = 0; i < D; ++i)
            o[i] = t[i] * r;
        return;
    }
    case V_SWIRL:                        // variations.hpp:509-522
    {
        const R x = coord<D>(t, ax), y = coord<D>(t, ay);
        const R r = x * x + y * y;
        R s, c;
        T::sincos_(r, &s, &c);
        x2 = x * s - y * c;
        y2 = x * c + y * s;
        break;
    }
    case V_HORSESHOE:                    // variations.hpp:527-540
    {
        const R x = coord<D>(t, ax), y = coord<D>(t, ay);
        const R r = T::recip_(T::sqrt_(x * x + y * y) + T::eps);
        x2 = ((x - y) * (x + y)) * r;
        y2 = (R(2) * x * y) * r;
        break;
    }
    case V_POLAR:                        // variations.hpp:545-555
    {
        const R x = coord<D>(t, ax), y = coord<D>(t, ay);
        const R a = T::atan2_(y, x);
        const R r = T::sqrt_(x * x + y * y);
        x2 = a * T::inv_pi;
        y2 = r - R(1);
        break;
    }
    case V_JULIA:                        // variations.hpp:807-819
    {
        const R x = coord<D>(t, ax), y = coord<D>(t, ay);
        const R a = R(0.5) * T::atan2_(y, x) + (R)(rng.next() & 1u) * T::pi;
        R s, c;
        T::sincos_(a, &s, &c);
        const R r = T::sqrt_(x * x + y * y);
        x2 = c * r;
        y2 = s * r;
        break;
    }
    default:
        // unreachable: the host rejects variations this build lacks
#pragma unroll
        for (int i = 0; i < D; ++i)
            o[i] = R(0) / R(0);
        return;
    }
    // 2-D result into the (axis_x, axis_y) plane, zero elsewhere
#pragma unroll
    for (int i = 0; i < D; ++i)
        o[i] = i == ax ? x2 : (i == ay ? y2 : R(0));
}

} // namespace ffr
