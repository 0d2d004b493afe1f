// Device-resident description of one normalised flame ("flame program").
//
// Built on the host from the parsed flame (flame.cpp) in the arithmetic type
// R of the kernel that runs it (double for the FP64 mirror, float for FP32),
// laid out as one contiguous blob so a CTA copies it into shared memory with
// a single coalesced loop.  Every thread indexes its own xform per sample, so
// shared memory (divergent addresses at full rate) is used instead of
// __constant__ (divergent addresses serialise).
//
// Blob layout (all offsets in bytes from the blob start, 16-byte aligned):
//   ProgHeader<R>
//   uint64_t thresh[nxf]        xform selection thresholds (see below)
//   float     fast[(nxf + 1) * kFast2Floats]   merged 2-D FP32 programs only
//   XformT<R> xf[nxf + 1]       sorted xforms, then the final xform
//   VarT<R>   var[nvar]         variations of all xforms, in xform order
//   R         color[(nxf+1) * color_dims]
//
// Selection: the reference draws r = (w >> 11) / 2^53 (FlameRNG::randNum,
// src/rng/flame_rng.hpp:67-87) and takes the first i with xfcw[i] >= r
// (Flame::getRandomXForm, src/types/flame.hpp:212-219).  With m = w >> 11,
// xfcw[i] < m / 2^53 holds exactly when m > floor(xfcw[i] * 2^53), so
// thresh[i] = floor(xfcw[i] * 2^53) and the choice is the first i with
// m <= thresh[i]: the same choice for every word, in integer arithmetic.
#pragma once

#include "std_types.h"

#include "variation_ids.h"

namespace ffr {

// dims 1..4: the reference's templates are generic over dims, its ffr-buf
// CLI compiles 1..3 (ffr_buf.cpp:134-141); 4 is rendered by ffr_render
// (plain kernel) here
constexpr int kMaxDims = 4;
constexpr int kMaxColorDims = 127;   // flame.hpp:156
constexpr int kVarParams = 16;
constexpr int kMaxXformIds = 4096;
constexpr int kMaxBadRecords = 4096;
constexpr uint32_t kMaxProgramBytes = 48 * 1024;

template <typename R>
struct alignas(16) XformT
{
    R pre[kMaxDims * kMaxDims + kMaxDims];   // A row-major, then b
    R post[kMaxDims * kMaxDims + kMaxDims];
    R color_speed;
    uint32_t id;            // index in the JSON xform list (stats are by id)
    int16_t var_begin;
    int16_t var_count;
    uint8_t has_pre;
    uint8_t has_post;
    uint8_t has_color;
    uint8_t rng_words;      // RNG words one application draws (fixed per xform)
    // merged form (ProgHeader::merged): the summed weight of each benchmark
    // variation type in this xform, in the order linear, sinusoidal,
    // spherical, swirl, horseshoe, polar, julia (0 where the xform lacks
    // the type), then 1 if the xform has julia (which draws a word even at
    // weight 0), else 0
    R coef[8];
    // merged form, 3-D flames: the plane (axis_x, axis_y) of this xform's
    // swirl, horseshoe, polar and julia, in that order ((0, 1) where absent)
    uint8_t plane[8];
};

// compact merged 2-D xform: pre-affine {a00, a01, b0, a10, a11, b1}, then
// post-affine {a00, a01, b0, a10, a11, b1} (both as XformT stores them),
// then XformT::coef
constexpr int kFast2Floats = 20;

template <typename R>
struct alignas(16) VarT
{
    int32_t type;           // VariationId
    int16_t axis_x;         // 2-D variations: the plane they act on
    int16_t axis_y;
    R weight;
    R p[kVarParams];        // per-variation parameters (variation_ids.h)
};

template <typename R>
struct alignas(16) ProgHeader
{
    int32_t dims;
    int32_t nxf;            // selectable xforms (zero weights removed)
    int32_t has_final;
    int32_t color_dims;
    int32_t nvar;
    int32_t xform_ids;      // xforms in the JSON (getXFormIDCount)
    uint32_t off_thresh;
    uint32_t off_xf;
    uint32_t off_var;
    uint32_t off_color;
    uint32_t total_bytes;
    uint32_t rng_words_max; // upper bound of RNG words one xform step draws
    // which of the seven benchmark variations the flame uses (kTierABit..,
    // variations.cuh); bit 7 = some other variation.  Uniform per program,
    // so kernels branch on it without divergence.
    uint32_t tier_a_present;
    // 1 when selectable xforms draw different numbers of RNG words per
    // application (lanes of a warp then consume their ISAAC blocks out of
    // phase and the render kernels keep a carry area for refill ahead)
    uint32_t draws_vary;
    // 1 when the FP32 kernels evaluate each variation type once per xform
    // application and weight it by XformT::coef (variations.cuh,
    // merged_variations): FP32 programs whose variations are all benchmark
    // types, with julia at most once per xform and, above 2 dims, each 2-D
    // type at most once per xform (XformT::plane).  FP64 programs keep the
    // reference's per-variation order.
    uint32_t merged;
    // byte offset of the compact table of a merged 2-D program (kFast2Floats
    // floats per xform, the final xform last), or 0: the two affines and the
    // merged coefficients in five 16-byte words instead of eight
    uint32_t off_fast;
    // the kernels copy the first smem_bytes of the blob into shared memory
    // and read the rest (sections at offsets at or above it) from the
    // program's global copy: merged 2-D programs keep only the header, the
    // thresholds and the compact table in shared memory (their xforms and
    // variations are read only on rare paths); all others keep everything
    uint32_t smem_bytes;
    uint32_t pad_;
    uint64_t size[kMaxDims];
    uint64_t mult_i[kMaxDims];
    uint64_t cells;
    R lo[kMaxDims];
    R hi[kMaxDims];
    R mult_d[kMaxDims];     // size/(hi-lo) * (1 - 2^-52)  (buffer_renderer.hpp:126-127)
};

} // namespace ffr
