// Host-side flame model: parse, validate and normalise a flame JSON the way
// the reference's Flame<dims>(Json) does (src/types/flame.hpp:91-210), then
// pack it into a device flame program (flame_program.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "flame_program.h"
#include "json.hpp"

namespace ffr {

struct HostVar
{
    int32_t type = 0;
    std::string name;
    double weight = 0.0;
    int16_t axis_x = 0, axis_y = 1;
    std::vector<double> p;       // parameters as the device reads them
    uint32_t rng_words = 0;      // upper bound of RNG words per call
};

struct HostXform
{
    uint64_t id = 0;
    double weight = 1.0;
    bool has_pre = false, has_post = false;
    double pre[kMaxDims * kMaxDims + kMaxDims] = {};
    double post[kMaxDims * kMaxDims + kMaxDims] = {};
    std::vector<HostVar> vars;
    std::vector<double> color;
    double color_speed = 0.5;
};

struct HostFlame
{
    int dims = 0;
    uint64_t size[kMaxDims] = {};
    double lo[kMaxDims] = {}, hi[kMaxDims] = {};
    int color_dims = 0;
    double color_speed = 0.5;
    std::vector<HostXform> xforms;     // zero weights removed, decreasing weight
    std::vector<HostXform> removed;
    uint64_t xform_ids = 0;
    bool has_final = false;
    HostXform final_xf;
    std::vector<double> xfcw;          // cumulative weights, back() == 1.0
    double mult_d[kMaxDims] = {};
    uint64_t mult_i[kMaxDims] = {};
    uint64_t cells = 0;
    std::string echo;                  // compact JSON for the CLI echo
};

// Parse a flame document; throws FlameError with the reference's wording.
HostFlame parse_flame(const std::string& json_text);

// Parse one variation object for a flame of `dims` dimensions
// (Variation::parseVariation, variations.hpp:2614-2626).
HostVar parse_variation(const JsonValue& j, int dims);

// The JSON name of a variation id ("?" outside 0..V_COUNT-1)
const char* variation_name(int id);

// Pack the flame into a program blob of arithmetic type R.
template <typename R>
std::vector<uint8_t> build_program(const HostFlame& f);

// thresh[i] = floor(xfcw[i] * 2^53) (see flame_program.h)
uint64_t selection_threshold(double xfcw);

} // namespace ffr
