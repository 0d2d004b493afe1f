// Variation factory and parameter parsing (host side).
//
// Variation::parseVariation (src/variations/variations.hpp:2614-2626) tries
// the 2-D factory (only compiled for dims >= 2), then the empty 3-D one,
// then the N-D one, else throws "unknown variation: <name>".  Each entry
// below parses the same JSON keys as the reference constructor and stores the
// values the device code reads (including the reference's precomputed
// constants), in VarT::p order.
#include <cmath>
#include <cstring>
#include <string>

#include "flame.hpp"

namespace ffr {

namespace {

const char* const kNames[V_COUNT] = {
    "linear", "sinusoidal", "spherical", "bent", "rectangles", "fisheye",
    "bubble", "noise", "blur", "gaussian_blur", "square_noise", "separation",
    "splits", "pre_blur", "modulus", "celln", "spherical_p", "unit_sphere",
    "unit_sphere_p", "unit_cube",
    "swirl", "horseshoe", "polar", "polar2", "handkerchief", "heart", "disc",
    "disc2", "waves", "fan", "rings", "spiral", "hyperbolic", "diamond", "ex",
    "julia", "exponential", "power", "cosine", "blob", "pdj", "cylinder",
    "perspective", "julian", "juliascope", "radial_blur", "pie", "ngon",
    "curl", "arch", "tangent", "rays", "blade", "secant", "twintrian",
    "cross", "exp", "log", "sin", "cos", "tan", "sec", "csc", "cot", "sinh",
    "cosh", "tanh", "sech", "csch", "coth", "auger", "flux", "mobius", "scry",
    "split", "stripes", "wedge", "wedge_julia", "wedge_sph", "whorl",
    "supershape", "flower", "conic", "parabola", "bipolar", "boarders",
    "butterfly", "cell", "cpow", "curve", "edisc", "elliptic", "escher",
    "foci", "lazysusan", "loonie", "oscope", "popcorn",
};

int find_name(const std::string& n, int first, int last)
{
    for (int i = first; i < last; ++i)
        if (n == kNames[i])
            return i;
    return -1;
}

} // namespace

const char* variation_name(int id)
{
    return id >= 0 && id < V_COUNT ? kNames[id] : "?";
}

HostVar parse_variation(const JsonValue& j, int dims)
{
    const std::string name = j.at("name", "variation").stringValue("variation name");
    int id = -1;
    if (dims >= 2)
        id = find_name(name, kFirst2D, V_COUNT);
    if (id < 0)
        id = find_name(name, 0, kFirst2D);
    if (id < 0)
        throw FlameError("unknown variation: " + name);
    HostVar v;
    v.type = id;
    v.name = name;
    v.weight = j.at("weight", name).floatValue(name + ": weight");
    if (id >= kFirst2D && dims > 2)
    {
        // VariationFrom2D (variations.hpp:72-89)
        const int64_t ax = j.at("axis_x", name).intValue("axis_x");
        const int64_t ay = j.at("axis_y", name).intValue("axis_y");
        if (ax < 0 || ax >= dims)
            throw FlameError("axis_x index out of range");
        if (ay < 0 || ay >= dims)
            throw FlameError("axis_y index out of range");
        if (ax == ay)
            throw FlameError("axes are not distinct");
        v.axis_x = (int16_t)ax;
        v.axis_y = (int16_t)ay;
    }
    switch (id)
    {
    case V_LINEAR:
    case V_SINUSOIDAL:
    case V_SPHERICAL:
    case V_SWIRL:
    case V_HORSESHOE:
    case V_POLAR:
        break;
    case V_JULIA:
        v.rng_words = 1;          // randBool (variations.hpp:813)
        break;
    default:
        throw FlameError("variation not supported by this build: " + name);
    }
    return v;
}

} // namespace ffr
