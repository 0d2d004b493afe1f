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
#include <vector>

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

// RNG words one call draws: FlameRNG draw counts (src/rng/flame_rng.hpp:
// randNum 1, randBool 1, randGaussian 2, randPoint2 dims, randDirection 1 in
// 1-D and 2-D, 2 in 3-D) summed over the class's calc()
uint32_t variation_rng_words(int id, int dims)
{
    // randDirection<dims>: 1 word for dims 1 and 2, 2 for 3, a gaussian
    // pair (2 words) per two coordinates above 3 (flame_rng.hpp:171-217)
    const uint32_t dw = dims == 3 ? 2 : (dims > 3 ? 2 * (uint32_t)((dims + 1) / 2) : 1);
    switch (id)
    {
    case V_NOISE: case V_BLUR: return 1 + dw;
    case V_GAUSSIAN_BLUR: case V_PRE_BLUR: return 2 + dw;
    case V_SQUARE_NOISE: return (uint32_t)dims;
    case V_JULIA: case V_JULIAN: case V_ARCH: case V_RAYS: case V_BLADE:
    case V_TWINTRIAN: case V_WEDGE_JULIA: case V_SUPERSHAPE: case V_FLOWER:
    case V_CONIC: case V_BOARDERS: case V_CPOW: return 1;
    case V_JULIASCOPE: case V_RADIAL_BLUR: case V_PARABOLA: return 2;
    case V_PIE: return 3;
    default: return 0;
    }
}

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
    auto f = [&](const char* k) { return j.at(k, name).floatValue(name + ": " + k); };
    auto pt = [&](const char* k, int n) {
        const JsonValue& a = j.at(k, name);
        if (!a.isArray())
            throw FlameError(name + ": " + k + ": Point(Json&): not an array");
        const auto& e = a.arrayValue(k);
        if ((int)e.size() != n)
            throw FlameError(name + ": " + k + ": Point(Json&): incorrect array size: "
                + std::to_string(e.size()));
        std::vector<double> o;
        for (const auto& x : e)
        {
            if (!x.isNumber())
                throw FlameError(name + ": " + k + ": Point(Json&): entry is not a number");
            o.push_back(x.floatValue(k));
        }
        return o;
    };
    auto append = [&](const std::vector<double>& x) { v.p.insert(v.p.end(), x.begin(), x.end()); };
    constexpr double kPi = 3.14159265358979323846;        // M_PI
    constexpr double kPi2 = 1.57079632679489661923;       // M_PI_2
    constexpr double k1Pi = 0.31830988618379067154;       // M_1_PI
    constexpr double kEps = 1e-20;                        // eps<double>
    // Constructor arithmetic of each class in src/variations/variations.hpp
    // (host compiled with -ffp-contract=off, like the reference oracle)
    switch (id)
    {
    case V_BENT:                                          // 216-240
        append(pt("scales_neg", dims));
        append(pt("scales_pos", dims));
        break;
    case V_RECTANGLES:                                    // 245-270
    case V_SPLITS:                                        // 410-429
        append(pt("params", dims));
        break;
    case V_FISHEYE:                                       // 275-292
    case V_BUBBLE:                                        // 297-314
        v.p = {f("addval")};
        break;
    case V_SEPARATION:                                    // 383-405
    {
        std::vector<double> sep = pt("params", dims);
        for (double& x : sep)
            x *= x;
        append(sep);
        append(pt("inside", dims));
        break;
    }
    case V_MODULUS:                                       // 451-471
    {
        std::vector<double> p2 = pt("params", dims);
        for (double& x : p2)
            x *= 2.0;
        append(p2);
        for (double x : p2)
            v.p.push_back(1.0 / x);
        break;
    }
    case V_CELLN:                                         // 476-505
    {
        std::vector<double> sz = pt("sizes", dims);
        append(sz);
        for (double x : sz)
            v.p.push_back(1.0 / x);
        break;
    }
    case V_SPHERICAL_P:                                   // 2312-2328
    case V_UNIT_SPHERE_P:                                 // 2347-2363
    {
        const double n = f("norm");
        if (n <= 0.0)
            throw FlameError("norm <= 0");
        v.p = {n};
        break;
    }
    case V_DISC2:                                         // 624-655
    {
        const double rot = f("rotation"), twist = f("twist");
        const double rotpi = rot * kPi;
        double sinadd = std::sin(twist), cosadd = std::cos(twist);
        cosadd -= 1.0;
        double k = 1.0 + twist;
        if (twist > 2.0 * kPi) k -= 2.0 * kPi;
        if (twist < -2.0 * kPi) k += 2.0 * kPi;
        cosadd *= k;
        sinadd *= k;
        v.p = {rotpi, cosadd, sinadd};
        break;
    }
    case V_WAVES:                                         // 660-680
    {
        const double xf = f("xfreq"), xs = f("xscale"), yf = f("yfreq"), ys = f("yscale");
        v.p = {xf, xs, yf, ys};
        break;
    }
    case V_FAN:                                           // 685-709
    {
        const double x = f("x"), y = f("y");
        v.p = {kPi * (x * x + kEps), y};
        break;
    }
    case V_RINGS:                                         // 714-733
    {
        const double val = f("value");
        v.p = {val * val + kEps};
        break;
    }
    case V_BLOB:                                          // 875-896
    {
        const double low = f("low"), high = f("high");
        const double mid = (high + low) / 2.0, amp = (high - low) / 2.0;
        v.p = {mid, amp, f("waves")};
        break;
    }
    case V_PDJ:                                           // 901-925
    {
        const double a = f("a"), b = f("b"), c = f("c"), d = f("d");
        v.p = {a, b, c, d};
        break;
    }
    case V_PERSPECTIVE:                                   // 943-962
    {
        const double dist = f("distance"), ang = f("angle");
        v.p = {dist, std::sin(ang), dist * std::cos(ang)};
        break;
    }
    case V_JULIAN:                                        // 967-989
    case V_JULIASCOPE:                                    // 994-1018
    {
        const double power = f("power"), dist = f("dist");
        v.p = {std::fabs(power), 1.0 / power, dist / (2.0 * power)};
        break;
    }
    case V_RADIAL_BLUR:                                   // 1023-1045
    {
        const double ang = f("angle");
        const double a = ang * kPi2;
        const double spin = std::sin(a), zoom = std::cos(a);
        v.p = {spin, zoom, f("flam3_weight")};
        break;
    }
    case V_PIE:                                           // 1050-1072
    {
        const double slices = f("slices"), rot = f("rotation"), thick = f("thickness");
        v.p = {slices, rot, thick, (2.0 * kPi) / slices};
        break;
    }
    case V_NGON:                                          // 1077-1102
    {
        const double sides = f("sides");
        const double powerval = f("power") / 2.0;
        const double ang = (2.0 * kPi) / sides;
        const double corners = f("corners"), circle = f("circle");
        v.p = {powerval, ang, corners, circle, sides / (2.0 * kPi)};
        break;
    }
    case V_CURL:                                          // 1107-1129
    {
        const double c1 = f("c1"), c2 = f("c2");
        v.p = {c1, c2};
        break;
    }
    case V_ARCH: case V_RAYS: case V_BLADE: case V_SECANT: case V_TWINTRIAN: case V_SCRY:
        v.p = {f("flam3_weight")};
        break;
    case V_AUGER:                                         // 1549-1571
    {
        const double freq = f("freq"), w = f("flam3_weight");
        const double scale = f("scale") / 2.0;
        v.p = {freq, w, scale, f("sym")};
        break;
    }
    case V_FLUX:                                          // 1576-1600
    {
        const double spread = 2.0 + f("spread");
        v.p = {spread, f("flam3_weight")};
        break;
    }
    case V_MOBIUS:                                        // 1605-1630
        append(pt("a", 2));
        append(pt("b", 2));
        append(pt("c", 2));
        append(pt("d", 2));
        break;
    case V_SPLIT:                                         // 1655-1673
    {
        const double sx = f("xsize") * kPi, sy = f("ysize") * kPi;
        v.p = {sx, sy};
        break;
    }
    case V_STRIPES:                                       // 1678-1696
    {
        const double space = 1.0 - f("space");
        v.p = {space, f("warp")};
        break;
    }
    case V_WEDGE:                                         // 1701-1724
    {
        const double sw = f("swirl"), count = f("count"), ang = f("angle"), hole = f("hole");
        v.p = {sw, count, ang, hole, 1.0 - ang * count * (k1Pi * 0.5)};
        break;
    }
    case V_WEDGE_JULIA:                                   // 1729-1756
    {
        const double ang = f("angle"), count = f("count"), power = f("power");
        const double invpower = 1.0 / power;
        const double dist = f("dist");
        const double cn = dist / (2.0 * power);
        v.p = {ang, count, invpower, cn, std::fabs(power), 1.0 - ang * count * (k1Pi * 0.5)};
        break;
    }
    case V_WEDGE_SPH:                                     // 1761-1785
    {
        const double ang = f("angle"), count = f("count"), sw = f("swirl"), hole = f("hole");
        v.p = {ang, count, sw, hole, 1.0 - ang * count * (k1Pi * 0.5)};
        break;
    }
    case V_WHORL:                                         // 1790-1810
    {
        const double in = f("inside"), out = f("outside"), w = f("flam3_weight");
        v.p = {in, out, w};
        break;
    }
    case V_SUPERSHAPE:                                    // 1815-1842
    {
        const double n1 = f("n1");
        const double pm_4 = f("m") / 4.0;
        const double pneg1_n1 = -1.0 / n1;
        const double n2 = f("n2"), n3 = f("n3"), rnd = f("rnd"), holes = f("holes");
        v.p = {pm_4, pneg1_n1, n2, n3, rnd, holes};
        break;
    }
    case V_FLOWER:                                        // 1847-1864
    {
        const double petals = f("petals"), holes = f("holes");
        v.p = {petals, holes};
        break;
    }
    case V_CONIC:                                         // 1869-1886
    {
        const double eccen = f("eccen"), holes = f("holes");
        v.p = {eccen, holes};
        break;
    }
    case V_PARABOLA:                                      // 1891-1909
    {
        const double hh = f("height"), ww = f("width");
        v.p = {hh, ww};
        break;
    }
    case V_BIPOLAR:                                       // 1914-1935
        v.p = {-kPi2 * f("shift")};
        break;
    case V_BOARDERS:                                      // 1940-1983
    {
        const double prob = f("prob");
        if (prob < 0.0 || prob > 1.0)
            throw FlameError("boarders probability out of range");
        v.p = {prob};
        break;
    }
    case V_CELL:                                          // 2008-2033
    {
        const double size = f("size");
        v.p = {size, 1.0 / size};
        break;
    }
    case V_CPOW:                                          // 2038-2061
    {
        const double r = f("r"), i = f("i"), power = f("power");
        v.p = {2.0 * kPi / power, r / power, i / power, power};
        break;
    }
    case V_CURVE:                                         // 2066-2091
    {
        const double xamp = f("xamp"), yamp = f("yamp");
        double xlen = f("xlen"), ylen = f("ylen");
        xlen *= xlen;
        ylen *= ylen;
        v.p = {xamp, yamp, 1.0 / (kEps < xlen ? xlen : kEps), 1.0 / (kEps < ylen ? ylen : kEps)};
        break;
    }
    case V_ESCHER:                                        // 2149-2171
    {
        const double beta = f("beta");
        const double seb = std::sin(beta), ceb = std::cos(beta);
        v.p = {0.5 * (1.0 + ceb), 0.5 * seb};
        break;
    }
    case V_LAZYSUSAN:                                     // 2197-2230
    {
        const double px = f("x"), py = f("y"), spin = f("spin"), twist = f("twist"),
            space = f("space"), w = f("flam3_weight");
        v.p = {px, py, spin, twist, space, w};
        break;
    }
    case V_LOONIE:                                        // 2235-2254
    {
        const double w = f("flam3_weight");
        v.p = {w, w * w};
        break;
    }
    case V_OSCOPE:                                        // 2259-2281
    {
        const double freq = f("frequency");
        const double tpf = 2.0 * kPi * freq;
        const double amp = f("amplitude"), damp = f("damping"), sep = f("separation");
        v.p = {tpf, amp, damp, sep};
        break;
    }
    case V_POPCORN:                                       // 2286-2305
    {
        const double px = f("x"), py = f("y"), pc = f("c");
        v.p = {px, py, pc};
        break;
    }
    default:
        break;                                            // no parameters
    }
    v.rng_words = variation_rng_words(id, dims);
    return v;
}

} // namespace ffr
