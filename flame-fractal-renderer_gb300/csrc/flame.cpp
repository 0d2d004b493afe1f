// Flame parsing, validation and normalisation (host side).
//
// Follows, check for check, the reference constructors:
//   Flame(Json)         src/types/flame.hpp:91-210
//   Flame::_optimize    src/types/flame.hpp:63-83
//   Flame::_setupCumulativeWeights  src/types/flame.hpp:44-60
//   XForm(Json)         src/types/xform.hpp:71-172 (+ _optimize 55-66)
//   Affine(Json)        src/types/affine.hpp:45-92
//   Point(Json)         src/types/point.hpp:60-77
//   BufferRenderer::_init index multipliers, buffer_renderer.hpp:114-140
#include "flame.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace ffr {

namespace {

constexpr double kMaxRect = 1e10;      // max_rect<double> (constants.hpp:35-37)
constexpr uint64_t kMaxDim = 65535;    // max_dim (constants.hpp:33)

void point_value(const JsonValue& j, int n, double* out, const std::string& what)
{
    if (!j.isArray())
        throw FlameError(what + ": Point(Json&): not an array");
    const auto& a = j.arrayValue(what);
    if ((int)a.size() != n)
        throw FlameError(what + ": Point(Json&): incorrect array size: "
            + std::to_string(a.size()));
    for (int i = 0; i < n; ++i)
    {
        if (!a[i].isNumber())
            throw FlameError(what + ": Point(Json&): entry is not a number");
        out[i] = a[i].floatValue(what);
    }
}

void identity(double* aff, int n)
{
    std::memset(aff, 0, sizeof(double) * (kMaxDims * kMaxDims + kMaxDims));
    for (int i = 0; i < n; ++i)
        aff[i * n + i] = 1.0;
}

// A (n*n row-major) then b (n), packed contiguously at aff[0 .. n*n+n)
void parse_affine(const JsonValue& j, int n, double* aff, const std::string& what)
{
    if (!j.isObject())
        throw FlameError(what + ": Affine(Json&): not an object");
    identity(aff, n);
    if (j.has("A"))
    {
        const JsonValue& A = j.at("A", what);
        if (!A.isArray())
            throw FlameError(what + ": Affine(Json&): A is not an array");
        const auto& rows = A.arrayValue(what);
        if ((int)rows.size() != n)
            throw FlameError(what + ": Affine(Json&): A is wrong size");
        for (int i = 0; i < n; ++i)
            point_value(rows[i], n, aff + i * n,
                what + ": Affine(Json&): error parsing A[" + std::to_string(i) + "]");
    }
    if (j.has("b"))
        point_value(j.at("b", what), n, aff + n * n,
            what + ": Affine(Json&): error parsing b");
}

HostXform parse_xform(const JsonValue& j, uint64_t id, bool is_final, int dims,
    int color_dims, double default_speed)
{
    HostXform x;
    x.id = id;
    if (!is_final)
        x.weight = j.at("weight", "XForm(): cannot parse weight")
            .floatValue("XForm(): cannot parse weight");
    else
        x.weight = 1.0;
    if (x.weight < 0.0)
        throw FlameError("XForm(): weight is negative");
    x.has_pre = j.has("pre_affine");
    if (x.has_pre)
        parse_affine(j.at("pre_affine", "XForm()"), dims, x.pre,
            "XForm(): cannot parse pre_affine");
    else
        identity(x.pre, dims);
    x.has_post = j.has("post_affine");
    if (x.has_post)
        parse_affine(j.at("post_affine", "XForm()"), dims, x.post,
            "XForm(): cannot parse post_affine");
    else
        identity(x.post, dims);
    const JsonValue& vj = j.at("variations", "XForm(): cannot parse variations");
    for (const JsonValue& v : vj.arrayValue("XForm(): cannot parse variations"))
    {
        try
        {
            x.vars.push_back(parse_variation(v, dims));
        }
        catch (const FlameError& e)
        {
            throw FlameError(std::string("XForm(): cannot parse variations: ") + e.what());
        }
    }
    if (color_dims && j.has("color"))
    {
        const auto& c = j.at("color", "XForm()").arrayValue("XForm(): cannot parse color");
        if ((int)c.size() != color_dims)
            throw FlameError("XForm(): cannot parse color: color length incorrect");
        for (const JsonValue& e : c)
        {
            double v = e.floatValue("XForm(): cannot parse color");
            if (v < 0.0 || v > 1.0)
                throw FlameError("XForm(): cannot parse color: color coordinate out of range");
            x.color.push_back(v);
        }
    }
    if (color_dims && j.has("color_speed"))
    {
        x.color_speed = j.at("color_speed", "XForm()").floatValue("XForm(): color speed issue");
        if (x.color_speed < 0.0 || x.color_speed > 1.0)
            throw FlameError("XForm(): color speed issue: color speed out of range");
    }
    else
        x.color_speed = default_speed;
    // XForm::_optimize: drop variations whose weight is exactly zero
    x.vars.erase(std::remove_if(x.vars.begin(), x.vars.end(),
        [](const HostVar& v) { return std::fabs(v.weight) == 0.0; }), x.vars.end());
    return x;
}

} // namespace

uint64_t selection_threshold(double c)
{
    if (std::isnan(c))
        return UINT64_MAX;          // NaN < r is false: never step past it
    if (c <= 0.0)
        return 0;
    const double s = std::ldexp(c, 53);
    if (s >= 18446744073709551615.0)
        return UINT64_MAX;
    return (uint64_t)std::floor(s);
}

HostFlame parse_flame(const std::string& text)
{
    JsonValue root = JsonValue::parse(text);
    HostFlame f;
    f.echo = root.dump();
    if (!root.isObject())
        throw FlameError("flame: not an object");
    const int64_t dims = root.at("dimensions", "flame").intValue("dimensions");
    if (dims < 1 || dims > kMaxDims)
        throw FlameError(std::to_string(dims) + "D not supported");
    f.dims = (int)dims;
    try
    {
        const auto& sizej = root.at("size", "Flame()").arrayValue("size");
        const auto& boundsj = root.at("bounds", "Flame()").arrayValue("bounds");
        if ((int)sizej.size() != f.dims)
            throw FlameError("incorrect size length");
        if ((int)boundsj.size() != f.dims)
            throw FlameError("incorrect bounds length");
        for (int i = 0; i < f.dims; ++i)
        {
            const std::string si = std::to_string(i);
            double s = sizej[i].floatValue("error parsing size[" + si + "]");
            // size[i] = floatValue() truncated to size_t; 0 or > 65535 rejected
            if (!(s >= 1.0) || !(s < (double)(kMaxDim + 1)))
                throw FlameError("size[" + si + "] out of range");
            f.size[i] = (uint64_t)s;
            const auto& b = boundsj[i].arrayValue("bounds[" + si + "]");
            if (b.size() != 2)
                throw FlameError("bounds[" + si + "] wrong format");
            const double lo = b[0].floatValue("error parsing bounds[" + si + "]");
            const double hi = b[1].floatValue("error parsing bounds[" + si + "]");
            if (lo < -kMaxRect || lo > kMaxRect || hi < -kMaxRect || hi > kMaxRect)
                throw FlameError("bounds[" + si + "] out of range");
            if (lo >= hi)
                throw FlameError("bounds[" + si + "] low >= high");
            f.lo[i] = lo;
            f.hi[i] = hi;
        }
    }
    catch (const FlameError& e)
    {
        throw FlameError(std::string("Flame(): ") + e.what());
    }
    const auto& xfs = root.at("xforms", "Flame(): cannot parse xforms")
        .arrayValue("Flame(): cannot parse xforms");
    try
    {
        f.color_dims = 0;
        if (root.has("color_dimensions"))
        {
            int64_t cd = root.at("color_dimensions", "flame").intValue("color_dimensions");
            if (cd < 0 || cd > kMaxColorDims)
                throw FlameError("too many color dimensions");
            f.color_dims = (int)cd;
        }
        f.color_speed = root.has("color_speed")
            ? root.at("color_speed", "flame").floatValue("color_speed") : 0.5;
        if (f.color_speed < 0.0 || f.color_speed > 1.0)
            throw FlameError("color speed out of range");
    }
    catch (const FlameError& e)
    {
        throw FlameError(std::string("Flame(): ") + e.what());
    }
    std::vector<HostXform> all;
    uint64_t id = 0;
    for (const JsonValue& xj : xfs)
    {
        try
        {
            all.push_back(parse_xform(xj, id, false, f.dims, f.color_dims, f.color_speed));
        }
        catch (const FlameError& e)
        {
            throw FlameError("Flame(): error parsing xforms[" + std::to_string(id)
                + "]: " + e.what());
        }
        ++id;
    }
    f.xform_ids = id;
    if (all.empty())
        throw FlameError("Flame(): no xforms");
    if (root.has("final_xform"))
    {
        f.has_final = true;
        try
        {
            f.final_xf = parse_xform(root.at("final_xform", "flame"), UINT64_MAX,
                true, f.dims, f.color_dims, f.color_speed);
        }
        catch (const FlameError& e)
        {
            throw FlameError(std::string("Flame(): error parsing final xform: ") + e.what());
        }
    }
    // Flame::_optimize: remove weight-0 xforms, then std::sort by decreasing
    // weight with the same comparator (libstdc++ on both build hosts), so
    // ties are ordered exactly as the reference orders them
    for (auto& x : all)
        (x.weight == 0.0 ? f.removed : f.xforms).push_back(x);
    if (f.xforms.empty())
        throw FlameError("Flame(): no xforms remaining after optimization");
    std::sort(f.xforms.begin(), f.xforms.end(),
        [](const HostXform& a, const HostXform& b) { return a.weight > b.weight; });
    // Flame::_setupCumulativeWeights
    double normdiv = 0.0;
    for (const auto& x : f.xforms)
        normdiv += x.weight;
    double wsum = 0.0;
    for (const auto& x : f.xforms)
    {
        wsum += x.weight / normdiv;
        f.xfcw.push_back(wsum);
    }
    f.xfcw.back() = 1.0;
    // BufferRenderer::_init
    uint64_t cells = 1;
    for (int i = 0; i < f.dims; ++i)
    {
        f.mult_d[i] = (double)f.size[i] / (f.hi[i] - f.lo[i]);
        f.mult_d[i] *= 1.0 - std::ldexp(1.0, -52);
        f.mult_i[i] = cells;
        cells *= f.size[i];
        if (cells >= (1ULL << 48))
            throw FlameError("BufferRenderer(): histogram too big");
    }
    f.cells = cells;
    return f;
}

namespace {

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename R>
void pack_xform(const HostXform& h, int dims, XformT<R>& x, int16_t var_begin)
{
    std::memset(&x, 0, sizeof x);
    // re-pack with a fixed stride of kMaxDims so device code indexes
    // A[i*kMaxDims + j] and b at kMaxDims*kMaxDims + i for every dims
    for (int i = 0; i < dims; ++i)
    {
        for (int j = 0; j < dims; ++j)
        {
            x.pre[i * kMaxDims + j] = (R)h.pre[i * dims + j];
            x.post[i * kMaxDims + j] = (R)h.post[i * dims + j];
        }
        x.pre[kMaxDims * kMaxDims + i] = (R)h.pre[dims * dims + i];
        x.post[kMaxDims * kMaxDims + i] = (R)h.post[dims * dims + i];
    }
    x.color_speed = (R)h.color_speed;
    x.id = (uint32_t)std::min<uint64_t>(h.id, UINT32_MAX);
    x.var_begin = var_begin;
    x.var_count = (int16_t)h.vars.size();
    x.has_pre = h.has_pre;
    x.has_post = h.has_post;
    x.has_color = !h.color.empty();
    uint32_t w = 0;
    for (const auto& v : h.vars)
        w += v.rng_words;
    x.rng_words = (uint8_t)std::min<uint32_t>(w, 255);
}

} // namespace

// The FP32 merged form applies (ProgHeader::merged): every variation one of
// the seven benchmark types, julia at most once per xform (julia's random
// word differs per instance, so two julias are not one julia of the summed
// weight; every other type is a fixed map), and above 2 dims each 2-D type
// at most once per xform (it acts on that instance's plane).
static bool merged_form(const HostFlame& f)
{
    static const int32_t kTierA[7] = {V_LINEAR, V_SINUSOIDAL, V_SPHERICAL, V_SWIRL,
                                      V_HORSESHOE, V_POLAR, V_JULIA};
    auto ok_xform = [&](const HostXform& x) {
        int jul = 0;
        for (const auto& v : x.vars)
        {
            bool a = false;
            for (int k = 0; k < 7; ++k)
                a = a || v.type == kTierA[k];
            if (!a)
                return false;
            jul += v.type == V_JULIA;
        }
        // above 2 dims each 2-D type acts on its own plane: at most one of
        // each per xform, so one plane per type
        if (f.dims > 2)
            for (int32_t t2 : {V_SWIRL, V_HORSESHOE, V_POLAR})
            {
                int n = 0;
                for (const auto& v : x.vars)
                    n += v.type == t2;
                if (n > 1)
                    return false;
            }
        return jul <= 1;
    };
    for (const auto& x : f.xforms)
        if (!ok_xform(x))
            return false;
    return !f.has_final || ok_xform(f.final_xf);
}

template <typename R>
std::vector<uint8_t> build_program(const HostFlame& f)
{
    const int nxf = (int)f.xforms.size();
    std::vector<const HostXform*> all;
    for (const auto& x : f.xforms)
        all.push_back(&x);
    all.push_back(f.has_final ? &f.final_xf : nullptr);
    size_t nvar = 0;
    for (const HostXform* x : all)
        if (x)
            nvar += x->vars.size();
    ProgHeader<R> h;
    std::memset(&h, 0, sizeof h);
    h.dims = f.dims;
    h.nxf = nxf;
    h.has_final = f.has_final;
    h.color_dims = f.color_dims;
    h.nvar = (int32_t)nvar;
    h.xform_ids = (int32_t)std::min<uint64_t>(f.xform_ids, INT32_MAX);
    size_t off = align16(sizeof(ProgHeader<R>));
    h.off_thresh = (uint32_t)off;
    off = align16(off + sizeof(uint64_t) * nxf);
    const bool fast2 = sizeof(R) == sizeof(float) && f.dims == 2 && merged_form(f);
    h.off_fast = fast2 ? (uint32_t)off : 0u;
    if (fast2)
        off = align16(off + sizeof(float) * (size_t)(nxf + 1) * kFast2Floats);
    // shared-memory part: up to here for merged 2-D programs, else all
    const size_t smem_end = off;
    h.off_xf = (uint32_t)off;
    off = align16(off + sizeof(XformT<R>) * (nxf + 1));
    h.off_var = (uint32_t)off;
    off = align16(off + sizeof(VarT<R>) * nvar);
    h.off_color = (uint32_t)off;
    off = align16(off + sizeof(R) * (size_t)(nxf + 1) * f.color_dims);
    h.smem_bytes = (uint32_t)(fast2 ? smem_end : off);
    if (off > kMaxProgramBytes || nvar > 32767)
        throw FlameError("flame too large for one device program ("
            + std::to_string(off) + " bytes; limit "
            + std::to_string(kMaxProgramBytes) + ")");
    h.total_bytes = (uint32_t)off;
    // the largest draw count of one selectable xform application (the final
    // xform is applied by the stream's owner thread and draws directly)
    uint32_t words = 0;
    for (int k = 0; k < nxf; ++k)
    {
        uint32_t w = 0;
        for (const auto& v : all[k]->vars)
            w += v.rng_words;
        words = std::max(words, w);
    }
    if (words > 255)
        throw FlameError("an xform draws more than 255 random words per application");
    h.rng_words_max = words;
    h.draws_vary = 0;
    for (int k = 1; k < nxf; ++k)
    {
        uint32_t a = 0, b = 0;
        for (const auto& v : all[0]->vars)
            a += v.rng_words;
        for (const auto& v : all[k]->vars)
            b += v.rng_words;
        if (a != b)
            h.draws_vary = 1;
    }
    // variation types present (selectable and final xforms): bits in the
    // order linear, sinusoidal, spherical, swirl, horseshoe, polar, julia,
    // then bit 7 for any other type
    static const int32_t kTierA[7] = {V_LINEAR, V_SINUSOIDAL, V_SPHERICAL, V_SWIRL,
                                      V_HORSESHOE, V_POLAR, V_JULIA};
    uint32_t present = 0;
    for (const HostXform* x : all)
        if (x)
            for (const auto& v : x->vars)
            {
                uint32_t bit = 1u << 7;
                for (int k = 0; k < 7; ++k)
                    if (v.type == kTierA[k])
                        bit = 1u << k;
                present |= bit;
            }
    h.tier_a_present = present;
    // the FP32 merged form: every type once per application, weighted by
    // the xform's summed weight of that type.  Sums of equal terms are the
    // same map (V(t) does not depend on the instance), except julia, whose
    // random word differs per instance.
    h.merged = sizeof(R) == sizeof(float) && merged_form(f) ? 1 : 0;
    for (int i = 0; i < f.dims; ++i)
    {
        h.size[i] = f.size[i];
        h.mult_i[i] = f.mult_i[i];
        h.lo[i] = (R)f.lo[i];
        h.hi[i] = (R)f.hi[i];
        if (sizeof(R) == sizeof(double))
            h.mult_d[i] = (R)f.mult_d[i];
        else
        {
            // the reference's float build: scale_adjust_down<float> = 1 - 2^-23
            float m = (float)f.size[i] / ((float)f.hi[i] - (float)f.lo[i]);
            m *= 1.0f - std::ldexp(1.0f, -23);
            h.mult_d[i] = (R)m;
        }
    }
    h.cells = f.cells;
    std::vector<uint8_t> blob(off, 0);
    std::memcpy(blob.data(), &h, sizeof h);
    uint64_t* th = reinterpret_cast<uint64_t*>(blob.data() + h.off_thresh);
    for (int i = 0; i < nxf; ++i)
        th[i] = selection_threshold(f.xfcw[i]);
    XformT<R>* xp = reinterpret_cast<XformT<R>*>(blob.data() + h.off_xf);
    VarT<R>* vp = reinterpret_cast<VarT<R>*>(blob.data() + h.off_var);
    R* cp = reinterpret_cast<R*>(blob.data() + h.off_color);
    int16_t vb = 0;
    for (int k = 0; k <= nxf; ++k)
    {
        const HostXform* x = all[k];
        if (!x)
            continue;
        pack_xform<R>(*x, f.dims, xp[k], vb);
        if (h.merged)
        {
            for (int t = 0; t < 4; ++t)
            {
                xp[k].plane[2 * t] = 0;
                xp[k].plane[2 * t + 1] = 1;
            }
            for (const auto& v : x->vars)
            {
                for (int t = 0; t < 7; ++t)
                    if (v.type == kTierA[t])
                        xp[k].coef[t] = (R)((double)xp[k].coef[t] + v.weight);
                // julia draws its word whatever its weight
                if (v.type == V_JULIA)
                    xp[k].coef[7] = R(1);
                // swirl, horseshoe, polar, julia are kTierA[3..6]
                for (int t = 3; t < 7; ++t)
                    if (v.type == kTierA[t] && f.dims > 2)
                    {
                        xp[k].plane[2 * (t - 3)] = (uint8_t)v.axis_x;
                        xp[k].plane[2 * (t - 3) + 1] = (uint8_t)v.axis_y;
                    }
            }
        }
        for (const auto& v : x->vars)
        {
            VarT<R>& d = vp[vb++];
            std::memset(&d, 0, sizeof d);
            d.type = v.type;
            d.axis_x = v.axis_x;
            d.axis_y = v.axis_y;
            d.weight = (R)v.weight;
            for (size_t p = 0; p < v.p.size() && p < (size_t)kVarParams; ++p)
                d.p[p] = (R)v.p[p];
        }
        for (int c = 0; c < (int)x->color.size(); ++c)
            cp[(size_t)k * f.color_dims + c] = (R)x->color[c];
        if (fast2)
        {
            float* q = reinterpret_cast<float*>(blob.data() + h.off_fast) + (size_t)k * kFast2Floats;
            const XformT<R>& d = xp[k];
            // A[i][j] at i * kMaxDims + j, b[i] at kMaxDims * kMaxDims + i
            const int b0 = kMaxDims * kMaxDims;
            const R* aff[2] = {d.pre, d.post};
            for (int a = 0; a < 2; ++a)
            {
                q[6 * a + 0] = (float)aff[a][0];
                q[6 * a + 1] = (float)aff[a][1];
                q[6 * a + 2] = (float)aff[a][b0];
                q[6 * a + 3] = (float)aff[a][kMaxDims];
                q[6 * a + 4] = (float)aff[a][kMaxDims + 1];
                q[6 * a + 5] = (float)aff[a][b0 + 1];
            }
            for (int c = 0; c < 8; ++c)
                q[12 + c] = (float)d.coef[c];
        }
    }
    return blob;
}

template std::vector<uint8_t> build_program<double>(const HostFlame&);
template std::vector<uint8_t> build_program<float>(const HostFlame&);

} // namespace ffr
