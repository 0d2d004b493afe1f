// Test-infrastructure driver for the REFERENCE build (oracle/_ref/ffr_ref).
//
// Compiled by oracle/build_ref.sh against the reference's own, unmodified
// hot-path headers (src/renderers, src/types, src/variations, src/rng) plus
// its src/rng/flame_rng.cpp and src/utils/json.cpp.  It replaces only the
// Boost.program_options front end of src/ffr_buf.cpp:61-274 and is used to
// generate the golden fixtures under tests/golden/ and, in this container,
// as the timed CPU baseline.  It never ships with the product.
//
// Stream model shared with the product and the C restatement:
//   stream s of seed S is Isaac<u64,4> seeded by setSeed(u64 key(S,s)) with
//   key(S,s) = S + fmix64(s)   (fmix64 = MurmurHash3 64-bit finaliser,
//   fmix64(0) = 0, so stream 0 is exactly the reference's setSeed(S)).
//   A job of N samples with trajectory length L has ceil(N/L) trajectories;
//   trajectory j belongs to stream j mod S, and each stream runs its
//   trajectories in increasing j (the last, possibly shorter, trajectory is
//   the last one of its stream), i.e. stream s is renderSeeded(n_s, L).
//
// Sub-commands (all output on stdout unless a path is given):
//   kat KEY N                         N Isaac<u64,4> words after setSeed(KEY)
//   flame FLAME.json                  normalised flame dump (sorted xforms)
//   render FLAME S STREAMS N L SETTLE BVLIMIT OUT.buf [seeded]
//                                     deterministic multi-stream render;
//                                     'seeded' uses BufferRenderer::
//                                     renderSeeded (SETTLE must be 53)
//   step FLAME XF KEY IN.bin OUT.bin  applyIteration of sorted xform XF
//                                     (-1 = final xform) on each point of
//                                     IN.bin (f64, dims per point); point j
//                                     uses stream key(KEY, j)
//   trace FLAME KEY SETTLE N          first N samples of one trajectory:
//                                     xform id and point per sample
//   bench FLAME N THREADS             BufferRenderer::render() timing with
//                                     clock seeds (samples/s), as ffr-buf

#include "renderers/buffer_renderer.hpp"

#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using namespace tkoz::flame;

static uint64_t fmix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

static uint64_t stream_key(uint64_t seed, uint64_t stream)
{
    return seed + fmix64(stream);
}

static Json load_json(const std::string& path)
{
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f)
        throw std::runtime_error("cannot open " + path);
    return Json(f);
}

static void print_double(double d)
{
    uint64_t u;
    std::memcpy(&u, &d, 8);
    std::printf("\"0x%016" PRIx64 "\"", u);
}

// ---------------------------------------------------------------- kat
static int cmd_kat(uint64_t key, uint64_t n)
{
    Isaac<u64,4> g(key);
    for (uint64_t i = 0; i < n; ++i)
        std::printf("%016" PRIx64 "\n", g.next());
    return 0;
}

// ---------------------------------------------------------------- flame
template <size_t dims>
static void dump_xform(const XForm<dims>& xf)
{
    std::printf("{\"id\":%zu,\"weight\":", xf.getID());
    print_double(xf.getWeight());
    std::printf(",\"has_pre\":%d,\"has_post\":%d,\"pre\":[",
        (int)xf.hasPreAffine(), (int)xf.hasPostAffine());
    const auto& pre = xf.getPreAffine();
    const auto& post = xf.getPostAffine();
    for (size_t i = 0; i < dims; ++i)
        for (size_t j = 0; j < dims; ++j)
        {
            print_double(pre.getA()[i][j]);
            std::printf(",");
        }
    for (size_t i = 0; i < dims; ++i)
    {
        print_double(pre.getB()[i]);
        std::printf(i + 1 < dims ? "," : "");
    }
    std::printf("],\"post\":[");
    for (size_t i = 0; i < dims; ++i)
        for (size_t j = 0; j < dims; ++j)
        {
            print_double(post.getA()[i][j]);
            std::printf(",");
        }
    for (size_t i = 0; i < dims; ++i)
    {
        print_double(post.getB()[i]);
        std::printf(i + 1 < dims ? "," : "");
    }
    std::printf("],\"var_weights\":[");
    const auto& vars = xf.getVariations();
    for (size_t v = 0; v < vars.size(); ++v)
    {
        print_double(vars[v]->getWeight());
        std::printf(v + 1 < vars.size() ? "," : "");
    }
    std::printf("],\"color\":[");
    for (size_t c = 0; c < xf.getColor().size(); ++c)
    {
        print_double(xf.getColor()[c]);
        std::printf(c + 1 < xf.getColor().size() ? "," : "");
    }
    std::printf("],\"color_speed\":");
    print_double(xf.getColorSpeed());
    std::printf("}");
}

template <size_t dims>
static int cmd_flame_t(const Json& j)
{
    Flame<dims> fl(j);
    BufferRenderer<dims> r(fl);
    std::printf("{\"dims\":%zu,\"xform_ids\":%zu,\"color_dims\":%zu,\"xforms\":[",
        dims, fl.getXFormIDCount(), fl.getColorDims());
    for (size_t i = 0; i < fl.getXForms().size(); ++i)
    {
        dump_xform<dims>(fl.getXForms()[i]);
        std::printf(i + 1 < fl.getXForms().size() ? "," : "");
    }
    std::printf("],\"xfcw\":[");
    for (size_t i = 0; i < fl.getCumulativeWeights().size(); ++i)
    {
        print_double(fl.getCumulativeWeights()[i]);
        std::printf(i + 1 < fl.getCumulativeWeights().size() ? "," : "");
    }
    std::printf("],\"has_final\":%d", (int)fl.hasFinalXForm());
    if (fl.hasFinalXForm())
    {
        std::printf(",\"final\":");
        dump_xform<dims>(fl.getFinalXForm());
    }
    std::printf(",\"mult_d\":[");
    for (size_t i = 0; i < dims; ++i)
    {
        print_double(r.getDimMults()[i]);
        std::printf(i + 1 < dims ? "," : "");
    }
    std::printf("],\"mult_i\":[");
    for (size_t i = 0; i < dims; ++i)
        std::printf("%zu%s", r.getIndexMults()[i], i + 1 < dims ? "," : "");
    std::printf("],\"cells\":%zu}\n", r.getBufferNumCells());
    return 0;
}

// ---------------------------------------------------------------- render
// Mirror of BufferRenderer::_render_batch (src/renderers/buffer_renderer.hpp:
// 151-250) and RenderIterator (src/renderers/render_iterator.hpp:52-139) with
// a run-time settle count; built from the reference's own Flame/XForm/rng.
// A NaN final point is not binned (the reference's behaviour is undefined
// there: (size_t)NaN at buffer_renderer.hpp:202).
template <size_t dims>
struct MirrorStats
{
    uint64_t s_iter = 0, s_plot = 0, bad = 0, dropped = 0;
    std::vector<uint64_t> xf_dist;
    std::vector<size_t> bv_xfs;
    std::array<std::pair<double,double>,dims> ext;
};

template <size_t dims>
static bool mirror_batch(const Flame<dims>& fl, const BufferRenderer<dims>& br,
    std::vector<uint64_t>& buf, size_t cell_size, size_t cells,
    uint64_t samples, uint64_t settle, uint64_t bv_limit, MirrorStats<dims>& st)
{
    typedef Point<num_t,dims> point_t;
    if (st.bv_xfs.size() > bv_limit)
        return false;
    const size_t r = fl.getColorDims();
    std::vector<double> c(r, 0.0), cf(r, 0.0);
    point_t p, pf;
    auto init = [&]()
    {
        p = rng::randPoint<dims>();
        for (uint64_t i = 0; i < settle; ++i)
            p = fl.getRandomXForm().applyIteration(p);
        for (size_t i = 0; i < r; ++i)
            c[i] = rng::randNum();
    };
    init();
    for (; samples > 0; --samples)
    {
        const XForm<dims>& xf = fl.getRandomXForm();
        double s = xf.getColorSpeed();
        size_t xf_id = xf.getID();
        p = xf.applyIteration(p);
        if (r && xf.hasColor())
            for (size_t i = 0; i < r; ++i)
                c[i] = (1.0-s)*c[i] + s*xf.getColor()[i];
        if (fl.hasFinalXForm())
        {
            const XForm<dims>& xff = fl.getFinalXForm();
            s = xff.getColorSpeed();
            pf = xff.applyIteration(p);
            if (r)
            {
                if (xff.hasColor())
                    for (size_t i = 0; i < r; ++i)
                        cf[i] = (1.0-s)*c[i] + s*xff.getColor()[i];
                else
                    for (size_t i = 0; i < r; ++i)
                        cf[i] = c[i];
            }
        }
        else
        {
            pf = p;
            for (size_t i = 0; i < r; ++i)
                cf[i] = c[i];
        }
        ++st.s_iter;
        ++st.xf_dist[xf_id];
        bool badv = false;
        for (size_t i = 0; i < dims; ++i)
            if (bad_value(p[i]))
                badv = true;
        if (badv)
        {
            st.bv_xfs.push_back(xf_id);
            ++st.bad;
            if (st.bv_xfs.size() > bv_limit)
                break;
            init();
        }
        for (size_t i = 0; i < dims; ++i)
        {
            if (p[i] < st.ext[i].first) st.ext[i].first = p[i];
            if (p[i] > st.ext[i].second) st.ext[i].second = p[i];
        }
        bool inb = true;
        for (size_t i = 0; i < dims; ++i)
            if (std::isnan(pf[i]) || pf[i] < fl.getBounds()[i].first
                    || pf[i] > fl.getBounds()[i].second)
                inb = false;
        if (!inb)
            continue;
        ++st.s_plot;
        size_t bi = (pf[0] - fl.getBounds()[0].first) * br.getDimMults()[0];
        for (size_t i = 1; i < dims; ++i)
        {
            size_t di = (pf[i] - fl.getBounds()[i].first) * br.getDimMults()[i];
            bi += di * br.getIndexMults()[i];
        }
        if (bi >= cells)
        {
            ++st.dropped;
            continue;
        }
        ++buf[bi * cell_size];
        for (size_t i = 0; i < r; ++i)
        {
            double d;
            std::memcpy(&d, &buf[bi * cell_size + 1 + i], 8);
            d += cf[i];
            std::memcpy(&buf[bi * cell_size + 1 + i], &d, 8);
        }
    }
    return samples == 0;
}

template <size_t dims>
static int cmd_render_t(const Json& j, uint64_t seed, uint64_t streams,
    uint64_t n, uint64_t L, uint64_t settle, uint64_t bvl,
    const std::string& out, bool seeded)
{
    Flame<dims> fl(j);
    BufferRenderer<dims> br(fl);
    const size_t cells = br.getBufferNumCells();
    const size_t cell_size = br.getBufferCellSize();
    std::vector<uint64_t> buf(cells * cell_size, 0);
    MirrorStats<dims> st;
    st.xf_dist.assign(fl.getXFormIDCount(), 0);
    for (size_t i = 0; i < dims; ++i)
        st.ext[i] = std::make_pair(INFINITY, -INFINITY);
    const uint64_t ntraj = (n + L - 1) / L;
    bool ok = true;
    uint64_t seeded_s_plot = 0;
    for (uint64_t s = 0; s < streams && s < ntraj; ++s)
    {
        uint64_t ns = 0;
        for (uint64_t t = s; t < ntraj; t += streams)
            ns += std::min<uint64_t>(L, n - t * L);
        rng::setSeed(stream_key(seed, s));
        if (seeded)
        {
            if (!br.renderSeeded(ns, L, bvl))
                ok = false;
            continue;
        }
        uint64_t left = ns;
        while (left)
        {
            uint64_t len = std::min<uint64_t>(L, left);
            if (!mirror_batch<dims>(fl, br, buf, cell_size, cells, len,
                    settle, bvl, st))
            {
                ok = false;
                break;
            }
            left -= len;
        }
        if (!ok)
            break;
    }
    std::ofstream f(out, std::ios::out | std::ios::binary);
    if (seeded)
    {
        br.writeBuffer(f);
        seeded_s_plot = br.getSamplesPlotted();
        std::printf("{\"ok\":%d,\"s_iter\":%zu,\"s_plot\":%" PRIu64
            ",\"xf_dist\":[", (int)ok, br.getSamplesIterated(), seeded_s_plot);
        const auto& xd = br.getXFormDistribution();
        for (size_t i = 0; i < xd.size(); ++i)
            std::printf("%zu%s", xd[i], i + 1 < xd.size() ? "," : "");
        std::printf("],\"ext\":[");
        for (size_t i = 0; i < dims; ++i)
        {
            std::printf("[");
            print_double(br.getPointExtremes()[i].first);
            std::printf(",");
            print_double(br.getPointExtremes()[i].second);
            std::printf("]%s", i + 1 < dims ? "," : "");
        }
        std::printf("]}\n");
        return 0;
    }
    f.write((const char*)buf.data(), buf.size() * 8);
    std::printf("{\"ok\":%d,\"s_iter\":%" PRIu64 ",\"s_plot\":%" PRIu64
        ",\"bad\":%" PRIu64 ",\"dropped\":%" PRIu64 ",\"xf_dist\":[",
        (int)ok, st.s_iter, st.s_plot, st.bad, st.dropped);
    for (size_t i = 0; i < st.xf_dist.size(); ++i)
        std::printf("%" PRIu64 "%s", st.xf_dist[i],
            i + 1 < st.xf_dist.size() ? "," : "");
    std::printf("],\"ext\":[");
    for (size_t i = 0; i < dims; ++i)
    {
        std::printf("[");
        print_double(st.ext[i].first);
        std::printf(",");
        print_double(st.ext[i].second);
        std::printf("]%s", i + 1 < dims ? "," : "");
    }
    std::printf("]}\n");
    return 0;
}

// ---------------------------------------------------------------- step
template <size_t dims>
static int cmd_step_t(const Json& j, long xf_index, uint64_t key,
    const std::string& in, const std::string& out)
{
    Flame<dims> fl(j);
    const XForm<dims>& xf = xf_index < 0 ? fl.getFinalXForm()
        : fl.getXForms().at((size_t)xf_index);
    std::ifstream fi(in, std::ios::in | std::ios::binary);
    std::vector<double> pts((std::istreambuf_iterator<char>(fi)),
        std::istreambuf_iterator<char>());
    (void)pts;
    fi.clear();
    fi.seekg(0, std::ios::end);
    size_t bytes = (size_t)fi.tellg();
    fi.seekg(0);
    std::vector<double> x(bytes / 8);
    fi.read((char*)x.data(), bytes);
    size_t np = x.size() / dims;
    std::vector<double> y(np * dims);
    for (size_t k = 0; k < np; ++k)
    {
        Point<num_t,dims> p;
        for (size_t i = 0; i < dims; ++i)
            p[i] = x[k * dims + i];
        rng::setSeed(stream_key(key, k));
        Point<num_t,dims> q = xf.applyIteration(p);
        for (size_t i = 0; i < dims; ++i)
            y[k * dims + i] = q[i];
    }
    std::ofstream fo(out, std::ios::out | std::ios::binary);
    fo.write((const char*)y.data(), y.size() * 8);
    return 0;
}

// ---------------------------------------------------------------- trace
template <size_t dims>
static int cmd_trace_t(const Json& j, uint64_t key, uint64_t settle, uint64_t n)
{
    Flame<dims> fl(j);
    rng::setSeed(key);
    Point<num_t,dims> p = rng::randPoint<dims>();
    for (uint64_t i = 0; i < settle; ++i)
        p = fl.getRandomXForm().applyIteration(p);
    for (uint64_t k = 0; k < n; ++k)
    {
        const XForm<dims>& xf = fl.getRandomXForm();
        p = xf.applyIteration(p);
        std::printf("%zu", xf.getID());
        for (size_t i = 0; i < dims; ++i)
        {
            uint64_t u;
            double d = p[i];
            std::memcpy(&u, &d, 8);
            std::printf(" %016" PRIx64, u);
        }
        std::printf("\n");
    }
    return 0;
}

// ---------------------------------------------------------------- bench
template <size_t dims>
static int cmd_bench_t(const Json& j, uint64_t n, uint64_t threads)
{
    Flame<dims> fl(j);
    BufferRenderer<dims> br(fl);
    // ffr_buf.cpp:94-101 automatic batch size
    uint64_t batch = std::clamp<uint64_t>((n + 255) >> 8, 1 << 12, 1 << 20);
    auto t0 = std::chrono::steady_clock::now();
    bool ok = br.render(n, threads, batch, 256);
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    std::printf("{\"ok\":%d,\"samples\":%" PRIu64 ",\"threads\":%" PRIu64
        ",\"batch\":%" PRIu64 ",\"seconds\":%.6f,\"samples_per_s\":%.1f,"
        "\"s_plot\":%zu}\n", (int)ok, n, threads, batch, secs, n / secs,
        br.getSamplesPlotted());
    return 0;
}

template <template <size_t> class F, typename... A>
static int by_dims(const Json& j, A... a)
{
    JsonInt d = j["dimensions"].intValue();
    switch (d)
    {
    case 1: return F<1>::run(j, a...);
    case 2: return F<2>::run(j, a...);
    case 3: return F<3>::run(j, a...);
    // the reference's templates are generic over dims; its ffr-buf CLI
    // instantiates 1..3 only (ffr_buf.cpp:134-141)
    case 4: return F<4>::run(j, a...);
    default:
        std::fprintf(stderr, "ERROR: %lldD not supported\n", (long long)d);
        return 1;
    }
}

template <size_t d> struct FlameCmd
{ template <typename... A> static int run(const Json& j, A... a) { return cmd_flame_t<d>(j, a...); } };
template <size_t d> struct RenderCmd
{ template <typename... A> static int run(const Json& j, A... a) { return cmd_render_t<d>(j, a...); } };
template <size_t d> struct StepCmd
{ template <typename... A> static int run(const Json& j, A... a) { return cmd_step_t<d>(j, a...); } };
template <size_t d> struct TraceCmd
{ template <typename... A> static int run(const Json& j, A... a) { return cmd_trace_t<d>(j, a...); } };
template <size_t d> struct BenchCmd
{ template <typename... A> static int run(const Json& j, A... a) { return cmd_bench_t<d>(j, a...); } };

static uint64_t u64arg(const char *s)
{
    return std::strtoull(s, nullptr, 0);
}

int main(int argc, char **argv)
{
    try
    {
        if (argc < 2)
            throw std::runtime_error("usage: ffr_ref kat|flame|render|step|trace|bench ...");
        std::string cmd = argv[1];
        if (cmd == "kat" && argc == 4)
            return cmd_kat(u64arg(argv[2]), u64arg(argv[3]));
        if (cmd == "flame" && argc == 3)
            return by_dims<FlameCmd>(load_json(argv[2]));
        if (cmd == "render" && (argc == 10 || argc == 11))
            return by_dims<RenderCmd>(load_json(argv[2]), u64arg(argv[3]),
                u64arg(argv[4]), u64arg(argv[5]), u64arg(argv[6]),
                u64arg(argv[7]), u64arg(argv[8]), std::string(argv[9]),
                argc == 11 && std::string(argv[10]) == "seeded");
        if (cmd == "step" && argc == 7)
            return by_dims<StepCmd>(load_json(argv[2]), std::strtol(argv[3], nullptr, 0),
                u64arg(argv[4]), std::string(argv[5]), std::string(argv[6]));
        if (cmd == "trace" && argc == 6)
            return by_dims<TraceCmd>(load_json(argv[2]), u64arg(argv[3]),
                u64arg(argv[4]), u64arg(argv[5]));
        if (cmd == "bench" && argc == 5)
            return by_dims<BenchCmd>(load_json(argv[2]), u64arg(argv[3]),
                u64arg(argv[4]));
        throw std::runtime_error("bad arguments for " + cmd);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "ffr_ref error: %s\n", e.what());
        return 2;
    }
}
