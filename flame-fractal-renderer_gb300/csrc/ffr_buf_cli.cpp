// ffr-buf: drop-in command line front end for the GB300 buffer generator.
//
// Same options, defaults, stderr report and output bytes as the reference's
// src/ffr_buf.cpp:61-274 (-f/--flame, -i/--input (repeatable), -o/--output,
// -s/--samples, -t/--threads, -b/--batch-size, -z/--bad-values; '-' means
// stdin/stdout), calling libffr_gpu.so through its C ABI only.
//
// GPU meaning of the reference's work-split options:
//   -b/--batch-size  samples per trajectory (the reference starts a new
//                    trajectory per batch, buffer_renderer.hpp:155).  0 is
//                    the reference's automatic size, clamp((samples + 255)
//                    >> 8, 4096, 2^20) (ffr_buf.cpp:94-101), so the same
//                    command restarts and settles trajectories as often as
//                    the reference does; with --streams, 0 instead picks
//                    samples / streams (one trajectory per GPU thread).
//                    Below 256 is rejected when rendering, as render() does
//                    (buffer_renderer.hpp:283-285).
//   -t/--threads     checked as render() checks it (1..65535,
//                    buffer_renderer.hpp:277-282) and echoed; the device
//                    decides its parallelism
// The render-time checks of -t and -b run before the flame is read (the
// reference runs them when render() starts, after reading the flame and the
// input buffers), so a command with a bad flame and a bad -t reports -t.
// Added options: --seed N (stream seeds; default from the clock, like the
// reference's per-thread clock seeding), --precision fp64|fp32, --settle N
// (default 53 = settle_iters<double>), --streams N, --trajectories T (T
// streams of one trajectory each, of ceil(samples / T) samples: "N samples
// from T trajectories"; excludes -b and --streams), --device N,
// --timeout-ms N, --kernel auto|plain|sorted|hot|jit|jit-sorted
// (ffr_opts.kernel; jit, jit-sorted = the plain and xform-sorted kernels
// compiled for this flame's structure at run time).
//
// Errors: the reference lets parse/IO exceptions escape main (abort); this
// front end prints "ERROR: <message>" and exits 1.  A bad-value stop prints
// "render failure" and still writes the buffer with exit status 0, as the
// reference does (ffr_buf.cpp:228-230).
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "ffr_gpu.h"

namespace {

struct Args
{
    std::string flame, output;
    std::vector<std::string> inputs;
    uint64_t samples = 0;
    uint64_t threads = std::max(1u, std::thread::hardware_concurrency());
    uint64_t batch = 0;
    uint64_t bad_values = 1 << 8;
    bool have_seed = false;
    uint64_t seed = 0;
    int precision = FFR_FP64;
    uint64_t settle = 53;
    uint64_t streams = 0;
    uint64_t trajectories = 0;
    int device = 0;
    uint64_t timeout_ms = 0;
    int kernel = FFR_KERNEL_AUTO;
    bool help = false;
    bool have_flame = false, have_output = false;
};

const char* kUsage =
    "ffr-buf usage:\n"
    "  -h [ --help ]                 show this help message\n"
    "  -f [ --flame ] arg            flame parameters JSON file\n"
    "  -i [ --input ] arg            buffers to add initially\n"
    "  -o [ --output ] arg           output file\n"
    "  -s [ --samples ] arg (=0)     samples to render\n"
    "  -t [ --threads ] arg          threads to use (accepted, device chooses)\n"
    "  -b [ --batch-size ] arg (=0)  batch size (samples per trajectory)\n"
    "  -z [ --bad-values ] arg (=256) bad values limit\n"
    "  --seed arg                    stream seed (default: clock)\n"
    "  --precision arg (=fp64)       fp64 (reference arithmetic) or fp32\n"
    "  --settle arg (=53)            settle iterations per trajectory\n"
    "  --streams arg (=0)            concurrent RNG streams (0 = device)\n"
    "  --trajectories arg            trajectories (one stream each)\n"
    "  --device arg (=0)             CUDA device\n"
    "  --timeout-ms arg (=0)         render time limit (0 = none)\n"
    "  --kernel arg (=auto)          auto, plain, sorted, hot, jit or jit-sorted\n";

[[noreturn]] void die(const std::string& m)
{
    std::cerr << "ERROR: " << m << std::endl;
    std::exit(1);
}

uint64_t to_u64(const std::string& v, const std::string& opt)
{
    if (v.empty() || v[0] == '-')
        die("the argument ('" + v + "') for option '--" + opt + "' is invalid");
    char* end = nullptr;
    errno = 0;
    unsigned long long x = std::strtoull(v.c_str(), &end, 10);
    if (errno || *end)
        die("the argument ('" + v + "') for option '--" + opt + "' is invalid");
    return x;
}

Args parse_args(int argc, char** argv)
{
    Args a;
    struct Opt { const char* lng; char shrt; bool value; };
    static const Opt opts[] = {
        {"help", 'h', false}, {"flame", 'f', true}, {"input", 'i', true},
        {"output", 'o', true}, {"samples", 's', true}, {"threads", 't', true},
        {"batch-size", 'b', true}, {"bad-values", 'z', true},
        {"seed", 0, true}, {"precision", 0, true}, {"settle", 0, true},
        {"streams", 0, true}, {"trajectories", 0, true}, {"device", 0, true},
        {"timeout-ms", 0, true}, {"kernel", 0, true},
    };
    for (int k = 1; k < argc; ++k)
    {
        std::string tok = argv[k];
        const Opt* o = nullptr;
        std::string val;
        bool have_val = false;
        if (tok.rfind("--", 0) == 0 && tok.size() > 2)
        {
            std::string name = tok.substr(2);
            size_t eq = name.find('=');
            if (eq != std::string::npos)
            {
                val = name.substr(eq + 1);
                name = name.substr(0, eq);
                have_val = true;
            }
            for (const Opt& c : opts)
                if (name == c.lng)
                    o = &c;
            if (!o)
                die("unrecognised option '" + tok + "'");
        }
        else if (tok.size() >= 2 && tok[0] == '-' && tok[1] != '-')
        {
            for (const Opt& c : opts)
                if (c.shrt && tok[1] == c.shrt)
                    o = &c;
            if (!o)
                die("unrecognised option '" + tok + "'");
            if (tok.size() > 2)
            {
                val = tok.substr(2);
                have_val = true;
            }
        }
        else
            die("unexpected argument '" + tok + "'");
        if (o->value && !have_val)
        {
            if (k + 1 >= argc)
                die(std::string("the required argument for option '--") + o->lng
                    + "' is missing");
            val = argv[++k];
        }
        const std::string n = o->lng;
        if (n == "help") a.help = true;
        else if (n == "flame") { a.flame = val; a.have_flame = true; }
        else if (n == "input") a.inputs.push_back(val);
        else if (n == "output") { a.output = val; a.have_output = true; }
        else if (n == "samples") a.samples = to_u64(val, n);
        else if (n == "threads") a.threads = to_u64(val, n);
        else if (n == "batch-size") a.batch = to_u64(val, n);
        else if (n == "bad-values") a.bad_values = to_u64(val, n);
        else if (n == "seed") { a.seed = to_u64(val, n); a.have_seed = true; }
        else if (n == "precision")
        {
            if (val == "fp64") a.precision = FFR_FP64;
            else if (val == "fp32") a.precision = FFR_FP32;
            else die("--precision must be fp64 or fp32");
        }
        else if (n == "settle") a.settle = to_u64(val, n);
        else if (n == "streams") a.streams = to_u64(val, n);
        else if (n == "trajectories") a.trajectories = to_u64(val, n);
        else if (n == "device") a.device = (int)to_u64(val, n);
        else if (n == "timeout-ms") a.timeout_ms = to_u64(val, n);
        else if (n == "kernel")
        {
            static_assert(FFR_KERNEL_AUTO == 0 && FFR_KERNEL_JIT_SORTED == 5, "kernel names");
            static const char* const kNames[] = {"auto", "plain", "sorted", "hot", "jit",
                                                 "jit-sorted"};
            int k = -1;
            for (int i = 0; i < 6; ++i)
                if (val == kNames[i])
                    k = i;
            if (k < 0)
                die("--kernel must be auto, plain, sorted, hot, jit or jit-sorted");
            a.kernel = k;       // FFR_KERNEL_AUTO .. FFR_KERNEL_JIT_SORTED in this order
        }
    }
    return a;
}

std::string read_all(std::istream& in)
{
    return std::string((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

bool read_exact(std::istream& in, std::vector<char>& buf)
{
    in.read(buf.data(), (std::streamsize)buf.size());
    return in.good() || (size_t)in.gcount() == buf.size();
}

void check(ffr_ctx* ctx, ffr_status s)
{
    if (s != FFR_OK && s != FFR_BAD_VALUES)
        die(ffr_last_error(ctx));
}

} // namespace

int main(int argc, char** argv)
{
    Args a = parse_args(argc, argv);
    if (a.help || argc < 2)
    {
        std::cerr << kUsage;
        return 1;
    }
    if (!a.have_flame)
        die("the option '--flame' is required but missing");
    if (!a.have_output)
        die("the option '--output' is required but missing");
    const bool user_batch = a.batch != 0;
    if (a.trajectories)
    {
        if (a.batch || a.streams)
            die("--trajectories excludes --batch-size and --streams");
        a.streams = a.trajectories;
        a.batch = a.samples ? (a.samples + a.trajectories - 1) / a.trajectories : 1;
    }
    // the reference's automatic batch size (ffr_buf.cpp:94-101)
    const bool calculated_batch = a.batch == 0 && a.streams == 0;
    if (calculated_batch)
        a.batch = std::clamp<uint64_t>((a.samples + 255) >> 8, 1u << 12, 1u << 20);
    // BufferRenderer::render's argument checks (buffer_renderer.hpp:277-285)
    if (a.samples > 0)
    {
        if (a.threads == 0)
            die("BufferRenderer::render(): threads must be positive");
        if (a.threads > 65535)
            die("BufferRenderer::render(): too many threads");
        if (user_batch && a.batch < 256)
            die("BufferRenderer::render(): batch size too small");
    }
    if (!a.have_seed)
        a.seed = (uint64_t)std::chrono::steady_clock::now().time_since_epoch().count()
            ^ (uint64_t)std::chrono::system_clock::now().time_since_epoch().count();

    // option echo (ffr_buf.cpp:104-119)
    std::cerr << "ffr-buf version gb300" << std::endl;
    std::cerr << "--flame " << a.flame << std::endl;
    for (auto& s : a.inputs)
        std::cerr << "--input " << s << std::endl;
    std::cerr << "--output " << a.output << std::endl;
    std::cerr << "--samples " << a.samples;
    if (a.samples == 0)
        std::cerr << " (not rendering)";
    std::cerr << std::endl;
    std::cerr << "--threads " << a.threads << std::endl;
    // a batch size known without the device is echoed where the reference
    // echoes it, before the flame is read (ffr_buf.cpp:115-118)
    const bool batch_known = a.batch != 0;
    if (batch_known)
    {
        if (calculated_batch)
            std::cerr << "--batch_size 0 (" << a.batch << ")" << std::endl;
        else
            std::cerr << "--batch_size " << a.batch << std::endl;
        std::cerr << "--bad_values " << a.bad_values << std::endl;
    }

    std::string text;
    if (a.flame == "-")
        text = read_all(std::cin);
    else
    {
        std::ifstream f(a.flame, std::ios::in | std::ios::binary);
        if (!f)
            die("cannot open flame file " + a.flame);
        text = read_all(f);
    }
    ffr_opts o;
    ffr_default_opts(&o);
    o.device = a.device;
    o.precision = a.precision;
    o.settle = a.settle;
    o.streams = a.streams;
    o.traj_len = a.batch;
    o.timeout_ms = a.timeout_ms;
    o.kernel = a.kernel;
    ffr_ctx* ctx = nullptr;
    ffr_status st = ffr_create(text.data(), text.size(), &o, &ctx);
    if (st != FFR_OK)
        die(ffr_last_error(nullptr));
    uint64_t streams = 0, traj_len = a.batch;
    if (a.samples)
        check(ctx, ffr_plan(ctx, a.samples, &streams, &traj_len));
    if (!batch_known)
    {
        // --streams with -b 0: the trajectory length comes from the plan
        std::cerr << "--batch_size 0 (" << traj_len << ")" << std::endl;
        std::cerr << "--bad_values " << a.bad_values << std::endl;
    }
    std::cerr << "--seed " << a.seed << std::endl;
    std::cerr << "--precision " << (a.precision == FFR_FP64 ? "fp64" : "fp32") << std::endl;
    std::cerr << "--settle " << a.settle << std::endl;
    std::cerr << "--streams " << streams << std::endl;
    std::cerr << "--" << std::endl;
    std::cerr << "flame: " << ffr_flame_json(ctx) << std::endl;

    uint32_t dims = 0, color_dims = 0;
    uint64_t cells = 0;
    size_t bytes = 0;
    check(ctx, ffr_info(ctx, &dims, &cells, &color_dims, &bytes));
    std::cerr << "buffer: " << bytes << " bytes, little endian, 8 byte numbers" << std::endl;
    std::cerr << "size:";
    std::vector<uint64_t> size(dims);
    check(ctx, ffr_size(ctx, size.data()));
    for (uint64_t d : size)
        std::cerr << " " << d;
    std::cerr << std::endl;
    std::cerr << "color: " << color_dims << " dimensions" << std::endl;

    // initial input buffers (ffr_buf.cpp:167-183)
    std::vector<char> buf(bytes);
    for (auto& s : a.inputs)
    {
        std::cerr << "adding input file " << s << std::endl;
        bool ok;
        if (s == "-")
            ok = read_exact(std::cin, buf);
        else
        {
            std::ifstream f(s, std::ios::in | std::ios::binary);
            ok = f && read_exact(f, buf);
        }
        if (!ok)
            die("error reading file");
        check(ctx, ffr_add_buffer(ctx, buf.data(), buf.size()));
    }

    if (a.samples > 0)
    {
        std::cerr << "render start" << std::endl;
        static ffr_stats stats;
        const auto t1 = std::chrono::steady_clock::now();
        st = ffr_render(ctx, a.samples, a.seed, a.bad_values, &stats);
        const auto t2 = std::chrono::steady_clock::now();
        check(ctx, st);
        double secs = std::chrono::duration<double>(t2 - t1).count();
        const uint64_t nbatch = (a.samples + stats.traj_len - 1) / stats.traj_len;
        std::cerr << "\rprogress: " << nbatch << "/" << nbatch << " batches, "
                  << a.samples << "/" << a.samples << " samples (100%) "
                  << secs << "sec elapsed, (~0sec remaining)";
        std::cerr << std::endl;
        if (secs < 1e-9)
            secs = 1e-9;
        std::cerr << "render done: " << secs << " sec ("
                  << (size_t)(a.samples / secs) << " samples/sec)" << std::endl;
        if (st == FFR_BAD_VALUES)
            std::cerr << "render failure " << " (flame may not be sufficiently contractive)"
                      << std::endl;
        const double iter_part = stats.samples_iterated / (double)a.samples;
        std::cerr << "samples iterated: " << stats.samples_iterated << " ("
                  << (100 * iter_part) << "%)" << std::endl;
        const double plot_part = stats.samples_plotted / (double)a.samples;
        std::cerr << "samples plotted: " << stats.samples_plotted << " ("
                  << (100 * plot_part) << "%)" << std::endl;
        std::cerr << "xform selection:";
        for (uint64_t i = 0; i < stats.xform_ids && i < FFR_MAX_XFORM_IDS; ++i)
            std::cerr << " " << stats.xf_dist[i];
        std::cerr << std::endl;
        std::cerr << "bad value xforms:";
        for (uint64_t i = 0; i < stats.bad_recorded; ++i)
            std::cerr << " " << stats.bad_xf[i];
        std::cerr << std::endl;
        std::cerr << "bad value points:";
        for (uint64_t i = 0; i < stats.bad_recorded; ++i)
        {
            std::cerr << " (" << stats.bad_pts[i][0];
            for (uint32_t d = 1; d < dims; ++d)
                std::cerr << "," << stats.bad_pts[i][d];
            std::cerr << ")";
        }
        std::cerr << std::endl;
        std::cerr << "extreme coordinates:";
        for (uint32_t d = 0; d < dims; ++d)
            std::cerr << " (" << stats.ext_lo[d] << "," << stats.ext_hi[d] << ")";
        std::cerr << std::endl;
    }

    std::cerr << "writing output" << std::endl;
    check(ctx, ffr_read_buffer(ctx, buf.data(), buf.size()));
    if (a.output == "-")
    {
        std::cout.write(buf.data(), (std::streamsize)buf.size());
        std::cout.flush();
        if (!std::cout.good())
            die("error writing output");
    }
    else
    {
        std::ofstream f(a.output, std::ios::out | std::ios::binary);
        f.write(buf.data(), (std::streamsize)buf.size());
        if (!f.good())
            die("error writing output");
    }
    ffr_destroy(ctx);
    return 0;
}
