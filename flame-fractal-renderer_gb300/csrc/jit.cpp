// Per-flame render kernels: source generation, NVRTC compilation, caches,
// loading (cudaLibraryLoadData) and launch.  See jit.h.
#include "jit.h"

#include <dlfcn.h>
#include <unistd.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>

#include "flame.hpp"
#include "flame_program.h"

namespace ffr {

namespace {

// the kernel headers, embedded at build time (kJitHeaderCount,
// kJitHeaderNames, kJitHeaderTexts)
#include "jit_headers.inc"

// ProgHeader::tier_a_present's bit of a variation type (the kTa* bits of
// variations.cuh: linear, sinusoidal, spherical, swirl, horseshoe, polar,
// julia), 0 for the other types
const int32_t kTierA[7] = {V_LINEAR, V_SINUSOIDAL, V_SPHERICAL, V_SWIRL, V_HORSESHOE, V_POLAR,
                           V_JULIA};

uint32_t tier_a_bit(int type)
{
    for (int k = 0; k < 7; ++k)
        if (type == kTierA[k])
            return 1u << k;
    return 0u;
}

int tier_a_type(int bit)
{
    return kTierA[bit];
}

template <typename R>
std::string source_for(const std::vector<unsigned char>& prog, int precision, bool color,
                       bool sorted)
{
    ProgHeader<R> h;
    if (prog.size() < sizeof h)
        return std::string();
    std::memcpy(&h, prog.data(), sizeof h);
    if (h.merged || (sorted && (h.dims > 3 || h.nxf > kSortedMaxXforms)))
        return std::string();
    // the types each variation slot holds over the selectable and final xforms
    const int nx = h.nxf + (h.has_final ? 1 : 0);
    std::vector<uint32_t> ta;               // kTa* bits per slot
    std::vector<std::set<int>> other;       // the other types per slot
    std::ostringstream per_xform;           // the cases of FlameSpec::xform
    for (int i = 0; i < nx; ++i)
    {
        XformT<R> x;
        std::memcpy(&x, prog.data() + h.off_xf + (size_t)i * sizeof x, sizeof x);
        uint32_t xpresent = 0;
        std::string xtypes, xnames;
        for (int k = 0; k < x.var_count; ++k)
        {
            VarT<R> v;
            std::memcpy(&v, prog.data() + h.off_var + (size_t)(x.var_begin + k) * sizeof v,
                        sizeof v);
            xpresent |= tier_a_bit(v.type);
            xtypes += ", " + std::to_string(v.type);
            xnames += std::string(xnames.empty() ? "" : " ") + variation_name(v.type);
            if ((int)ta.size() <= k)
            {
                ta.resize(k + 1, 0u);
                other.resize(k + 1);
            }
            if (const uint32_t bit = tier_a_bit(v.type))
                ta[k] |= bit;
            else
                other[k].insert(v.type);
        }
        per_xform << "        " << (i + 1 == nx ? std::string("default")
                                                 : "case " + std::to_string(i))
                  << ":   // " << (i == h.nxf ? "final" : "xform " + std::to_string(i))
                  << ": " << (xnames.empty() ? "no variations" : xnames) << "\n"
                  << "            FixedXform<D, R, " << xpresent << "u, "
                  << (x.has_pre ? "true" : "false") << ", " << (x.has_post ? "true" : "false")
                  << ", " << x.var_begin << xtypes << ">::apply(pg, pg.xf[" << i
                  << "], p, out, rng);\n            return;\n";
    }
    std::ostringstream s;
    s << "// per-flame render kernel (" << h.dims << " dims, "
      << (precision ? "FP32" : "FP64") << (color ? ", colour" : "") << ", " << h.nxf
      << " xforms" << (h.has_final ? " + final" : "") << ")\n"
      << (sorted ? "#include \"chaos_sorted.cuh\"\n" : "#include \"chaos_kernel.cuh\"\n")
      << "namespace ffr {\n"
      << "struct FlameSpec\n{\n"
      << "    static constexpr bool on = true;\n"
      << "    static constexpr uint32_t present = " << h.tier_a_present << "u;\n"
      << "    static constexpr int slots = " << ta.size() << ";\n"
      << "    template <int S, int D, typename R, typename Rng>\n"
      << "    __device__ static __forceinline__ void slot(const VarT<R>& var, const R* t, R* o,"
         " Rng& rng, const PlanePrims<R>& pp)\n    {\n";
    for (size_t k = 0; k < ta.size(); ++k)
    {
        std::string types, names;
        for (int b = 0; b < 7; ++b)
            if (ta[k] >> b & 1u)
                names += std::string(names.empty() ? "" : " ") + variation_name(tier_a_type(b));
        for (int t : other[k])
        {
            types += ", " + std::to_string(t);
            names += std::string(names.empty() ? "" : " ") + variation_name(t);
        }
        s << "        " << (k ? "else if" : "if") << " constexpr (S == " << k << ")   // " << names
          << "\n            SlotTypes<D, R, " << ta[k] << "u" << types
          << ">::eval(var, t, o, rng, pp);\n";
    }
    s << "    }\n";
    if (sorted)
        s << "    // warps that apply one xform on every lane (sorted chunks, final xform)\n"
          << "    template <int D, typename R, typename Rng>\n"
          << "    __device__ static __forceinline__ void xform(const Prog<R>& pg, int xi, "
             "const R* p, R* out, Rng& rng)\n    {\n        switch (xi)\n        {\n"
          << per_xform.str() << "        }\n    }\n";
    s << "};\n} // namespace ffr\n\n";
    if (sorted)
    {
        s << "extern \"C\" __global__ void __launch_bounds__(" << kSortedBlock << ", 2)\n"
          << "ffr_flame_sorted(const ffr::RenderArgs a)\n{\n"
          << "    extern __shared__ __align__(16) unsigned char smem[];\n"
          << "    ffr::load_program<" << kSortedBlock << ">(smem, a.prog, a.prog_bytes);\n"
          << "    __syncthreads();\n"
          << "    ffr::sorted_body<" << h.dims << ", " << (precision ? "float" : "double")
          << ", " << (color ? "true" : "false") << ", " << kSortedBlock
          << ", ffr::FlameSpec>(a, smem);\n}\n";
        return s.str();
    }
    s << "extern \"C\" __global__ void __launch_bounds__(" << kJitBlock << ", "
      << "ffr::render_min_blocks<" << (precision ? "float" : "double") << ">())\n"
      << "ffr_flame_render(const ffr::RenderArgs a)\n{\n"
      << "    extern __shared__ __align__(16) unsigned char smem[];\n"
      << "    ffr::load_program<" << kJitBlock << ">(smem, a.prog, a.prog_bytes);\n"
      << "    __syncthreads();\n"
      << "    ffr::chaos_body<" << h.dims << ", " << (precision ? "float" : "double") << ", "
      << (color ? "true" : "false") << ", " << kJitBlock << ", 0, ffr::FlameSpec>(\n"
      << "        a, smem, (unsigned long long)blockIdx.x * " << kJitBlock << " + threadIdx.x,\n"
      << "        (unsigned long long)gridDim.x * " << kJitBlock << ");\n}\n";
    return s.str();
}

// ---- NVRTC, loaded on first use --------------------------------------------

typedef int (*nvrtcCreateProgram_t)(void**, const char*, const char*, int, const char* const*,
                                    const char* const*);
typedef int (*nvrtcCompileProgram_t)(void*, int, const char* const*);
typedef int (*nvrtcGetSize_t)(void*, size_t*);
typedef int (*nvrtcGetBytes_t)(void*, char*);
typedef int (*nvrtcDestroyProgram_t)(void**);
typedef const char* (*nvrtcGetErrorString_t)(int);

struct Nvrtc
{
    bool ok = false;
    std::string why;
    nvrtcCreateProgram_t create = nullptr;
    nvrtcCompileProgram_t compile = nullptr;
    nvrtcGetSize_t log_size = nullptr, cubin_size = nullptr;
    nvrtcGetBytes_t log = nullptr, cubin = nullptr;
    nvrtcDestroyProgram_t destroy = nullptr;
    nvrtcGetErrorString_t error = nullptr;
};

const Nvrtc& nvrtc()
{
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
        for (const char* env : {"CUDA_HOME", "CUDA_PATH"})
            if (const char* c = std::getenv(env))
                names.push_back(std::string(c) + "/lib64/libnvrtc.so.13");
        names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
        void* h = nullptr;
        for (const std::string& nm : names)
            if ((h = dlopen(nm.c_str(), RTLD_NOW | RTLD_LOCAL)) != nullptr)
                break;
        if (!h)
        {
            n.why = "NVRTC (libnvrtc.so.13) not found";
            return;
        }
        n.create = (nvrtcCreateProgram_t)dlsym(h, "nvrtcCreateProgram");
        n.compile = (nvrtcCompileProgram_t)dlsym(h, "nvrtcCompileProgram");
        n.log_size = (nvrtcGetSize_t)dlsym(h, "nvrtcGetProgramLogSize");
        n.log = (nvrtcGetBytes_t)dlsym(h, "nvrtcGetProgramLog");
        n.cubin_size = (nvrtcGetSize_t)dlsym(h, "nvrtcGetCUBINSize");
        n.cubin = (nvrtcGetBytes_t)dlsym(h, "nvrtcGetCUBIN");
        n.destroy = (nvrtcDestroyProgram_t)dlsym(h, "nvrtcDestroyProgram");
        n.error = (nvrtcGetErrorString_t)dlsym(h, "nvrtcGetErrorString");
        n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin
            && n.destroy && n.error;
        if (!n.ok)
            n.why = "NVRTC library lacks an entry point";
    });
    return n;
}

// compile options: the ones the precompiled kernel objects use (FP64
// without multiply-add contraction)
std::vector<std::string> options(int precision)
{
    std::vector<std::string> o = {"-arch=sm_103a", "-std=c++17", "-lineinfo"};
    if (precision == 0)
        o.push_back("--fmad=false");
    return o;
}

bool compile(const std::string& src, int precision, std::vector<char>* cubin, std::string* err)
{
    const Nvrtc& n = nvrtc();
    if (!n.ok)
    {
        *err = n.why;
        return false;
    }
    void* prog = nullptr;
    int r = n.create(&prog, src.c_str(), "ffr_flame.cu", kJitHeaderCount, kJitHeaderTexts,
                     kJitHeaderNames);
    if (r != 0)
    {
        *err = std::string("nvrtcCreateProgram: ") + n.error(r);
        return false;
    }
    const std::vector<std::string> opts = options(precision);
    std::vector<const char*> ov;
    for (const std::string& o : opts)
        ov.push_back(o.c_str());
    r = n.compile(prog, (int)ov.size(), ov.data());
    bool ok = r == 0;
    if (!ok)
    {
        size_t ls = 0;
        n.log_size(prog, &ls);
        std::string log(ls, '\0');
        if (ls)
            n.log(prog, &log[0]);
        *err = std::string("per-flame kernel failed to compile: ") + n.error(r) + "\n" + log;
    }
    else
    {
        size_t cs = 0;
        n.cubin_size(prog, &cs);
        cubin->assign(cs, 0);
        if (cs == 0 || n.cubin(prog, cubin->data()) != 0)
        {
            ok = false;
            *err = "NVRTC returned no cubin";
        }
    }
    n.destroy(&prog);
    return ok;
}

// ---- caches ----------------------------------------------------------------

uint64_t fnv1a(const std::string& s)
{
    uint64_t h = 1469598103934665603ull;
    for (unsigned char c : s)
    {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

// the kernel headers' text, hashed once: part of every key, so that a
// library built from other headers never takes a cached cubin of these
uint64_t headers_hash()
{
    static const uint64_t h = [] {
        std::string all;
        for (int i = 0; i < kJitHeaderCount; ++i)
            all += std::string(kJitHeaderNames[i]) + "\n" + kJitHeaderTexts[i];
        return fnv1a(all);
    }();
    return h;
}

// cache key: compile options, the headers' hash, the source
std::string key_of(const std::string& src, int precision)
{
    std::string k;
    for (const std::string& o : options(precision))
        k += o + "\n";
    char hh[40];
    std::snprintf(hh, sizeof hh, "headers %016llx\n", (unsigned long long)headers_hash());
    return k + hh + src;
}

// disk cache (FFR_JIT_CACHE): <hash>.cubin beside <hash>.key holding the
// full key, so a hash collision is a miss
std::string disk_path(const std::string& key, const char* ext)
{
    const char* dir = std::getenv("FFR_JIT_CACHE");
    if (!dir || !*dir)
        return std::string();
    char name[64];
    std::snprintf(name, sizeof name, "/ffr_%016llx.%s", (unsigned long long)fnv1a(key), ext);
    return std::string(dir) + name;
}

bool read_file(const std::string& path, std::string* out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    std::ostringstream s;
    s << f.rdbuf();
    *out = s.str();
    return true;
}

void write_file(const std::string& path, const char* data, size_t n)
{
    static std::atomic<unsigned long> serial{0};
    const std::string tmp = path + ".tmp" + std::to_string((unsigned long)getpid()) + "."
        + std::to_string(serial++);
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f)
            return;
        f.write(data, (std::streamsize)n);
        if (!f)
            return;
    }
    std::rename(tmp.c_str(), path.c_str());
}

struct Entry
{
    std::vector<char> cubin;
    double compile_ms = 0.0;
    std::unique_ptr<JitKernel> loaded;
};

std::mutex g_mu;
std::map<std::string, Entry>& cache()
{
    static std::map<std::string, Entry> c;
    return c;
}

// the entry for a key with its cubin (compiled unless compile_ok is false,
// or read from disk).  g_mu guards the map only: different sources compile
// in parallel (two threads compiling the same one keep the first result).
Entry* entry_for(const std::string& src, int precision, std::string* err, bool compile_ok)
{
    const std::string key = key_of(src, precision);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = cache().find(key);
        if (it != cache().end())
            return &it->second;
    }
    Entry e;
    const std::string kp = disk_path(key, "key"), cp = disk_path(key, "cubin");
    std::string k2, cub;
    if (!kp.empty() && read_file(kp, &k2) && k2 == key && read_file(cp, &cub) && !cub.empty())
        e.cubin.assign(cub.begin(), cub.end());
    else
    {
        if (!compile_ok)
        {
            *err = "per-flame kernel not compiled yet";
            return nullptr;
        }
        const auto t0 = std::chrono::steady_clock::now();
        if (!compile(src, precision, &e.cubin, err))
            return nullptr;
        e.compile_ms = std::chrono::duration<double, std::milli>(
            std::chrono::steady_clock::now() - t0).count();
        if (!cp.empty())
        {
            write_file(cp, e.cubin.data(), e.cubin.size());
            write_file(kp, key.data(), key.size());
        }
    }
    std::lock_guard<std::mutex> lk(g_mu);
    return &cache().emplace(key, std::move(e)).first->second;
}

} // namespace

std::string jit_source(const std::vector<unsigned char>& prog, int precision, bool color,
                       bool sorted)
{
    return precision == 0 ? source_for<double>(prog, 0, color, sorted)
                          : source_for<float>(prog, 1, color, sorted);
}

bool jit_compile_only(const std::string& source, int precision, std::string* err)
{
    if (source.empty())
    {
        *err = "no per-flame kernel for this program";
        return false;
    }
    return entry_for(source, precision, err, true) != nullptr;
}

const JitKernel* jit_kernel(const std::string& source, int precision, std::string* err,
                            bool compile)
{
    // the entry point the source defines
    const bool sorted = source.find("ffr_flame_sorted(") != std::string::npos;
    if (source.empty())
    {
        *err = "no per-flame kernel for this program";
        return nullptr;
    }
    Entry* e = entry_for(source, precision, err, compile);
    if (!e)
        return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (e->loaded)
        return e->loaded.get();
    std::unique_ptr<JitKernel> k(new JitKernel());
    cudaError_t ce = cudaLibraryLoadData(&k->lib, e->cubin.data(), nullptr, nullptr, 0,
                                         nullptr, nullptr, 0);
    if (ce == cudaSuccess)
    {
        ce = cudaLibraryGetKernel(&k->kernel, k->lib,
                                  sorted ? "ffr_flame_sorted" : "ffr_flame_render");
        if (ce != cudaSuccess)
            cudaLibraryUnload(k->lib);
    }
    if (ce != cudaSuccess)
    {
        *err = std::string("loading the per-flame kernel: ") + cudaGetErrorString(ce);
        return nullptr;
    }
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(k->kernel)) == cudaSuccess)
    {
        k->regs = fa.numRegs;
        k->local_bytes = (int)fa.localSizeBytes;
    }
    k->compile_ms = e->compile_ms;
    k->block = sorted ? kSortedBlock : kJitBlock;
    e->loaded = std::move(k);
    return e->loaded.get();
}

cudaError_t jit_occupancy(const JitKernel* k, size_t smem, int* blocks_per_sm)
{
    const void* f = reinterpret_cast<const void*>(k->kernel);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, k->block, smem);
}

cudaError_t jit_launch(const JitKernel* k, const RenderArgs& a, int grid, size_t smem,
                       cudaStream_t st)
{
    const void* f = reinterpret_cast<const void*>(k->kernel);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    RenderArgs copy = a;
    void* params[] = {&copy};
    return cudaLaunchKernel(f, dim3((unsigned)grid), dim3((unsigned)k->block), params, smem, st);
}

} // namespace ffr
