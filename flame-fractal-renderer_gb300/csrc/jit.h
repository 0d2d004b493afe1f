// Per-flame render kernels compiled at run time (NVRTC).
//
// The reference applies an xform by walking its variation list through
// virtual calls (XForm::applyIteration, src/types/xform.hpp:211-227, over
// the factory of src/variations/variations.hpp:2614-2626); the precompiled
// general kernel does the same walk with a 98-way switch per variation.  A
// per-flame kernel is the same render kernel (chaos_body) with each xform's
// variation types fixed when it is compiled (chaos_kernel.cuh, FixedXform):
// no dispatch, no loop, no code for types the flame lacks.  Affines,
// weights and parameters stay in the program blob, so the kernel depends
// only on the flame's structure and is shared by every flame of the same
// structure; its buffers are those of the general kernel.
//
// Kernels are cached per process by their source text (and, with the
// environment variable FFR_JIT_CACHE naming a directory, on disk as cubins),
// so a structure is compiled once.
#pragma once

#include <cstddef>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "launch.h"

namespace ffr {

struct JitKernel
{
    cudaLibrary_t lib;
    cudaKernel_t kernel;
    int block;              // threads per CTA
    int regs;               // registers per thread
    int local_bytes;        // local memory (stack, spills) per thread
    double compile_ms;      // NVRTC time (0 when loaded from the disk cache)
};

// The per-flame render kernel's source for a program blob (ProgHeader<R>
// first; precision 0 = FP64, 1 = FP32), with or without colour: the plain
// kernel (entry ffr_flame_render, each variation slot's dispatch narrowed
// to the slot's types) or, with sorted, the xform-sorted kernel (entry
// ffr_flame_sorted, whose warps apply one xform at a time, each xform's
// code with its types fixed).  Empty for programs in the FP32 merged form,
// which the precompiled merged instantiations already run without dispatch,
// and for sorted kernels of flames the sorted kernel does not take (above 3
// dims or kSortedMaxXforms xforms).
std::string jit_source(const std::vector<unsigned char>& prog, int precision, bool color,
                       bool sorted = false);

// The loaded kernel for a source (compiled on first use; with compile
// false, only if the process or the disk cache already holds it); null and
// a message on failure (NVRTC missing, compile or load error).
const JitKernel* jit_kernel(const std::string& source, int precision, std::string* err,
                            bool compile = true);

// NVRTC only, no device: compile the source (or find it in the caches).
// Used to prepare kernels ahead of their renders.
bool jit_compile_only(const std::string& source, int precision, std::string* err);

cudaError_t jit_occupancy(const JitKernel* k, size_t smem, int* blocks_per_sm);
cudaError_t jit_launch(const JitKernel* k, const RenderArgs& a, int grid, size_t smem,
                       cudaStream_t st);

// threads per CTA of the per-flame plain kernels (the sorted ones:
// kSortedBlock)
constexpr int kJitBlock = 128;

} // namespace ffr
