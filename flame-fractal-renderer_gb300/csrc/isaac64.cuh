// Per-thread ISAAC-64 with a 16-word state: the generator the reference
// runs per CPU thread, Isaac<u64,4> (src/rng/isaac.hpp:45-362), bit-exact.
//
//   gen()  isaac.hpp:77-90 with rngstep 146-153 and rngstep4 196-203
//   next() isaac.hpp:321-329: words are consumed from randrsl[15] down to
//          randrsl[0], then the state is regenerated
//   seed   setSeed(u64 s) -> setSeed(s, ~s, s ^ 11713835213681433683)
//          (isaac.hpp:267-282) with no seed array, so init() runs with
//          flag = false (isaac.hpp:93-131): randmem after init is the same
//          16 words for every seed (the golden-ratio mix, computed once on
//          the host: isaac_init_table()), and only a, b, c carry the seed.
//
// GB300 layout: randmem (16 words) and the result array (CAP words) of each
// thread live in shared memory as [word][thread] (stride BLOCK).  gen()
// indexes randmem with data-dependent words; with this layout lane L always
// hits bank pair (2L mod 32) whatever the word index, so every access is
// conflict-free.
//
// Refill ahead (CAP > 16): refill() moves the cnt unconsumed words up to
// rsl[16..16+cnt) and generates the next block into rsl[0..16); next() keeps
// consuming downwards, so the word sequence is exactly Isaac::next's, only
// the moment of generation moves earlier.  A warp can then regenerate all
// its lanes at one point (one masked gen() for the warp) instead of running
// gen() at every step for the few lanes that happen to run dry, which is
// what happens once lanes draw different numbers of words per step.
#pragma once

#include "std_types.h"

namespace ffr {

constexpr uint64_t kIsaacGolden = 0x9e3779b97f4a7c13ULL;
constexpr uint64_t kIsaacSeedXor = 11713835213681433683ULL;

// MurmurHash3 fmix64; fmix64(0) == 0 so stream 0 of seed S is setSeed(S)
__host__ __device__ inline uint64_t fmix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

__host__ __device__ inline uint64_t stream_key(uint64_t seed, uint64_t stream)
{
    return seed + fmix64(stream);
}

#ifdef __CUDACC__
template <int BLOCK, int CAP = 16>
struct DevIsaac
{
    static_assert(CAP >= 16, "the result array holds at least one block");
    uint64_t* mem;      // &smem_mem[threadIdx.x], stride BLOCK, 16 words
    uint64_t* rsl;      // &smem_rsl[threadIdx.x], stride BLOCK, CAP words
    uint64_t a, b, c;
    uint32_t cnt;

    __device__ __forceinline__ uint64_t& M(int i) { return mem[i * BLOCK]; }
    __device__ __forceinline__ uint64_t& Rs(int i) { return rsl[i * BLOCK]; }

    // one rngstep (isaac.hpp:146-153) at state index i with mixed a value mx
    __device__ __forceinline__ void step(int i, uint64_t mx, uint64_t& aa, uint64_t& bb)
    {
        const uint64_t x = M(i);
        aa = mx + M((i + 8) & 15);
        const uint64_t y = M((int)((x >> 3) & 15)) + aa + bb;
        M(i) = y;
        bb = M((int)((y >> 7) & 15)) + x;
        Rs(i) = bb;
    }

    // Isaac::gen: 16 rngsteps in four rngstep4 groups; kept as a rolled
    // loop so each inlined copy is small and no call ABI is involved
    __device__ __forceinline__ void gen()
    {
        uint64_t aa = a;
        uint64_t bb = b + (++c);
#pragma unroll 1
        for (int i = 0; i < 16; i += 4)
        {
            step(i + 0, ~(aa ^ (aa << 21)), aa, bb);
            step(i + 1, aa ^ (aa >> 5), aa, bb);
            step(i + 2, aa ^ (aa << 12), aa, bb);
            step(i + 3, aa ^ (aa >> 33), aa, bb);
        }
        a = aa;
        b = bb;
    }

    template <typename W>
    __device__ __forceinline__ void seed(uint64_t key, const W* init16)
    {
#pragma unroll
        for (int i = 0; i < 16; ++i)
            M(i) = init16[i];
        a = key;
        b = ~key;
        c = key ^ kIsaacSeedXor;
        gen();
        cnt = 16;
    }

    __device__ __forceinline__ uint64_t next()
    {
        if (cnt == 0)
        {
            gen();
            cnt = 16;
        }
        --cnt;
        return Rs((int)cnt);
    }

    // generate the next block now, keeping the cnt unconsumed words (needs
    // cnt <= CAP - 16)
    __device__ __forceinline__ void refill()
    {
        for (int k = (int)cnt - 1; k >= 0; --k)
            Rs(16 + k) = Rs(k);
        gen();
        cnt += 16;
    }
};
#endif // __CUDACC__

} // namespace ffr
