// Placement of a render's hot cells in the kernels' shared-memory table
// (chaos_kernel.cuh, bin_count): choose up to kHotCells candidates and an odd
// multiplier m under which slot(k) = (k * m) >> (32 - kHotSlotBits) is
// distinct for all of them.  Host-only; no reference counterpart.
#include "launch.h"

#include <algorithm>
#include <functional>
#include <vector>

bool ffr::hot_place(std::vector<unsigned long long>& found, unsigned long long sum,
                    unsigned int* mult, std::vector<unsigned int>& keys)
{
    // hottest first (ties by cell index, so the table is deterministic)
    std::sort(found.begin(), found.end(), std::greater<unsigned long long>());
    if (found.size() > (size_t)kHotCells)
        found.resize(kHotCells);
    unsigned long long mass = 0;
    for (unsigned long long f : found)
        mass += f >> 32;
    if (found.empty() || mass * 50 < sum)
        return false;
    // odd multipliers from a fixed sequence until the keys land in distinct
    // slots; with 64 keys in 256 slots about 1 in 4000 does, so give up on
    // the coldest keys only after many tries
    uint64_t x = 0x9E3779B97F4A7C15ull;
    for (size_t n = found.size(); n > 0; n = n > 8 ? n - 8 : 0)
    {
        for (int t = 0; t < 200000; ++t)
        {
            x = x * 6364136223846793005ull + 1442695040888963407ull;
            const unsigned int m = (unsigned int)(x >> 32) | 1u;
            uint64_t used[kHotSlots / 64] = {};
            bool ok = true;
            for (size_t i = 0; i < n && ok; ++i)
            {
                const unsigned int k = (unsigned int)(found[i] & 0xFFFFFFFFull);
                const unsigned int slot = (k * m) >> (32 - kHotSlotBits);
                ok = !(used[slot / 64] >> (slot % 64) & 1);
                used[slot / 64] |= 1ull << (slot % 64);
            }
            if (!ok)
                continue;
            keys.assign(kHotSlots, kHotEmpty);
            for (size_t i = 0; i < n; ++i)
            {
                const unsigned int k = (unsigned int)(found[i] & 0xFFFFFFFFull);
                keys[(k * m) >> (32 - kHotSlotBits)] = k;
            }
            *mult = m;
            return true;
        }
    }
    return false;
}
