// Host check (no GPU): the Hilbert state-table encoder equals the per-level encoder for 64- and 32-bit keys, on
// random coordinates (also with bits above the key levels) and on a lattice of cell corners. Exit status 0 when equal.
#include "cs_common.cuh"

#include <cstdio>
#include <random>

int main()
{
    constexpr csg::HilbertTable t = csg::makeHilbertTable();
    std::mt19937_64 rng(5);
    long bad = 0, n = 0;
    for (int i = 0; i < 2000000; ++i)
    {
        uint64_t r = rng();
        unsigned x = r & 0x1fffff, y = (r >> 21) & 0x1fffff, z = (r >> 42) & 0x1fffff;
        if (i & 1)
        {
            x = unsigned(rng());
            y = unsigned(rng());
            z = unsigned(rng());
        }
        bad += csg::iHilbert<uint64_t>(x, y, z) != csg::iHilbertByTable<uint64_t>(x, y, z, t.e);
        bad += csg::iHilbert<uint32_t>(x, y, z) != csg::iHilbertByTable<uint32_t>(x, y, z, t.e);
        n += 2;
    }
    for (unsigned x = 0; x < 32; ++x)
        for (unsigned y = 0; y < 32; ++y)
            for (unsigned z = 0; z < 32; ++z, n += 2)
            {
                bad += csg::iHilbert<uint64_t>(x << 16, y << 16, z << 16) !=
                       csg::iHilbertByTable<uint64_t>(x << 16, y << 16, z << 16, t.e);
                bad += csg::iHilbert<uint32_t>(x << 5, y << 5, z << 5) !=
                       csg::iHilbertByTable<uint32_t>(x << 5, y << 5, z << 5, t.e);
            }
    std::printf("checked %ld, mismatches %ld\n", n, bad);
    return bad != 0;
}
