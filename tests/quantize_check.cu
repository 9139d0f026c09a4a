// Host check (compiled with nvcc, run on the CPU): the integer form of sfc3D's FP64 quantisation (quantizeAxis with
// intForm) equals the reference's expression int(floor(x m) - o) on boxes with integer, near-integer and arbitrary
// offsets, for points on, beside and between cell boundaries, inside and outside the box.
#include "cs_common.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <random>

using namespace csg;

template<class K>
static void checkQuantisation(std::mt19937_64& rng, long long& checked, long long& mismatches, long long& boxesInt,
                              long long& boxes)
{
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    const double cells = double(1u << KeyTraits<K>::maxLevel);
    const double los[] = {-100.0, -1.0, 0.0, 0.3, -0.5, 1e-3, -3.7e2, 12345.678, -0.1, 2.0 / 3.0};
    for (int bi = 0; bi < 4000; ++bi)
    {
        double lo, len;
        if (bi < 10) { lo = los[bi], len = bi % 2 ? 2.0 : 200.0; }
        else
        {
            // arbitrary, power-of-two and near-integer-offset boxes
            lo  = (u01(rng) - 0.5) * std::pow(10.0, int(u01(rng) * 6) - 2);
            len = std::pow(2.0, int(u01(rng) * 12) - 4) * (bi % 3 ? 1.0 + u01(rng) : 1.0);
        }
        cs_box box{{lo, lo, lo}, {lo + len, lo + len, lo + len}, {CS_OPEN, CS_OPEN, CS_OPEN}};
        if (bi % 7 == 0)
        {
            // nudge the offset so that o = lo m lies within a few ulps of an integer
            const double m = cells / len;
            double o       = std::round(lo * m);
            box.lo[0] = box.lo[1] = box.lo[2] = std::nextafter(o / m, bi % 2 ? 1e300 : -1e300);
            box.hi[0] = box.hi[1] = box.hi[2] = box.lo[0] + len;
        }
        auto bp = makeBoxParams<double>(box);
        auto p  = makeKeyParams<double, K>(bp);
        ++boxes;
        if (!p.intForm) continue;
        ++boxesInt;
        auto ref = p;
        ref.intForm = 0;
        for (int t = 0; t < 2000; ++t)
        {
            double x;
            const int mode = t % 5;
            if (mode == 0) x = bp.lo[0] + u01(rng) * (bp.hi[0] - bp.lo[0]);
            else if (mode <= 2)
            {
                // on a cell boundary of the key grid and the neighbouring doubles
                const double cell = std::floor(u01(rng) * cells);
                x                 = bp.lo[0] + cell / p.m[0];
                for (int s = 0; s < t % 3; ++s)
                    x = std::nextafter(x, mode == 1 ? 1e300 : -1e300);
            }
            else if (mode == 3) x = bp.lo[0] + (u01(rng) * 3.0 - 1.0) * (bp.hi[0] - bp.lo[0]); // outside as well
            else x = t % 2 ? bp.lo[0] : bp.hi[0];
            const int a = quantizeAxis<double, K>(x, p, 0);
            const int b = quantizeAxis<double, K>(x, ref, 0);
            ++checked;
            if (a != b && mismatches++ < 5)
                std::printf("mismatch: lo %.17g len %.17g x %.17g int %d fp64 %d\n", bp.lo[0], bp.hi[0] - bp.lo[0], x,
                            a, b);
        }
    }
}

int main()
{
    std::mt19937_64 rng(20261204);
    long long checked = 0, mismatches = 0, boxesInt = 0, boxes = 0;
    checkQuantisation<uint64_t>(rng, checked, mismatches, boxesInt, boxes);
    checkQuantisation<uint32_t>(rng, checked, mismatches, boxesInt, boxes);
    std::printf("boxes %lld with the integer form %lld checked %lld mismatches %lld\n", boxes, boxesInt, checked,
                mismatches);

    // splitDouble: hi = RN_float(x), lo = RN_float(x - hi), against the conversions themselves, on random doubles of
    // every exponent and on the rounding ties and carries of the mantissa
    long long splitChecked = 0, splitBad = 0;
    auto checkSplit = [&](double x) {
        float hi, lo;
        splitDouble(x, hi, lo);
        const float rh = float(x), rl = float(x - double(rh));
        uint32_t a, b, c, d;
        std::memcpy(&a, &hi, 4);
        std::memcpy(&b, &rh, 4);
        std::memcpy(&c, &lo, 4);
        std::memcpy(&d, &rl, 4);
        ++splitChecked;
        if ((a != b || c != d) && !(x != x) && splitBad++ < 5)
            std::printf("split mismatch: x %a hi %a/%a lo %a/%a\n", x, double(hi), double(rh), double(lo), double(rl));
    };
    for (int e = -1100; e <= 1100; ++e)
        for (int t = 0; t < 400; ++t)
        {
            uint64_t mant = rng() & 0xfffffffffffffull;
            if (t % 4 == 1) mant = (mant & ~0x1fffffffull) | 0x10000000ull;           // a tie on the 29 bits
            if (t % 4 == 2) mant = 0xfffffe0000000ull | (mant & 0x1fffffffull);       // carry into the exponent
            if (t % 4 == 3) mant = (mant & ~0x1fffffffull) | (rng() & 0x3ull);       // tiny remainder
            const int be   = std::min(std::max(e + 1023, 0), 2047);
            uint64_t bits = (uint64_t(t & 1) << 63) | (uint64_t(be) << 52) | mant;
            double x;
            std::memcpy(&x, &bits, 8);
            checkSplit(x);
        }
    for (double x : {0.0, -0.0, 1.0, -1.0, 0x1p-70, 0x1p100, 0x1.fffffffp100, 0x1p-71, 3.4e38, -3.5e38})
        checkSplit(x);
    std::printf("split checked %lld mismatches %lld\n", splitChecked, splitBad);
    return mismatches || splitBad ? 1 : 0;
}
