// Host check (compiled with nvcc, run on the CPU) of the error bound behind the FP32 screen of the FP64 search boxes
// (searchBoxesScreenKernel). For coordinates p and smoothing lengths h over the whole covered range and beyond it,
// h in double or in float, scales in [2^-20, 16], and float estimates made either by rounding to nearest (the
// neighbour search's shadows) or by truncEstimate:
// - truncEstimate keeps 2^-20 relative accuracy from 2^-120 up, is +-0 below (error under 2^-120), and refuses
//   magnitudes from 2^120 on, infinities and NaN;
// - whenever every estimate is accepted, f = RN32(pt -+ rt) lies within E = 24 u (|pt| + |rt|) + 2^-98 (u = 2^-24) of
//   the reference's RN64(p -+ r), r = RN_Th(h scale);
// - a leaf centre c estimated by truncEstimate lies within 2^-19 |ct| + 2^-98 of c.
#include "cs_common.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace csg;

static double randExp(std::mt19937_64& rng, int emin, int emax)
{
    std::uniform_int_distribution<int> ed(emin, emax);
    std::uniform_int_distribution<unsigned long long> md(0, (1ull << 52) - 1);
    const double v = std::ldexp(1.0 + double(md(rng)) * 0x1p-52, ed(rng));
    return (rng() & 1) ? -v : v;
}

// a coordinate-like value: any exponent from far below to beyond the covered range, the range's edges and their
// neighbours, zeros and subnormals, or an everyday magnitude
static double pick(std::mt19937_64& rng, int emin, int emax)
{
    const int kind = int(rng() % 10);
    if (kind < 6) return randExp(rng, emin, emax);
    if (kind < 8)
    {
        const double edges[] = {0x1p120, 0x1p-120, 0x1p119, 0x1p-121, 0.0, -0.0, 5e-324, 1e-310, 0x1p-126, 0x1p-149,
                                1.0, 0.75};
        double v = edges[rng() % (sizeof(edges) / sizeof(edges[0]))];
        const int step = int(rng() % 3);
        if (step == 1) v = std::nextafter(v, 1e300);
        if (step == 2) v = std::nextafter(v, -1e300);
        return (rng() & 1) ? -v : v;
    }
    std::uniform_real_distribution<double> u(-1000.0, 1000.0);
    return u(rng);
}

static bool checkTrunc(double v, long long& bad)
{
    float e;
    const bool ok     = truncEstimate(v, e);
    const double a    = std::fabs(v);
    const bool expect = std::isfinite(v) && a < 0x1p120;
    if (ok != expect)
    {
        if (bad++ < 5) std::printf("truncEstimate(%.17g): ok %d, expected %d\n", v, int(ok), int(expect));
        return false;
    }
    if (!ok) return false;
    const long double err = std::fabs((long double)e - (long double)v);
    const bool good       = a >= 0x1p-120 ? err <= 0x1p-20L * a : (e == 0.f && err < 0x1p-120L);
    if (!good && bad++ < 5) std::printf("truncEstimate(%.17g) = %.9g\n", v, double(e));
    return good;
}

template<class Th>
static void checkScreen(std::mt19937_64& rng, bool shadow, long long& checked, long long& refused, long long& viol)
{
    const double scales[] = {2.0, 0.75, 0x1p-20, 16.0, 1.0, 1.5, 3.0};
    std::uniform_real_distribution<double> us(0x1p-20, 16.0);
    for (int it = 0; it < 400000; ++it)
    {
        const double p     = pick(rng, -140, 125);
        const double hd    = std::fabs(pick(rng, std::is_same_v<Th, float> ? -149 : -140, 125));
        const Th h         = Th(hd);
        const double scale = it % 2 ? scales[rng() % (sizeof(scales) / sizeof(scales[0]))] : us(rng);
        const Th sTh       = Th(scale);
        // the reference: r = RN_Th(h scale), then RN64(p -+ r)
        const Th rTh     = h * sTh;
        const double r   = double(rTh);
        const double vlo = p - r, vhi = p + r;
        if (!std::isfinite(r) || !std::isfinite(vlo) || !std::isfinite(vhi)) continue;
        // the screen's estimates, as sbEstimate makes them
        float pt  = 0.f;
        bool ok;
        if (shadow)
        {
            pt = float(p);
            ok = std::fabs(pt) < 0x1p120f;
        }
        else ok = truncEstimate(p, pt);
        const float sF = float(double(sTh));
        float rt;
        if constexpr (std::is_same_v<Th, float>)
        {
            rt = h * sF;
            ok = ok && std::fabs(rt) < 0x1p120f;
        }
        else
        {
            float ht = 0.f;
            ok       = truncEstimate(double(h), ht) && ok;
            rt       = ht * sF;
        }
        if (!ok)
        {
            refused++;
            continue;
        }
        const float flo = pt - rt, fhi = pt + rt;
        const long double E =
            24.0L * 0x1p-24L * ((long double)std::fabs(pt) + (long double)std::fabs(rt)) + 0x1p-98L;
        const long double dlo = std::fabs((long double)flo - (long double)vlo);
        const long double dhi = std::fabs((long double)fhi - (long double)vhi);
        if (dlo > E || dhi > E)
        {
            if (viol++ < 5)
                std::printf("bound violated: p %.17g h %.17g scale %.17g shadow %d: f %.9g %.9g v %.17g %.17g\n", p,
                            double(h), double(sTh), int(shadow), double(flo), double(fhi), vlo, vhi);
        }
        checked++;
    }
}

int main()
{
    std::mt19937_64 rng(20261204);
    long long truncChecked = 0, truncBad = 0;
    for (int it = 0; it < 2000000; ++it)
    {
        const double v = it % 1000 == 0 ? (it % 2000 ? std::nan("") : 1.0 / 0.0) : pick(rng, -1074, 1023);
        checkTrunc(v, truncBad);
        truncChecked++;
    }
    std::printf("truncEstimate: checked %lld, mismatches %lld\n", truncChecked, truncBad);

    long long centreChecked = 0, centreBad = 0;
    for (int it = 0; it < 1000000; ++it)
    {
        const double c = pick(rng, -140, 125);
        float ct;
        if (!truncEstimate(c, ct)) continue;
        const long double err = std::fabs((long double)ct - (long double)c);
        if (err > 0x1p-19L * std::fabs((long double)ct) + 0x1p-98L && centreBad++ < 5)
            std::printf("centre bound violated: %.17g -> %.9g\n", c, double(ct));
        centreChecked++;
    }
    std::printf("centre: checked %lld, mismatches %lld\n", centreChecked, centreBad);

    long long checked = 0, refused = 0, viol = 0;
    for (int shadow = 0; shadow < 2; ++shadow)
    {
        checkScreen<double>(rng, shadow, checked, refused, viol);
        checkScreen<float>(rng, shadow, checked, refused, viol);
    }
    std::printf("screen bound: checked %lld, refused %lld, mismatches %lld\n", checked, refused, viol);
    return (truncBad || centreBad || viol) ? 1 : 0;
}
