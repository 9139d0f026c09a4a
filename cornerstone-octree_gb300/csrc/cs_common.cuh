// Shared device/host helpers for the GB300 octree library: SFC key algebra, exactly-rounded arithmetic wrappers,
// the box parameter block, status codes and launch helpers.
//
// Parity rule for every floating-point expression that feeds a key, a node box or a distance test: it is written
// with explicit round-to-nearest intrinsics (__dmul_rn, __dadd_rn, ... / __fmul_rn, ...) so nvcc cannot fuse it into
// an FMA. The reference evaluates those expressions unfused (g++, x86-64), so only unfused arithmetic reproduces its
// results bit for bit.
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>

#include "../../include/cstone_gb300.h"

namespace csg
{

using TreeNodeIndex = int32_t;
using LocalIndex    = uint32_t;

// ---------------------------------------------------------------------------------------------------------------
// key width traits (tree/definitions.h:29-75)
// ---------------------------------------------------------------------------------------------------------------
template<class K>
struct KeyTraits;
template<>
struct KeyTraits<uint32_t>
{
    static constexpr int maxLevel   = 10;
    static constexpr int unusedBits = 2;
    static constexpr int bits       = 32;
};
template<>
struct KeyTraits<uint64_t>
{
    static constexpr int maxLevel   = 21;
    static constexpr int unusedBits = 1;
    static constexpr int bits       = 64;
};

template<class K>
__host__ __device__ __forceinline__ int clzKey(K x)
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(K) == 4) return __clz(x);
    else return __clzll((long long)x);
#else
    if (x == 0) return 8 * sizeof(K);
    if constexpr (sizeof(K) == 4) return __builtin_clz(x);
    else return __builtin_clzll(x);
#endif
}

template<class K>
__host__ __device__ __forceinline__ int ctzKey(K x)
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(K) == 4) return __ffs(x) - 1;
    else return __ffsll((long long)x) - 1;
#else
    if constexpr (sizeof(K) == 4) return __builtin_ctz(x);
    else return __builtin_ctzll(x);
#endif
}

// nodeRange(level) = 8^(maxLevel - level)
template<class K>
__host__ __device__ __forceinline__ K nodeRange(unsigned level)
{
    return K(1) << (3u * (KeyTraits<K>::maxLevel - level));
}
template<class K>
__host__ __device__ __forceinline__ K removeKey()
{
    return nodeRange<K>(0);
}
// level of a node whose key range is `range` (a power of 8)
template<class K>
__host__ __device__ __forceinline__ unsigned treeLevel(K range)
{
    return unsigned(clzKey<K>(range - 1) - KeyTraits<K>::unusedBits) / 3u;
}
template<class K>
__host__ __device__ __forceinline__ unsigned octalDigit(K code, unsigned pos)
{
    return unsigned(code >> (3u * (KeyTraits<K>::maxLevel - pos))) & 7u;
}
template<class K>
__host__ __device__ __forceinline__ int commonPrefix(K a, K b)
{
    return clzKey<K>(a ^ b) - KeyTraits<K>::unusedBits;
}
template<class K>
__host__ __device__ __forceinline__ K encodePlaceholderBit(K code, int prefixLength)
{
    int nShifts = 3 * KeyTraits<K>::maxLevel - prefixLength;
    return (K(1) << prefixLength) | (code >> nShifts);
}
template<class K>
__host__ __device__ __forceinline__ unsigned decodePrefixLength(K code)
{
    return unsigned(8 * sizeof(K) - 1 - clzKey<K>(code));
}
template<class K>
__host__ __device__ __forceinline__ K decodePlaceholderBit(K code)
{
    unsigned len = decodePrefixLength(code);
    return (code ^ (K(1) << len)) << (3u * KeyTraits<K>::maxLevel - len);
}
template<class K>
__host__ __device__ __forceinline__ K enclosingBoxCode(K key, unsigned level)
{
    return key & ~(nodeRange<K>(level) - 1);
}
__host__ __device__ __forceinline__ int digitWeight(int digit)
{
    int fourGeqMask = -int(digit >= 4);
    return ((7 - digit) & fourGeqMask) - (digit & ~fourGeqMask);
}

// ---------------------------------------------------------------------------------------------------------------
// Morton and Hilbert encoders/decoders (sfc/morton.hpp, sfc/hilbert.hpp)
// ---------------------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t spreadBits10(uint32_t v)
{
    // each of the 10 low bits of v moves to bit 3b
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__host__ __device__ __forceinline__ uint64_t spreadBits21(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x001f00000000ffffull;
    v = (v | (v << 16)) & 0x001f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ __forceinline__ uint32_t compactBits10(uint32_t v)
{
    v &= 0x09249249u;
    v = (v ^ (v >> 2)) & 0x030c30c3u;
    v = (v ^ (v >> 4)) & 0x0300f00fu;
    v = (v ^ (v >> 8)) & 0x030000ffu;
    v = (v ^ (v >> 16)) & 0x000003ffu;
    return v;
}
__host__ __device__ __forceinline__ uint32_t compactBits21(uint64_t v)
{
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
    v = (v ^ (v >> 8)) & 0x001f0000ff0000ffull;
    v = (v ^ (v >> 16)) & 0x001f00000000ffffull;
    v = (v ^ (v >> 32)) & 0x00000000001fffffull;
    return uint32_t(v);
}

template<class K>
__host__ __device__ __forceinline__ K iMorton(unsigned ix, unsigned iy, unsigned iz)
{
    if constexpr (sizeof(K) == 4) return K(spreadBits10(ix) * 4u + spreadBits10(iy) * 2u + spreadBits10(iz));
    else return K(spreadBits21(ix) * 4u + spreadBits21(iy) * 2u + spreadBits21(iz));
}

template<class K>
__host__ __device__ __forceinline__ void decodeMorton(K key, unsigned& ix, unsigned& iy, unsigned& iz)
{
    if constexpr (sizeof(K) == 4)
    {
        ix = compactBits10(key >> 2);
        iy = compactBits10(key >> 1);
        iz = compactBits10(key);
    }
    else
    {
        ix = compactBits21(key >> 2);
        iy = compactBits21(key >> 1);
        iz = compactBits21(key);
    }
}

// 3D Hilbert key, one octant per level from the most significant (the curve of sfc/hilbert.hpp:43-94). The octant of
// the current (rotated) coordinates is mapped by the table 0,1,3,2,7,6,4,5 (packed 3 bits per entry); afterwards the
// remaining lower bits of each coordinate are conditionally complemented and the axes permuted.
template<class K>
__host__ __device__ __forceinline__ K iHilbert(unsigned px, unsigned py, unsigned pz)
{
    constexpr uint32_t m2h = (0u) | (1u << 3) | (3u << 6) | (2u << 9) | (7u << 12) | (6u << 15) | (4u << 18) | (5u << 21);
    K key = 0;
#pragma unroll
    for (int level = KeyTraits<K>::maxLevel - 1; level >= 0; --level)
    {
        unsigned xi     = (px >> level) & 1u;
        unsigned yi     = (py >> level) & 1u;
        unsigned zi     = (pz >> level) & 1u;
        unsigned octant = (xi << 2) | (yi << 1) | zi;
        key             = (key << 3) + ((m2h >> (3 * octant)) & 7u);

        unsigned nyi = yi ^ 1u, nzi = zi ^ 1u;
        px ^= 0u - (xi & (nyi | zi));
        py ^= 0u - ((xi & (yi | zi)) | (yi & nzi));
        pz ^= 0u - ((xi & nyi & nzi) | (yi & nzi));

        unsigned t0 = px, t1 = py, t2 = pz;
        // zi: (x,y,z) <- (y,z,x); !zi && !yi: swap x and z
        px = zi ? t1 : (yi ? t0 : t2);
        py = zi ? t2 : t1;
        pz = zi ? t0 : (yi ? t2 : t0);
    }
    return key;
}

// The same curve by a state table. Every level of iHilbert complements some axes of the remaining bits and permutes
// the axes, so its running transform is a state: for each transformed axis, the original axis it reads (one of six
// permutations) and whether it is complemented (3 bits), 48 states of which 24 are reached from the identity (state
// 0). Entry [state * 8 + octant of the original bits at a level] = digit | next state << 3, generated from the level
// rule above.
struct HilbertTable
{
    uint16_t e[384];
};

constexpr HilbertTable makeHilbertTable()
{
    HilbertTable t{};
    constexpr int perms[6][3]  = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    constexpr unsigned m2h[8] = {0, 1, 3, 2, 7, 6, 4, 5};
    for (int st = 0; st < 48; ++st)
    {
        const int s[3]      = {perms[st / 8][0], perms[st / 8][1], perms[st / 8][2]};
        const unsigned f[3] = {(unsigned(st) >> 2) & 1u, (unsigned(st) >> 1) & 1u, unsigned(st) & 1u};
        for (unsigned o = 0; o < 8; ++o)
        {
            const unsigned ob[3] = {(o >> 2) & 1u, (o >> 1) & 1u, o & 1u};
            const unsigned xi = ob[s[0]] ^ f[0], yi = ob[s[1]] ^ f[1], zi = ob[s[2]] ^ f[2];
            const unsigned nyi = yi ^ 1u, nzi = zi ^ 1u;
            const unsigned g[3] = {f[0] ^ (xi & (nyi | zi)), f[1] ^ ((xi & (yi | zi)) | (yi & nzi)),
                                   f[2] ^ ((xi & nyi & nzi) | (yi & nzi))};
            // zi: (x, y, z) <- (y, z, x); !zi && !yi: swap x and z
            const int from[3] = {zi ? 1 : (yi ? 0 : 2), zi ? 2 : 1, zi ? 0 : (yi ? 2 : 0)};
            const int ns[3]   = {s[from[0]], s[from[1]], s[from[2]]};
            int pi            = 0;
            for (int q = 0; q < 6; ++q)
                if (perms[q][0] == ns[0] && perms[q][1] == ns[1] && perms[q][2] == ns[2]) pi = q;
            const unsigned next = unsigned(pi) * 8u + (g[from[0]] << 2 | g[from[1]] << 1 | g[from[2]]);
            t.e[st * 8 + int(o)] = uint16_t(m2h[xi << 2 | yi << 1 | zi] | (next << 3));
        }
    }
    return t;
}

// iHilbert through the state table T (in shared memory): the octants of all levels from one Morton interleave, then
// one lookup per level
template<class K>
__host__ __device__ __forceinline__ K iHilbertByTable(unsigned px, unsigned py, unsigned pz, const uint16_t* T)
{
    constexpr int L = KeyTraits<K>::maxLevel;
    uint64_t m;
    if constexpr (L == 21) m = (spreadBits21(px) << 2) | (spreadBits21(py) << 1) | spreadBits21(pz);
    else m = (spreadBits10(px) << 2) | (spreadBits10(py) << 1) | spreadBits10(pz);
    K key       = 0;
    unsigned st = 0;
#pragma unroll
    for (int level = L - 1; level >= 0; --level)
    {
        const unsigned e = T[st * 8u + (unsigned(m >> (3 * level)) & 7u)];
        key              = (key << 3) | K(e & 7u);
        st               = e >> 3;
    }
    return key;
}

template<class K>
__host__ __device__ __forceinline__ void decodeHilbert(K key, unsigned& ox, unsigned& oy, unsigned& oz)
{
    unsigned px = 0, py = 0, pz = 0;
#pragma unroll
    for (unsigned level = 0; level < unsigned(KeyTraits<K>::maxLevel); ++level)
    {
        unsigned octant = unsigned(key >> (3 * level)) & 7u;
        unsigned xi     = octant >> 2u;
        unsigned yi     = (octant >> 1u) & 1u;
        unsigned zi     = octant & 1u;
        unsigned t0 = px, t1 = py, t2 = pz;
        if (yi ^ zi)
        {
            px = t2;
            py = t0;
            pz = t1;
        }
        else if ((!xi & !yi & !zi) || (xi & yi & zi))
        {
            px = t2;
            pz = t0;
        }
        unsigned mask = (1u << level) - 1u;
        unsigned nxi = xi ^ 1u, nyi = yi ^ 1u, nzi = zi ^ 1u;
        px ^= mask & (0u - (xi & (yi | zi)));
        py ^= mask & (0u - ((xi & (nyi | nzi)) | (nxi & yi & zi)));
        pz ^= mask & (0u - ((xi & nyi & nzi) | (yi & zi)));
        px |= (xi << level);
        py |= ((xi ^ yi) << level);
        pz |= ((yi ^ zi) << level);
    }
    ox = px;
    oy = py;
    oz = pz;
}

template<class K>
__host__ __device__ __forceinline__ K iSfc(unsigned ix, unsigned iy, unsigned iz, int kind)
{
    return kind == CS_HILBERT ? iHilbert<K>(ix, iy, iz) : iMorton<K>(ix, iy, iz);
}

// ---------------------------------------------------------------------------------------------------------------
// exactly rounded scalar arithmetic (no FMA contraction)
// ---------------------------------------------------------------------------------------------------------------
template<class T>
struct RN;
template<>
struct RN<double>
{
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ int toIntRz(double a) { return __double2int_rz(a); }
    static __device__ __forceinline__ double floor_(double a) { return floor(a); }
    static __device__ __forceinline__ double rint_(double a) { return rint(a); }
    static __device__ __forceinline__ double abs_(double a) { return fabs(a); }
};
template<>
struct RN<float>
{
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ int toIntRz(float a) { return __float2int_rz(a); }
    static __device__ __forceinline__ float floor_(float a) { return floorf(a); }
    static __device__ __forceinline__ float rint_(float a) { return rintf(a); }
    static __device__ __forceinline__ float abs_(float a) { return fabsf(a); }
};

// ---------------------------------------------------------------------------------------------------------------
// box parameters, derived on the host in T precision exactly as cstone::Box<T> does (sfc/box.hpp:96-122)
// ---------------------------------------------------------------------------------------------------------------
template<class T>
struct BoxParams
{
    T lo[3], hi[3], len[3], ilen[3];
    int pbc[3];
};

template<class T>
inline BoxParams<T> makeBoxParams(const cs_box& b)
{
    BoxParams<T> p;
    for (int k = 0; k < 3; ++k)
    {
        p.lo[k]   = T(b.lo[k]);
        p.hi[k]   = T(b.hi[k]);
        p.len[k]  = p.hi[k] - p.lo[k];
        p.ilen[k] = T(1) / (p.hi[k] - p.lo[k]);
        p.pbc[k]  = b.boundary[k] == CS_PERIODIC;
    }
    return p;
}

// sfc3D (sfc/sfc.hpp:142-179) parameters: mx = 2^L * ilx and xmin * mx, both rounded in T as the reference does.
// T = double also carries the integer form of the quantisation (quantizeAxis): oi = floor(o), ofrac = (o != oi), and
// intForm when every axis passes the host's exactness checks
template<class T, class K>
struct KeyParams
{
    T m[3];
    T o[3];
    int oi[3];
    int ofrac[3];
    int intForm;
};

template<class T, class K>
inline KeyParams<T, K> makeKeyParams(const BoxParams<T>& b)
{
    KeyParams<T, K> p;
    unsigned cube = 1u << KeyTraits<K>::maxLevel;
    p.intForm     = std::is_same_v<T, double> ? 1 : 0;
    for (int k = 0; k < 3; ++k)
    {
        p.m[k] = T(cube) * b.ilen[k];
        p.o[k] = b.lo[k] * p.m[k];
        // integer form (quantizeAxis): |x m| and |o| below 2^29 over the box (so floor(x m) - o is within 2^30 and
        // its FP64 rounding below 2^-23), and the fraction of o zero or at least 2^-21 from 0 and 1
        const double o    = double(p.o[k]);
        const double oi   = std::floor(o);
        const double frac = o - oi; // exact
        const double ext  = std::max(std::fabs(double(b.lo[k])), std::fabs(double(b.hi[k]))) * double(p.m[k]);
        const bool ok     = std::isfinite(ext) && ext < 0x1p29 && std::fabs(o) < 0x1p29 &&
                        (frac == 0.0 || (frac > 0x1p-21 && 1.0 - frac > 0x1p-21));
        p.oi[k]    = ok ? int(oi) : 0;
        p.ofrac[k] = frac != 0.0 ? 1 : 0;
        if (!ok) p.intForm = 0;
    }
    return p;
}

// x = hi + lo with hi = RN_float(x) and lo = RN_float(x - hi) (x - hi is exact in FP64), computed from the bits of x
// with integer and FP32 instructions: GB300 issues FP64 instructions (the conversions and the subtraction) at a small
// fraction of the FP32 rate. For a normal float result (binary exponent of x in [-70, 100]) hi keeps the top 23 of
// the 52 mantissa bits, rounded to nearest with ties to even on the other 29 (a carry into the exponent included); x -
// hi is then rem * 2^(e - 52) with rem the discarded bits minus 2^29 when rounded up (|rem| <= 2^28), and lo is
// RN_float(rem) * 2^(e - 52), exact scaling by a power of two. Other exponents (zero, tiny or huge values, infinities,
// NaN) take the FP64 instructions. Both give the same bits.
__host__ __device__ __forceinline__ void splitDouble(double x, float& hi, float& lo)
{
#ifdef __CUDA_ARCH__
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long b;
    std::memcpy(&b, &x, sizeof b);
#endif
    const int e = int((b >> 52) & 0x7ffu) - 1023;
    if (e >= -70 && e <= 100)
    {
        const unsigned long long mant = b & 0xfffffffffffffull;
        unsigned m23                  = unsigned(mant >> 29);
        const int rem                 = int(mant & 0x1fffffffu);
        const bool up                 = rem > (1 << 28) || (rem == (1 << 28) && (m23 & 1u));
        const int diff                = up ? rem - (1 << 29) : rem;
        unsigned ex                   = unsigned(e + 127);
        if (up && ++m23 == (1u << 23))
        {
            m23 = 0;
            ++ex;
        }
        const unsigned sign = unsigned(b >> 32) & 0x80000000u;
        const unsigned hb   = sign | (ex << 23) | m23;
        const unsigned sb   = unsigned(e - 52 + 127) << 23; // 2^(e - 52), a normal float for e >= -74
#ifdef __CUDA_ARCH__
        hi = __uint_as_float(hb);
        lo = __fmul_rn(__int2float_rn(sign ? -diff : diff), __uint_as_float(sb));
#else
        std::memcpy(&hi, &hb, sizeof hi);
        float scale;
        std::memcpy(&scale, &sb, sizeof scale);
        lo = float(sign ? -diff : diff) * scale;
#endif
        return;
    }
#ifdef __CUDA_ARCH__
    hi = __double2float_rn(x);
    lo = __double2float_rn(__dsub_rn(x, double(hi)));
#else
    hi = float(x);
    lo = float(x - double(hi));
#endif
}

// Float estimate of a double from its high word (sign, exponent and the top 20 mantissa bits, rounded toward zero):
// |e - v| <= 2^-20 |v| for 2^-120 <= |v| < 2^120 and e = +-0 (|e - v| < 2^-120) below that range; false for
// |v| >= 2^120, Inf and NaN. Integer instructions only.
__host__ __device__ __forceinline__ bool truncEstimate(double v, float& e)
{
#ifdef __CUDA_ARCH__
    const unsigned hw = unsigned(__double2hiint(v));
#else
    unsigned long long b;
    std::memcpy(&b, &v, sizeof b);
    const unsigned hw = unsigned(b >> 32);
#endif
    const unsigned a = hw & 0x7fffffffu;
    if (a >= 0x47700000u) return false; // biased exponent >= 1023 + 120
    const unsigned fb = a < 0x38700000u ? hw & 0x80000000u : (hw & 0x80000000u) | ((a - 0x38000000u) << 3);
#ifdef __CUDA_ARCH__
    e = __uint_as_float(fb);
#else
    std::memcpy(&e, &fb, sizeof e);
#endif
    return true;
}

// One axis of sfc3D's quantisation, int(floor(x m) - o) evaluated as the reference does in T (sfc/sfc.hpp:142-160).
// Integer form (T = double, intForm): with f = floor(x m) (exact, an int while |x m| < 2^30) and o = oi + phi
// (oi = floor(o), phi in [0, 1)), the exact difference f - o is d - phi with d = f - oi. The reference rounds it to
// FP64 (an error of at most 2^-24 below 2^30), which keeps it inside (d - 1, d) when phi is 0 or at least 2^-21 from
// 0 and 1; its truncation is then d - 1 when phi > 0 and d >= 1, and d otherwise. That is two FP64-pipe operations
// (the product and the rounding-down conversion) instead of four. Products beyond 2^30 (points far outside the box)
// take the FP64 expression.
template<class T, class K>
__host__ __device__ __forceinline__ int quantizeAxis(T x, const KeyParams<T, K>& p, int k)
{
    if constexpr (std::is_same_v<T, double>)
    {
        if (p.intForm)
        {
#ifdef __CUDA_ARCH__
            const double y = __dmul_rn(x, p.m[k]);
            const int f    = __double2int_rd(y);
#else
            const double y = x * p.m[k];
            const double fy = std::floor(y);
            const int f     = fy >= -0x1p31 && fy < 0x1p31 ? int(fy) : (fy < 0 ? INT_MIN : INT_MAX);
#endif
            if (f > -(1 << 30) && f < (1 << 30))
            {
                const int d = f - p.oi[k];
                return p.ofrac[k] && d >= 1 ? d - 1 : d;
            }
        }
    }
#ifdef __CUDA_ARCH__
    return RN<T>::toIntRz(RN<T>::sub(RN<T>::floor_(RN<T>::mul(x, p.m[k])), p.o[k]));
#else
    const T v = T(std::floor(T(x * p.m[k])) - p.o[k]);
    return v >= T(-0x1p31) && v < T(0x1p31) ? int(v) : (v < T(0) ? INT_MIN : INT_MAX);
#endif
}

// htab: the Hilbert state table in shared memory (iHilbertByTable), or null for the per-level encoder; same keys
template<class T, class K>
__device__ __forceinline__ K sfc3D(T x, T y, T z, const KeyParams<T, K>& p, int kind, const uint16_t* htab = nullptr)
{
    constexpr int mcoord = (1 << KeyTraits<K>::maxLevel) - 1;
    int ix = quantizeAxis<T, K>(x, p, 0);
    int iy = quantizeAxis<T, K>(y, p, 1);
    int iz = quantizeAxis<T, K>(z, p, 2);
    ix     = min(ix, mcoord);
    iy     = min(iy, mcoord);
    iz     = min(iz, mcoord);
    if (kind == CS_HILBERT && htab) return iHilbertByTable<K>(unsigned(ix), unsigned(iy), unsigned(iz), htab);
    return iSfc<K>(unsigned(ix), unsigned(iy), unsigned(iz), kind);
}

// ---------------------------------------------------------------------------------------------------------------
// status plumbing
// ---------------------------------------------------------------------------------------------------------------
void setLastError(const char* fmt, ...);

#define CSG_CUDA_TRY(call)                                                                                             \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t err_ = (call);                                                                                     \
        if (err_ != cudaSuccess)                                                                                       \
        {                                                                                                              \
            ::csg::setLastError("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(err_));                 \
            return CS_ERR_CUDA;                                                                                        \
        }                                                                                                              \
    } while (0)

#define CSG_CHECK_LAUNCH() CSG_CUDA_TRY(cudaGetLastError())

inline unsigned iceil(size_t a, size_t b) { return unsigned((a + b - 1) / b); }

// number of SMs of the current device (cached per device)
int smCount();

// Reads `bytes` (a multiple of 4, at most 4096) of device memory to host memory after the work already on stream s:
// a one-warp kernel copies them into mapped pinned memory, then the stream is synchronised. No copy engine takes
// part, so the read never waits behind large device-to-host copies queued on other streams.
int readSmallToHost(cudaStream_t s, void* hostDst, const void* devSrc, size_t bytes);

// dst[k] = src[k], k < words: one warp; dst may be mapped pinned host memory
__global__ void copyWordsKernel(const uint32_t* src, uint32_t* dst, unsigned words);

// Device memory to host memory on stream s. Pinned (page-locked) destinations are written by a small kernel through
// their device mapping (16-byte stores where source and destination are aligned alike): the copy does not queue
// behind other streams' copies on the copy engines. Other destinations go through cudaMemcpyAsync.
int copyToHostAsync(cudaStream_t s, void* hostDst, const void* devSrc, size_t bytes);

// Bounds of the device-side waits, read by the host at each launch and passed as kernel arguments. The defaults
// give up after about a second; cs_set_wait_limits lowers them and can make one wait stall on purpose (a flag that
// nothing sets), so that tests reach the timeout path on ordinary inputs.
struct WaitLimits
{
    uint32_t sortSpins    = 1u << 22; // look-back rounds of the onesweep passes
    uint32_t barrierSpins = 1u << 24; // polls of the build's grid barrier
    int stall             = 0;        // CS_WAIT_STALL_* of include/cstone_gb300.h
};
WaitLimits waitLimits();

// bump allocator over a caller workspace; `size` only accumulates when base == nullptr (size query)
struct Arena
{
    char* base   = nullptr;
    size_t size  = 0;
    size_t limit = 0;

    template<class T>
    T* take(size_t n, size_t align = 256)
    {
        size_t off = (size + align - 1) / align * align;
        size       = off + n * sizeof(T);
        return base ? reinterpret_cast<T*>(base + off) : nullptr;
    }
    bool ok() const { return base == nullptr || size <= limit; }
};

// workspace helper: uses the caller's buffer when given, else a stream-ordered allocation freed on release()
struct Workspace
{
    void* ptr        = nullptr;
    bool owned       = false;
    cudaStream_t str = nullptr;

    int acquire(void* userPtr, size_t userBytes, size_t needed, cudaStream_t s)
    {
        str = s;
        if (needed == 0) return CS_OK;
        if (userPtr)
        {
            if (userBytes < needed)
            {
                setLastError("workspace too small: %zu bytes given, %zu needed", userBytes, needed);
                return CS_ERR_INVALID;
            }
            ptr = userPtr;
            return CS_OK;
        }
        CSG_CUDA_TRY(cudaMallocAsync(&ptr, needed, s));
        owned = true;
        return CS_OK;
    }
    ~Workspace()
    {
        if (owned && ptr) cudaFreeAsync(ptr, str);
    }
};

// a device buffer that only grows (the pipeline and batch objects keep theirs across calls)
struct DevBuf
{
    void* p      = nullptr;
    size_t bytes = 0;
    DevBuf()     = default;
    DevBuf(const DevBuf&)            = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    int ensure(size_t need)
    {
        if (need <= bytes) return CS_OK;
        if (p) cudaFree(p);
        p     = nullptr;
        bytes = 0;
        size_t alloc = need + need / 8 + 256;
        CSG_CUDA_TRY(cudaMalloc(&p, alloc));
        bytes = alloc;
        return CS_OK;
    }
    template<class T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

} // namespace csg
