// Neighbour search with the CPU reference's exact semantics (findneighbors.hpp:33-177).
//
// Semantics to reproduce. For each target i the reference walks the tree from the root in its stackless order
// (traversal/traversal.hpp:26-69), descends into a node only if norm2(minDistance(x_i, node box)) < cellR2 with
// cellR2 = (2 h_i)^2 ext^2, and in each leaf it reaches counts the particles j != i with |x_j - x_i|^2 < (2 h_i)^2,
// storing the first ngmax of them in visiting order; the count is not capped. Leaves are met in SFC order, so the
// stored neighbours are the first ngmax in ascending j among those on leaves whose whole root path passed the test.
//
// Main kernel (findNeighborsGroupKernel): one warp serves 32 consecutive targets and walks the tree ONCE for all of
// them, depth first with an explicit stack of (child offset or leaf code, lane mask) in shared memory, lowest child
// first. A child is pushed when it can hold a neighbour of some lane: lane l tests child l % 8 against the bounding
// box and bounding sphere of its sub-group of 8 targets (l / 8), and a child carries the lanes of the sub-groups that
// may reach it; a warp whose targets are spread far apart, or that has already expanded many nodes, tests each child
// per lane instead. At a leaf, each lane decides with a conservative box test whether it needs the leaf; the leaf's
// candidates come 32 at a time, and a batch is tested either per lane (each needing lane against all staged
// candidates, two per packed FP32 instruction, comparison signs appended to bit masks) or, when few lanes need it,
// per target (lanes hold the candidates, the warp loops over the needing targets with two ballots each); both give
// the same masks. The targets per warp (32, 16, 8) and the switch between the two loops are runtime tuning
// (NbArgs::groupSize, byTargetCost). Visiting superset leaves is harmless as long as the final decision equals the
// reference's, which depends on the whole root path (next paragraph).
//
// Path safety. A candidate at distance^2 d2 < r2 is counted by the reference only if each ancestor of its leaf passed
// the cell test. Every ancestor contains the candidate's key cell, so minDistance(x_i, ancestor) <= |x_j - x_i| up to
// the rounding of node boxes; with kappa = 32 u C (u the unit roundoff of T, C a bound on |coordinate|) and
// rho = 2^-20 (f64) / 2^-17 (f32),
//   Tsafe = cellR2 (1 - rho) - 4 kappa sqrt(cellR2) - 4 kappa^2
// is a lower bound below which every ancestor test passes in the reference's own arithmetic. Candidates with
// d2 < min(r2, Tsafe) are accepted outright; the rare ones in [Tsafe, r2) (only when ext < 1 + O(kappa)) walk the
// ancestor chain explicitly through parents[] with the reference's cell test.
//
// Arithmetic. T = float decides with the reference's expressions in round-to-nearest intrinsics (no contraction). The
// one-target-per-lane loops first evaluate the squared distance of the reference's own differences with packed FMAs,
// fma(dz, dz, fma(dy, dy, dx dx)); it and the reference's RN(RN(RN(dx dx) + RN(dy dy)) + RN(dz dz)) are each within
// 3 u d2 + 3 2^-150 of the exact sum (u = 2^-24), so below min(r2, Tsafe) (1 - 8 u) - 2^-146 the pair is a path-safe
// neighbour, from r2 (1 + 8 u) + 2^-146 on it is not, and only the band between is evaluated again unfused.
// T = double (GB300 has little FP64 throughput) first evaluates each test in FP32 on coordinates relative to a
// per-warp reference point P, with a proven bound on the difference to the FP64 result:
//   candidate  a_j = fl((xhi_j - P) + xlo_j)  (x = xhi + xlo, two floats),  target b_i = fl(x_i - P)
//   per axis   |fl(a_j - b_i) - fl64(x_j - x_i)| <= 3 eps |dx| + A,   A = 4 eps R + 4 eps^2 C,   eps = 2^-24
//              (R bounds |x_i - P| over the warp's targets, C bounds |x| over all particles)
//   distance   |d2_f - d2_64| <= 9.2 eps d2 + 3.5 A sqrt(d2) + 6 A^2
// so d2_f < T_acc proves d2_64 < min(r2, Tsafe) and d2_f >= T_out proves d2_64 >= r2 with
//   T_acc = min(r2, Tsafe) (1 - 24 eps) - 8 A r - 32 A^2,   T_out = r2 (1 + 24 eps) + 8 A r + 32 A^2.
// Only the tests that fall in [T_acc, T_out) are decided again in exact FP64, in out-of-line functions: inlined, the
// compiler hoists their FP64 multiplies into the hot FP32 loop.
//
// Periodic boundaries. Warps that contain a target whose search sphere crosses a periodic boundary are served by the
// per-lane path kernel (findNeighborsKernel): each lane keeps a mask per depth of its own root-to-node path and
// decides every test in T exactly as the reference does, with minimum-image folding.
#include "cs_common.cuh"
#include "neighbors.cuh"

#include <algorithm>
#include <cstdlib>
#include <type_traits>

namespace csg
{

constexpr int NB_THREADS  = 128;
constexpr int NB_WARPS    = NB_THREADS / 32;
constexpr int NB_MAXDEPTH = 24;
constexpr float EPS32     = 5.9604644775390625e-8f; // 2^-24

template<class T>
__device__ __forceinline__ T pbcFoldNb(T d, int pbc, T len, T ilen)
{
    return RN<T>::sub(d, RN<T>::mul(RN<T>::mul(T(pbc), len), RN<T>::rint_(RN<T>::mul(d, ilen))));
}

// norm2(minDistance(X, center, size[, box])) < cellR2 in precision T (traversal/boxoverlap.hpp:230-250)
template<class T>
__device__ __forceinline__ bool cellOverlapsExact(T xi, T yi, T zi, bool pbc, T cellR2, const T* c, const T* s,
                                                  const BoxParams<T>& b)
{
    T p[3] = {xi, yi, zi};
    T dd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        T d = RN<T>::sub(c[k], p[k]);
        if (pbc) d = pbcFoldNb<T>(d, b.pbc[k], b.len[k], b.ilen[k]);
        d     = RN<T>::abs_(d);
        d     = RN<T>::sub(d, s[k]);
        d     = RN<T>::add(d, RN<T>::abs_(d));
        dd[k] = RN<T>::mul(d, T(0.5));
    }
    T n2 = RN<T>::add(RN<T>::add(RN<T>::mul(dd[0], dd[0]), RN<T>::mul(dd[1], dd[1])), RN<T>::mul(dd[2], dd[2]));
    return n2 < cellR2;
}

// distanceSq<Pbc>(x_j, ..., x_i, ...) (findneighbors.hpp:33-60)
template<class T>
__device__ __forceinline__ T pairDist2Exact(T xi, T yi, T zi, bool pbc, T xj, T yj, T zj, const BoxParams<T>& b)
{
    T dx = RN<T>::sub(xj, xi), dy = RN<T>::sub(yj, yi), dz = RN<T>::sub(zj, zi);
    if (pbc)
    {
        dx = pbcFoldNb<T>(dx, b.pbc[0], b.len[0], b.ilen[0]);
        dy = pbcFoldNb<T>(dy, b.pbc[1], b.len[1], b.ilen[1]);
        dz = pbcFoldNb<T>(dz, b.pbc[2], b.len[2], b.ilen[2]);
    }
    return RN<T>::add(RN<T>::add(RN<T>::mul(dx, dx), RN<T>::mul(dy, dy)), RN<T>::mul(dz, dz));
}

// Exact FP64 decisions of the pre-filter's rare ambiguous cases. They are kept out of line: inlined, the compiler
// may hoist their FP64 multiplies into the FP32 fast path, and FP64 issues at a small fraction of the FP32 rate here.
struct PbcArgs
{
    double len[3], ilen[3];
    int pbc[3];
};

__device__ __noinline__ bool cellExactF64(double xi, double yi, double zi, bool pbc, double cellR2, const double* c,
                                          const double* s, PbcArgs pa)
{
    BoxParams<double> b;
    for (int k = 0; k < 3; ++k)
    {
        b.len[k]  = pa.len[k];
        b.ilen[k] = pa.ilen[k];
        b.pbc[k]  = pa.pbc[k];
    }
    return cellOverlapsExact<double>(xi, yi, zi, pbc, cellR2, c, s, b);
}

__device__ __noinline__ bool pairExactF64(double xi, double yi, double zi, bool pbc, double r2, const double* x,
                                          const double* y, const double* z, uint32_t j, PbcArgs pa)
{
    BoxParams<double> b;
    for (int k = 0; k < 3; ++k)
    {
        b.len[k]  = pa.len[k];
        b.ilen[k] = pa.ilen[k];
        b.pbc[k]  = pa.pbc[k];
    }
    return pairDist2Exact<double>(xi, yi, zi, pbc, x[j], y[j], z[j], b) < r2;
}

__device__ __forceinline__ float warpMaxF(float v)
{
    for (int o = 16; o > 0; o >>= 1)
        v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// radiusSq = 4 h h and cellRadiusSq = radiusSq ext ext in the precision of h (findneighbors.hpp:93-94), and the 2 h
// of the periodic-crossing test (:100): h of type T, or float with T coordinates when hf is set (the reference's
// findNeighbors with Tc = double and Th = float: both radii rounded to float, compared with T distances)
template<class T>
__device__ __forceinline__ void targetRadii(const T* h, const float* hf, uint32_t i, float ext, T& r2, T& cellR2,
                                            T& twoh)
{
    if (hf)
    {
        const float hh  = hf[i];
        const float r2f = __fmul_rn(__fmul_rn(4.f, hh), hh);
        r2              = T(r2f);
        cellR2          = T(__fmul_rn(__fmul_rn(r2f, ext), ext));
        twoh            = RN<T>::mul(T(2), T(hh));
    }
    else
    {
        const T hi = h[i];
        r2         = RN<T>::mul(RN<T>::mul(T(4.0), hi), hi);
        cellR2     = RN<T>::mul(RN<T>::mul(r2, T(ext)), T(ext));
        twoh       = RN<T>::mul(T(2), hi);
    }
}

template<class T, bool Stats>
__global__ void __launch_bounds__(NB_THREADS) findNeighborsKernel(NbArgs<T> a, NbPrep prep)
{
    constexpr bool F64 = std::is_same_v<T, double>;
    __shared__ unsigned sMask[NB_WARPS][NB_MAXDEPTH + 1];
    __shared__ float4 sCand[NB_WARPS][32];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t wid   = size_t(blockIdx.x) * NB_WARPS + warp;
    const size_t base0 = size_t(a.first) + wid * 32;
    if (base0 >= size_t(a.last)) return; // whole warp idle
    const size_t i64  = base0 + lane;
    const bool active = i64 < size_t(a.last);
    const uint32_t i  = active ? uint32_t(i64) : uint32_t(base0);

    // ---- target state in the reference precision ----
    T xi = a.x[i], yi = a.y[i], zi = a.z[i];
    T r2, cellR2, twoh;
    targetRadii<T>(a.h, a.hf, i, a.ext, r2, cellR2, twoh);
    bool pbc  = false;
    if (a.anyPbc)
    {
        bool inside = RN<T>::sub(xi, twoh) >= a.b.lo[0] && RN<T>::sub(yi, twoh) >= a.b.lo[1] &&
                      RN<T>::sub(zi, twoh) >= a.b.lo[2] && RN<T>::add(xi, twoh) <= a.b.hi[0] &&
                      RN<T>::add(yi, twoh) <= a.b.hi[1] && RN<T>::add(zi, twoh) <= a.b.hi[2];
        pbc = !inside;
    }
    // in the default mode this kernel only serves warps with a particle whose search sphere crosses a periodic
    // boundary; findNeighborsGroupKernel serves all others
    if (a.pathOnlyPbcWarps && !__any_sync(0xffffffffu, active && pbc)) return;

    // ---- FP32 pre-filter state (T = double) ----
    float Px = 0, Py = 0, Pz = 0, bx = 0, by = 0, bz = 0, A = 0, Tin = 0, Tout = 0, cLo = 0, cHi = 0;
    if constexpr (F64)
    {
        Px = __shfl_sync(0xffffffffu, __double2float_rn(xi), 0);
        Py = __shfl_sync(0xffffffffu, __double2float_rn(yi), 0);
        Pz = __shfl_sync(0xffffffffu, __double2float_rn(zi), 0);
        bx = __double2float_rn(__dsub_rn(xi, double(Px)));
        by = __double2float_rn(__dsub_rn(yi, double(Py)));
        bz = __double2float_rn(__dsub_rn(zi, double(Pz)));
        // thresholds in FP32 with directed rounding, so each is a true lower / upper bound of its real value:
        // R >= max |x_i - P| over the warp, C >= max |x|, A = 4 eps R + 4 eps^2 C
        float rloc = active ? fmaxf(fabsf(bx), fmaxf(fabsf(by), fabsf(bz))) : 0.f;
        float R    = __fmul_ru(warpMaxF(rloc), 1.f + 4 * EPS32);
        float C    = __fmul_ru(*prep.cmax, 1.f + 4 * EPS32);
        A          = __fmaf_ru(4 * EPS32, R, __fmul_ru(4 * EPS32 * EPS32, C));
        float r2lo = __double2float_rd(r2);
        float r2hi = __double2float_ru(r2);
        float rr   = __fsqrt_ru(r2hi);
        float m    = __fmul_ru(__fmul_ru(8.f, A), rr);
        float q    = __fmul_ru(__fmul_ru(32.f, A), A);
        Tin        = __fadd_rd(__fadd_rd(__fmul_rd(r2lo, 1.f - 24 * EPS32), -m), -q);
        Tout       = __fadd_ru(__fadd_ru(__fmul_ru(r2hi, 1.f + 24 * EPS32), m), q);
        cLo        = __double2float_rd(cellR2);
        cHi        = __double2float_ru(cellR2);
    }

    PbcArgs pa;
    for (int k = 0; k < 3; ++k)
    {
        pa.len[k]  = double(a.b.len[k]);
        pa.ilen[k] = double(a.b.ilen[k]);
        pa.pbc[k]  = a.b.pbc[k];
    }
    const unsigned ngmax = a.ngmax;
    uint32_t* myNb       = a.nb + size_t(i - a.first) * ngmax;
    unsigned nc          = 0;
    // optional statistics, accumulated per lane and flushed once per warp
    unsigned long long stCell = 0, stCellExact = 0, stPair = 0, stPairExact = 0, stLeaves = 0, stCand = 0, stNodes = 0;

    auto cellTest = [&](int node, unsigned parentMask) -> unsigned {
        bool ok = false;
        if constexpr (Stats) stNodes++;
        if ((parentMask >> lane) & 1u)
        {
            if constexpr (Stats) stCell++;
            const T* c = a.centers + 3 * size_t(node);
            const T* s = a.sizes + 3 * size_t(node);
            if constexpr (F64)
            {
                if (pbc) { ok = cellExactF64(xi, yi, zi, true, cellR2, c, s, pa); }
                else
                {
                    float4 ch = prep.nrec[3 * size_t(node)], cl = prep.nrec[3 * size_t(node) + 1],
                           sz = prep.nrec[3 * size_t(node) + 2];
                    float D[3] = {__fsub_rn(__fadd_rn(__fsub_rn(ch.x, Px), cl.x), bx),
                                  __fsub_rn(__fadd_rn(__fsub_rn(ch.y, Py), cl.y), by),
                                  __fsub_rn(__fadd_rn(__fsub_rn(ch.z, Pz), cl.z), bz)};
                    float S[3] = {sz.x, sz.y, sz.z};
                    float d[3], E = 0.f;
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                    {
                        // t = |c - x| - s differs from its FP64 value by at most u (see the file header); an axis
                        // with t + u < 0 is 0 in both precisions and adds no error, otherwise its square is off by
                        // at most 2 u (max(t, 0) + u)
                        float ad = fabsf(D[k]);
                        float t  = ad - S[k];
                        float u  = fmaf(4.5f * EPS32, ad + S[k], 1.05f * A);
                        d[k]     = fmaxf(t, 0.f);
                        if (t + u >= 0.f) E = fmaf(2.f * u, d[k] + u, E);
                    }
                    float n2 = fmaf(d[2], d[2], fmaf(d[1], d[1], d[0] * d[0]));
                    E        = fmaf(1.02f, E, fmaf(6.f * EPS32, n2, 1e-37f));
                    if (n2 + E < cLo) ok = true;
                    else if (n2 - E >= cHi) ok = false;
                    else
                    {
                        if constexpr (Stats) stCellExact++;
                        ok = cellExactF64(xi, yi, zi, false, cellR2, c, s, pa);
                    }
                }
            }
            else { ok = cellOverlapsExact<T>(xi, yi, zi, pbc, cellR2, c, s, a.b); }
        }
        return __ballot_sync(0xffffffffu, ok);
    };

    auto processLeaf = [&](int node, unsigned mask) {
        int leafIdx    = a.i2l[node];
        uint32_t first = a.layout[leafIdx];
        uint32_t last  = a.layout[leafIdx + 1];
        const bool mine = (mask >> lane) & 1u;
        if constexpr (Stats)
        {
            stLeaves++;
            stCand += last - first;
        }
        for (uint32_t base = first; base < last; base += 32)
        {
            uint32_t j = base + lane;
            float4 q   = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j < last)
            {
                if constexpr (F64)
                {
                    float4 ph = prep.phi[j], pl = prep.plo[j];
                    q.x = __fadd_rn(__fsub_rn(ph.x, Px), pl.x);
                    q.y = __fadd_rn(__fsub_rn(ph.y, Py), pl.y);
                    q.z = __fadd_rn(__fsub_rn(ph.z, Pz), pl.z);
                }
                else { q = make_float4(a.x[j], a.y[j], a.z[j], 0.f); }
            }
            __syncwarp();
            sCand[warp][lane] = q;
            __syncwarp();
            int cnt = int(min(32u, last - base));
            if (mine)
            {
                for (int k = 0; k < cnt; ++k)
                {
                    float4 c    = sCand[warp][k];
                    uint32_t jj = base + k;
                    bool in;
                    if constexpr (F64)
                    {
                        if (pbc) { in = pairExactF64(xi, yi, zi, true, r2, a.x, a.y, a.z, jj, pa); }
                        else
                        {
                            float dx = c.x - bx, dy = c.y - by, dz = c.z - bz;
                            float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                            if constexpr (Stats) stPair++;
                            if (d2 >= Tout) continue;
                            in = d2 < Tin;
                            if (!in)
                            {
                                if constexpr (Stats) stPairExact++;
                                in = pairExactF64(xi, yi, zi, false, r2, a.x, a.y, a.z, jj, pa);
                            }
                        }
                    }
                    else { in = pairDist2Exact<T>(xi, yi, zi, pbc, T(c.x), T(c.y), T(c.z), a.b) < r2; }
                    if (in && jj != i)
                    {
                        if (nc < ngmax) myNb[nc] = jj;
                        nc++;
                    }
                }
            }
        }
    };

    unsigned activeMask = __ballot_sync(0xffffffffu, active);
    unsigned rootMask   = cellTest(0, activeMask);
    if (rootMask)
    {
        if (a.childOffsets[0] == 0) { processLeaf(0, rootMask); }
        else
        {
            int depth          = 1;
            sMask[warp][depth] = rootMask;
            int node           = a.childOffsets[0];
            bool backtrack     = false;
            while (node != 0)
            {
                int child   = a.childOffsets[node];
                bool isLeaf = child == 0;
                unsigned m  = backtrack ? 0u : cellTest(node, sMask[warp][depth]);
                if (isLeaf && m) processLeaf(node, m);
                int sib = (node - 1) % 8;
                if (!isLeaf && m)
                {
                    node = child;
                    ++depth;
                    sMask[warp][depth] = m;
                    backtrack          = false;
                }
                else if (sib < 7)
                {
                    node++;
                    backtrack = false;
                }
                else
                {
                    node = a.parents[(node - 1) / 8];
                    --depth;
                    backtrack = true;
                }
                __syncwarp();
            }
        }
    }
    if (active) a.nc[i - a.first] = nc;
    if constexpr (Stats)
    {
        unsigned long long v[7] = {stCell, stCellExact, stPair, stPairExact, stLeaves, stCand, stNodes};
#pragma unroll
        for (int k = 0; k < 7; ++k)
        {
            unsigned long long x = v[k];
            if (k >= 4) x = lane == 0 ? x : 0; // per-warp quantities: count once
            for (int o = 16; o > 0; o >>= 1)
                x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) atomicAdd(a.stats + k, x);
        }
        if (lane == 0) atomicAdd(a.stats + 7, 1ull);
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Group traversal (all warps whose particles' search spheres stay inside the box, or open boxes).
//
// The reference visits a leaf for particle i only if every node on the root path passes i's pruning test. For a pair
// (i, j) with d2(i, j) clearly below the pruning radius that condition always holds: j lies in every ancestor's box
// up to the rounding slack delta of the key quantisation and of the node box arithmetic, so every ancestor is within
// sqrt(d2) + sqrt(3) kappa of x_i (kappa = delta + the FP rounding of the cell test). Hence
//   accept iff d2 < r2 and (d2 < Tsafe = cellR2 (1 - rho) - 4 kappa sqrt(cellR2) - 4 kappa^2
//                           or every ancestor of j's leaf passes i's exact cell test)
// gives exactly the reference's neighbour set; the explicit ancestor walk is needed only inside the thin band
// [Tsafe, r2). The tree is therefore walked once per warp with a conservative group test (node box against the
// bounding box of the warp's 32 search spheres, all boxes widened by their rounding margins), testing the 8
// children of a node in parallel and keeping the reference's depth-first order with a per-warp stack, so leaves are
// still met in SFC order and every lane sees its candidates in ascending j. Each reached leaf gets one conservative
// per-lane test (lower bound of the distance from x_i to the leaf box) that decides which lanes scan it.
// ---------------------------------------------------------------------------------------------------------------
// Stack entries per warp. Expanding a node at level d (at most 20: 64-bit keys have 21 levels) leaves at most 7
// pending siblings on each of the levels 1..d and pushes at most 8 children: 7 * 20 + 8 = 148 entries. The overflow
// check stays, and the shared memory saved goes to L1 (the kernel's node records and candidates).
constexpr int NBG_STACK = 152;
// resident blocks of 4 warps per SM: 64 registers per thread (a few spilled to the L1-cached stack); 7 and 9 measured
// slower on the 16M Plummer search
#ifndef NBG_MIN_BLOCKS
#define NBG_MIN_BLOCKS 8
#endif
// leaves merged into one candidate range at most (one target per lane), and the longest merged range
#ifndef NBG_MERGE
#define NBG_MERGE 8
#endif
#ifndef NBG_MERGE_SPAN
#define NBG_MERGE_SPAN 32
#endif

// exact decision of a pair in the ambiguous band (T = double): d2 < r2 and the reference's path condition
__device__ __noinline__ bool pairDecideF64(double xi, double yi, double zi, double r2, double cellR2, double kappa,
                                           const double* x, const double* y, const double* z, uint32_t j, int leafNode,
                                           const int32_t* parents, const double* centers, const double* sizes,
                                           bool contained, int rootNode)
{
    double dx = __dsub_rn(x[j], xi), dy = __dsub_rn(y[j], yi), dz = __dsub_rn(z[j], zi);
    double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (!(d2 < r2)) return false;
    // the path-safe shortcut needs the candidate inside its leaf's box (then inside every ancestor's)
    double ts = cellR2 * (1.0 - 0x1p-46) - 4.0 * kappa * sqrt(cellR2) - 4.0 * kappa * kappa;
    if (contained && d2 < ts) return true;
    BoxParams<double> nb{};
    for (int n = leafNode;;)
    {
        if (!cellOverlapsExact<double>(xi, yi, zi, false, cellR2, centers + 3 * size_t(n), sizes + 3 * size_t(n), nb))
            return false;
        if (n <= rootNode) return true;
        n = parents[(n - 1) / 8];
    }
}

// the reference's cell tests on the path from a leaf to the root, exact in FP64 (no periodic axis)
__device__ __noinline__ bool pathExactF64(double xi, double yi, double zi, double cellR2, int leafNode,
                                          const int32_t* parents, const double* centers, const double* sizes,
                                          int rootNode)
{
    BoxParams<double> nb{};
    for (int n = leafNode;;)
    {
        if (!cellOverlapsExact<double>(xi, yi, zi, false, cellR2, centers + 3 * size_t(n), sizes + 3 * size_t(n), nb))
            return false;
        if (n <= rootNode) return true;
        n = parents[(n - 1) / 8];
    }
}

// the reference's path condition for a float pair already known to be within r (T = float)
__device__ __noinline__ bool pathCheckF32(float xi, float yi, float zi, float cellR2, int leafNode,
                                          const int32_t* parents, const float* centers, const float* sizes,
                                          int rootNode)
{
    BoxParams<float> nb{};
    for (int n = leafNode;;)
    {
        if (!cellOverlapsExact<float>(xi, yi, zi, false, cellR2, centers + 3 * size_t(n), sizes + 3 * size_t(n), nb))
            return false;
        if (n <= rootNode) return true;
        n = parents[(n - 1) / 8];
    }
}

// The group traversal's rare exact decisions reload the target (coordinates, h; r2 and cellR2 recomputed with the
// expressions of the kernel's start) instead of keeping them in registers through the whole traversal.
template<class T>
struct TargetRef
{
    const T *x, *y, *z, *h;
    const float* hf;
    float ext;
    uint32_t i;
};

template<class T>
__device__ __forceinline__ void loadTarget(const TargetRef<T>& t, T& xi, T& yi, T& zi, T& r2, T& cellR2)
{
    xi       = t.x[t.i];
    yi       = t.y[t.i];
    zi       = t.z[t.i];
    T twoh;
    targetRadii<T>(t.h, t.hf, t.i, t.ext, r2, cellR2, twoh);
}

// a candidate in the band of the FP32 filter: the pair decision in the reference's arithmetic (T = double: FP64;
// T = float: the unfused FP32 distance) and the path condition (path-safe below tsafe when the candidate lies inside
// its leaf's box, else the ancestor walk)
template<class T>
__device__ __noinline__ bool slowPairAt(TargetRef<T> t, float kappa, float tsafe, uint32_t j, int leafNode,
                                        const int32_t* parents, const T* centers, const T* sizes, bool contained,
                                        int rootNode)
{
    T xi, yi, zi, r2, cellR2;
    loadTarget(t, xi, yi, zi, r2, cellR2);
    if constexpr (std::is_same_v<T, double>)
        return pairDecideF64(xi, yi, zi, r2, cellR2, double(kappa), t.x, t.y, t.z, j, leafNode, parents, centers,
                             sizes, contained, rootNode);
    else
    {
        const float dx = __fsub_rn(t.x[j], xi), dy = __fsub_rn(t.y[j], yi), dz = __fsub_rn(t.z[j], zi);
        const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (!(d2 < r2)) return false;
        if (contained && d2 < tsafe) return true;
        return pathCheckF32(xi, yi, zi, cellR2, leafNode, parents, centers, sizes, rootNode);
    }
}

// the path condition to a leaf (its candidates outside its box have no path-safe shortcut)
template<class T>
__device__ __noinline__ bool leafPathAt(TargetRef<T> t, int leafNode, const int32_t* parents, const T* centers,
                                        const T* sizes, int rootNode)
{
    T xi, yi, zi, r2, cellR2;
    loadTarget(t, xi, yi, zi, r2, cellR2);
    if constexpr (std::is_same_v<T, double>)
        return pathExactF64(xi, yi, zi, cellR2, leafNode, parents, centers, sizes, rootNode);
    else
        return pathCheckF32(float(xi), float(yi), float(zi), float(cellR2), leafNode, parents,
                            reinterpret_cast<const float*>(centers), reinterpret_cast<const float*>(sizes), rootNode);
}

// exact d2 < r2 of a pair (T = double, no periodic axis)
__device__ __noinline__ bool pairWithinAt(TargetRef<double> t, uint32_t j)
{
    double xi, yi, zi, r2, cellR2;
    loadTarget(t, xi, yi, zi, r2, cellR2);
    const PbcArgs open{};
    return pairExactF64(xi, yi, zi, false, r2, t.x, t.y, t.z, j, open);
}

// exact d2 < r2 of a pair in the reference's FP32 arithmetic (T = float, no periodic axis)
__device__ __noinline__ bool pairWithinAt(TargetRef<float> t, uint32_t j)
{
    float xi, yi, zi, r2, cellR2;
    loadTarget(t, xi, yi, zi, r2, cellR2);
    const float dx = __fsub_rn(t.x[j], xi), dy = __fsub_rn(t.y[j], yi), dz = __fsub_rn(t.z[j], zi);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) < r2;
}

__device__ __forceinline__ float warpMinF(float v)
{
    for (int o = 16; o > 0; o >>= 1)
        v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template<class T, bool Stats, int G>
__global__ void __launch_bounds__(NB_THREADS, NBG_MIN_BLOCKS) findNeighborsGroupKernel(NbArgs<T> a, NbPrep prep)
{
    // G targets per warp; the 32 / G lanes of one target test consecutive candidates side by side
    static_assert(G == 8 || G == 16 || G == 32, "targets per warp");
    constexpr int S      = 32 / G;
    constexpr bool F64   = std::is_same_v<T, double>;
    constexpr float EPS  = EPS32;
    // rounding slack of the key quantisation / node boxes, and of the cell test, in units of C
    constexpr float KAPPA_REL = F64 ? 32.f * 2.220446e-16f : 32.f * 1.1920929e-7f;
    constexpr float RHO       = F64 ? 9.5367432e-7f : 7.6293945e-6f; // 2^-20, 2^-17

    // stack entries (code, lane mask): code > 0 is the child offset of an internal node; a leaf is -(2 node + out) - 1,
    // out = 1 when it holds particles outside its box
    __shared__ int2 sStack[NB_WARPS][NBG_STACK];
    __shared__ float4 sCand[NB_WARPS][32];
    // S == 1: the staged candidates as separate x, y, z rows, read four at a time (two float2 pairs)
    __shared__ __align__(16) float sCx[NB_WARPS][32], sCy[NB_WARPS][32], sCz[NB_WARPS][32];
    // S == 1: each lane's target for the by-target loop: negated frame coordinates and -Tin, and -Tup
    __shared__ float4 sTgtA[NB_WARPS][32];
    __shared__ float sTgtB[NB_WARPS][32];
    // S == 1: leaves merged into one candidate range (their particle ranges adjoin): end of each range and its node
    __shared__ int2 sMerge[NB_WARPS][NBG_MERGE];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = lane % G, s = lane / G;
    const size_t wid   = size_t(blockIdx.x) * NB_WARPS + warp;
    const size_t base0 = size_t(a.first) + wid * G;
    if (base0 >= size_t(a.last)) return;
    if (a.anyPbc)
    {
        // the path kernel serves whole blocks of 32 targets that contain a sphere crossing a periodic boundary
        size_t b32 = size_t(a.first) + (base0 - size_t(a.first)) / 32 * 32;
        size_t ip  = b32 + lane;
        bool act   = ip < size_t(a.last);
        uint32_t q = act ? uint32_t(ip) : uint32_t(b32);
        T xq = a.x[q], yq = a.y[q], zq = a.z[q];
        T r2q, cr2q, twoh;
        targetRadii<T>(a.h, a.hf, q, a.ext, r2q, cr2q, twoh);
        bool inside = RN<T>::sub(xq, twoh) >= a.b.lo[0] && RN<T>::sub(yq, twoh) >= a.b.lo[1] &&
                      RN<T>::sub(zq, twoh) >= a.b.lo[2] && RN<T>::add(xq, twoh) <= a.b.hi[0] &&
                      RN<T>::add(yq, twoh) <= a.b.hi[1] && RN<T>::add(zq, twoh) <= a.b.hi[2];
        if (__any_sync(0xffffffffu, act && !inside)) return; // served by findNeighborsKernel
    }
    const size_t i64  = base0 + t;
    const bool active = i64 < size_t(a.last);
    const uint32_t i  = active ? uint32_t(i64) : uint32_t(base0);

    T xi = a.x[i], yi = a.y[i], zi = a.z[i];
    T r2, cellR2, twohI;
    targetRadii<T>(a.h, a.hf, i, a.ext, r2, cellR2, twohI);

    // ---- the warp's float frame: P = lane 0's position rounded to float, b = x_i - P ----
    float P[3], b[3];
    P[0] = __shfl_sync(0xffffffffu, float(xi), 0);
    P[1] = __shfl_sync(0xffffffffu, float(yi), 0);
    P[2] = __shfl_sync(0xffffffffu, float(zi), 0);
    if constexpr (F64)
    {
        b[0] = __double2float_rn(__dsub_rn(xi, double(P[0])));
        b[1] = __double2float_rn(__dsub_rn(yi, double(P[1])));
        b[2] = __double2float_rn(__dsub_rn(zi, double(P[2])));
    }
    else
    {
        b[0] = __fsub_rn(xi, P[0]);
        b[1] = __fsub_rn(yi, P[1]);
        b[2] = __fsub_rn(zi, P[2]);
    }
    float rloc = active ? fmaxf(fabsf(b[0]), fmaxf(fabsf(b[1]), fabsf(b[2]))) : 0.f;
    float R    = __fmul_ru(warpMaxF(rloc), 1.f + 4 * EPS);
    float C    = __fmul_ru(*prep.cmax, 1.f + 64 * EPS);
    float A    = __fmaf_ru(4 * EPS, R, __fmul_ru(4 * EPS * EPS, C));
    float delta = __fmul_ru(KAPPA_REL * 0.5f, C); // particle outside its node's float box by at most delta
    float kappa = __fmul_ru(KAPPA_REL, C);
    float r2lo, r2hi, cLo, cHi;
    if constexpr (F64)
    {
        r2lo = __double2float_rd(r2);
        r2hi = __double2float_ru(r2);
        cLo  = __double2float_rd(cellR2);
        cHi  = __double2float_ru(cellR2);
    }
    else { r2lo = r2hi = r2; cLo = cHi = cellR2; }
    float rr = __fsqrt_ru(r2hi);
    // path-safe threshold (lower bound)
    float tsafe = __fadd_rd(__fadd_rd(__fmul_rd(cLo, 1.f - RHO), -__fmul_ru(__fmul_ru(4.f, kappa), __fsqrt_ru(cHi))),
                            -__fmul_ru(__fmul_ru(4.f, kappa), kappa));
    // FP32 pre-filter thresholds (T = double): d2_f < Tacc proves d2_64 < min(r2, Tsafe); d2_f >= Tout proves >= r2
    float Tacc = 0, Tout = 0;
    if constexpr (F64)
    {
        float m  = __fmul_ru(__fmul_ru(8.f, A), rr);
        float q  = __fmul_ru(__fmul_ru(32.f, A), A);
        float lo = fminf(r2lo, tsafe);
        Tacc     = __fadd_rd(__fadd_rd(__fmul_rd(lo, 1.f - 24 * EPS), -m), -q);
        Tout     = __fadd_ru(__fadd_ru(__fmul_ru(r2hi, 1.f + 24 * EPS), m), q);
    }

    // ---- the warp's group bounds, per pass over the lanes whose targets share a traversal root ----
    // bounding box of the lanes' search spheres (widened by the frame's rounding), bounding sphere around its
    // centre, largest radius; the first node of the traversal (0, or the root of the lanes' set)
    float gc[3], gh[3], gR2 = 0.f, rmax = 0.f;
    unsigned activeMask = 0;
    int rootNode        = 0;
    // With one target per lane (S == 1) the bounds are those of the lane's sub-group of 8 consecutive targets (lanes
    // 8g .. 8g + 7), so that a node is only carried for the sub-groups that can reach it; otherwise the whole warp's.
    constexpr bool SUB = S == 1;
    auto segMin = [&](float v) {
        if constexpr (SUB)
        {
            for (int o = 4; o > 0; o >>= 1)
                v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
            return v;
        }
        else return warpMinF(v);
    };
    auto segMax = [&](float v) {
        if constexpr (SUB)
        {
            for (int o = 4; o > 0; o >>= 1)
                v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
            return v;
        }
        else return warpMaxF(v);
    };
    auto groupBounds = [&](bool inPass) {
        float rad = __fmul_ru(rr, 1.f + 64 * EPS);
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            float slack = __fmaf_ru(2 * EPS, fabsf(b[k]), delta);
            float lo    = inPass ? __fsub_rd(__fsub_rd(b[k], rad), slack) : INFINITY;
            float hi    = inPass ? __fadd_ru(__fadd_ru(b[k], rad), slack) : -INFINITY;
            lo          = segMin(lo);
            hi          = segMax(hi);
            gc[k]       = 0.5f * (lo + hi);
            gh[k]       = __fmul_ru(__fsub_ru(hi, lo), 0.5f);
        }
        // bounding sphere around the box centre gc: every point of every lane's sphere is within gR of gc, so it cuts
        // the corners of the box (which matter where the density rises steeply, e.g. towards a Plummer core)
        activeMask = __ballot_sync(0xffffffffu, inPass);
        rmax       = segMax(inPass ? rr : 0.f);
        float e0 = b[0] - gc[0], e1 = b[1] - gc[1], e2 = b[2] - gc[2];
        float dc = __fsqrt_ru(__fmaf_ru(e2, e2, __fmaf_ru(e1, e1, __fmul_ru(e0, e0))));
        float sl = __fmaf_ru(2 * EPS, fmaxf(fabsf(b[0]), fmaxf(fabsf(b[1]), fabsf(b[2]))), delta);
        float gr = inPass ? __fadd_ru(__fadd_ru(__fmul_ru(dc, 1.f + 8 * EPS), __fmul_ru(rr, 1.f + 64 * EPS)), sl) : 0.f;
        gr       = segMax(gr);
        gR2      = __fmul_ru(gr, gr);
    };

    const unsigned ngmax = a.ngmax;
    uint32_t* myNb       = a.nb + size_t(i - a.first) * ngmax;
    unsigned nc          = 0;
    // the lanes serving this lane's target: t, t + G, t + 2G, ...
    unsigned tmask = 0;
#pragma unroll
    for (int q = 0; q < S; ++q)
        tmask |= 1u << (t + q * G);
    unsigned long long stLeaves = 0, stCand = 0, stNodes = 0, stPair = 0, stExact = 0;
    // cost model of the candidate batches (lane 0): steps of the lane-per-target loop, needing lanes, the cheaper of
    // 11 instructions per step and 20 per needing lane, batches, cycles spent in the batches
    unsigned long long stSteps = 0, stNeed = 0, stMinCost = 0, stBatches = 0, stCandCyc = 0;
    // cycles in leaf visits (box test, staging and batches) and leaf visits no lane needed
    unsigned long long stLeafCyc = 0, stLeafIdle = 0;
    // output loop shapes per batch: the most hits of one lane, lanes with hits, rounds of 32 hits
    unsigned long long stOutMax = 0, stOutLanes = 0, stOutRounds = 0;
    unsigned long long stPathWalks = 0; // exact path walks to leaves holding particles outside their box

    // node box in the warp frame: center cc = (chi - P) + clo, half size sz
    auto frameOf = [&](float4 ch, float4 cl, float4 s4, float cc[3], float sz[3]) {
        cc[0] = __fadd_rn(__fsub_rn(ch.x, P[0]), cl.x);
        cc[1] = __fadd_rn(__fsub_rn(ch.y, P[1]), cl.y);
        cc[2] = __fadd_rn(__fsub_rn(ch.z, P[2]), cl.z);
        sz[0] = s4.x;
        sz[1] = s4.y;
        sz[2] = s4.z;
    };
    auto nodeFrame = [&](int node, float cc[3], float sz[3]) {
        const float4* r = prep.nrec + 3 * size_t(node);
        frameOf(r[0], r[1], r[2], cc, sz);
    };

    // conservative per-lane test: can a particle of this node lie within the search radius of x_i? (a lower
    // bound of |x_i - node box|, the box widened by the particle slack delta)
    // per axis (D - sz) - u with u = 4.5 EPS (D + sz) + 1.05 A + delta, evaluated as two FMAs with the factors
    // rounded outward, D (1 - 5 EPS) - (sz (1 + 6 EPS) + c0), the first rounded up and the second down
    const float hitC0 = __fmaf_ru(1.05f, A, delta);
    auto mayHitBox = [&](const float cc[3], const float sz[3]) -> bool {
        float n2 = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            float D = fabsf(__fsub_rn(cc[k], b[k]));
            float d = fmaxf(__fmaf_rd(D, 1.f - 5 * EPS, -__fmaf_ru(sz[k], 1.f + 6 * EPS, hitC0)), 0.f);
            n2      = __fmaf_rd(d, d, n2);
        }
        return n2 < r2hi;
    };
    auto mayHit = [&](int node) -> bool {
        float cc[3], sz[3];
        nodeFrame(node, cc, sz);
        return mayHitBox(cc, sz);
    };

    // decision for one candidate of the lane's target that survived the first distance filter; outside: the
    // candidate lies outside its leaf's box (no path-safe shortcut)
    auto decide = [&](uint32_t jj, float d2, int node, bool outside) -> bool {
        bool in;
        if constexpr (F64)
        {
            in = !outside && d2 < Tacc;
            if (!in)
            {
                if constexpr (Stats) stExact++;
                in = pairDecideF64(xi, yi, zi, r2, cellR2, double(kappa), a.x, a.y, a.z, jj, node, a.parents,
                                   a.centers, a.sizes, !outside, rootNode);
            }
        }
        else
        {
            in = !outside && d2 < tsafe;
            if (!in)
            {
                if constexpr (Stats) stExact++;
                in = pathCheckF32(float(xi), float(yi), float(zi), float(cellR2), node, a.parents,
                                  reinterpret_cast<const float*>(a.centers),
                                  reinterpret_cast<const float*>(a.sizes), rootNode);
            }
        }
        return in && jj != i;
    };
    // batch thresholds of the S == 1 loop: d2 < Tin is a neighbour (self aside), d2 >= Tup is not, the rest is
    // decided by decideSlow
    float Tin, Tup;
    if constexpr (F64)
    {
        Tin = Tacc;
        Tup = Tout;
    }
    else
    {
        // the packed FMA distance of the batch loops is within 6 u d2 + 6 2^-150 of the reference's unfused FP32
        // value (u = 2^-24, three roundings each, subnormal results included): below Tin the pair is a path-safe
        // neighbour, from Tup on it is not; the band between is decided exactly (decideSlow)
        Tin = __fsub_rd(__fmul_rd(fminf(float(r2), tsafe), 1.f - 8 * EPS), 0x1p-146f);
        Tup = __fadd_ru(__fmul_ru(float(r2), 1.f + 8 * EPS), 0x1p-146f);
    }
    // minus the target in the candidates' frame, as float pairs for the packed distance evaluation
    float nbS[3];
    if constexpr (F64)
    {
        nbS[0] = -b[0];
        nbS[1] = -b[1];
        nbS[2] = -b[2];
    }
    else
    {
        nbS[0] = -float(xi);
        nbS[1] = -float(yi);
        nbS[2] = -float(zi);
    }
    const float nTinS = -Tin, nTupS = -Tup;
    if constexpr (S == 1)
    {
        sTgtA[warp][lane] = make_float4(nbS[0], nbS[1], nbS[2], nTinS);
        sTgtB[warp][lane] = nTupS;
        __syncwarp();
    }
    const TargetRef<T> tref{a.x, a.y, a.z, a.h, a.hf, a.ext, i};
    auto decideSlow = [&](uint32_t jj, int node, bool contained) -> bool {
        return slowPairAt<T>(tref, kappa, tsafe, jj, node, a.parents, a.centers, a.sizes, contained, rootNode);
    };
    // first filter: FP32 distance of the staged candidate; returns d2 and whether it can be a neighbour
    auto filter = [&](float4 c, float& d2) -> bool {
        if constexpr (F64)
        {
            float dx = c.x - b[0], dy = c.y - b[1], dz = c.z - b[2];
            d2       = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            return d2 < Tout;
        }
        else
        {
            float dx = __fsub_rn(c.x, float(xi)), dy = __fsub_rn(c.y, float(yi)), dz = __fsub_rn(c.z, float(zi));
            d2       = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            return d2 < float(r2);
        }
    };

    // candidate j in the warp frame; beyond the leaf a point at infinity, which fails every distance test
    auto stage = [&](uint32_t j, uint32_t last) -> float4 {
        float4 q = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
        if (j < last)
        {
            if constexpr (F64)
            {
                float4 ph = prep.phi[j], pl = prep.plo[j];
                q.x       = __fadd_rn(__fsub_rn(ph.x, P[0]), pl.x);
                q.y       = __fadd_rn(__fsub_rn(ph.y, P[1]), pl.y);
                q.z       = __fadd_rn(__fsub_rn(ph.z, P[2]), pl.z);
            }
            else { q = make_float4(a.x[j], a.y[j], a.z[j], 0.f); }
        }
        return q;
    };

    // a leaf with its record r0..r2: the lanes whose sphere may reach it test its particles, 32 per batch
    // a leaf with its record r0..r2: the lanes whose sphere may reach it test its particles, 32 per batch. With
    // nMerged > 1 (S == 1) the following leaves of sMerge are tested with it as one range [first, lastM): needM is
    // this lane's need of any of them
    auto processLeaf = [&](int node, unsigned pmask, float4 recA, float4 recB, float4 recC, bool anyOut, int nMerged,
                           uint32_t lastM, bool needM) {
        const uint32_t first = __float_as_uint(recB.w), last = nMerged > 1 ? lastM : __float_as_uint(recC.w);
        // the first batch is loaded before the lanes' box test, so that the two latencies overlap
        float4 q0 = stage(first + lane, last);
        float cc[3], sz[3];
        frameOf(recA, recB, recC, cc, sz);
        bool need     = (((pmask >> lane) & 1u) && mayHitBox(cc, sz)) || needM;
        unsigned mask = __ballot_sync(0xffffffffu, need);
        if (mask == 0) return;
        // a leaf holding particles outside its box: whether this lane's path to it passes the reference's cell tests.
        // An upper bound of |x_i - box|^2 below Tsafe proves it (the ancestors contain the leaf); otherwise the path
        // is walked once, exactly
        bool leafPass = true;
        if (anyOut && need)
        {
            float n2u = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
            {
                float D = fabsf(__fsub_rn(cc[k], b[k]));
                float u = __fmaf_ru(4.5f * EPS, D + sz[k], __fmaf_ru(1.05f, A, delta));
                float d = fmaxf(__fadd_ru(__fsub_ru(D, sz[k]), u), 0.f);
                n2u     = __fmaf_ru(d, d, n2u);
            }
            if (!(n2u < tsafe))
            {
                if constexpr (Stats) stPathWalks++;
                leafPass = leafPathAt<T>(tref, node, a.parents, a.centers, a.sizes, rootNode);
            }
        }
        if constexpr (Stats)
        {
            stLeaves++;
            stCand += last - first;
        }
        for (uint32_t base = first; base < last; base += 32)
        {
            float4 q = base == first ? q0 : stage(base + lane, last);
            // candidates of this batch that lie outside their leaf's box (only in marked leaves)
            const unsigned outB =
                anyOut ? __ballot_sync(0xffffffffu, base + lane < last && prep.pout[base + lane]) : 0u;
            int cnt = int(min(32u, last - base));
            // S == 1: few needing lanes against many candidates are cheaper with the roles swapped (lanes hold the
            // candidates, the warp loops over the needing targets): about 19 instructions per needing target against
            // about byTargetCost (default 7) per candidate step of the per-lane loop (steps of eight; on the 16M
            // Plummer search the ratio 19 : 7 measured as good as any between 19 : 9 and 24 : 7)
            const bool byTarget = S == 1 && 19 * __popc(mask) < a.byTargetCost * ((cnt + 7) & ~7);
            if (!byTarget)
            {
                __syncwarp();
                if constexpr (S == 1)
                {
                    sCx[warp][lane] = q.x;
                    sCy[warp][lane] = q.y;
                    sCz[warp][lane] = q.z;
                }
                else { sCand[warp][lane] = q; }
                __syncwarp();
            }
            long long tc0 = 0;
            unsigned hitsThis = 0;
            if constexpr (Stats)
            {
                unsigned steps = (unsigned(cnt) + 7u) & ~7u;
                unsigned m     = __popc(mask);
                stSteps += steps;
                stNeed += m;
                stMinCost += min(11u * steps, 20u * m);
                stBatches++;
                tc0 = clock64();
            }
            if constexpr (S == 1)
            {
                // Bit 31 - k of inM: candidate k passes the FP32 test outright; of ambM: it is below the upper
                // threshold. The sign of e - T (exact for the packed add) is the comparison e < T, and a funnel shift
                // appends it to the mask, so that the candidates of a run end in order below its first one.
                unsigned inM = 0, ambM = 0;
                // four candidates (two packed FP32 pairs) against the target -n (negated frame coordinates) with the
                // negated thresholds nin, nup; the expressions are those of filter()
                auto four = [&](const float4& x4, const float4& y4, const float4& z4, const float2 n[3], float2 nin,
                                float2 nup, unsigned& mi, unsigned& ma) {
#pragma unroll
                    for (int p = 0; p < 2; ++p)
                    {
                        float2 cx = p ? make_float2(x4.z, x4.w) : make_float2(x4.x, x4.y);
                        float2 cy = p ? make_float2(y4.z, y4.w) : make_float2(y4.x, y4.y);
                        float2 cz = p ? make_float2(z4.z, z4.w) : make_float2(z4.x, z4.y);
                        float2 dx = __fadd2_rn(cx, n[0]);
                        float2 dy = __fadd2_rn(cy, n[1]);
                        float2 dz = __fadd2_rn(cz, n[2]);
                        // an FP32 filter with proven margins (the thresholds): any rounding of these FMAs stays
                        // inside them. T = float: the differences are the reference's own, and the band around r2
                        // is decided again with its unfused expression
                        float2 e = __fmul2_rn(dx, dx);
                        e        = __ffma2_rn(dy, dy, e);
                        e        = __ffma2_rn(dz, dz, e);
                        const float2 ti = __fadd2_rn(e, nin), tu = __fadd2_rn(e, nup);
                        mi = __funnelshift_l(__float_as_uint(ti.x), mi, 1);
                        mi = __funnelshift_l(__float_as_uint(ti.y), mi, 1);
                        ma = __funnelshift_l(__float_as_uint(tu.x), ma, 1);
                        ma = __funnelshift_l(__float_as_uint(tu.y), ma, 1);
                    }
                };
                const float4* vx = reinterpret_cast<const float4*>(sCx[warp]);
                const float4* vy = reinterpret_cast<const float4*>(sCy[warp]);
                const float4* vz = reinterpret_cast<const float4*>(sCz[warp]);
                // the target as packed pairs (negated frame coordinates and thresholds), built per batch from scalars
                const float2 n[3] = {make_float2(nbS[0], nbS[0]), make_float2(nbS[1], nbS[1]),
                                     make_float2(nbS[2], nbS[2])};
                const float2 nin = make_float2(nTinS, nTinS), nup = make_float2(nTupS, nTupS);
                if (byTarget)
                {
                    // lane k holds candidate k (past the leaf's end: a point at infinity); per needing target t the
                    // same FP32 expressions as four(), and the two signs collected by ballots (bit k: candidate k)
                    unsigned mm = mask, bi = 0, ba = 0;
                    while (mm)
                    {
                        const int t = __ffs(mm) - 1;
                        mm &= mm - 1;
                        const float4 tg = sTgtA[warp][t];
                        const float tup = sTgtB[warp][t];
                        const float dx = __fadd_rn(q.x, tg.x), dy = __fadd_rn(q.y, tg.y), dz = __fadd_rn(q.z, tg.z);
                        float e;
                        e = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                        const unsigned mi = __ballot_sync(0xffffffffu, __float_as_int(__fadd_rn(e, tg.w)) < 0);
                        const unsigned ma = __ballot_sync(0xffffffffu, __float_as_int(__fadd_rn(e, tup)) < 0);
                        if (lane == t)
                        {
                            bi = mi;
                            ba = ma;
                        }
                    }
                    inM  = __brev(bi);
                    ambM = __brev(ba);
                }
                else if (need)
                {
                    // eight independent distance chains per step; the staged points past the leaf's end never pass
                    int steps = 0;
                    for (int k0 = 0; k0 < cnt; k0 += 8, steps += 8)
                    {
                        const int v = k0 >> 2;
                        four(vx[v], vy[v], vz[v], n, nin, nup, inM, ambM);
                        four(vx[v + 1], vy[v + 1], vz[v + 1], n, nin, nup, inM, ambM);
                    }
                    if (steps < 32)
                    {
                        inM <<= 32 - steps;
                        ambM <<= 32 - steps;
                    }
                }
                if (need)
                {
                    ambM &= ~inM;
                    const unsigned outR = __brev(outB); // bit 31 - k: candidate k lies outside its leaf's box
                    // candidates outside their leaf's box: no path-safe shortcut; a neighbour iff within r and the
                    // lane's path to the leaf passes. Below Tin the FP32 bound already proves d2 < r2; the band
                    // [Tin, Tup) is decided exactly
                    const unsigned fIn = inM & outR, fAmb = ambM & outR;
                    inM &= ~outR;
                    ambM &= ~outR;
                    if (leafPass)
                    {
                        inM |= fIn;
                        // group warps have no periodic sphere
                        unsigned f = fAmb;
                        while (f)
                        {
                            int k = __clz(f);
                            f &= ~(0x80000000u >> k);
                            if (pairWithinAt(tref, base + k)) inM |= 0x80000000u >> k;
                        }
                    }
                    if constexpr (Stats)
                    {
                        stPair += cnt;
                        stExact += __popc(ambM);
                    }
                    while (ambM)
                    {
                        int k = __clz(ambM);
                        ambM &= ~(0x80000000u >> k);
                        int kn = node;
                        if (nMerged > 1)
                            for (int m = 0; m < nMerged; ++m)
                                if (base + k < uint32_t(sMerge[warp][m].x))
                                {
                                    kn = sMerge[warp][m].y;
                                    break;
                                }
                        if (decideSlow(base + k, kn, true)) inM |= 0x80000000u >> k;
                    }
                    if (i >= base && i - base < 32u) inM &= ~(0x80000000u >> (i - base));
                    if constexpr (Stats) hitsThis = __popc(inM);
                    // the hits in ascending candidate order; while the row has room for all of them (the common
                    // case) two per round, without a bound check per hit
                    const unsigned nh = __popc(inM);
                    if (nc + nh <= ngmax)
                    {
                        uint32_t* p = myNb + nc;
                        while (inM)
                        {
                            const int k1 = __clz(inM);
                            inM ^= 0x80000000u >> k1;
                            p[0] = base + k1;
                            if (inM)
                            {
                                const int k2 = __clz(inM);
                                inM ^= 0x80000000u >> k2;
                                p[1] = base + k2;
                            }
                            p += 2;
                        }
                        nc += nh;
                    }
                    else
                    {
                        while (inM)
                        {
                            int k = __clz(inM);
                            inM &= ~(0x80000000u >> k);
                            if (nc < ngmax) myNb[nc] = base + k;
                            nc++;
                        }
                    }
                }
            }
            else
            {
                // lane (t, s) tests candidate k0 + s for target t; a ballot keeps each target's hits in order
                for (int k0 = 0; k0 < cnt; k0 += S)
                {
                    int k       = k0 + s;
                    uint32_t jj = base + k;
                    bool in     = false;
                    if (need && k < cnt)
                    {
                        float e;
                        if constexpr (Stats) stPair++;
                        in = filter(sCand[warp][k], e) && decide(jj, e, node, (outB >> k) & 1u);
                    }
                    unsigned hits = __ballot_sync(0xffffffffu, in);
                    unsigned mine = hits & tmask;
                    if (in)
                    {
                        unsigned pos = nc + __popc(mine & ((1u << lane) - 1u));
                        if (pos < ngmax) myNb[pos] = jj;
                    }
                    nc += __popc(mine);
                }
            }
            if constexpr (Stats)
            {
                __syncwarp();
                stCandCyc += (unsigned long long)(clock64() - tc0);
                const unsigned mx  = __reduce_max_sync(0xffffffffu, hitsThis);
                const unsigned tot = __reduce_add_sync(0xffffffffu, hitsThis);
                stOutMax += mx;
                stOutLanes += __popc(__ballot_sync(0xffffffffu, hitsThis != 0));
                stOutRounds += (tot + 31) / 32;
            }
        }
    };

    // A warp whose targets are spread far apart (sparse regions, jumps of the curve) has a bounding box much larger
    // than its spheres; it then tests every child per lane against the lane's own sphere and carries the lanes that
    // remain alive on the stack, as the per-particle traversal does, instead of using the box. So does a warp whose
    // group bounds turn out to enclose many more nodes than its spheres (after LOOSE_AFTER expansions, several times
    // what a compact warp needs).
    constexpr int LOOSE_AFTER = 96;
    bool loose                = false;
    int expansions            = 0;
    long long t0              = Stats ? clock64() : 0;
    // absolute part of the child test's margin: the rounding terms and the float centre's missing low part
    const float childMargin = __fadd_ru(__fmaf_ru(4 * EPS * EPS, C, delta), __fmul_ru(EPS, C));
    float rminW               = Stats ? warpMinF(active ? rr : INFINITY) : 0.f;
    int2* stack               = sStack[warp];
    auto entryCode            = [](int node, int c0) { return c0 > 0 ? c0 : -(2 * node + (c0 < 0 ? 1 : 0)) - 1; };

    // one pass per set among the warp's targets (batched trees; a single pass otherwise)
    int mySet = 0, passSet = 0, lastSet = 0;
    if (a.numSets)
    {
        int lo = 0, hi = a.numSets;
        while (lo + 1 < hi)
        {
            int mid = (lo + hi) >> 1;
            if (__ldg(a.setOffsets + mid) <= i) lo = mid;
            else hi = mid;
        }
        mySet   = lo;
        passSet = __reduce_min_sync(0xffffffffu, active ? unsigned(mySet) : 0xffffffffu);
        lastSet = int(__reduce_max_sync(0xffffffffu, active ? unsigned(mySet) : 0u));
    }
    for (;; ++passSet)
    {
    const bool inPass = active && (!a.numSets || mySet == passSet);
    groupBounds(inPass);
    rootNode   = a.numSets ? __ldg(a.setRoots + passSet) : 0;
    loose      = __any_sync(0xffffffffu, __fsqrt_ru(gR2) > 3.f * rmax);
    expansions = 0;
    int top      = 0;
    const int rootC0 = __float_as_int(prep.nrec[3 * size_t(rootNode)].w);
    if (lane == 0)
    {
        stack[0] = make_int2(entryCode(rootNode, rootC0), int(activeMask));
    }
    top = activeMask ? 1 : 0;
    __syncwarp();
    while (top > 0)
    {
        const int2 ent       = stack[top - 1];
        const unsigned pmask = unsigned(ent.y);
        const int c0         = ent.x;
        --top;
        if (c0 <= 0) // a leaf
        {
            const int node = (-c0 - 1) >> 1;
            const bool out = (-c0 - 1) & 1;
            const float4* rec = prep.nrec + 3 * size_t(node);
            float4 recA = rec[0], recB = rec[1], recC = rec[2];
            long long tl0 = Stats ? clock64() : 0;
            unsigned long long before = stLeaves;
            // S == 1: the next leaves on the stack whose particles continue this leaf's range (siblings and cousins
            // met consecutively in SFC order) join its candidate range while it stays within NBG_MERGE_SPAN
            // particles; a
            // lane then tests all of them, which changes no decision (a candidate outside a lane's sphere fails its
            // distance test), and the batch overhead is paid once. Leaves holding particles outside their box stay alone
            int nMerged    = 1;
            uint32_t lastM = __float_as_uint(recC.w);
            bool needM     = false;
            if constexpr (S == 1)
            {
                const uint32_t first = __float_as_uint(recB.w);
                while (!out && top > 0 && nMerged < NBG_MERGE && lastM - first < unsigned(NBG_MERGE_SPAN))
                {
                    const int2 nx = stack[top - 1];
                    if (nx.x > 0 || ((-nx.x - 1) & 1)) break; // an internal node, or a leaf with outside particles
                    const int nnode    = (-nx.x - 1) >> 1;
                    const float4* nrc  = prep.nrec + 3 * size_t(nnode);
                    const float4 nB = nrc[1], nC = nrc[2];
                    if (__float_as_uint(nB.w) != lastM || __float_as_uint(nC.w) - first > unsigned(NBG_MERGE_SPAN))
                        break;
                    const float4 nA = nrc[0];
                    float cc[3], sz[3];
                    frameOf(nA, nB, nC, cc, sz);
                    needM = needM || (((unsigned(nx.y) >> lane) & 1u) && mayHitBox(cc, sz));
                    if (lane == 0)
                    {
                        if (nMerged == 1) sMerge[warp][0] = make_int2(int(lastM), node);
                        sMerge[warp][nMerged] = make_int2(int(__float_as_uint(nC.w)), nnode);
                    }
                    lastM = __float_as_uint(nC.w);
                    ++nMerged;
                    --top;
                }
                if (nMerged > 1) __syncwarp();
            }
            processLeaf(node, pmask, recA, recB, recC, out, nMerged, lastM, needM);
            if constexpr (Stats)
            {
                stLeafCyc += (unsigned long long)(clock64() - tl0);
                stLeafIdle += stLeaves == before;
            }
            continue;
        }
        if constexpr (Stats) stNodes++;
        if (++expansions > LOOSE_AFTER) loose = true;
        bool ok         = false;
        unsigned cmask  = pmask; // lanes alive in the accepted child (this lane's child when lane < 8)
        int childC0     = 0;     // child offset of this lane's child (lane < 8)
        if (!loose)
        {
            // lane l tests child l & 7 against its sub-group's bounds (every lane of one sub-group tests the 8
            // children; S > 1: lanes 0-7 against the warp's bounds)
            const int cidx = SUB ? (lane & 7) : lane;
            bool hit       = false;
            if (SUB || lane < 8)
            {
                // the child's centre in the frame from its float centre alone (the low part, at most EPS C, is
                // covered by childMargin), so one load of its record is saved
                const float4* r = prep.nrec + 3 * size_t(c0 + cidx);
                const float4 rA = r[0], rC = r[2];
                const float cc[3] = {__fsub_rn(rA.x, P[0]), __fsub_rn(rA.y, P[1]), __fsub_rn(rA.z, P[2])};
                const float sz[3] = {rC.x, rC.y, rC.z};
                childC0     = __float_as_int(rA.w);
                hit         = true;
                float dist2 = 0.f;
#pragma unroll
                for (int k = 0; k < 3; ++k)
                {
                    // ad - sz rounded down once for both tests (that only widens the overlap test)
                    float ad     = fabsf(cc[k] - gc[k]);
                    float margin = __fmaf_ru(4 * EPS, fabsf(cc[k]) + sz[k] + fabsf(gc[k]) + gh[k], childMargin);
                    float t      = __fsub_rd(ad, sz[k]);
                    hit          = hit && (t - gh[k] < margin);
                    float dk     = fmaxf(__fsub_rd(t, margin), 0.f);
                    dist2        = __fmaf_rd(dk, dk, dist2);
                }
                hit = hit && dist2 <= gR2;
            }
            if constexpr (SUB)
            {
                // bit 8g + c: sub-group g may reach child c; the lanes of child c are those sub-groups' alive lanes
                const unsigned m32 = __ballot_sync(0xffffffffu, hit);
                cmask              = pmask & (((m32 >> cidx) & 0x01010101u) * 0xFFu);
                ok                 = lane < 8 && cmask != 0;
            }
            else { ok = hit; }
        }
        else
        {
            bool alive = (pmask >> lane) & 1u;
#pragma unroll 1
            for (int c = 0; c < 8; ++c)
            {
                const float4* r = prep.nrec + 3 * size_t(c0 + c);
                float4 rA = r[0], rB = r[1], rC = r[2];
                float cc[3], sz[3];
                frameOf(rA, rB, rC, cc, sz);
                unsigned m = __ballot_sync(0xffffffffu, alive && mayHitBox(cc, sz));
                if (lane == c)
                {
                    cmask   = m;
                    ok      = m != 0;
                    childC0 = __float_as_int(rA.w);
                }
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, ok);
        __syncwarp();
        if (top + 8 > NBG_STACK)
        {
            if (lane == 0 && a.errWord) atomicOr(a.errWord, 4u);
            break;
        }
        // accepted children, highest index deepest in the stack, so the lowest is popped first
        if (ok)
        {
            int pos        = top + __popc(m >> (lane + 1));
            stack[pos] = make_int2(entryCode(c0 + lane, childC0), int(cmask));
        }
        top += __popc(m);
        __syncwarp();
    }
    if (!a.numSets || passSet >= lastSet) break;
    } // passes
    if (active && s == 0) a.nc[i - a.first] = nc;
    if constexpr (Stats)
    {
        {
            unsigned long long x = stPathWalks;
            for (int o = 16; o > 0; o >>= 1)
                x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) atomicAdd(a.stats + 31, x);
        }
        unsigned long long v[5] = {stPair, stExact, stLeaves, stCand, stNodes};
#pragma unroll
        for (int k = 0; k < 5; ++k)
        {
            unsigned long long x = v[k];
            if (k >= 2) x = lane == 0 ? x : 0;
            for (int o = 16; o > 0; o >>= 1)
                x += __shfl_xor_sync(0xffffffffu, x, o);
            // same slots as findNeighborsKernel: [2] pair tests, [3] exact, [4] leaves, [5] candidates, [6] nodes
            if (lane == 0) atomicAdd(a.stats + 2 + k, x);
        }
        if (lane == 0)
        {
            atomicAdd(a.stats + 20, stSteps);
            atomicAdd(a.stats + 21, stNeed);
            atomicAdd(a.stats + 22, stMinCost);
            atomicAdd(a.stats + 23, stBatches);
            atomicAdd(a.stats + 24, stCandCyc);
            atomicAdd(a.stats + 25, (unsigned long long)(clock64() - t0));
            atomicAdd(a.stats + 26, stLeafCyc);
            atomicAdd(a.stats + 27, stLeafIdle);
            atomicAdd(a.stats + 28, stOutMax);
            atomicAdd(a.stats + 29, stOutLanes);
            atomicAdd(a.stats + 30, stOutRounds);
            atomicAdd(a.stats + 7, 1ull);
            // slowest warp: [8] cycles, [9] its expansions, [10] leaves, [11] candidates, [12] loose flag,
            // [13] its first target; [14] number of loose warps
            unsigned long long cyc = (unsigned long long)(clock64() - t0);
            if (atomicMax(a.stats + 8, cyc) < cyc)
            {
                a.stats[9]  = stNodes;
                a.stats[10] = stLeaves;
                a.stats[11] = stCand;
                a.stats[12] = loose;
                a.stats[13] = base0;
                a.stats[15] = __float_as_uint(rmax);
                a.stats[16] = __float_as_uint(__fsqrt_ru(gR2));
                a.stats[17] = __float_as_uint(fmaxf(gh[0], fmaxf(gh[1], gh[2])));
                a.stats[18] = __float_as_uint(rminW);
                a.stats[19] = __float_as_uint(C);
            }
            if (loose) atomicAdd(a.stats + 14, 1ull);
        }
    }
}

// float shadows of the FP64 particle coordinates and node boxes, and the magnitude bound C
__global__ void prepParticlesKernel(const double* __restrict__ x, const double* __restrict__ y,
                                    const double* __restrict__ z, size_t n, float4* __restrict__ phi,
                                    float4* __restrict__ plo, float* cmax)
{
    float m = 0.f;
    for (size_t j = size_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += size_t(gridDim.x) * blockDim.x)
    {
        double v[3] = {x[j], y[j], z[j]};
        float h[3], l[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            splitDouble(v[k], h[k], l[k]);
            m = fmaxf(m, fabsf(h[k]));
        }
        phi[j] = make_float4(h[0], h[1], h[2], 0.f);
        plo[j] = make_float4(l[0], l[1], l[2], 0.f);
    }
    m = warpMaxF(m);
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
}

// the child offset and particle range of node i, stored in the w components of its record
__device__ __forceinline__ void nodeLinks(int i, const int32_t* childOffsets, const int32_t* i2l, const uint32_t* layout,
                                          float& w0, float& w1, float& w2)
{
    int c0     = childOffsets[i];
    uint32_t f = 0, e = 0;
    if (c0 == 0)
    {
        int leaf = i2l[i];
        f        = layout[leaf];
        e        = layout[leaf + 1];
    }
    w0 = __int_as_float(c0);
    w1 = __uint_as_float(f);
    w2 = __uint_as_float(e);
}

// the node count from the host, or from a leaf count in device memory (N = L + (L - 1) / 7)
__device__ __forceinline__ int nodeCount(const int* Ldev, int Nhost)
{
    if (!Ldev) return Nhost;
    int L = *Ldev;
    return L + (L - 1) / 7;
}

__global__ void prepNodesKernel(const double* __restrict__ centers, const double* __restrict__ sizes,
                                const int32_t* __restrict__ childOffsets, const int32_t* __restrict__ i2l,
                                const uint32_t* __restrict__ layout, int Nhost, const int* Ldev,
                                float4* __restrict__ nrec, float* cmax)
{
    float m     = 0.f;
    const int N = nodeCount(Ldev, Nhost);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    {
        float h[3], l[3], s[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            splitDouble(centers[3 * size_t(i) + k], h[k], l[k]);
            s[k] = __double2float_rn(sizes[3 * size_t(i) + k]);
            m        = fmaxf(m, fabsf(h[k]) + s[k]);
        }
        float w0, w1, w2;
        nodeLinks(i, childOffsets, i2l, layout, w0, w1, w2);
        nrec[3 * size_t(i)]     = make_float4(h[0], h[1], h[2], w0);
        nrec[3 * size_t(i) + 1] = make_float4(l[0], l[1], l[2], w1);
        nrec[3 * size_t(i) + 2] = make_float4(s[0], s[1], s[2], w2);
    }
    m = warpMaxF(m);
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
}

// records of a float tree (centre, zero low part, size) and the magnitude bound C
__global__ void prepNodesF32Kernel(const float* __restrict__ centers, const float* __restrict__ sizes,
                                   const int32_t* __restrict__ childOffsets, const int32_t* __restrict__ i2l,
                                   const uint32_t* __restrict__ layout, int Nhost, const int* Ldev,
                                   float4* __restrict__ nrec, float* cmax)
{
    float m     = 0.f;
    const int N = nodeCount(Ldev, Nhost);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    {
        float c[3], s[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            c[k] = centers[3 * size_t(i) + k];
            s[k] = sizes[3 * size_t(i) + k];
            m    = fmaxf(m, fabsf(c[k]) + s[k]);
        }
        float w0, w1, w2;
        nodeLinks(i, childOffsets, i2l, layout, w0, w1, w2);
        nrec[3 * size_t(i)]     = make_float4(c[0], c[1], c[2], w0);
        nrec[3 * size_t(i) + 1] = make_float4(0.f, 0.f, 0.f, w1);
        nrec[3 * size_t(i) + 2] = make_float4(s[0], s[1], s[2], w2);
    }
    m = warpMaxF(m);
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
}

// eight lanes per node (four nodes per warp; leaves hold about 8 to 30 particles): the particles of a leaf that lie
// outside its box (the exact test in T, as the reference's node boxes are T values), and a marker in the leaf's record
// (child offset -1) when it holds any. For T = double most particles are decided in FP32 on the float shadows: with
// u = 2^-24 the FP32 value of |x - c| - s is within 4 u (|x| + |c| + s) of the exact one, so a value below
// -8 u (|hi| + |c_hi| + s_f) proves the particle inside.
constexpr int MARK_LANES = 8;

template<class T>
__global__ void markOutsideKernel(const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z,
                                  const float4* __restrict__ phi, const T* __restrict__ centers,
                                  const T* __restrict__ sizes, int Nhost, const int* Ldev, float4* __restrict__ nrec,
                                  uint8_t* __restrict__ pout)
{
    const size_t gtid = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int sub = int(gtid % MARK_LANES), lane = threadIdx.x & 31;
    const unsigned segMask = 0xFFu << (lane & ~(MARK_LANES - 1));
    const long long node   = (long long)(gtid / MARK_LANES);
    // whole warps leave together past the last node; the others keep every lane for the segment votes
    const int N = nodeCount(Ldev, Nhost);
    if (__all_sync(0xffffffffu, node >= N)) return;
    bool leaf      = false;
    uint32_t first = 0, last = 0;
    float4 ch = make_float4(0.f, 0.f, 0.f, 0.f), sz = ch;
    if (node < N)
    {
        // the node's record: float box, child offset, particle range (one load round)
        ch = nrec[3 * size_t(node)];
        const float4 cl = nrec[3 * size_t(node) + 1];
        sz              = nrec[3 * size_t(node) + 2];
        leaf            = __float_as_int(ch.w) == 0;
        first           = __float_as_uint(cl.w);
        last            = __float_as_uint(sz.w);
    }
    if (!leaf) first = last = 0;
    bool any = false;
    // rounds over the longest leaf of the warp's four, all eight lanes of a segment voting together
    uint32_t cnt = last - first;
    for (int o = MARK_LANES; o < 32; o <<= 1)
        cnt = max(cnt, __shfl_xor_sync(0xffffffffu, cnt, o));
    for (uint32_t j0 = 0; j0 < cnt; j0 += MARK_LANES)
    {
        const uint32_t j = first + j0 + uint32_t(sub);
        bool o           = false;
        if (j < last)
        {
            bool inside = false;
            if constexpr (std::is_same_v<T, double>)
            {
                constexpr float U8 = 8.f * 5.9604644775390625e-8f;
                float4 p           = phi[j];
                float P[3] = {p.x, p.y, p.z}, C[3] = {ch.x, ch.y, ch.z}, S[3] = {sz.x, sz.y, sz.z};
                inside = true;
#pragma unroll
                for (int k = 0; k < 3; ++k)
                {
                    float d = __fsub_rn(fabsf(__fsub_rn(P[k], C[k])), S[k]);
                    float E = __fmul_ru(U8, __fadd_ru(__fadd_ru(fabsf(P[k]), fabsf(C[k])), S[k]));
                    inside  = inside && d < -E;
                }
            }
            if (!inside)
            {
                const T* c = centers + 3 * size_t(node);
                const T* s = sizes + 3 * size_t(node);
                o = RN<T>::abs_(RN<T>::sub(x[j], c[0])) > s[0] || RN<T>::abs_(RN<T>::sub(y[j], c[1])) > s[1] ||
                    RN<T>::abs_(RN<T>::sub(z[j], c[2])) > s[2];
            }
            pout[j] = o ? 1 : 0;
        }
        any |= (__ballot_sync(0xffffffffu, o) & segMask) != 0u;
    }
    if (any && sub == 0) nrec[3 * size_t(node)].w = __int_as_float(-1);
}

template<class T>
int nbMarkOutside(cudaStream_t s, const T* x, const T* y, const T* z, const float4* phi, const T* centers,
                  const T* sizes, const int32_t* childOffsets, const int32_t* i2l, const uint32_t* layout,
                  int numNodes, const NbPrep& prep, uint8_t* pout, const int* Ldev)
{
    if (numNodes <= 0) return CS_OK;
    if (std::is_same_v<T, double> && !phi)
    {
        setLastError("find neighbors: the outside marks of FP64 particles need the float shadows");
        return CS_ERR_INVALID;
    }
    markOutsideKernel<T><<<iceil(size_t(numNodes) * MARK_LANES, 256), 256, 0, s>>>(
        x, y, z, phi, centers, sizes, numNodes, Ldev, const_cast<float4*>(prep.nrec), pout);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int nbMarkOutside<float>(cudaStream_t, const float*, const float*, const float*, const float4*,
                                  const float*, const float*, const int32_t*, const int32_t*, const uint32_t*, int,
                                  const NbPrep&, uint8_t*, const int*);
template int nbMarkOutside<double>(cudaStream_t, const double*, const double*, const double*, const float4*,
                                   const double*, const double*, const int32_t*, const int32_t*, const uint32_t*, int,
                                   const NbPrep&, uint8_t*, const int*);

size_t nbPrepBytes(size_t n, int numNodes)
{
    Arena ar;
    ar.take<float4>(n);
    ar.take<float4>(n);
    ar.take<float4>(3 * size_t(numNodes));
    ar.take<float>(1);
    ar.take<uint8_t>(n);
    return ar.size + 256;
}

template<class T>
int nbPrepare(cudaStream_t s, const T* x, const T* y, const T* z, size_t n, const T* centers, const T* sizes,
              const int32_t* childOffsets, const int32_t* i2l, const uint32_t* layout, int numNodes, void* ws,
              size_t wsBytes, NbPrep* prep)
{
    constexpr bool F64 = std::is_same_v<T, double>;
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    float4* phi  = ar.take<float4>(F64 ? n : 0);
    float4* plo  = ar.take<float4>(F64 ? n : 0);
    float4* nrec  = ar.take<float4>(3 * size_t(numNodes));
    float* cmax   = ar.take<float>(1);
    uint8_t* pout = ar.take<uint8_t>(n);
    if (!ar.ok())
    {
        setLastError("find neighbors: workspace too small");
        return CS_ERR_INVALID;
    }
    CSG_CUDA_TRY(cudaMemsetAsync(cmax, 0, sizeof(float), s));
    unsigned gn = unsigned(std::min<size_t>((size_t(numNodes) + 255) / 256, size_t(smCount()) * 16));
    if constexpr (F64)
    {
        unsigned g = unsigned(std::min<size_t>((n + 255) / 256, size_t(smCount()) * 16));
        if (n) prepParticlesKernel<<<g, 256, 0, s>>>(x, y, z, n, phi, plo, cmax);
        CSG_CHECK_LAUNCH();
        if (numNodes)
            prepNodesKernel<<<gn, 256, 0, s>>>(centers, sizes, childOffsets, i2l, layout, numNodes, nullptr, nrec,
                                               cmax);
    }
    else
    {
        if (numNodes)
            prepNodesF32Kernel<<<gn, 256, 0, s>>>(centers, sizes, childOffsets, i2l, layout, numNodes, nullptr, nrec,
                                                  cmax);
    }
    CSG_CHECK_LAUNCH();
    *prep  = NbPrep{phi, plo, nrec, cmax, pout};
    int rc = nbMarkOutside<T>(s, x, y, z, F64 ? phi : nullptr, centers, sizes, childOffsets, i2l, layout, numNodes,
                              *prep, pout);
    return rc;
}

template<class T>
int nbPrepareNodes(cudaStream_t s, const T* centers, const T* sizes, const int32_t* childOffsets,
                   const int32_t* i2l, const uint32_t* layout, int numNodes, void* ws, size_t wsBytes, NbPrep* prep,
                   const int* Ldev)
{
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    ar.take<float4>(0);
    ar.take<float4>(0);
    float4* nrec = ar.take<float4>(3 * size_t(numNodes));
    if (!ar.ok() || !prep->cmax)
    {
        setLastError("find neighbors: node workspace too small or no bound");
        return CS_ERR_INVALID;
    }
    float* cmax = const_cast<float*>(prep->cmax);
    unsigned gn = unsigned(std::min<size_t>((size_t(numNodes) + 255) / 256, size_t(smCount()) * 16));
    if (numNodes)
    {
        if constexpr (std::is_same_v<T, double>)
            prepNodesKernel<<<gn, 256, 0, s>>>(centers, sizes, childOffsets, i2l, layout, numNodes, Ldev, nrec, cmax);
        else
            prepNodesF32Kernel<<<gn, 256, 0, s>>>(centers, sizes, childOffsets, i2l, layout, numNodes, Ldev, nrec,
                                                  cmax);
        CSG_CHECK_LAUNCH();
    }
    prep->nrec = nrec;
    return CS_OK;
}

template int nbPrepareNodes<float>(cudaStream_t, const float*, const float*, const int32_t*, const int32_t*,
                                   const uint32_t*, int, void*, size_t, NbPrep*, const int*);
template int nbPrepareNodes<double>(cudaStream_t, const double*, const double*, const int32_t*, const int32_t*,
                                    const uint32_t*, int, void*, size_t, NbPrep*, const int*);

template int nbPrepare<float>(cudaStream_t, const float*, const float*, const float*, size_t, const float*,
                              const float*, const int32_t*, const int32_t*, const uint32_t*, int, void*, size_t,
                              NbPrep*);
template int nbPrepare<double>(cudaStream_t, const double*, const double*, const double*, size_t, const double*,
                               const double*, const int32_t*, const int32_t*, const uint32_t*, int, void*, size_t,
                               NbPrep*);

// The smallest shared-memory carveout that keeps NBG_MIN_BLOCKS blocks of the kernel resident (1 KB per block is
// reserved by the runtime), so that the rest of the unified L1 / shared storage caches node records and candidates.
// Set once per kernel.
template<auto Kernel>
static void preferL1()
{
    static const bool done = [] {
        cudaFuncAttributes fa{};
        int dev = 0, smemSM = 0;
        if (cudaFuncGetAttributes(&fa, Kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            smemSM <= 0)
        {
            (void)cudaGetLastError();
            return false;
        }
        const size_t need = size_t(NBG_MIN_BLOCKS) * (fa.sharedSizeBytes + 1024);
        const int pct     = int(std::min<size_t>(100, (need * 100 + size_t(smemSM) - 1) / size_t(smemSM) + 1));
        if (cudaFuncSetAttribute(Kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct) != cudaSuccess)
            (void)cudaGetLastError();
        return true;
    }();
    (void)done;
}

template<class T, bool Stats, int G>
static void launchGroup(unsigned gblk, cudaStream_t s, const NbArgs<T>& a, const NbPrep& prep)
{
    preferL1<findNeighborsGroupKernel<T, Stats, G>>();
    findNeighborsGroupKernel<T, Stats, G><<<gblk, NB_THREADS, 0, s>>>(a, prep);
}

template<class T>
int findNeighbors(cudaStream_t s, const NbArgs<T>& a0, const NbPrep& prep)
{
    if (a0.last <= a0.first) return CS_OK;
    size_t warps  = (size_t(a0.last - a0.first) + 31) / 32;
    size_t blocks = (warps + NB_WARPS - 1) / NB_WARPS;
    NbArgs<T> a   = a0;
    a.pathOnlyPbcWarps = 0;
    int G = a.groupSize == 8 || a.groupSize == 16 || a.groupSize == 32 ? a.groupSize : 32;
    size_t gwarps  = (size_t(a.last - a.first) + G - 1) / G;
    unsigned gblk  = unsigned((gwarps + NB_WARPS - 1) / NB_WARPS);
    if (G == 8)
    {
        if (a.stats) launchGroup<T, true, 8>(gblk, s, a, prep);
        else launchGroup<T, false, 8>(gblk, s, a, prep);
    }
    else if (G == 16)
    {
        if (a.stats) launchGroup<T, true, 16>(gblk, s, a, prep);
        else launchGroup<T, false, 16>(gblk, s, a, prep);
    }
    else
    {
        if (a.stats) launchGroup<T, true, 32>(gblk, s, a, prep);
        else launchGroup<T, false, 32>(gblk, s, a, prep);
    }
    CSG_CHECK_LAUNCH();
    if (a.anyPbc)
    {
        // warps with a particle whose search sphere crosses a periodic boundary: per-lane path traversal
        a.pathOnlyPbcWarps = 1;
        if (a.stats) findNeighborsKernel<T, true><<<unsigned(blocks), NB_THREADS, 0, s>>>(a, prep);
        else findNeighborsKernel<T, false><<<unsigned(blocks), NB_THREADS, 0, s>>>(a, prep);
        CSG_CHECK_LAUNCH();
    }
    return CS_OK;
}

template<class T>
NbArgs<T> makeNbArgs(const T* x, const T* y, const T* z, const T* h, uint32_t first, uint32_t last,
                     const cs_box& box, const cs_ns_view& v, unsigned ngmax, uint32_t* nb, uint32_t* nc)
{
    NbArgs<T> a;
    a.x            = x;
    a.y            = y;
    a.z            = z;
    a.h            = h;
    a.first        = first;
    a.last         = last;
    a.b            = makeBoxParams<T>(box);
    a.anyPbc       = a.b.pbc[0] || a.b.pbc[1] || a.b.pbc[2];
    a.childOffsets = v.child_offsets;
    a.parents      = v.parents;
    a.i2l          = v.internal_to_leaf;
    a.layout       = v.layout;
    a.centers      = static_cast<const T*>(v.centers);
    a.sizes        = static_cast<const T*>(v.sizes);
    a.ext          = v.search_ext_factor;
    a.ngmax        = ngmax;
    a.nb           = nb;
    a.nc           = nc;
    return a;
}

template<class T>
int findNeighborsEntry(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, uint32_t first, uint32_t last,
                       const cs_box& box, const cs_ns_view& v, unsigned ngmax, uint32_t* nb, uint32_t* nc,
                       const float* hf = nullptr)
{
    if (last < first || (last > first && (!x || !y || !z || (!h && !hf) || !nc || (ngmax && !nb) || !v.child_offsets ||
                                          !v.parents || !v.internal_to_leaf || !v.layout || !v.centers || !v.sizes)))
    {
        setLastError("find neighbors: invalid arguments");
        return CS_ERR_INVALID;
    }
    if (last == first) return CS_OK;
    NbArgs<T> a = makeNbArgs<T>(x, y, z, h, first, last, box, v, ngmax, nb, nc);
    a.hf        = hf;
    // the float shadows and the outside flags cover every particle a leaf can reference: [0, layout[L])
    uint32_t nAll = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&nAll, v.layout + v.num_leaf_nodes, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    Workspace w;
    size_t need = nbPrepBytes(nAll, v.num_nodes);
    int rc      = w.acquire(nullptr, 0, need, s);
    if (rc) return rc;
    NbPrep prep;
    rc = nbPrepare<T>(s, x, y, z, nAll, a.centers, a.sizes, v.child_offsets, v.internal_to_leaf, v.layout, v.num_nodes,
                      w.ptr, need, &prep);
    if (rc) return rc;
    return findNeighbors<T>(s, a, prep);
}

template int findNeighbors<float>(cudaStream_t, const NbArgs<float>&, const NbPrep&);
template int findNeighbors<double>(cudaStream_t, const NbArgs<double>&, const NbPrep&);
template NbArgs<float> makeNbArgs<float>(const float*, const float*, const float*, const float*, uint32_t, uint32_t,
                                         const cs_box&, const cs_ns_view&, unsigned, uint32_t*, uint32_t*);
template NbArgs<double> makeNbArgs<double>(const double*, const double*, const double*, const double*, uint32_t,
                                           uint32_t, const cs_box&, const cs_ns_view&, unsigned, uint32_t*, uint32_t*);

} // namespace csg

using namespace csg;

extern "C" int cs_find_neighbors_f32(cs_stream_t stream, const float* x, const float* y, const float* z,
                                     const float* h, uint32_t first, uint32_t last, const cs_box* box,
                                     const cs_ns_view* tree, unsigned ngmax, uint32_t* neighbors, uint32_t* counts)
{
    if (!box || !tree)
    {
        setLastError("find neighbors: null box or tree");
        return CS_ERR_INVALID;
    }
    return findNeighborsEntry<float>(cudaStream_t(stream), x, y, z, h, first, last, *box, *tree, ngmax, neighbors,
                                     counts);
}
extern "C" int cs_find_neighbors_f64(cs_stream_t stream, const double* x, const double* y, const double* z,
                                     const double* h, uint32_t first, uint32_t last, const cs_box* box,
                                     const cs_ns_view* tree, unsigned ngmax, uint32_t* neighbors, uint32_t* counts)
{
    if (!box || !tree)
    {
        setLastError("find neighbors: null box or tree");
        return CS_ERR_INVALID;
    }
    return findNeighborsEntry<double>(cudaStream_t(stream), x, y, z, h, first, last, *box, *tree, ngmax, neighbors,
                                      counts);
}

extern "C" int cs_find_neighbors_f64_hf32(cs_stream_t stream, const double* x, const double* y, const double* z,
                                          const float* h, uint32_t first, uint32_t last, const cs_box* box,
                                          const cs_ns_view* tree, unsigned ngmax, uint32_t* neighbors,
                                          uint32_t* counts)
{
    if (!box || !tree || (last > first && !h))
    {
        setLastError("find neighbors: null box, tree or h");
        return CS_ERR_INVALID;
    }
    return findNeighborsEntry<double>(cudaStream_t(stream), x, y, z, nullptr, first, last, *box, *tree, ngmax,
                                      neighbors, counts, h);
}
