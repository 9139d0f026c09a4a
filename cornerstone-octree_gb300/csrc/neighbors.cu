// Neighbour search with the CPU reference's exact semantics (findneighbors.hpp:33-177).
//
// One warp serves 32 consecutive (SFC-ordered) target particles. The warp walks the tree once, depth first in the
// reference's stackless order (childOffsets/parents, traversal/traversal.hpp:26-69), and keeps one 32-bit mask per
// depth: the lanes whose own root-to-node path passed the reference's pruning test
// |minDistance(x_i, node)|^2 < (2 h_i)^2 ext^2. A node is entered when any lane's path is alive; a lane tests a
// leaf's particles only if its path reached that leaf. Leaves are visited in SFC order, so each lane meets its
// candidates in ascending j: the first ngmax stored neighbours are the reference's, and the count is uncapped.
//
// Arithmetic. The reference decides every test in the coordinate precision T without FMA. For T = float this kernel
// evaluates the same expressions with round-to-nearest intrinsics. For T = double (GB300 has little FP64 throughput)
// each test is first evaluated in FP32 on coordinates relative to a per-warp reference point P, with a proven bound
// on the difference to the FP64 result:
//   candidate  a_j = fl((xhi_j - P) + xlo_j)  (x = xhi + xlo, two floats),  target b_i = fl(x_i - P)
//   per axis   |fl(a_j - b_i) - fl64(x_j - x_i)| <= 3 eps |dx| + A,   A = 4 eps R + 4 eps^2 C,   eps = 2^-24
//              (R bounds |x_i - P| over the warp's targets, C bounds |x| over all particles)
//   distance   |d2_f - d2_64| <= 9.2 eps d2 + 3.5 A sqrt(d2) + 6 A^2
// so d2_f < T_in proves d2_64 < r2 and d2_f >= T_out proves d2_64 >= r2 with
//   T_in = r2 (1 - 24 eps) - 8 A r - 32 A^2,   T_out = r2 (1 + 24 eps) + 8 A r + 32 A^2.
// The cell test uses the analogous bound E = 16 eps sum G_k^2 + 3 A sum G_k + 4 A^2 with G_k = |c_k - x_k| + s_k.
// Only tests that fall inside [T_in, T_out) (or the cell band) are re-evaluated in exact FP64, as are all tests of a
// particle whose search sphere crosses a periodic boundary.
#include "cs_common.cuh"
#include "neighbors.cuh"

#include <algorithm>
#include <type_traits>

namespace csg
{

constexpr int NB_THREADS  = 128;
constexpr int NB_WARPS    = NB_THREADS / 32;
constexpr int NB_MAXDEPTH = 24;
constexpr float EPS32     = 5.9604644775390625e-8f; // 2^-24
constexpr double EPSD     = 5.9604644775390625e-8;

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
    T hi      = a.h[i];
    T r2      = RN<T>::mul(RN<T>::mul(T(4.0), hi), hi);
    T cellR2  = RN<T>::mul(RN<T>::mul(r2, T(a.ext)), T(a.ext));
    bool pbc  = false;
    if (a.anyPbc)
    {
        T twoh      = RN<T>::mul(T(2), hi);
        bool inside = RN<T>::sub(xi, twoh) >= a.b.lo[0] && RN<T>::sub(yi, twoh) >= a.b.lo[1] &&
                      RN<T>::sub(zi, twoh) >= a.b.lo[2] && RN<T>::add(xi, twoh) <= a.b.hi[0] &&
                      RN<T>::add(yi, twoh) <= a.b.hi[1] && RN<T>::add(zi, twoh) <= a.b.hi[2];
        pbc = !inside;
    }

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
                    float4 ch = prep.chi[node], cl = prep.clo[node], sz = prep.sz[node];
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
            h[k] = __double2float_rn(v[k]);
            l[k] = __double2float_rn(__dsub_rn(v[k], double(h[k])));
            m    = fmaxf(m, fabsf(h[k]));
        }
        phi[j] = make_float4(h[0], h[1], h[2], 0.f);
        plo[j] = make_float4(l[0], l[1], l[2], 0.f);
    }
    m = warpMaxF(m);
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
}

__global__ void prepNodesKernel(const double* __restrict__ centers, const double* __restrict__ sizes, int N,
                                float4* __restrict__ chi, float4* __restrict__ clo, float4* __restrict__ sz,
                                float* cmax)
{
    float m = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    {
        float h[3], l[3], s[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            double c = centers[3 * size_t(i) + k];
            h[k]     = __double2float_rn(c);
            l[k]     = __double2float_rn(__dsub_rn(c, double(h[k])));
            s[k]     = __double2float_rn(sizes[3 * size_t(i) + k]);
            m        = fmaxf(m, fabsf(h[k]) + s[k]);
        }
        chi[i] = make_float4(h[0], h[1], h[2], 0.f);
        clo[i] = make_float4(l[0], l[1], l[2], 0.f);
        sz[i]  = make_float4(s[0], s[1], s[2], 0.f);
    }
    m = warpMaxF(m);
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
}

size_t nbPrepBytes(size_t n, int numNodes)
{
    Arena ar;
    ar.take<float4>(n);
    ar.take<float4>(n);
    ar.take<float4>(size_t(numNodes));
    ar.take<float4>(size_t(numNodes));
    ar.take<float4>(size_t(numNodes));
    ar.take<float>(1);
    return ar.size + 256;
}

int nbPrepare(cudaStream_t s, const double* x, const double* y, const double* z, size_t n, const double* centers,
              const double* sizes, int numNodes, void* ws, size_t wsBytes, NbPrep* prep)
{
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    float4* phi = ar.take<float4>(n);
    float4* plo = ar.take<float4>(n);
    float4* chi = ar.take<float4>(size_t(numNodes));
    float4* clo = ar.take<float4>(size_t(numNodes));
    float4* sz  = ar.take<float4>(size_t(numNodes));
    float* cmax = ar.take<float>(1);
    if (!ar.ok())
    {
        setLastError("find neighbors: workspace too small");
        return CS_ERR_INVALID;
    }
    CSG_CUDA_TRY(cudaMemsetAsync(cmax, 0, sizeof(float), s));
    unsigned g = unsigned(std::min<size_t>((n + 255) / 256, size_t(smCount()) * 16));
    if (n) prepParticlesKernel<<<g, 256, 0, s>>>(x, y, z, n, phi, plo, cmax);
    CSG_CHECK_LAUNCH();
    unsigned gn = unsigned(std::min<size_t>((size_t(numNodes) + 255) / 256, size_t(smCount()) * 16));
    if (numNodes) prepNodesKernel<<<gn, 256, 0, s>>>(centers, sizes, numNodes, chi, clo, sz, cmax);
    CSG_CHECK_LAUNCH();
    *prep = NbPrep{phi, plo, chi, clo, sz, cmax};
    return CS_OK;
}

template<class T>
int findNeighbors(cudaStream_t s, const NbArgs<T>& a, const NbPrep& prep)
{
    if (a.last <= a.first) return CS_OK;
    size_t warps  = (size_t(a.last - a.first) + 31) / 32;
    size_t blocks = (warps + NB_WARPS - 1) / NB_WARPS;
    if (a.stats) findNeighborsKernel<T, true><<<unsigned(blocks), NB_THREADS, 0, s>>>(a, prep);
    else findNeighborsKernel<T, false><<<unsigned(blocks), NB_THREADS, 0, s>>>(a, prep);
    CSG_CHECK_LAUNCH();
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
                       const cs_box& box, const cs_ns_view& v, unsigned ngmax, uint32_t* nb, uint32_t* nc)
{
    if (last < first || (last > first && (!x || !y || !z || !h || !nc || (ngmax && !nb) || !v.child_offsets ||
                                          !v.parents || !v.internal_to_leaf || !v.layout || !v.centers || !v.sizes)))
    {
        setLastError("find neighbors: invalid arguments");
        return CS_ERR_INVALID;
    }
    if (last == first) return CS_OK;
    NbArgs<T> a = makeNbArgs<T>(x, y, z, h, first, last, box, v, ngmax, nb, nc);
    if constexpr (std::is_same_v<T, double>)
    {
        // the shadows cover every particle a leaf can reference: [0, layout[L])
        uint32_t nAll = 0;
        CSG_CUDA_TRY(cudaMemcpyAsync(&nAll, v.layout + v.num_leaf_nodes, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        CSG_CUDA_TRY(cudaStreamSynchronize(s));
        Workspace w;
        size_t need = nbPrepBytes(nAll, v.num_nodes);
        int rc      = w.acquire(nullptr, 0, need, s);
        if (rc) return rc;
        NbPrep prep;
        rc = nbPrepare(s, x, y, z, nAll, a.centers, a.sizes, v.num_nodes, w.ptr, need, &prep);
        if (rc) return rc;
        return findNeighbors<T>(s, a, prep);
    }
    else { return findNeighbors<T>(s, a, NbPrep{}); }
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
