// Neighbour-list consumers (the reference's ijLoop neighbourhoods, traversal/ijloop/).
//
// Two ways to loop over neighbours, both evaluated with a fixed interaction here (an SPH density sum, the
// interaction the tests and the benchmark use); the C++ header include/cstone_gb300/ijloop_gb300.cuh runs any
// interaction functor over the same cluster lists.
//
// 1. Over stored neighbour lists (CpuFullNbListNeighborhood::jLoop, traversal/ijloop/cpu_fullnblist.hpp:94-112):
//    one thread per target walks its ngmax-strided row in order. Results equal the CPU full list bit for bit.
//
// 2. Over cluster-pair lists (the role of the reference's supercluster lists, traversal/ijloop/
//    gpu_superclusternblist.cuh and gpu_superclusternblist/{build,loop}.cuh, built differently here). Particles are
//    cut into clusters of 8 consecutive (SFC-ordered) particles. An i-cluster's search box is the union of its
//    particles' 2h boxes, rounded outwards to float and widened by one finest cell (which covers particles that lie
//    slightly outside their leaf's box). A warp walks the octree once for 4 consecutive i-clusters, with the union of
//    their search boxes, and lists for each, in ascending order and without repeats, every j-cluster whose float
//    bounding box meets its own search box; capacity ncmax j-clusters per i-cluster.
//    The loop then runs 4 i-clusters per warp, one target per lane: each j-cluster's 8 particles are loaded by the 8
//    lanes of the segment and broadcast with shuffles, so every target adds its neighbours in ascending j. The list is
//    a superset of the neighbours of every target, so the sum equals the brute-force sum over all j with
//    d2 < (2 h_i)^2, in ascending j, bit for bit. Open boxes only (no periodic images).
//
// Interaction: contribution m_j w(q), q = sqrt(d2) hinv_i, w = (1 - 1.5 q^2) + (0.75 q^2) q for q < 1, else
// 0.25 (2 - q)^3 evaluated as 0.25 ((t t) t); the sum starts with i's own contribution (w(0) = 1, as the reference's
// loops start from interaction(i, i)); rho_i = sum * hinv^3. Round-to-nearest intrinsics, no contraction.
#include "cs_common.cuh"

#include <type_traits>
#include <vector>

namespace csg
{

constexpr int CLUSTER = 8;

template<class T>
__device__ __forceinline__ T sqrtRn(T a)
{
    if constexpr (std::is_same_v<T, double>) return __dsqrt_rn(a);
    else return __fsqrt_rn(a);
}

template<class T>
__device__ __forceinline__ T divRn(T a, T b)
{
    if constexpr (std::is_same_v<T, double>) return __ddiv_rn(a, b);
    else return __fdiv_rn(a, b);
}

template<class T>
__device__ __forceinline__ T densityW(T d2, T hinv)
{
    using R = RN<T>;
    T q  = R::mul(sqrtRn<T>(d2), hinv);
    T q2 = R::mul(q, q);
    if (q < T(1)) return R::add(R::sub(T(1), R::mul(T(1.5), q2)), R::mul(R::mul(T(0.75), q2), q));
    T t = R::sub(T(2), q);
    return R::mul(T(0.25), R::mul(R::mul(t, t), t));
}

template<class T>
__device__ __forceinline__ T foldRn(T d, int pbc, T len, T ilen)
{
    return RN<T>::sub(d, RN<T>::mul(RN<T>::mul(T(pbc), len), RN<T>::rint_(RN<T>::mul(d, ilen))));
}

// ---------------------------------------------------------------------------------------------------------------
// 1. stored neighbour lists
// ---------------------------------------------------------------------------------------------------------------
template<class T>
__global__ void densityListKernel(const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z,
                                  const T* __restrict__ h, const T* __restrict__ m, uint32_t first, uint32_t last,
                                  BoxParams<T> b, int anyPbc, const uint32_t* __restrict__ nb,
                                  const uint32_t* __restrict__ nc, unsigned ngmax, T* __restrict__ rho)
{
    using R          = RN<T>;
    const uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= last) return;
    const T xi = x[i], yi = y[i], zi = z[i], hi = h[i];
    const T hinv = divRn<T>(T(1), hi);
    const T r2   = R::mul(R::mul(T(4), hi), hi);
    bool pbc     = false;
    if (anyPbc)
    {
        T r2h       = R::mul(T(2), hi);
        bool inside = R::sub(xi, r2h) >= b.lo[0] && R::sub(yi, r2h) >= b.lo[1] && R::sub(zi, r2h) >= b.lo[2] &&
                      R::add(xi, r2h) <= b.hi[0] && R::add(yi, r2h) <= b.hi[1] && R::add(zi, r2h) <= b.hi[2];
        pbc = !inside;
    }
    T sum              = R::mul(m[i], densityW<T>(T(0), hinv));
    const unsigned cnt = min(nc[i - first], ngmax);
    const uint32_t* row = nb + size_t(i - first) * ngmax;
    for (unsigned k = 0; k < cnt; ++k)
    {
        uint32_t j = __ldg(row + k);
        T dx = R::sub(xi, __ldg(x + j)), dy = R::sub(yi, __ldg(y + j)), dz = R::sub(zi, __ldg(z + j));
        if (pbc)
        {
            dx = foldRn<T>(dx, b.pbc[0], b.len[0], b.ilen[0]);
            dy = foldRn<T>(dy, b.pbc[1], b.len[1], b.ilen[1]);
            dz = foldRn<T>(dz, b.pbc[2], b.len[2], b.ilen[2]);
        }
        T d2 = R::add(R::add(R::mul(dx, dx), R::mul(dy, dy)), R::mul(dz, dz));
        if (d2 < r2) sum = R::add(sum, R::mul(__ldg(m + j), densityW<T>(d2, hinv)));
    }
    rho[i - first] = R::mul(sum, R::mul(R::mul(hinv, hinv), hinv));
}

// ---------------------------------------------------------------------------------------------------------------
// 2. cluster-pair lists
// ---------------------------------------------------------------------------------------------------------------
template<class T>
__device__ __forceinline__ float toFloatRd(T v)
{
    if constexpr (std::is_same_v<T, double>) return __double2float_rd(v);
    else return v;
}
template<class T>
__device__ __forceinline__ float toFloatRu(T v)
{
    if constexpr (std::is_same_v<T, double>) return __double2float_ru(v);
    else return v;
}

// float bounding box (rounded outwards) of each cluster of 8 consecutive particles: lo xyz, hi xyz
template<class T>
__global__ void jClusterBoxKernel(const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z, size_t n,
                                  size_t numClusters, float4* __restrict__ boxes)
{
    size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= numClusters) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t j = c * CLUSTER; j < min(n, c * CLUSTER + CLUSTER); ++j)
    {
        T p[3] = {x[j], y[j], z[j]};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = fminf(lo[k], toFloatRd<T>(p[k]));
            hi[k] = fmaxf(hi[k], toFloatRu<T>(p[k]));
        }
    }
    boxes[2 * c]     = make_float4(lo[0], lo[1], lo[2], 0.f);
    boxes[2 * c + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
}

constexpr int CB_WARPS = 4;
constexpr int CB_GROUP = 4; // i-clusters per warp
constexpr int CB_STACK = 192;

template<class T>
struct ClusterBuildArgs
{
    const T *x, *y, *z, *h;
    size_t n, numIClusters;
    const int32_t* childOffsets;
    const int32_t* internalToLeaf;
    const uint32_t* layout;
    const T *centers, *sizes;
    const float4* jBoxes;
    float margin[3];
    unsigned ncmax;
    uint32_t* lists;
    uint32_t* counts;
    uint32_t* err; // bit 0: a list overflowed ncmax; bit 1: traversal stack overflow
};

// One warp builds the lists of CB_GROUP consecutive i-clusters (lane 8 g + k holds particle k of i-cluster g): one
// tree walk with the union of their search boxes, and at each reached leaf every j-cluster box tested against each
// i-cluster's own box.
template<class T>
__global__ void __launch_bounds__(CB_WARPS * 32) clusterBuildKernel(ClusterBuildArgs<T> a)
{
    __shared__ int sStack[CB_WARPS][CB_STACK];
    const int lane   = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t ic0 = (size_t(blockIdx.x) * CB_WARPS + warp) * CB_GROUP;
    if (ic0 >= a.numIClusters) return;

    // each i-cluster's search box: union over its particles of [x - 2h, x + 2h], rounded outwards, plus the margin
    float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const size_t i = ic0 * CLUSTER + lane;
    if (i < a.n)
    {
        T p[3]  = {a.x[i], a.y[i], a.z[i]};
        float r = toFloatRu<T>(RN<T>::mul(T(2), a.h[i]));
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            blo[k] = __fsub_rd(toFloatRd<T>(p[k]), r);
            bhi[k] = __fadd_ru(toFloatRu<T>(p[k]), r);
        }
    }
    float glo[CB_GROUP][3], ghi[CB_GROUP][3], ulo[3], uhi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        for (int o = CLUSTER / 2; o > 0; o >>= 1)
        {
            blo[k] = fminf(blo[k], __shfl_xor_sync(0xffffffffu, blo[k], o));
            bhi[k] = fmaxf(bhi[k], __shfl_xor_sync(0xffffffffu, bhi[k], o));
        }
        blo[k] = __fsub_rd(blo[k], a.margin[k]);
        bhi[k] = __fadd_ru(bhi[k], a.margin[k]);
        ulo[k] = INFINITY, uhi[k] = -INFINITY;
#pragma unroll
        for (int g = 0; g < CB_GROUP; ++g)
        {
            glo[g][k] = __shfl_sync(0xffffffffu, blo[k], g * CLUSTER);
            ghi[g][k] = __shfl_sync(0xffffffffu, bhi[k], g * CLUSTER);
            ulo[k]    = fminf(ulo[k], glo[g][k]);
            uhi[k]    = fmaxf(uhi[k], ghi[g][k]);
        }
    }

    auto nodeMeets = [&](int node) {
        bool meet = true;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            T c      = a.centers[3 * size_t(node) + k];
            T sz     = a.sizes[3 * size_t(node) + k];
            float lo = __fsub_rd(__fsub_rd(toFloatRd<T>(c), toFloatRu<T>(sz)), a.margin[k]);
            float hi = __fadd_ru(__fadd_ru(toFloatRu<T>(c), toFloatRu<T>(sz)), a.margin[k]);
            meet     = meet && lo <= uhi[k] && ulo[k] <= hi;
        }
        return meet;
    };

    unsigned count[CB_GROUP] = {};
    long long lastJ[CB_GROUP];
#pragma unroll
    for (int g = 0; g < CB_GROUP; ++g)
        lastJ[g] = -1;
    int* stack = sStack[warp];
    int top    = 0;
    if (nodeMeets(0))
    {
        if (lane == 0) stack[0] = 0;
        top = 1;
    }
    __syncwarp();
    while (top > 0)
    {
        const int node = stack[top - 1];
        --top;
        const int c0 = a.childOffsets[node];
        if (c0 == 0)
        {
            // a leaf: its particles' j-clusters, tested 32 at a time, appended in ascending order without repeats
            const int leaf    = a.internalToLeaf[node];
            const uint32_t pf = a.layout[leaf], pl = a.layout[leaf + 1];
            if (pl > pf)
            {
                const long long J0 = pf / CLUSTER, J1 = (pl - 1) / CLUSTER;
                for (long long Jb = J0; Jb <= J1; Jb += 32)
                {
                    const long long J = Jb + lane;
                    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY,
                                                                                                -INFINITY, 0.f);
                    if (J <= J1) lo = a.jBoxes[2 * J], hi = a.jBoxes[2 * J + 1];
#pragma unroll
                    for (int g = 0; g < CB_GROUP; ++g)
                    {
                        const bool hit = J != lastJ[g] && lo.x <= ghi[g][0] && glo[g][0] <= hi.x &&
                                         lo.y <= ghi[g][1] && glo[g][1] <= hi.y && lo.z <= ghi[g][2] &&
                                         glo[g][2] <= hi.z;
                        const unsigned m = __ballot_sync(0xffffffffu, hit);
                        if (hit)
                        {
                            const unsigned pos = count[g] + __popc(m & ((1u << lane) - 1u));
                            if (pos < a.ncmax && ic0 + g < a.numIClusters)
                                a.lists[(ic0 + g) * size_t(a.ncmax) + pos] = uint32_t(J);
                        }
                        count[g] += __popc(m);
                        if (m) lastJ[g] = Jb + 31 - __clz(m);
                    }
                }
            }
            continue;
        }
        // an internal node: lanes 0-7 test the children; accepted ones pushed highest first
        bool ok          = lane < 8 && nodeMeets(c0 + lane);
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        __syncwarp();
        if (top + 8 > CB_STACK)
        {
            if (lane == 0) atomicOr(a.err, 2u);
            break;
        }
        if (ok) stack[top + __popc(m >> (lane + 1))] = c0 + lane;
        top += __popc(m);
        __syncwarp();
    }
#pragma unroll
    for (int g = 0; g < CB_GROUP; ++g)
        if (lane == g && ic0 + g < a.numIClusters)
        {
            a.counts[ic0 + g] = count[g];
            if (count[g] > a.ncmax) atomicOr(a.err, 1u);
        }
}

// The cluster loop in two phases per warp (4 i-clusters, one target per lane; each j-cluster's particles are broadcast
// within the lane's 8-lane segment):
//  - screen: every candidate j of the lane's target is tested in FP32; the ones that may lie within 2 h_i go, in
//    ascending j, into the lane's queue in shared memory;
//  - flush (when a queue may not take another j-cluster, and at the end): the queued pairs of all 32 lanes are dealt
//    out 32 at a time, each lane evaluating the exact test and the interaction term of one pair (of any target), so
//    that no lane idles in the expensive arithmetic; then each target adds its own terms in queue order.
// For float coordinates the screen is the exact test itself. For double coordinates it is a proven lower bound:
// with xf = float(x) (round to nearest), a = |float(xi_f - xj_f)| and S = |xi_f| + |xj_f|,
//   |xi - xj| >= a (1 - 2^-24) - 2^-24 S - 2^-149,
// and u = max(fma(-2^-21, a + S, a), 0) stays below that bound after its own roundings. A j is dropped only when
// ux^2 + uy^2 + uz^2 (three float roundings, under 2^-21.4 relative) exceeds float_ru(r2) (1 + 2^-20): then the exact
// d2 exceeds r2 (1 + 2^-22), and the double d2 (five roundings, under 2^-50) still exceeds r2, so the double test
// would have dropped it too. NaN and infinite coordinates give u = 0 (never dropped); a threshold below 2^-100 is
// raised to 2^-100 so that subnormal roundings cannot matter. The sums are those of the one-phase loop, bit for bit.
constexpr int DC_WARPS = 4;
constexpr int DC_QCAP  = 32; // queued candidates per target; a j-cluster adds at most CLUSTER

template<class T>
__device__ __forceinline__ unsigned long long toBits(T v)
{
    if constexpr (std::is_same_v<T, double>) return static_cast<unsigned long long>(__double_as_longlong(v));
    else return __float_as_uint(v);
}
template<class T>
__device__ __forceinline__ T fromBits(unsigned long long b)
{
    if constexpr (std::is_same_v<T, double>) return __longlong_as_double(static_cast<long long>(b));
    else return __uint_as_float(uint32_t(b));
}

template<class T>
__device__ __forceinline__ float toFloatRn(T v)
{
    if constexpr (std::is_same_v<T, double>) return __double2float_rn(v);
    else return v;
}

__device__ __forceinline__ float screenAxis(float fi, float absFi, float fj)
{
    const float a = fabsf(__fsub_rn(fi, fj));
    const float t = __fadd_rn(a, __fadd_rn(absFi, fabsf(fj)));
    return fmaxf(__fmaf_rn(-0x1p-21f, t, a), 0.f);
}

template<class T>
__global__ void __launch_bounds__(DC_WARPS * 32) densityClusterKernel(const T* __restrict__ x, const T* __restrict__ y,
                                                                      const T* __restrict__ z, const T* __restrict__ h,
                                                                      const T* __restrict__ m, size_t n,
                                                                      size_t numIClusters,
                                                                      const uint32_t* __restrict__ lists,
                                                                      const uint32_t* __restrict__ counts,
                                                                      unsigned ncmax, T* __restrict__ rho)
{
    constexpr bool kExactScreen = std::is_same_v<T, float>;
    __shared__ unsigned long long sQueue[DC_WARPS][DC_QCAP][32]; // a queued j, then its term
    using R            = RN<T>;
    const int lane     = threadIdx.x & 31;
    const int warp     = threadIdx.x >> 5;
    const size_t gw    = size_t(blockIdx.x) * DC_WARPS + warp;
    const size_t ic    = gw * 4 + (lane >> 3);
    const int k        = lane & 7;
    const int seg0     = lane & ~7;
    const size_t i     = ic * CLUSTER + k;
    const bool activeI = ic < numIClusters && i < n;
    const size_t iSafe = activeI ? i : 0;
    const T xi = x[iSafe], yi = y[iSafe], zi = z[iSafe], hi = h[iSafe];
    const T hinv = divRn<T>(T(1), hi);
    const T r2   = R::mul(R::mul(T(4), hi), hi);
    T sum        = R::mul(m[iSafe], densityW<T>(T(0), hinv));

    const float fxi = toFloatRn<T>(xi), fyi = toFloatRn<T>(yi), fzi = toFloatRn<T>(zi);
    const float axi = fabsf(fxi), ayi = fabsf(fyi), azi = fabsf(fzi);
    float thr = 0.f;
    if constexpr (!kExactScreen) thr = fmaxf(__fmul_ru(__double2float_ru(r2), 1.f + 0x1p-20f), 0x1p-100f);

    unsigned long long(*queue)[32] = sQueue[warp];
    unsigned qn                    = 0;
    auto flush                     = [&]() {
        // (1) every queued pair's term, the warp's queues taken 32 pairs at a time in lane-major order, so that all
        //     lanes evaluate the expensive part; a term replaces its j in the queue (-0 where d2 >= r2: adding -0
        //     leaves every sum unchanged)
        unsigned incl = qn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
        const unsigned excl  = incl - qn;
        __syncwarp();
        for (unsigned e0 = 0; e0 < total; e0 += 32)
        {
            const unsigned e = e0 + lane;
            // the pair's owner: the last lane whose queue starts at or before e (its queue is not empty)
            int owner = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, excl, owner + step) <= e) owner += step;
            const unsigned slot = e - __shfl_sync(0xffffffffu, excl, owner);
            const T oxi = __shfl_sync(0xffffffffu, xi, owner), oyi = __shfl_sync(0xffffffffu, yi, owner);
            const T ozi = __shfl_sync(0xffffffffu, zi, owner), ohinv = __shfl_sync(0xffffffffu, hinv, owner);
            const T or2 = __shfl_sync(0xffffffffu, r2, owner);
            if (e < total)
            {
                const uint32_t j = uint32_t(queue[slot][owner]);
                T dx = R::sub(oxi, __ldg(x + j)), dy = R::sub(oyi, __ldg(y + j)), dz = R::sub(ozi, __ldg(z + j));
                T d2 = R::add(R::add(R::mul(dx, dx), R::mul(dy, dy)), R::mul(dz, dz));
                T term = d2 < or2 ? R::mul(__ldg(m + j), densityW<T>(d2, ohinv)) : T(-0.0);
                queue[slot][owner] = toBits<T>(term);
            }
        }
        __syncwarp();
        // (2) each target adds its own terms in queue order (ascending j)
        const unsigned qmax = __reduce_max_sync(0xffffffffu, qn);
        for (unsigned k = 0; k < qmax; ++k)
            if (k < qn) sum = R::add(sum, fromBits<T>(queue[k][lane]));
        __syncwarp();
        qn = 0;
    };

    const unsigned cnt    = ic < numIClusters ? min(counts[ic], ncmax) : 0u;
    const unsigned maxCnt = __reduce_max_sync(0xffffffffu, cnt);
    const uint32_t* list  = lists + (ic < numIClusters ? ic : 0) * size_t(ncmax);
    for (unsigned t = 0; t < maxCnt; ++t)
    {
        const bool segOn = t < cnt;
        const size_t J   = segOn ? __ldg(list + t) : 0;
        const size_t jk  = J * CLUSTER + k;
        const bool jOk   = segOn && jk < n;
        const float fxj = jOk ? toFloatRn<T>(x[jk]) : 0.f, fyj = jOk ? toFloatRn<T>(y[jk]) : 0.f;
        const float fzj = jOk ? toFloatRn<T>(z[jk]) : 0.f;
#pragma unroll
        for (int q = 0; q < CLUSTER; ++q)
        {
            const float xq = __shfl_sync(0xffffffffu, fxj, seg0 + q);
            const float yq = __shfl_sync(0xffffffffu, fyj, seg0 + q);
            const float zq = __shfl_sync(0xffffffffu, fzj, seg0 + q);
            const size_t j = J * CLUSTER + q;
            bool cand      = activeI && segOn && j < n && j != i;
            if constexpr (kExactScreen)
            {
                const float dx = __fsub_rn(fxi, xq), dy = __fsub_rn(fyi, yq), dz = __fsub_rn(fzi, zq);
                const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                cand           = cand && d2 < float(r2);
            }
            else
            {
                const float ux = screenAxis(fxi, axi, xq), uy = screenAxis(fyi, ayi, yq);
                const float uz = screenAxis(fzi, azi, zq);
                const float lb = __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux)));
                cand           = cand && !(lb > thr);
            }
            if (cand) queue[qn++][lane] = uint32_t(j);
        }
        if (__reduce_max_sync(0xffffffffu, qn) > DC_QCAP - CLUSTER) flush();
    }
    flush();
    if (activeI) rho[i] = R::mul(sum, R::mul(R::mul(hinv, hinv), hinv));
}

} // namespace csg

using namespace csg;

#define CS_IJLOOP_ENTRIES(SUF, T)                                                                                      \
    extern "C" int cs_ijloop_density_list_##SUF(cs_stream_t stream, const T* x, const T* y, const T* z, const T* h,   \
                                               const T* m, uint32_t first, uint32_t last, const cs_box* box,          \
                                               const uint32_t* neighbors, const uint32_t* neighbor_counts,            \
                                               unsigned ngmax, T* rho)                                                 \
    {                                                                                                                  \
        if (last <= first) return CS_OK;                                                                               \
        if (!x || !y || !z || !h || !m || !box || !rho || (ngmax && (!neighbors || !neighbor_counts)))               \
        {                                                                                                              \
            setLastError("ijloop density (lists): null argument");                                                    \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        BoxParams<T> b = makeBoxParams<T>(*box);                                                                       \
        int anyPbc     = b.pbc[0] | b.pbc[1] | b.pbc[2];                                                               \
        densityListKernel<T><<<iceil(last - first, 256), 256, 0, cudaStream_t(stream)>>>(                             \
            x, y, z, h, m, first, last, b, anyPbc, neighbors, neighbor_counts, ngmax, rho);                            \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }                                                                                                                  \
    extern "C" int cs_cluster_nblist_build_##SUF(cs_stream_t stream, const T* x, const T* y, const T* z, const T* h,  \
                                                size_t n, const cs_ns_view* tree, const cs_box* box, int key_bits,    \
                                                unsigned ncmax, uint32_t* lists, uint32_t* counts, void* workspace,   \
                                                size_t workspace_bytes, int* max_count_host)                          \
    {                                                                                                                  \
        return clusterBuild<T>(cudaStream_t(stream), x, y, z, h, n, tree, box, key_bits, ncmax, lists, counts,        \
                               workspace, workspace_bytes, max_count_host);                                           \
    }                                                                                                                  \
    extern "C" int cs_ijloop_density_clusters_##SUF(cs_stream_t stream, const T* x, const T* y, const T* z,           \
                                                   const T* h, const T* m, size_t n, const uint32_t* lists,           \
                                                   const uint32_t* counts, unsigned ncmax, T* rho)                     \
    {                                                                                                                  \
        if (n == 0) return CS_OK;                                                                                      \
        if (!x || !y || !z || !h || !m || !lists || !counts || !rho || ncmax == 0 || n >= (size_t(1) << 32))          \
        {                                                                                                              \
            setLastError("ijloop density (clusters): invalid argument");                                              \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        size_t nic   = (n + CLUSTER - 1) / CLUSTER;                                                                    \
        size_t warps = (nic + 3) / 4;                                                                                  \
        densityClusterKernel<T><<<iceil(warps, DC_WARPS), DC_WARPS * 32, 0, cudaStream_t(stream)>>>(                  \
            x, y, z, h, m, n, nic, lists, counts, ncmax, rho);                                                         \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }

namespace csg
{
size_t clusterWorkspaceBytes(size_t n) { return ((n + CLUSTER - 1) / CLUSTER) * 2 * sizeof(float4) + 512; }

template<class T>
int clusterBuild(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, size_t n, const cs_ns_view* tree,
                 const cs_box* box, int keyBits, unsigned ncmax, uint32_t* lists, uint32_t* counts, void* ws,
                 size_t wsb, int* maxCountHost)
{
    if (n == 0) return CS_OK;
    if (keyBits != 32 && keyBits != 64)
    {
        setLastError("cluster neighbour lists: key_bits must be 32 or 64");
        return CS_ERR_INVALID;
    }
    if (!x || !y || !z || !h || !tree || !box || !lists || !counts || ncmax == 0 || n >= (size_t(1) << 32) ||
        !tree->child_offsets || !tree->internal_to_leaf || !tree->layout || !tree->centers || !tree->sizes)
    {
        setLastError("cluster neighbour lists: invalid argument");
        return CS_ERR_INVALID;
    }
    if (box->boundary[0] == CS_PERIODIC || box->boundary[1] == CS_PERIODIC || box->boundary[2] == CS_PERIODIC)
    {
        setLastError("cluster neighbour lists: periodic boxes are not supported");
        return CS_ERR_INVALID;
    }
    const size_t nic = (n + CLUSTER - 1) / CLUSTER;
    const size_t need = clusterWorkspaceBytes(n) + 256;
    Workspace w;
    int rc = w.acquire(ws, wsb, need, s);
    if (rc) return rc;
    Arena ar{static_cast<char*>(w.ptr), 0, need};
    float4* jBoxes = ar.take<float4>(2 * nic);
    uint32_t* err  = ar.take<uint32_t>(4);
    CSG_CUDA_TRY(cudaMemsetAsync(err, 0, 4 * sizeof(uint32_t), s));
    jClusterBoxKernel<T><<<iceil(nic, 256), 256, 0, s>>>(x, y, z, n, nic, jBoxes);
    CSG_CHECK_LAUNCH();
    BoxParams<T> bp = makeBoxParams<T>(*box);
    ClusterBuildArgs<T> a{};
    a.x = x, a.y = y, a.z = z, a.h = h, a.n = n, a.numIClusters = nic;
    a.childOffsets   = tree->child_offsets;
    a.internalToLeaf = tree->internal_to_leaf;
    a.layout         = tree->layout;
    a.centers        = static_cast<const T*>(tree->centers);
    a.sizes          = static_cast<const T*>(tree->sizes);
    a.jBoxes         = jBoxes;
    // one finest cell of the keys (box length / 2^maxLevel), rounded up: the slack between a particle and the box of
    // the leaf its key selects
    const int maxLevel = keyBits == 32 ? 10 : 21;
    for (int k = 0; k < 3; ++k)
        a.margin[k] = float(double(bp.len[k]) / double(1ull << maxLevel) * 1.0001);
    a.ncmax  = ncmax;
    a.lists  = lists;
    a.counts = counts;
    a.err    = err;
    clusterBuildKernel<T><<<iceil(nic, CB_WARPS * CB_GROUP), CB_WARPS * 32, 0, s>>>(a);
    CSG_CHECK_LAUNCH();
    uint32_t herr = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr & 2u)
    {
        setLastError("cluster neighbour lists: traversal stack overflow (malformed tree)");
        return CS_ERR_DEVICE;
    }
    if (herr & 1u)
    {
        if (maxCountHost)
        {
            // the largest count, for the caller to size ncmax
            unsigned mx = 0;
            std::vector<uint32_t> hc(nic);
            CSG_CUDA_TRY(cudaMemcpy(hc.data(), counts, nic * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (uint32_t c : hc)
                mx = c > mx ? c : mx;
            *maxCountHost = int(mx);
        }
        setLastError("cluster neighbour lists: an i-cluster needs more than ncmax = %u j-clusters", ncmax);
        return CS_ERR_CAPACITY;
    }
    return CS_OK;
}
} // namespace csg

CS_IJLOOP_ENTRIES(f64, double)
CS_IJLOOP_ENTRIES(f32, float)

extern "C" size_t cs_cluster_nblist_workspace_bytes(size_t n) { return clusterWorkspaceBytes(n) + 256; }
