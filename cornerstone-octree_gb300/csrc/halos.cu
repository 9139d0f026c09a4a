// Halo discovery: per-leaf h-expanded search boxes (focus/source_center.hpp:28-43, focus/source_center_gpu.cu:23-92)
// and the collision traversal that flags every node outside the focus key range that overlaps a focus leaf's search
// box (traversal/collisions.hpp:25-94, traversal/collisions_gpu.cu:23-77, traversal/boxoverlap.hpp:127-291).
//
// Search boxes: 8 lanes per leaf stride over its particles; min/max are exact (taken on order-preserving integer
// images of the values), so any reduction order gives the reference's bits (up to the sign of a zero extremum that
// ties with the other zero). FP64 particles go through an FP32 screen first, and only the particles that can hold an
// extremum are evaluated in FP64 (searchBoxesScreenKernel). Collisions: the containment test per focus leaf, then one
// warp-wide traversal testing 32 nodes at a time for each leaf that needs it, either in the warp that owns 32
// neighbouring leaves (findHalosWarpKernel) or, given a scratch list, by persistent warps over the list of leaves
// that need one (haloNeedKernel, findHalosListKernel); the flagged set equals that of the reference's per-leaf
// singleTraversal (traversal/traversal.hpp:26-69), and every floating-point expression is unfused and in the
// reference's order.
#include "cs_common.cuh"
#include "halos.cuh"

#include <algorithm>
#include <atomic>
#include <type_traits>

namespace csg
{

// order-preserving integer image of a float / double (sign-magnitude to two's complement): min and max of the images
// are those of the values for all non-NaN inputs, with -0 ordered before +0, and they run on the integer pipes
__device__ __forceinline__ long long ordKey(double v)
{
    long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double ordVal(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }
__device__ __forceinline__ int ordKey(float v)
{
    int b = __float_as_int(v);
    return b ^ ((b >> 31) & 0x7fffffff);
}
__device__ __forceinline__ float ordVal(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); }

template<class T, class Th>
__global__ void searchBoxesKernel(const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z,
                                  const Th* __restrict__ h, const uint32_t* __restrict__ layout, int firstLeaf,
                                  int lastLeaf, Th scale, const int32_t* __restrict__ l2i,
                                  const T* __restrict__ nodeCenters, T* __restrict__ sc, T* __restrict__ ss)
{
    using I           = std::conditional_t<std::is_same_v<T, double>, long long, int>;
    constexpr int TPL = 8;
    int gtid          = blockIdx.x * blockDim.x + threadIdx.x;
    int leaf          = firstLeaf + gtid / TPL;
    int sub           = gtid % TPL;
    bool valid        = leaf < lastLeaf;
    I mn[3], mx[3];
    if (valid)
    {
        // the leaf's geometric centre, or (no leaf-to-node map) the caller's initial value in sc, as
        // computeBoundingBoxGpu reads it
        const T* init = l2i ? nodeCenters + 3 * size_t(l2i[leaf]) : sc + 3 * size_t(leaf);
        for (int k = 0; k < 3; ++k)
            mn[k] = mx[k] = ordKey(init[k]);
        uint32_t first = layout[leaf], last = layout[leaf + 1];
        // four particles per lane and round, loaded before any is used (leaves hold about 20 particles)
        constexpr int U = 4;
        for (uint32_t i0 = first + sub; i0 < last; i0 += U * TPL)
        {
            Th ph[U];
            T px[U], py[U], pz[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const uint32_t i = i0 + u * TPL;
                const bool ok    = i < last;
                ph[u]            = ok ? h[i] : Th(0);
                px[u]            = ok ? x[i] : T(0);
                py[u]            = ok ? y[i] : T(0);
                pz[u]            = ok ? z[i] : T(0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
            {
                if (i0 + u * TPL >= last) continue;
                // r = h * scale in the precision of h (computeBoundingBox, focus/source_center.hpp:33)
                T r    = T(RN<Th>::mul(ph[u], scale));
                T p[3] = {px[u], py[u], pz[u]};
#pragma unroll
                for (int k = 0; k < 3; ++k)
                {
                    I lo  = ordKey(RN<T>::sub(p[k], r));
                    I hi  = ordKey(RN<T>::add(p[k], r));
                    mn[k] = lo < mn[k] ? lo : mn[k];
                    mx[k] = mx[k] < hi ? hi : mx[k];
                }
            }
        }
    }
    else
    {
        for (int k = 0; k < 3; ++k)
            mn[k] = mx[k] = 0;
    }
#pragma unroll
    for (int o = 1; o < TPL; o <<= 1)
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            I a   = __shfl_down_sync(0xffffffffu, mn[k], o, TPL);
            I b   = __shfl_down_sync(0xffffffffu, mx[k], o, TPL);
            mn[k] = a < mn[k] ? a : mn[k];
            mx[k] = mx[k] < b ? b : mx[k];
        }
    }
    if (valid && sub == 0)
    {
        for (int k = 0; k < 3; ++k)
        {
            T lo = ordVal(mn[k]), hi = ordVal(mx[k]);
            sc[3 * size_t(leaf) + k] = RN<T>::mul(RN<T>::add(hi, lo), T(0.5));
            ss[3 * size_t(leaf) + k] = RN<T>::mul(RN<T>::sub(hi, lo), T(0.5));
        }
    }
}

// FP32 estimates of one particle for the screened search boxes: pt ~ (x, y, z), rt ~ h * scale. Shadow: pt are the
// coordinates rounded to nearest float (the neighbour search's shadows), else truncEstimate of the doubles. With
// Th = float, rt is the reference's r itself; with Th = double it comes from truncEstimate(h) times the float
// nearest to scale. False if an estimate is outside the range the screen's error bound covers.
template<class Th, bool Shadow>
__device__ __forceinline__ bool sbEstimate(uint32_t i, const double* __restrict__ x, const double* __restrict__ y,
                                           const double* __restrict__ z, const Th* __restrict__ h,
                                           const float4* __restrict__ phi, float scaleF, float pt[3], float& rt)
{
    bool ok;
    if constexpr (Shadow)
    {
        const float4 s = phi[i];
        pt[0] = s.x, pt[1] = s.y, pt[2] = s.z;
        ok    = fabsf(s.x) < 0x1p120f && fabsf(s.y) < 0x1p120f && fabsf(s.z) < 0x1p120f;
    }
    else
    {
        const bool a = truncEstimate(x[i], pt[0]), b = truncEstimate(y[i], pt[1]), c = truncEstimate(z[i], pt[2]);
        ok = a && b && c;
    }
    if constexpr (std::is_same_v<Th, float>)
    {
        rt = __fmul_rn(h[i], scaleF);
        ok = ok && fabsf(rt) < 0x1p120f;
    }
    else
    {
        float ht = 0.f;
        ok = truncEstimate(h[i], ht) && ok;
        rt = __fmul_rn(ht, scaleF);
    }
    return ok;
}

// Search boxes of FP64 particles with an FP32 screen, so that the FP64 pipe (2 lanes per clock and SM) only sees the
// few particles that can hold a leaf's extremum. Per leaf and axis the reference's value is min_i RN(p_i - r_i) (and
// max_i RN(p_i + r_i)), r_i = RN(h_i * scale) in the precision of h, together with the leaf centre it starts from.
// Error bound: with u = 2^-24, pt within 2^-20 |p| (or RN), rt within 19.01 u |rt| + 2^-99 of r (2^-20 from h, u
// from the float scale, u from the product, u from r's own rounding), f = RN32(pt -+ rt) within u (|pt| + |rt|) of
// pt -+ rt and the exact RN64 value within 2^-53 |p -+ r|: |f - v| <= 17.02 u |pt| + 20.02 u |rt| + 2^-98.9, so
// E = 24 u (|pt| + |rt|) + 2^-98 (rounded up) bounds it. Pass 1 takes M = min_i (f_i + E_i) (and the centre's upper
// bound), an upper bound of the true minimum; a particle with f_i - E_i > M cannot reach it. Pass 2 queues every
// other (particle, side) pair, and the queue is evaluated 32 pairs at a time, one per lane, in FP64 with the
// reference's expression, reduced by 64-bit atomics on the order-preserving integer images in shared memory, so the
// result is the same as the exact min/max over all particles. Particles whose estimates fall outside the covered
// range are queued on every side. Eight lanes per leaf, four leaves per warp; the host requires
// 2^-20 <= scale <= 16 so that rt stays finite and the absolute term covers h below 2^-120.
constexpr int SB_WARPS = 8;
constexpr int SB_QCAP  = 256; // a step queues at most 6 x 32 pairs onto fewer than 32
constexpr int SB_KEEP  = 4;   // particles per lane whose estimates pass 1 keeps for pass 2

template<class Th, bool Shadow>
__global__ void __launch_bounds__(32 * SB_WARPS, Shadow ? 6 : 5)
    searchBoxesScreenKernel(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                            const Th* __restrict__ h, const float4* __restrict__ phi,
                            const uint32_t* __restrict__ layout, int firstLeaf, int lastLeaf, Th scale, float scaleF,
                            const int32_t* __restrict__ l2i, const double* __restrict__ nodeCenters,
                            double* __restrict__ sc, double* __restrict__ ss)
{
    constexpr float E24  = 24.f * 5.9604644775390625e-8f;
    constexpr float EABS = 0x1p-98f;
    const float INF      = __int_as_float(0x7f800000);
    __shared__ uint2 sQ[SB_WARPS][SB_QCAP];
    __shared__ long long sMn[SB_WARPS][4][3], sMx[SB_WARPS][4][3];

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 3, sub = lane & 7;
    const long long leaf0 = firstLeaf + (long long)(blockIdx.x * SB_WARPS + w) * 4;
    if (leaf0 >= lastLeaf) return;
    const int leaf   = int(leaf0) + g;
    const bool valid = leaf < lastLeaf;

    uint32_t first = 0, cnt = 0;
    float mlo[3], mhi[3];
    if (valid)
    {
        first = layout[leaf];
        cnt   = layout[leaf + 1] - first;
        // the leaf's geometric centre, or (no leaf-to-node map) the caller's initial value in sc, as
        // computeBoundingBoxGpu reads it; it takes part in the min and max exactly
        const double* init = l2i ? nodeCenters + 3 * size_t(l2i[leaf]) : sc + 3 * size_t(leaf);
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const double c = init[k];
            if (sub == 0) sMn[w][g][k] = sMx[w][g][k] = ordKey(c);
            float ct;
            if (truncEstimate(c, ct))
            {
                mlo[k] = __fadd_ru(__fmaf_ru(0x1p-19f, fabsf(ct), ct), EABS);
                mhi[k] = __fsub_rd(__fmaf_rd(-0x1p-19f, fabsf(ct), ct), EABS);
            }
            else
                mlo[k] = INF, mhi[k] = -INF;
        }
    }
    else
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
            mlo[k] = INF, mhi[k] = -INF;
    }

    // pass 1: upper bound of each minimum, lower bound of each maximum. The first SB_KEEP particles of each lane
    // (SB_KEEP x 8 per leaf, loaded together) keep their estimates in registers for pass 2; the rest of a large leaf
    // is loaded two particles per lane and round, and again in pass 2.
    auto fold = [&](const float (&pt)[3], float rt) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float E = __fmaf_ru(E24, __fadd_ru(fabsf(pt[k]), fabsf(rt)), EABS);
            mlo[k]        = fminf(mlo[k], __fadd_ru(__fsub_rn(pt[k], rt), E));
            mhi[k]        = fmaxf(mhi[k], __fsub_rd(__fadd_rn(pt[k], rt), E));
        }
    };
    float ept[SB_KEEP][3], ert[SB_KEEP];
    bool eok[SB_KEEP];
#pragma unroll
    for (int u = 0; u < SB_KEEP; ++u)
    {
        const uint32_t j = sub + 8u * u;
        eok[u]           = j < cnt && sbEstimate<Th, Shadow>(first + j, x, y, z, h, phi, scaleF, ept[u], ert[u]);
    }
#pragma unroll
    for (int u = 0; u < SB_KEEP; ++u)
        if (eok[u]) fold(ept[u], ert[u]);
    for (uint32_t j = sub + 8u * SB_KEEP; j < cnt; j += 2 * 8)
    {
        float pt[2][3], rt[2];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u)
        {
            const uint32_t jj = j + u * 8;
            ok[u]             = jj < cnt && sbEstimate<Th, Shadow>(first + jj, x, y, z, h, phi, scaleF, pt[u], rt[u]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
            if (ok[u]) fold(pt[u], rt[u]);
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1)
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            mlo[k] = fminf(mlo[k], __shfl_xor_sync(0xffffffffu, mlo[k], o));
            mhi[k] = fmaxf(mhi[k], __shfl_xor_sync(0xffffffffu, mhi[k], o));
        }
    }

    // exact FP64 values of the queued pairs [base, base + count), one per lane
    auto evaluate = [&](int base, int count) {
        if (lane < count)
        {
            const uint2 q    = sQ[w][base + lane];
            const int side   = int(q.y & 7u), gq = int(q.y >> 3);
            const int axis   = side < 3 ? side : side - 3;
            const double* pa = axis == 0 ? x : (axis == 1 ? y : z);
            const double r   = double(RN<Th>::mul(h[q.x], scale));
            const double v   = RN<double>::add(pa[q.x], side < 3 ? -r : r);
            if (side < 3)
                atomicMin(&sMn[w][gq][axis], ordKey(v));
            else
                atomicMax(&sMx[w][gq][axis], ordKey(v));
        }
        __syncwarp();
    };

    // pass 2: queue the (particle, side) pairs the screen cannot rule out (bits 0-2: minima, 3-5: maxima; all six
    // for a particle outside the screen's range); evaluate whenever 32 are queued
    const unsigned below = (1u << lane) - 1u;
    int qn               = 0;
    auto sides           = [&](const float (&pt)[3], float rt) -> unsigned {
        unsigned m = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float E = __fmaf_ru(E24, __fadd_ru(fabsf(pt[k]), fabsf(rt)), EABS);
            if (__fsub_rd(__fsub_rn(pt[k], rt), E) <= mlo[k]) m |= 1u << k;
            if (__fadd_ru(__fadd_rn(pt[k], rt), E) >= mhi[k]) m |= 8u << k;
        }
        return m;
    };
    auto queue = [&](unsigned m, uint32_t i) {
#pragma unroll
        for (int sd = 0; sd < 6; ++sd)
        {
            const bool mine   = (m >> sd) & 1u;
            const unsigned bm = __ballot_sync(0xffffffffu, mine);
            if (mine) sQ[w][qn + __popc(bm & below)] = make_uint2(i, unsigned(g << 3 | sd));
            qn += __popc(bm);
        }
        __syncwarp();
        while (qn >= 32)
        {
            qn -= 32;
            evaluate(qn, 32);
        }
    };
    const uint32_t maxCnt = __reduce_max_sync(0xffffffffu, cnt);
    __syncwarp();
#pragma unroll
    for (int u = 0; u < SB_KEEP; ++u)
    {
        if (8u * u >= maxCnt) break;
        const uint32_t j = sub + 8u * u;
        queue(j < cnt ? (eok[u] ? sides(ept[u], ert[u]) : 63u) : 0u, first + j);
    }
    for (uint32_t j0 = 8u * SB_KEEP; j0 < maxCnt; j0 += 8)
    {
        const uint32_t j = j0 + sub;
        unsigned m       = 0;
        if (j < cnt)
        {
            float pt[3], rt;
            m = sbEstimate<Th, Shadow>(first + j, x, y, z, h, phi, scaleF, pt, rt) ? sides(pt, rt) : 63u;
        }
        queue(m, first + j);
    }
    if (qn > 0) evaluate(0, qn);

    // centre and half size: lanes 0-2 of a group the centres, lanes 3-5 the half sizes (reference order)
    if (valid && sub < 6)
    {
        const int axis  = sub < 3 ? sub : sub - 3;
        const double lo = ordVal(sMn[w][g][axis]), hi = ordVal(sMx[w][g][axis]);
        const double v  = RN<double>::mul(RN<double>::add(hi, sub < 3 ? lo : -lo), 0.5);
        (sub < 3 ? sc : ss)[3 * size_t(leaf) + axis] = v;
    }
}

template<class T, class Th>
int searchBoxes(cudaStream_t s, const T* x, const T* y, const T* z, const Th* h, const uint32_t* layout, int first,
                int last, Th scale, const int32_t* l2i, const T* nodeCenters, T* sc, T* ss, const float4* phi)
{
    if (last <= first) return CS_OK;
    if constexpr (std::is_same_v<T, double>)
    {
        const double sd = double(scale);
        if (sd >= 0x1p-20 && sd <= 16.0)
        {
            const float scaleF = float(sd);
            const unsigned g   = iceil(size_t(last - first), 4 * SB_WARPS);
            if (phi)
                searchBoxesScreenKernel<Th, true><<<g, 32 * SB_WARPS, 0, s>>>(x, y, z, h, phi, layout, first, last,
                                                                              scale, scaleF, l2i, nodeCenters, sc, ss);
            else
                searchBoxesScreenKernel<Th, false><<<g, 32 * SB_WARPS, 0, s>>>(
                    x, y, z, h, nullptr, layout, first, last, scale, scaleF, l2i, nodeCenters, sc, ss);
            CSG_CHECK_LAUNCH();
            return CS_OK;
        }
    }
    size_t threads = size_t(last - first) * 8;
    searchBoxesKernel<T, Th><<<iceil(threads, 256), 256, 0, s>>>(x, y, z, h, layout, first, last, scale, l2i,
                                                                 nodeCenters, sc, ss);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template<class T>
__device__ __forceinline__ T pbcFold(T d, int pbc, T len, T ilen)
{
    // d - pbc * len * rint(d * ilen)   (applyPbc, sfc/box.hpp:178-190)
    return RN<T>::sub(d, RN<T>::mul(RN<T>::mul(T(pbc), len), RN<T>::rint_(RN<T>::mul(d, ilen))));
}

template<class K, class T>
__device__ bool boxContainedIn(K codeStart, K codeEnd, const T* center, const T* size, const BoxParams<T>& b,
                               const KeyParams<T, K>& kp)
{
    T bmin[3], bmax[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        bmin[k] = RN<T>::sub(center[k], size[k]);
        bmax[k] = RN<T>::add(center[k], size[k]);
    }
    T d0 = RN<T>::sub(bmin[0], b.lo[0]), d1 = RN<T>::sub(bmin[1], b.lo[1]), d2 = RN<T>::sub(bmin[2], b.lo[2]);
    T dmin = d0;
    dmin   = dmin < d1 ? dmin : d1;
    dmin   = dmin < d2 ? dmin : d2;
    T e0 = RN<T>::sub(bmax[0], b.hi[0]), e1 = RN<T>::sub(bmax[1], b.hi[1]), e2 = RN<T>::sub(bmax[2], b.hi[2]);
    T dmax = e0;
    dmax   = dmax > e1 ? dmax : e1;
    dmax   = dmax > e2 ? dmax : e2;
    if (dmin < T(0) || dmax > T(0)) return codeStart == 0 && codeEnd == nodeRange<K>(0);

    const T unit = T(1) / T(1 << KeyTraits<K>::maxLevel);
#pragma unroll
    for (int k = 0; k < 3; ++k)
        bmax[k] = RN<T>::add(bmax[k], RN<T>::mul(b.len[k], unit));
    K lo       = sfc3D<T, K>(bmin[0], bmin[1], bmin[2], kp, CS_HILBERT);
    K hi       = sfc3D<T, K>(bmax[0], bmax[1], bmax[2], kp, CS_HILBERT);
    unsigned l = unsigned(commonPrefix<K>(lo, hi)) / 3u;
    K s        = enclosingBoxCode<K>(lo, l);
    K e        = s + nodeRange<K>(l);
    return s >= codeStart && e <= codeEnd;
}

// Warp-cooperative version of the same traversal: a node is tested iff its parent was tested and overlapped, and
// it is flagged iff it overlaps, so the flagged set does not depend on the visiting order. One warp serves 32
// consecutive focus leaves: each lane decides the containment test (FP64 key arithmetic) for its own leaf, then the
// warp traverses for each leaf whose search box leaves the focus, one after the other. Per traversal the warp pops up
// to four groups of eight siblings from a per-warp LIFO stack, tests the 32 nodes in parallel and pushes the child
// group of every overlapping internal node. Popping the newest groups first bounds the stack by 28 groups per level
// (< 21 * 28 + 32 entries).
constexpr int HALO_WARPS = 4;
constexpr int HALO_STACK = 1024;

// The reference's FP64 overlap test |tc - nc| - ns - ts < 0 on every axis (no periodic axis), out of line so that its
// FP64 arithmetic stays off the float pre-filter's path.
__device__ __noinline__ bool haloOverlapF64(double tc0, double tc1, double tc2, double ts0, double ts1, double ts2,
                                            const double* __restrict__ nc, const double* __restrict__ ns, int idx)
{
    double tc[3] = {tc0, tc1, tc2}, ts[3] = {ts0, ts1, ts2};
    bool ov      = true;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        double d = __dsub_rn(fabs(__dsub_rn(tc[k], nc[3 * size_t(idx) + k])), ns[3 * size_t(idx) + k]);
        ov       = ov && (__dsub_rn(d, ts[k]) < 0.0);
    }
    return ov;
}

// FloatFilter (T = double, no periodic axis): each node test is first evaluated in FP32 on the float node records
// of the neighbour search (centre rounded to nearest, half size rounded to nearest) and the float-rounded search box. With S = |tc| + |nc| +
// ns + ts and u = 2^-24 the FP32 value of |tc - nc| - ns - ts is within 4.01 u S of the exact one, and the FP64 value
// within 4 * 2^-53 S, so D_f < -8 u S proves the reference's test passes on that axis and D_f >= 8 u S proves it
// fails; anything in between is decided by haloOverlapF64.
//
// The node test of a traversal on the node's prefix and (FloatFilter) float records, loaded by the caller; flags an
// overlapping node. tcf, tsf: the search box rounded to float.
template<class K, class T, bool FloatFilter>
__device__ __forceinline__ bool haloNodeTest(int idx, K pfx, float4 c4, float4 s4, const T (&tc)[3],
                                             const T (&ts)[3], const float (&tcf)[3], const float (&tsf)[3],
                                             K lowest, K highest, const T* __restrict__ nc, const T* __restrict__ ns,
                                             const BoxParams<T>& b, uint8_t* flags)
{
    constexpr float U8 = 8.f * 5.9604644775390625e-8f;
    K nk1         = decodePlaceholderBit<K>(pfx);
    unsigned plen = decodePrefixLength<K>(pfx);
    K nk2         = nk1 + (K(1) << (3u * KeyTraits<K>::maxLevel - plen));
    bool inside   = !(nk1 < lowest || nk2 > highest);
    if (inside) return false;
    bool ov = true;
    if constexpr (FloatFilter)
    {
        float cc[3] = {c4.x, c4.y, c4.z}, sz[3] = {s4.x, s4.y, s4.z};
        bool sureIn = true, sureOut = false;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            float d = __fsub_rn(__fsub_rn(fabsf(__fsub_rn(tcf[k], cc[k])), sz[k]), tsf[k]);
            float S = __fadd_ru(__fadd_ru(__fadd_ru(fabsf(tcf[k]), fabsf(cc[k])), sz[k]), tsf[k]);
            float E = __fmul_ru(U8, S);
            sureIn  = sureIn && d < -E;
            sureOut = sureOut || d >= E;
        }
        ov = !sureOut && (sureIn || haloOverlapF64(tc[0], tc[1], tc[2], ts[0], ts[1], ts[2], nc, ns, idx));
    }
    else
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            T d = RN<T>::sub(tc[k], nc[3 * size_t(idx) + k]);
            d   = RN<T>::abs_(pbcFold<T>(d, b.pbc[k], b.len[k], b.ilen[k]));
            d   = RN<T>::sub(d, ns[3 * size_t(idx) + k]);
            d   = RN<T>::sub(d, ts[k]);
            ov  = ov && (d < T(0));
        }
    }
    if (ov) flags[idx] = 1;
    return ov;
}

template<class T, bool FloatFilter>
__device__ __forceinline__ void haloRecords(const float4* __restrict__ nrec, int idx, float4& c4, float4& s4)
{
    if constexpr (FloatFilter)
    {
        c4 = nrec[3 * size_t(idx)];
        s4 = nrec[3 * size_t(idx) + 2];
    }
}

//
// One leaf's traversal by the whole warp (tc, ts: its search box, the same in every lane): per step the warp pops up
// to four groups of eight siblings from the per-warp LIFO stack, tests the 32 nodes in parallel, flags the
// overlapping ones and pushes the child group of every overlapping internal node. Returns false (and sets bit 0 of
// errWord) if the stack would overflow.
template<class K, class T, bool FloatFilter>
__device__ __forceinline__ bool haloTraverse(const T (&tc)[3], const T (&ts)[3], int* stack, int lane, K lowest,
                                             K highest, const K* __restrict__ prefixes,
                                             const int32_t* __restrict__ childOffsets, const T* __restrict__ nc,
                                             const T* __restrict__ ns, const BoxParams<T>& b, uint8_t* flags,
                                             uint32_t* errWord, const float4* __restrict__ nrec)
{
    float tcf[3], tsf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        tcf[k] = float(tc[k]);
        tsf[k] = float(ts[k]);
    }
    auto overlapsLoaded = [&](int idx, K pfx, float4 c4, float4 s4) -> bool {
        return haloNodeTest<K, T, FloatFilter>(idx, pfx, c4, s4, tc, ts, tcf, tsf, lowest, highest, nc, ns, b, flags);
    };
    auto records = [&](int idx, float4& c4, float4& s4) { haloRecords<T, FloatFilter>(nrec, idx, c4, s4); };
    auto overlaps = [&](int idx) -> bool {
        float4 c4{}, s4{};
        records(idx, c4, s4);
        return overlapsLoaded(idx, prefixes[idx], c4, s4);
    };

    // the root is tested by lane 0 alone (a single node)
    bool rootOv = false;
    if (lane == 0) rootOv = overlaps(0);
    rootOv = __shfl_sync(0xffffffffu, rootOv, 0);
    if (!rootOv || childOffsets[0] == 0) return true;

    __syncwarp();
    if (lane == 0) stack[0] = childOffsets[0];
    int top = 1;
    __syncwarp();
    while (top > 0)
    {
        int ng = min(4, top);
        top -= ng;
        int g     = lane >> 3;
        bool push = false;
        int child = 0;
        if (g < ng)
        {
            // every load of the step is issued before the test needs any of them (one round trip per step)
            const int node = stack[top + g] + (lane & 7);
            const K pfx    = prefixes[node];
            const int ch   = childOffsets[node];
            float4 c4{}, s4{};
            records(node, c4, s4);
            if (overlapsLoaded(node, pfx, c4, s4))
            {
                child = ch;
                push  = child != 0;
            }
        }
        __syncwarp();
        unsigned pm = __ballot_sync(0xffffffffu, push);
        if (top + __popc(pm) > HALO_STACK)
        {
            if (lane == 0 && errWord) atomicOr(errWord, 1u);
            return false;
        }
        if (push) stack[top + __popc(pm & ((1u << lane) - 1u))] = child;
        top += __popc(pm);
        __syncwarp();
    }
    return true;
}

template<class K, class T, bool FloatFilter>
__global__ void __launch_bounds__(32 * HALO_WARPS)
    findHalosWarpKernel(const K* __restrict__ prefixes, const int32_t* __restrict__ childOffsets,
                        const T* __restrict__ nc, const T* __restrict__ ns, const K* __restrict__ leaves,
                        const T* __restrict__ sc, const T* __restrict__ ss, BoxParams<T> b, KeyParams<T, K> kp,
                        int firstNode, int lastNode, uint8_t* flags, uint32_t* errWord,
                        const float4* __restrict__ nrec)
{
    __shared__ int sStack[HALO_WARPS][HALO_STACK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long leaf0 = firstNode + (long long)(blockIdx.x * HALO_WARPS + warp) * 32;
    if (leaf0 >= lastNode) return;
    const K lowest  = leaves[firstNode];
    const K highest = leaves[lastNode];

    T myc[3], mys[3];
    const int myLeaf = int(leaf0) + lane;
    bool need        = false;
    if (myLeaf < lastNode)
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            myc[k] = sc[3 * size_t(myLeaf) + k];
            mys[k] = ss[3 * size_t(myLeaf) + k];
        }
        need = !boxContainedIn<K, T>(lowest, highest, myc, mys, b, kp);
    }
    else
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
            myc[k] = mys[k] = T(0);
    }
    unsigned todo = __ballot_sync(0xffffffffu, need);

    while (todo)
    {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        T tc[3], ts[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            tc[k] = __shfl_sync(0xffffffffu, myc[k], src);
            ts[k] = __shfl_sync(0xffffffffu, mys[k], src);
        }
        if (!haloTraverse<K, T, FloatFilter>(tc, ts, sStack[warp], lane, lowest, highest, prefixes, childOffsets, nc,
                                             ns, b, flags, errWord, nrec))
            return;
    }
}

// With a scratch list the work is split in two launches, so that the traversals spread over the whole GPU instead of
// running one after another in the warp that owns 32 neighbouring leaves (the leaves near the focus boundary are
// few and clustered). haloNeedKernel: one thread per focus leaf decides the containment test and appends the leaves
// that need a traversal (warp-aggregated; the order of the list does not matter, since the flagged set does not
// depend on the visiting order). findHalosListKernel: persistent warps take list entries one at a time from a
// counter and traverse for each. scratch: [0] list length, [1] next entry, [2 ...] the list.
template<class K, class T>
__global__ void haloNeedKernel(const K* __restrict__ leaves, const T* __restrict__ sc, const T* __restrict__ ss,
                               BoxParams<T> b, KeyParams<T, K> kp, int firstNode, int lastNode, int32_t* scratch)
{
    const long long leaf = firstNode + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool need            = false;
    if (leaf < lastNode)
    {
        T c[3], sz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            c[k]  = sc[3 * size_t(leaf) + k];
            sz[k] = ss[3 * size_t(leaf) + k];
        }
        need = !boxContainedIn<K, T>(leaves[firstNode], leaves[lastNode], c, sz, b, kp);
    }
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m == 0) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base       = 0;
    if (lane == leader) base = atomicAdd(&scratch[0], __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) scratch[2 + base + __popc(m & ((1u << lane) - 1u))] = int32_t(leaf);
}

// Per 8-lane group: its own traversal of one list entry at a time, one sibling group of 8 nodes per step from its
// own LIFO stack, so that a warp keeps four traversals in flight (a traversal's stack is mostly shallow, and each
// step waits for its node loads). One group popped and at most 8 pushed per step bounds a stack by 7 entries per
// level plus 8 (7 * 21 + 8 = 155 for 64-bit keys).
constexpr int HALO_GSTACK = 160;

template<class K, class T, bool FloatFilter>
__global__ void __launch_bounds__(32 * HALO_WARPS, 10)
    findHalosListKernel(const K* __restrict__ prefixes, const int32_t* __restrict__ childOffsets,
                        const T* __restrict__ nc, const T* __restrict__ ns, const K* __restrict__ leaves,
                        const T* __restrict__ sc, const T* __restrict__ ss, BoxParams<T> b, int firstNode,
                        int lastNode, uint8_t* flags, uint32_t* errWord, const float4* __restrict__ nrec,
                        int32_t* scratch)
{
    __shared__ int sStack[HALO_WARPS][4][HALO_GSTACK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 3, sub = lane & 7, lead = lane & ~7;
    const int total = scratch[0];
    if (total == 0) return;
    const K lowest  = leaves[firstNode];
    const K highest = leaves[lastNode];
    int* stack      = sStack[warp][g];
    int top         = 0;     // the group's stack height (the same in its 8 lanes)
    bool done       = false; // the group found the list exhausted
    T tc[3] = {}, ts[3] = {};
    float tcf[3] = {}, tsf[3] = {};
    for (;;)
    {
        // a group without work takes the next list entry; its lane 0 tests the root
        const bool want = !done && top == 0;
        int item        = 0;
        if (want && sub == 0) item = atomicAdd(&scratch[1], 1);
        item = __shfl_sync(0xffffffffu, item, lead);
        if (want)
        {
            if (item >= total)
                done = true;
            else
            {
                const int leaf = scratch[2 + item];
#pragma unroll
                for (int k = 0; k < 3; ++k)
                {
                    tc[k]  = sc[3 * size_t(leaf) + k];
                    ts[k]  = ss[3 * size_t(leaf) + k];
                    tcf[k] = float(tc[k]);
                    tsf[k] = float(ts[k]);
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) return;
        int rootChild = 0;
        if (want && !done && sub == 0)
        {
            float4 c4{}, s4{};
            haloRecords<T, FloatFilter>(nrec, 0, c4, s4);
            const int ch = childOffsets[0];
            if (haloNodeTest<K, T, FloatFilter>(0, prefixes[0], c4, s4, tc, ts, tcf, tsf, lowest, highest, nc, ns, b,
                                                flags))
                rootChild = ch;
        }
        rootChild = __shfl_sync(0xffffffffu, rootChild, lead);
        if (rootChild != 0)
        {
            if (sub == 0) stack[0] = rootChild;
            top = 1;
        }
        __syncwarp();

        // one step of every group with a non-empty stack: pop one sibling group, test its 8 nodes, push the child
        // groups of the overlapping internal ones
        bool push = false;
        int child = 0;
        if (top > 0)
        {
            --top;
            const int node = stack[top] + sub;
            const K pfx    = prefixes[node];
            const int ch   = childOffsets[node];
            float4 c4{}, s4{};
            haloRecords<T, FloatFilter>(nrec, node, c4, s4);
            if (haloNodeTest<K, T, FloatFilter>(node, pfx, c4, s4, tc, ts, tcf, tsf, lowest, highest, nc, ns, b,
                                                flags))
            {
                child = ch;
                push  = child != 0;
            }
        }
        __syncwarp();
        const unsigned pm = (__ballot_sync(0xffffffffu, push) >> lead) & 0xffu;
        if (__any_sync(0xffffffffu, top + __popc(pm) > HALO_GSTACK))
        {
            if (lane == 0 && errWord) atomicOr(errWord, 1u);
            return;
        }
        if (push) stack[top + __popc(pm & ((1u << sub) - 1u))] = child;
        top += __popc(pm);
        __syncwarp();
    }
}

template<class K, class T, bool FloatFilter>
static int haloListGrid()
{
    constexpr int MAX_DEVICES = 64;
    static std::atomic<int> cached[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < MAX_DEVICES && cached[dev].load() > 0) return cached[dev].load();
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, findHalosListKernel<K, T, FloatFilter>, 32 * HALO_WARPS, 0);
    const int g = std::max(1, perSm) * smCount();
    if (dev >= 0 && dev < MAX_DEVICES) cached[dev].store(g);
    return g;
}

template<class K, class T>
int findHalos(cudaStream_t s, const K* prefixes, const int32_t* childOffsets, const int32_t* parents, const T* nc,
              const T* ns, const K* leaves, const T* sc, const T* ss, const cs_box& box, int first, int last,
              uint8_t* flags, uint32_t* errWord, const float4* nrec, int32_t* scratch)
{
    if (last <= first) return CS_OK;
    auto bp = makeBoxParams<T>(box);
    auto kp = makeKeyParams<T, K>(bp);
    bool anyPbc = bp.pbc[0] || bp.pbc[1] || bp.pbc[2];
    bool ff     = false;
    if constexpr (std::is_same_v<T, double>) ff = nrec && !anyPbc;
    if (scratch)
    {
        CSG_CUDA_TRY(cudaMemsetAsync(scratch, 0, 2 * sizeof(int32_t), s));
        haloNeedKernel<K, T><<<iceil(size_t(last - first), 256), 256, 0, s>>>(leaves, sc, ss, bp, kp, first, last,
                                                                             scratch);
        CSG_CHECK_LAUNCH();
        if constexpr (std::is_same_v<T, double>)
        {
            if (ff)
            {
                findHalosListKernel<K, T, true><<<haloListGrid<K, T, true>(), 32 * HALO_WARPS, 0, s>>>(
                    prefixes, childOffsets, nc, ns, leaves, sc, ss, bp, first, last, flags, errWord, nrec, scratch);
                CSG_CHECK_LAUNCH();
                return CS_OK;
            }
        }
        findHalosListKernel<K, T, false><<<haloListGrid<K, T, false>(), 32 * HALO_WARPS, 0, s>>>(
            prefixes, childOffsets, nc, ns, leaves, sc, ss, bp, first, last, flags, errWord, nullptr, scratch);
        CSG_CHECK_LAUNCH();
        return CS_OK;
    }
    unsigned blocks = iceil(size_t(last - first), 32 * HALO_WARPS);
    if constexpr (std::is_same_v<T, double>)
    {
        if (ff)
        {
            findHalosWarpKernel<K, T, true><<<blocks, 32 * HALO_WARPS, 0, s>>>(
                prefixes, childOffsets, nc, ns, leaves, sc, ss, bp, kp, first, last, flags, errWord, nrec);
            CSG_CHECK_LAUNCH();
            return CS_OK;
        }
    }
    findHalosWarpKernel<K, T, false><<<blocks, 32 * HALO_WARPS, 0, s>>>(
        prefixes, childOffsets, nc, ns, leaves, sc, ss, bp, kp, first, last, flags, errWord, nullptr);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int searchBoxes<float, float>(cudaStream_t, const float*, const float*, const float*, const float*,
                                       const uint32_t*, int, int, float, const int32_t*, const float*, float*, float*,
                                       const float4*);
template int searchBoxes<double, double>(cudaStream_t, const double*, const double*, const double*, const double*,
                                         const uint32_t*, int, int, double, const int32_t*, const double*, double*,
                                         double*, const float4*);
template int searchBoxes<double, float>(cudaStream_t, const double*, const double*, const double*, const float*,
                                        const uint32_t*, int, int, float, const int32_t*, const double*, double*,
                                        double*, const float4*);
template int findHalos<uint32_t, float>(cudaStream_t, const uint32_t*, const int32_t*, const int32_t*, const float*,
                                        const float*, const uint32_t*, const float*, const float*, const cs_box&, int,
                                        int, uint8_t*, uint32_t*, const float4*, int32_t*);
template int findHalos<uint64_t, float>(cudaStream_t, const uint64_t*, const int32_t*, const int32_t*, const float*,
                                        const float*, const uint64_t*, const float*, const float*, const cs_box&, int,
                                        int, uint8_t*, uint32_t*, const float4*, int32_t*);
template int findHalos<uint64_t, double>(cudaStream_t, const uint64_t*, const int32_t*, const int32_t*, const double*,
                                         const double*, const uint64_t*, const double*, const double*, const cs_box&,
                                         int, int, uint8_t*, uint32_t*, const float4*, int32_t*);

} // namespace csg

using namespace csg;

extern "C" int cs_search_boxes_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                                   const uint32_t* layout, int32_t first, int32_t last, float scale,
                                   const int32_t* l2i, const float* nc, float* sc, float* ss)
{
    return searchBoxes<float, float>(cudaStream_t(stream), x, y, z, h, layout, first, last, scale, l2i, nc, sc, ss);
}
extern "C" int cs_search_boxes_f64(cs_stream_t stream, const double* x, const double* y, const double* z,
                                   const double* h, const uint32_t* layout, int32_t first, int32_t last, double scale,
                                   const int32_t* l2i, const double* nc, double* sc, double* ss)
{
    return searchBoxes<double, double>(cudaStream_t(stream), x, y, z, h, layout, first, last, scale, l2i, nc, sc, ss);
}
extern "C" int cs_search_boxes_f64_hf32(cs_stream_t stream, const double* x, const double* y, const double* z,
                                        const float* h, const uint32_t* layout, int32_t first, int32_t last,
                                        float scale, const int32_t* l2i, const double* nc, double* sc, double* ss)
{
    return searchBoxes<double, float>(cudaStream_t(stream), x, y, z, h, layout, first, last, scale, l2i, nc, sc, ss);
}

#define CS_HALOS_ENTRY(kb, K, tb, T)                                                                                   \
    extern "C" int cs_find_halos_##kb##_##tb(cs_stream_t stream, const K* prefixes, const int32_t* childOffsets,       \
                                             const int32_t* parents, const T* nc, const T* ns, const K* leaves,         \
                                             const T* sc, const T* ss, const cs_box* box, int32_t first,               \
                                             int32_t last, uint8_t* flags)                                              \
    {                                                                                                                  \
        if (!box)                                                                                                      \
        {                                                                                                              \
            setLastError("find halos: null box");                                                                      \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        return findHalos<K, T>(cudaStream_t(stream), prefixes, childOffsets, parents, nc, ns, leaves, sc, ss, *box,    \
                               first, last, flags, nullptr, nullptr, nullptr);                                                  \
    }
CS_HALOS_ENTRY(u32, uint32_t, f32, float)
CS_HALOS_ENTRY(u64, uint64_t, f32, float)
CS_HALOS_ENTRY(u64, uint64_t, f64, double)
