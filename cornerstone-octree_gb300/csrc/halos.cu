// Halo discovery: per-leaf h-expanded search boxes (focus/source_center.hpp:28-43, focus/source_center_gpu.cu:23-92)
// and the collision traversal that flags every node outside the focus key range that overlaps a focus leaf's search
// box (traversal/collisions.hpp:25-94, traversal/collisions_gpu.cu:23-77, traversal/boxoverlap.hpp:127-291).
//
// Search boxes: 8 lanes per leaf stride over its particles; min/max are exact (taken on order-preserving integer
// images of the values), so any reduction order gives the reference's bits (up to the sign of a zero extremum that
// ties with the other zero). Collisions: one warp per 32 focus leaves, each lane deciding the containment test for
// its own leaf, and one warp-wide traversal testing 32 nodes at a time for each leaf that needs it
// (findHalosWarpKernel); the flagged set equals that of the reference's per-leaf singleTraversal
// (traversal/traversal.hpp:26-69), and every floating-point expression is unfused and in the reference's order.
#include "cs_common.cuh"
#include "halos.cuh"

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

template<class T, class Th>
int searchBoxes(cudaStream_t s, const T* x, const T* y, const T* z, const Th* h, const uint32_t* layout, int first,
                int last, Th scale, const int32_t* l2i, const T* nodeCenters, T* sc, T* ss)
{
    if (last <= first) return CS_OK;
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
template<class K, class T, bool FloatFilter>
__global__ void __launch_bounds__(32 * HALO_WARPS)
    findHalosWarpKernel(const K* __restrict__ prefixes, const int32_t* __restrict__ childOffsets,
                        const T* __restrict__ nc, const T* __restrict__ ns, const K* __restrict__ leaves,
                        const T* __restrict__ sc, const T* __restrict__ ss, BoxParams<T> b, KeyParams<T, K> kp,
                        int firstNode, int lastNode, uint8_t* flags, uint32_t* errWord,
                        const float4* __restrict__ nrec)
{
    constexpr float U8 = 8.f * 5.9604644775390625e-8f;
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
    int* stack    = sStack[warp];

    while (todo)
    {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        T tc[3], ts[3];
        float tcf[3], tsf[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            tc[k]  = __shfl_sync(0xffffffffu, myc[k], src);
            ts[k]  = __shfl_sync(0xffffffffu, mys[k], src);
            tcf[k] = float(tc[k]);
            tsf[k] = float(ts[k]);
        }

        auto overlaps = [&](int idx) -> bool {
            K pfx         = prefixes[idx];
            K nk1         = decodePlaceholderBit<K>(pfx);
            unsigned plen = decodePrefixLength<K>(pfx);
            K nk2         = nk1 + (K(1) << (3u * KeyTraits<K>::maxLevel - plen));
            bool inside   = !(nk1 < lowest || nk2 > highest);
            if (inside) return false;
            bool ov = true;
            if constexpr (FloatFilter)
            {
                float4 c4    = nrec[3 * size_t(idx)], s4 = nrec[3 * size_t(idx) + 2];
                float cc[3]  = {c4.x, c4.y, c4.z}, sz[3] = {s4.x, s4.y, s4.z};
                bool sureIn  = true, sureOut = false;
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
        };

        // the root is tested by lane 0 alone (a single node)
        bool rootOv = false;
        if (lane == 0) rootOv = overlaps(0);
        rootOv = __shfl_sync(0xffffffffu, rootOv, 0);
        if (!rootOv || childOffsets[0] == 0) continue;

        int top = 0;
        __syncwarp();
        if (lane == 0) stack[0] = childOffsets[0];
        top = 1;
        __syncwarp();
        while (top > 0)
        {
            int ng = min(4, top);
            top -= ng;
            int g      = lane >> 3;
            bool push  = false;
            int child  = 0;
            if (g < ng)
            {
                int node = stack[top + g] + (lane & 7);
                if (overlaps(node))
                {
                    child = childOffsets[node];
                    push  = child != 0;
                }
            }
            __syncwarp();
            unsigned pm = __ballot_sync(0xffffffffu, push);
            if (top + __popc(pm) > HALO_STACK)
            {
                if (lane == 0 && errWord) atomicOr(errWord, 1u);
                return;
            }
            if (push) stack[top + __popc(pm & ((1u << lane) - 1u))] = child;
            top += __popc(pm);
            __syncwarp();
        }
    }
}

template<class K, class T>
int findHalos(cudaStream_t s, const K* prefixes, const int32_t* childOffsets, const int32_t* parents, const T* nc,
              const T* ns, const K* leaves, const T* sc, const T* ss, const cs_box& box, int first, int last,
              uint8_t* flags, uint32_t* errWord, const float4* nrec)
{
    if (last <= first) return CS_OK;
    auto bp = makeBoxParams<T>(box);
    auto kp = makeKeyParams<T, K>(bp);
    unsigned blocks = iceil(size_t(last - first), 32 * HALO_WARPS);
    bool anyPbc     = bp.pbc[0] || bp.pbc[1] || bp.pbc[2];
    if constexpr (std::is_same_v<T, double>)
    {
        if (nrec && !anyPbc)
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
                                       const uint32_t*, int, int, float, const int32_t*, const float*, float*, float*);
template int searchBoxes<double, double>(cudaStream_t, const double*, const double*, const double*, const double*,
                                         const uint32_t*, int, int, double, const int32_t*, const double*, double*,
                                         double*);
template int searchBoxes<double, float>(cudaStream_t, const double*, const double*, const double*, const float*,
                                        const uint32_t*, int, int, float, const int32_t*, const double*, double*,
                                        double*);
template int findHalos<uint32_t, float>(cudaStream_t, const uint32_t*, const int32_t*, const int32_t*, const float*,
                                        const float*, const uint32_t*, const float*, const float*, const cs_box&, int,
                                        int, uint8_t*, uint32_t*, const float4*);
template int findHalos<uint64_t, float>(cudaStream_t, const uint64_t*, const int32_t*, const int32_t*, const float*,
                                        const float*, const uint64_t*, const float*, const float*, const cs_box&, int,
                                        int, uint8_t*, uint32_t*, const float4*);
template int findHalos<uint64_t, double>(cudaStream_t, const uint64_t*, const int32_t*, const int32_t*, const double*,
                                         const double*, const uint64_t*, const double*, const double*, const cs_box&,
                                         int, int, uint8_t*, uint32_t*, const float4*);

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
                               first, last, flags, nullptr, nullptr);                                                  \
    }
CS_HALOS_ENTRY(u32, uint32_t, f32, float)
CS_HALOS_ENTRY(u64, uint64_t, f32, float)
CS_HALOS_ENTRY(u64, uint64_t, f64, double)
