// Tree operations around the octree path: upsweeps of node counts and source centres, target groups, SFC gap
// filling and spanning trees.
//
// Upsweeps (upsweepSumGpu, tree/octree_gpu.cu:218-236; upsweepCentersGpu, focus/source_center_gpu.cu:173-205). The
// reference launches one kernel per tree level, deepest first, with the level boundaries read on the host. Here one
// launch does the whole upsweep: every leaf thread walks up through parents[]; each internal node has an arrival
// counter, and the child that arrives eighth combines the 8 children (in child order, so floating-point results equal
// the level-by-level evaluation) and carries on upwards. The level-by-level form is kept for callers that hold only
// levelRange (no parents array), as the reference's signature does.
//
// Source centres (computeLeafSourceCenterGpu, focus/source_center_gpu.cu:103-170). Mass centres are evaluated in the
// CPU reference's order (massCenter, focus/source_center.hpp:70-81: a serial sum over the leaf's particles, then one
// division) with round-to-nearest intrinsics, so the results equal the CPU path bit for bit; the reference's own GPU
// kernel sums 8-way interleaved partial sums with fused multiply-adds and differs from its CPU path in the last bits.
//
// Target groups (computeFixedGroups / computeGroupSplits, traversal/groups_gpu.cu, groupSplitsKernel and findSplits in
// traversal/groups_gpu.cuh). Fixed groups of 32 or 64 consecutive particles are cut where consecutive particles are
// farther apart than min(tol * edge of the smallest leaf among the group's first 32 particles, 2h / minExtent), in
// unit-box coordinates. One warp per fixed group computes the cut mask and the count; an exclusive scan gives each
// group's first output slot, and a second pass writes the group starts directly (the reference scans twice with a
// host synchronisation in between).
//
// SFC gaps (countSfcGapsGpu / fillSfcGapsGpu, tree/csarray_gpu.cu:238-270) and computeSpanningTree
// (tree/csarray.hpp:482-506): spanSfcRange per interval, an exclusive scan, and the keys written per interval.
#include "cs_common.cuh"
#include "octree_link.cuh"

#include <algorithm>
#include <type_traits>

namespace csg
{

int exclusiveScanI32(cudaStream_t s, const int32_t* in, int32_t* out, size_t n, int32_t init, void* ws, size_t wsb);
size_t exclusiveScanWorkspaceBytes(size_t n);

// ---------------------------------------------------------------------------------------------------------------
// upsweeps
// ---------------------------------------------------------------------------------------------------------------

// NodeCount (tree/octree.hpp:603-615): min(2^32 - 1, sum of the 8 children)
struct CountCombine
{
    using V = uint32_t;
    __device__ static void combine(V* q, int node, int child)
    {
        unsigned long long sum = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            sum += __ldcg(q + child + k);
        q[node] = uint32_t(min(sum, 0xFFFFFFFFull));
    }
};

// addBody / normalizeMass / CombineSourceCenter (focus/source_center.hpp:46-98) in the reference's order, no fusion
template<class T>
__device__ __forceinline__ void addBody(T c[4], T x, T y, T z, T m)
{
    T w  = RN<T>::abs_(m);
    c[0] = RN<T>::add(c[0], RN<T>::mul(w, x));
    c[1] = RN<T>::add(c[1], RN<T>::mul(w, y));
    c[2] = RN<T>::add(c[2], RN<T>::mul(w, z));
    c[3] = RN<T>::add(c[3], w);
}

template<class T>
__device__ __forceinline__ T rdiv(T a, T b)
{
    if constexpr (std::is_same_v<T, double>) return __ddiv_rn(a, b);
    else return __fdiv_rn(a, b);
}

template<class T>
__device__ __forceinline__ void normalizeMass(T c[4])
{
    T inv = (c[3] != T(0)) ? rdiv<T>(T(1), c[3]) : T(1);
    c[0]  = RN<T>::mul(c[0], inv);
    c[1]  = RN<T>::mul(c[1], inv);
    c[2]  = RN<T>::mul(c[2], inv);
}

template<class T>
struct CenterCombine
{
    using V = T; // 4 per node
    __device__ static void combine(T* q, int node, int child)
    {
        T c[4] = {0, 0, 0, 0};
        for (int k = 0; k < 8; ++k)
        {
            const T* s = q + 4 * size_t(child + k);
            addBody<T>(c, __ldcg(s), __ldcg(s + 1), __ldcg(s + 2), __ldcg(s + 3));
        }
        normalizeMass<T>(c);
        T* o = q + 4 * size_t(node);
        o[0] = c[0], o[1] = c[1], o[2] = c[2], o[3] = c[3];
    }
};

// one launch: leaf threads walk up; the eighth child to arrive at a node combines its children and continues
template<class Op>
__global__ void upsweepLinkedKernel(const int32_t* __restrict__ childOffsets, const int32_t* __restrict__ parents,
                                    int numNodes, typename Op::V* q, unsigned* arrivals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numNodes || i == 0 || childOffsets[i] != 0) return;
    int node = i;
    while (node > 0)
    {
        int p = __ldg(parents + (node - 1) / 8);
        __threadfence(); // this node's value before the arrival that may let a sibling read it
        if (atomicAdd(arrivals + p, 1u) != 7u) return;
        __threadfence(); // the siblings' values after their arrivals
        Op::combine(q, p, __ldg(childOffsets + p));
        node = p;
    }
}

template<class Op>
__global__ void upsweepLevelKernel(int first, int last, const int32_t* __restrict__ childOffsets, typename Op::V* q)
{
    int i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= last) return;
    int c = childOffsets[i];
    if (c) Op::combine(q, i, c);
}

template<class Op>
static int upsweep(cudaStream_t s, int numLevels, const int32_t* levelRangeHost, const int32_t* childOffsets,
                   const int32_t* parents, int numNodes, typename Op::V* q, void* ws, size_t wsb)
{
    if (numNodes <= 1) return CS_OK;
    if (!childOffsets || !q)
    {
        setLastError("upsweep: null pointer");
        return CS_ERR_INVALID;
    }
    if (parents)
    {
        Workspace w;
        int rc = w.acquire(ws, wsb, size_t(numNodes) * sizeof(unsigned), s);
        if (rc) return rc;
        unsigned* arr = static_cast<unsigned*>(w.ptr);
        CSG_CUDA_TRY(cudaMemsetAsync(arr, 0, size_t(numNodes) * sizeof(unsigned), s));
        upsweepLinkedKernel<Op><<<iceil(size_t(numNodes), 256), 256, 0, s>>>(childOffsets, parents, numNodes, q, arr);
        CSG_CHECK_LAUNCH();
        return CS_OK;
    }
    if (!levelRangeHost || numLevels < 1)
    {
        setLastError("upsweep: need parents or the host level range");
        return CS_ERR_INVALID;
    }
    for (int level = numLevels - 1; level >= 0; --level)
    {
        int a = levelRangeHost[level], b = levelRangeHost[level + 1];
        if (b > a)
        {
            upsweepLevelKernel<Op><<<iceil(size_t(b - a), 256), 256, 0, s>>>(a, b, childOffsets, q);
            CSG_CHECK_LAUNCH();
        }
    }
    return CS_OK;
}

// leaf mass centres, one thread per leaf, the reference's serial order
template<class Tc, class Tm, class T>
__global__ void leafCentersKernel(const Tc* __restrict__ x, const Tc* __restrict__ y, const Tc* __restrict__ z,
                                  const Tm* __restrict__ m, const int32_t* __restrict__ l2i, int numLeaves,
                                  const uint32_t* __restrict__ layout, T* centers)
{
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= numLeaves) return;
    T c[4] = {0, 0, 0, 0};
    for (uint32_t i = layout[l], e = layout[l + 1]; i < e; ++i)
        addBody<T>(c, T(x[i]), T(y[i]), T(z[i]), T(m[i]));
    normalizeMass<T>(c);
    T* o = centers + 4 * size_t(l2i[l]);
    o[0] = c[0], o[1] = c[1], o[2] = c[2], o[3] = c[3];
}

// ---------------------------------------------------------------------------------------------------------------
// target groups
// ---------------------------------------------------------------------------------------------------------------

template<class T>
__device__ __forceinline__ T fmaRn(T a, T b, T c)
{
    if constexpr (std::is_same_v<T, double>) return __fma_rn(a, b, c);
    else return __fmaf_rn(a, b, c);
}

template<class T, class K>
struct GroupArgs
{
    uint32_t first, last;
    const T *x, *y, *z, *h;
    const K* leaves;
    int numLeaves;
    const uint32_t* layout;
    T ilx, ily, ilz, minExt;
    float tol;
};

// leaf of particle b: upper_bound(layout, layout + numLeaves, b) - 1
__device__ __forceinline__ int leafOf(const uint32_t* layout, int numLeaves, uint32_t b)
{
    int lo = 0, hi = numLeaves;
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (__ldg(layout + mid) <= b) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

// one warp per fixed group of NW * 32 particles: cut masks (bit k of segment w: cut after particle 32 w + k) and the
// number of groups it becomes
template<int NW, class T, class K>
__global__ void groupSplitsKernel(GroupArgs<T, K> a, uint32_t numFixed, uint32_t* masks, int32_t* numSplits)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane      = threadIdx.x & 31;
    if (warp >= numFixed) return;
    const uint32_t b0 = a.first + warp * 32u * NW;
    // smallest leaf volume among the first segment's particles; leaf volumes in the unit box are 2^(-3 level), and
    // their cube root is exactly 2^(-level): distCrit = 2^(-deepest level) * tol
    uint32_t b0l = min(b0 + uint32_t(lane), a.last - 1);
    int leaf     = leafOf(a.layout, a.numLeaves, b0l);
    unsigned lev = treeLevel<K>(a.leaves[leaf + 1] - a.leaves[leaf]);
    lev          = __reduce_max_sync(0xffffffffu, lev);
    T dc         = RN<T>::mul(T(ldexp(1.0, -int(lev))), T(a.tol));
    T dc2        = RN<T>::mul(dc, dc);
    int count    = 1;
#pragma unroll
    for (int w = 0; w < NW; ++w)
    {
        uint32_t j  = min(b0 + 32u * w + lane, a.last - 1);
        uint32_t jn = min(b0 + 32u * w + lane + 1, a.last - 1);
        // the last particle of the fixed group is compared with itself (no cut)
        if (w == NW - 1 && lane == 31) jn = j;
        T dx  = RN<T>::sub(RN<T>::mul(a.x[jn], a.ilx), RN<T>::mul(a.x[j], a.ilx));
        T dy  = RN<T>::sub(RN<T>::mul(a.y[jn], a.ily), RN<T>::mul(a.y[j], a.ily));
        T dz  = RN<T>::sub(RN<T>::mul(a.z[jn], a.ilz), RN<T>::mul(a.z[j], a.ilz));
        T d2  = fmaRn<T>(dz, dz, fmaRn<T>(dy, dy, RN<T>::mul(dx, dx)));
        T hr  = a.h ? rdiv<T>(RN<T>::mul(T(2), a.h[j]), a.minExt) : T(1);
        T h2  = RN<T>::mul(hr, hr);
        T crit = dc2 < h2 ? dc2 : h2;
        unsigned m = __ballot_sync(0xffffffffu, d2 > crit);
        if (lane == 0) masks[size_t(warp) * NW + w] = m;
        count += __popc(m);
    }
    if (lane == 0) numSplits[warp] = count;
}

template<int NW>
__global__ void groupWriteKernel(const uint32_t* __restrict__ masks, const int32_t* __restrict__ offsets,
                                 uint32_t numFixed, uint32_t first, uint32_t last, uint32_t* groups, size_t capacity)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= numFixed) return;
    const uint32_t b0 = first + g * 32u * NW;
    size_t o          = size_t(offsets[g]);
    if (o < capacity) groups[o] = b0;
    ++o;
#pragma unroll
    for (int w = 0; w < NW; ++w)
    {
        unsigned m = masks[size_t(g) * NW + w];
        while (m)
        {
            int k = __ffs(m) - 1;
            m &= m - 1;
            if (o < capacity) groups[o] = b0 + 32u * w + uint32_t(k) + 1u;
            ++o;
        }
    }
    if (g == numFixed - 1 && o < capacity) groups[o] = last;
}

// ---------------------------------------------------------------------------------------------------------------
// SFC gaps and spanning trees
// ---------------------------------------------------------------------------------------------------------------

template<class K>
__device__ __forceinline__ int lastNzPlace(K x)
{
    return x ? KeyTraits<K>::maxLevel - ctzKey<K>(x) / 3 : KeyTraits<K>::maxLevel;
}

// spanSfcRange (sfc/common.hpp:422-460): the cornerstone keys covering [a, b); counts them, stores them if out != 0
template<class K>
__device__ int spanSfcRange(K a, K b, K* out)
{
    int n         = 0;
    const int ub  = KeyTraits<K>::bits - 3 * KeyTraits<K>::maxLevel;
    int firstDiff = (clzKey<K>(a ^ b) + 3 - ub) / 3;
    int aLast = lastNzPlace<K>(a), bLast = lastNzPlace<K>(b);
    for (int pos = aLast; pos > firstDiff; --pos)
    {
        int digits = (8 - int(octalDigit<K>(a, unsigned(pos)))) % 8;
        n += digits;
        while (digits--)
        {
            if (out) *out++ = a;
            a += K(1) << (3 * (KeyTraits<K>::maxLevel - pos));
        }
    }
    for (int pos = firstDiff; pos <= bLast; ++pos)
    {
        int digits = int(octalDigit<K>(b, unsigned(pos))) - int(octalDigit<K>(a, unsigned(pos)));
        n += digits;
        while (digits--)
        {
            if (out) *out++ = a;
            a += K(1) << (3 * (KeyTraits<K>::maxLevel - pos));
        }
    }
    return n;
}

template<class K>
__global__ void countSfcGapsKernel(const K* __restrict__ tree, int numNodes, int32_t* ops)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < numNodes) ops[i] = spanSfcRange<K>(tree[i], tree[i + 1], nullptr);
}

template<class K>
__global__ void fillSfcGapsKernel(const K* __restrict__ tree, int numNodes, const int32_t* __restrict__ ops,
                                  K* newTree, int64_t capacity)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < numNodes)
    {
        int64_t o = ops[i], e = ops[i + 1];
        if (e <= capacity) spanSfcRange<K>(tree[i], tree[i + 1], newTree + o);
    }
    if (i == numNodes && int64_t(ops[numNodes]) < capacity) newTree[ops[numNodes]] = tree[numNodes];
}

} // namespace csg

using namespace csg;

// ---- upsweeps ----
extern "C" size_t cs_upsweep_workspace_bytes(int32_t num_nodes) { return size_t(num_nodes) * 4 + 256; }

extern "C" int cs_upsweep_sum(cs_stream_t stream, int num_levels, const int32_t* level_range_host,
                              const int32_t* child_offsets, const int32_t* parents, int32_t num_nodes,
                              uint32_t* node_counts, void* ws, size_t wsb)
{
    return upsweep<CountCombine>(cudaStream_t(stream), num_levels, level_range_host, child_offsets, parents,
                                 num_nodes, node_counts, ws, wsb);
}

#define CS_CENTER_ENTRIES(SUF, Tc, Tm, T)                                                                              \
    extern "C" int cs_leaf_source_centers_##SUF(cs_stream_t stream, const Tc* x, const Tc* y, const Tc* z,            \
                                               const Tm* m, const int32_t* leaf_to_internal, int32_t num_leaves,      \
                                               const uint32_t* layout, T* centers)                                   \
    {                                                                                                                  \
        if (num_leaves <= 0) return CS_OK;                                                                             \
        if (!x || !y || !z || !m || !leaf_to_internal || !layout || !centers)                                          \
        {                                                                                                              \
            setLastError("leaf source centres: null pointer");                                                         \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        leafCentersKernel<Tc, Tm, T><<<iceil(size_t(num_leaves), 128), 128, 0, cudaStream_t(stream)>>>(             \
            x, y, z, m, leaf_to_internal, num_leaves, layout, centers);                                                \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }

CS_CENTER_ENTRIES(f64, double, double, double)
CS_CENTER_ENTRIES(f64_m32, double, float, double)
CS_CENTER_ENTRIES(f32, float, float, float)

extern "C" int cs_upsweep_source_centers_f64(cs_stream_t stream, int num_levels, const int32_t* level_range_host,
                                             const int32_t* child_offsets, const int32_t* parents, int32_t num_nodes,
                                             double* centers, void* ws, size_t wsb)
{
    return upsweep<CenterCombine<double>>(cudaStream_t(stream), num_levels, level_range_host, child_offsets, parents,
                                          num_nodes, centers, ws, wsb);
}
extern "C" int cs_upsweep_source_centers_f32(cs_stream_t stream, int num_levels, const int32_t* level_range_host,
                                             const int32_t* child_offsets, const int32_t* parents, int32_t num_nodes,
                                             float* centers, void* ws, size_t wsb)
{
    return upsweep<CenterCombine<float>>(cudaStream_t(stream), num_levels, level_range_host, child_offsets, parents,
                                         num_nodes, centers, ws, wsb);
}

// ---- target groups ----
extern "C" size_t cs_group_splits_workspace_bytes(uint32_t num_particles, unsigned group_size)
{
    size_t nf = (size_t(num_particles) + group_size - 1) / std::max(1u, group_size);
    return nf * (2 * 4 + 4 + 4) + exclusiveScanWorkspaceBytes(nf + 1) + 1024;
}

template<class T>
static int groupSplits(cudaStream_t s, uint32_t first, uint32_t last, const T* x, const T* y, const T* z, const T* h,
                       const uint64_t* leaves, int32_t numLeaves, const uint32_t* layout, const cs_box* box,
                       unsigned groupSize, float tol, uint32_t* groups, size_t capacity, uint32_t* numGroupsHost,
                       void* ws, size_t wsb)
{
    if (groupSize != 32 && groupSize != 64)
    {
        setLastError("group splits: group size must be 32 or 64 (got %u)", groupSize);
        return CS_ERR_INVALID;
    }
    if (last < first || !box || !numGroupsHost || (last > first && (!x || !y || !z || !leaves || !layout)) ||
        (capacity && !groups) || numLeaves < 1)
    {
        setLastError("group splits: invalid arguments");
        return CS_ERR_INVALID;
    }
    const uint32_t nfix = (last - first + groupSize - 1) / groupSize;
    if (nfix == 0)
    {
        *numGroupsHost = 0;
        if (capacity) CSG_CUDA_TRY(cudaMemcpyAsync(groups, &last, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        return CS_OK;
    }
    Workspace w;
    int rc = w.acquire(ws, wsb, cs_group_splits_workspace_bytes(last - first, groupSize), s);
    if (rc) return rc;
    Arena ar{static_cast<char*>(w.ptr), 0, cs_group_splits_workspace_bytes(last - first, groupSize)};
    uint32_t* masks  = ar.take<uint32_t>(size_t(nfix) * 2);
    int32_t* nsplit  = ar.take<int32_t>(size_t(nfix) + 1);
    int32_t* offsets = ar.take<int32_t>(size_t(nfix) + 1);
    size_t scanBytes = exclusiveScanWorkspaceBytes(size_t(nfix) + 1);
    void* scanWs     = ar.take<char>(scanBytes);
    BoxParams<T> bp  = makeBoxParams<T>(*box);
    GroupArgs<T, uint64_t> a{first, last, x, y, z, h, leaves, numLeaves, layout, bp.ilen[0], bp.ilen[1], bp.ilen[2],
                             std::min(std::min(bp.len[0], bp.len[1]), bp.len[2]), tol};
    CSG_CUDA_TRY(cudaMemsetAsync(nsplit + nfix, 0, sizeof(int32_t), s));
    unsigned blocks = iceil(size_t(nfix) * 32, 256);
    if (groupSize == 32) groupSplitsKernel<1, T, uint64_t><<<blocks, 256, 0, s>>>(a, nfix, masks, nsplit);
    else groupSplitsKernel<2, T, uint64_t><<<blocks, 256, 0, s>>>(a, nfix, masks, nsplit);
    CSG_CHECK_LAUNCH();
    if ((rc = exclusiveScanI32(s, nsplit, offsets, size_t(nfix) + 1, 0, scanWs, scanBytes))) return rc;
    if (groupSize == 32)
        groupWriteKernel<1><<<iceil(nfix, 256), 256, 0, s>>>(masks, offsets, nfix, first, last, groups, capacity);
    else groupWriteKernel<2><<<iceil(nfix, 256), 256, 0, s>>>(masks, offsets, nfix, first, last, groups, capacity);
    CSG_CHECK_LAUNCH();
    int32_t total = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&total, offsets + nfix, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    *numGroupsHost = uint32_t(total);
    if (size_t(total) + 1 > capacity)
    {
        setLastError("group splits: %d groups need %d entries, capacity %zu", total, total + 1, capacity);
        return CS_ERR_CAPACITY;
    }
    return CS_OK;
}

extern "C" int cs_group_splits_f64(cs_stream_t stream, uint32_t first, uint32_t last, const double* x,
                                   const double* y, const double* z, const double* h, const uint64_t* leaves,
                                   int32_t num_leaves, const uint32_t* layout, const cs_box* box, unsigned group_size,
                                   float tol, uint32_t* groups, size_t groups_capacity, uint32_t* num_groups,
                                   void* ws, size_t wsb)
{
    return groupSplits<double>(cudaStream_t(stream), first, last, x, y, z, h, leaves, num_leaves, layout, box,
                               group_size, tol, groups, groups_capacity, num_groups, ws, wsb);
}
extern "C" int cs_group_splits_f32(cs_stream_t stream, uint32_t first, uint32_t last, const float* x, const float* y,
                                   const float* z, const float* h, const uint64_t* leaves, int32_t num_leaves,
                                   const uint32_t* layout, const cs_box* box, unsigned group_size, float tol,
                                   uint32_t* groups, size_t groups_capacity, uint32_t* num_groups, void* ws,
                                   size_t wsb)
{
    return groupSplits<float>(cudaStream_t(stream), first, last, x, y, z, h, leaves, num_leaves, layout, box,
                              group_size, tol, groups, groups_capacity, num_groups, ws, wsb);
}

// ---- SFC gaps and spanning trees ----
template<class K>
static int countGaps(cudaStream_t s, const K* tree, int32_t numNodes, int32_t* ops)
{
    if (numNodes <= 0) return CS_OK;
    if (!tree || !ops)
    {
        setLastError("count sfc gaps: null pointer");
        return CS_ERR_INVALID;
    }
    countSfcGapsKernel<K><<<iceil(size_t(numNodes), 256), 256, 0, s>>>(tree, numNodes, ops);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template<class K>
static int fillGaps(cudaStream_t s, const K* tree, int32_t numNodes, const int32_t* ops, K* newTree, int64_t cap)
{
    if (numNodes < 0 || !tree || !ops || !newTree)
    {
        setLastError("fill sfc gaps: invalid arguments");
        return CS_ERR_INVALID;
    }
    fillSfcGapsKernel<K><<<iceil(size_t(numNodes) + 1, 128), 128, 0, s>>>(tree, numNodes, ops, newTree, cap);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template<class K>
static int spanningTree(cudaStream_t s, const K* keys, int32_t numKeys, K* out, int32_t capacity, int32_t* outSize,
                        void* ws, size_t wsb)
{
    if (numKeys < 2 || !keys || !outSize)
    {
        setLastError("spanning tree: need at least 2 keys");
        return CS_ERR_INVALID;
    }
    const int32_t nn  = numKeys - 1;
    size_t scanBytes  = exclusiveScanWorkspaceBytes(size_t(nn) + 1);
    size_t need       = (size_t(nn) + 1) * 4 * 2 + scanBytes + 1024;
    Workspace w;
    int rc = w.acquire(ws, wsb, need, s);
    if (rc) return rc;
    Arena ar{static_cast<char*>(w.ptr), 0, need};
    int32_t* cnt = ar.take<int32_t>(size_t(nn) + 1);
    int32_t* off = ar.take<int32_t>(size_t(nn) + 1);
    void* sws    = ar.take<char>(scanBytes);
    CSG_CUDA_TRY(cudaMemsetAsync(cnt + nn, 0, sizeof(int32_t), s));
    if ((rc = countGaps<K>(s, keys, nn, cnt))) return rc;
    if ((rc = exclusiveScanI32(s, cnt, off, size_t(nn) + 1, 0, sws, scanBytes))) return rc;
    if ((rc = fillGaps<K>(s, keys, nn, off, out, int64_t(capacity)))) return rc;
    int32_t total = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&total, off + nn, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    *outSize = total + 1;
    if (total + 1 > capacity)
    {
        setLastError("spanning tree: %d keys needed, capacity %d", total + 1, capacity);
        return CS_ERR_CAPACITY;
    }
    return CS_OK;
}

extern "C" int cs_count_sfc_gaps_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes, int32_t* node_ops)
{
    return countGaps<uint32_t>(cudaStream_t(stream), tree, num_nodes, node_ops);
}
extern "C" int cs_count_sfc_gaps_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes, int32_t* node_ops)
{
    return countGaps<uint64_t>(cudaStream_t(stream), tree, num_nodes, node_ops);
}
extern "C" int cs_fill_sfc_gaps_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes,
                                    const int32_t* node_ops, uint32_t* new_tree)
{
    return fillGaps<uint32_t>(cudaStream_t(stream), tree, num_nodes, node_ops, new_tree, INT64_MAX);
}
extern "C" int cs_fill_sfc_gaps_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes,
                                    const int32_t* node_ops, uint64_t* new_tree)
{
    return fillGaps<uint64_t>(cudaStream_t(stream), tree, num_nodes, node_ops, new_tree, INT64_MAX);
}
extern "C" size_t cs_spanning_tree_workspace_bytes(int32_t num_keys)
{
    return (size_t(num_keys) + 1) * 8 + exclusiveScanWorkspaceBytes(size_t(num_keys) + 1) + 1024;
}
extern "C" int cs_spanning_tree_u32(cs_stream_t stream, const uint32_t* keys, int32_t num_keys, uint32_t* out,
                                    int32_t capacity, int32_t* out_size, void* ws, size_t wsb)
{
    return spanningTree<uint32_t>(cudaStream_t(stream), keys, num_keys, out, capacity, out_size, ws, wsb);
}
extern "C" int cs_spanning_tree_u64(cs_stream_t stream, const uint64_t* keys, int32_t num_keys, uint64_t* out,
                                    int32_t capacity, int32_t* out_size, void* ws, size_t wsb)
{
    return spanningTree<uint64_t>(cudaStream_t(stream), keys, num_keys, out, capacity, out_size, ws, wsb);
}
