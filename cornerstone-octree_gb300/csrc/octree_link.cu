// Internal octree linkage and node geometry (tree/octree.hpp:55-196, tree/octree_gpu.cu:41-203,
// focus/source_center_gpu.cu:212-240).
//
//  1. layout: leaf prefixes at [I, I+L) and internal-node prefixes at (j + binaryKeyWeight(k, cpr/3)) / 7
//  2. stable radix sort of (prefix, index) pairs -> (level, key) order
//  3. invert the permutation (leafToInternal), shift internalToLeaf by -I, levelRange by one warp of binary searches
//  4. link: first child of every internal node by binary search in the next level, parent of each sibling group
//  5. node geometric centres and half sizes from the decoded integer box, unfused arithmetic
#include "cs_common.cuh"
#include "octree_link.cuh"
#include "radix_sort.cuh"

#include <vector>

namespace csg
{

template<class K>
__device__ __forceinline__ int binaryKeyWeight(K key, unsigned level)
{
    int ret = 0;
    for (unsigned l = 1; l <= level + 1; ++l)
        ret += digitWeight(int(octalDigit<K>(key, l)));
    return ret;
}

// L, I, N from the host, or from a leaf count in device memory (then the launch covers a capacity and the slots
// [N, capacity) of the node arrays are padding)
struct LinkSizes
{
    int L, I, N;
};
__device__ __forceinline__ LinkSizes linkSizes(const int* Ldev, int Lhost)
{
    int L = Ldev ? *Ldev : Lhost;
    int I = (L - 1) / 7;
    return {L, I, L + I};
}

template<class K>
__global__ void createLayoutKernel(const K* __restrict__ leaves, const int* Ldev, int Lhost, int Ncap,
                                   K* __restrict__ prefixes, uint32_t* __restrict__ order)
{
    int tid          = blockIdx.x * blockDim.x + threadIdx.x;
    const LinkSizes z = linkSizes(Ldev, Lhost);
    const int L = z.L, I = z.I;
    if (Ldev && tid >= z.N && tid < Ncap)
    {
        // padding sorts behind every real prefix (ties with an all-ones prefix keep their larger index)
        prefixes[tid] = ~K(0);
        order[tid]    = uint32_t(tid);
    }
    if (tid >= L) return;
    K key                 = leaves[tid];
    K next                = leaves[tid + 1];
    unsigned level        = treeLevel<K>(next - key);
    prefixes[tid + I]     = encodePlaceholderBit<K>(key, 3 * int(level));
    order[tid + I]        = uint32_t(tid + I);
    unsigned prefixLength = unsigned(commonPrefix<K>(key, next));
    if (prefixLength % 3 == 0 && tid < L - 1)
    {
        int oct = (tid + binaryKeyWeight<K>(key, prefixLength / 3)) / 7;
        // a valid cornerstone array maps into [0, I); anything else is a malformed input, never written
        if (oct >= 0 && oct < I)
        {
            prefixes[oct] = encodePlaceholderBit<K>(key, int(prefixLength));
            order[oct]    = uint32_t(oct);
        }
    }
}

__global__ void invertOrderKernel(const uint32_t* __restrict__ order, const int* Ldev, int Lhost,
                                  int32_t* __restrict__ i2l, int32_t* __restrict__ l2i)
{
    int i             = blockIdx.x * blockDim.x + threadIdx.x;
    const LinkSizes z = linkSizes(Ldev, Lhost);
    const int N = z.N, I = z.I;
    if (i >= N) return;
    uint32_t v = order[i];
    if (v < uint32_t(N)) l2i[v] = i;
    i2l[i] = int32_t(v) - I;
}

template<class K>
__global__ void levelRangeKernel(const K* __restrict__ prefixes, const int* Ldev, int Lhost,
                                 int32_t* __restrict__ levelRange)
{
    constexpr int maxL = KeyTraits<K>::maxLevel;
    const int N        = linkSizes(Ldev, Lhost).N;
    int level          = threadIdx.x;
    if (level <= maxL)
    {
        K v    = encodePlaceholderBit<K>(K(0), 3 * level);
        int lo = 0, hi = N;
        while (lo < hi)
        {
            int mid = (lo + hi) >> 1;
            if (prefixes[mid] < v) lo = mid + 1;
            else hi = mid;
        }
        levelRange[level] = lo;
    }
    if (level == maxL + 1) levelRange[level] = N;
}

template<class K>
__global__ void linkKernel(const K* __restrict__ prefixes, const int* Ldev, int Lhost,
                           const int32_t* __restrict__ l2i, const int32_t* __restrict__ levelRange,
                           int32_t* __restrict__ childOffsets, int32_t* __restrict__ parents)
{
    int i       = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = linkSizes(Ldev, Lhost).I;
    if (i >= I) return;
    int idxA       = l2i[i];
    K prefix       = prefixes[idxA];
    K nodeKey      = decodePlaceholderBit<K>(prefix);
    unsigned plen  = decodePrefixLength<K>(prefix);
    unsigned level = plen / 3;
    if (level >= unsigned(KeyTraits<K>::maxLevel)) return; // internal nodes are never at the deepest level
    K child        = encodePlaceholderBit<K>(nodeKey, int(plen) + 3);
    int lo = levelRange[level + 1], hi = levelRange[level + 2];
    int end = hi;
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (prefixes[mid] < child) lo = mid + 1;
        else hi = mid;
    }
    if (lo != end && prefixes[lo] == child)
    {
        childOffsets[idxA]    = lo;
        parents[(lo - 1) / 8] = idxA;
    }
}

template<class K>
size_t buildLinkWorkspaceBytes(int L)
{
    int I = (L - 1) / 7, N = L + I;
    Arena a;
    a.take<K>(N);
    a.take<uint32_t>(N);
    a.take<uint32_t>(N);
    a.take<uint32_t>(4);
    return a.size + radixSortWorkspaceBytes<K>(N, 0, 8 * sizeof(K)) + 512;
}

template<class K>
int buildLink(cudaStream_t s, const K* leaves, int L, const cs_octree_view& v, int prefixBits, void* ws,
              size_t wsBytes, uint32_t* errWord, const int* Ldev)
{
    if (L < 1)
    {
        setLastError("build octree: need at least one leaf");
        return CS_ERR_INVALID;
    }
    // with Ldev, L is the leaf capacity and the arrays of v hold the capacity's node count
    int I = (L - 1) / 7, N = L + I;
    if (v.num_leaf_nodes != L || v.num_internal_nodes != I || v.num_nodes != N)
    {
        setLastError("build octree: view sizes (%d, %d, %d) do not match L = %d", v.num_leaf_nodes,
                     v.num_internal_nodes, v.num_nodes, L);
        return CS_ERR_INVALID;
    }
    K* prefixes = static_cast<K*>(v.prefixes);
    Arena a{static_cast<char*>(ws), 0, wsBytes};
    K* altKeys     = a.take<K>(N);
    uint32_t* ord  = a.take<uint32_t>(N);
    uint32_t* ordB = a.take<uint32_t>(N);
    uint32_t* err  = a.take<uint32_t>(4);
    int bits       = prefixBits > 0 ? prefixBits : int(8 * sizeof(K));
    size_t sortWs  = radixSortWorkspaceBytes<K>(N, 0, bits);
    void* sortBase = a.take<char>(sortWs);
    if (!a.ok())
    {
        setLastError("build octree: workspace too small");
        return CS_ERR_INVALID;
    }
    if (!errWord)
    {
        CSG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
        errWord = err;
    }

    createLayoutKernel<K><<<iceil(Ldev ? N : L, 256), 256, 0, s>>>(leaves, Ldev, L, N, prefixes, ord);
    CSG_CHECK_LAUNCH();
    bool inAlt = false;
    int rc = radixSortPairs<K>(s, prefixes, ord, altKeys, ordB, N, 0, bits, false, sortBase, sortWs, errWord, &inAlt);
    if (rc) return rc;
    uint32_t* sortedOrd = inAlt ? ordB : ord;
    if (inAlt) CSG_CUDA_TRY(cudaMemcpyAsync(prefixes, altKeys, size_t(N) * sizeof(K), cudaMemcpyDeviceToDevice, s));

    invertOrderKernel<<<iceil(N, 256), 256, 0, s>>>(sortedOrd, Ldev, L, v.internal_to_leaf, v.leaf_to_internal);
    CSG_CHECK_LAUNCH();
    levelRangeKernel<K><<<1, 32, 0, s>>>(prefixes, Ldev, L, v.level_range);
    CSG_CHECK_LAUNCH();
    CSG_CUDA_TRY(cudaMemsetAsync(v.child_offsets, 0, (size_t(N) + 1) * sizeof(int32_t), s));
    if (I > 0)
    {
        linkKernel<K><<<iceil(I, 256), 256, 0, s>>>(prefixes, Ldev, L, v.leaf_to_internal, v.level_range,
                                                   v.child_offsets, v.parents);
        CSG_CHECK_LAUNCH();
    }
    return CS_OK;
}

template size_t buildLinkWorkspaceBytes<uint32_t>(int);
template size_t buildLinkWorkspaceBytes<uint64_t>(int);
template int buildLink<uint32_t>(cudaStream_t, const uint32_t*, int, const cs_octree_view&, int, void*, size_t,
                                 uint32_t*, const int*);
template int buildLink<uint64_t>(cudaStream_t, const uint64_t*, int, const cs_octree_view&, int, void*, size_t,
                                 uint32_t*, const int*);

// ---------------------------------------------------------------------------------------------------------------
// node geometry: centerAndSize (sfc/box.hpp:318-335) of hilbertIBox / mortonIBox
// ---------------------------------------------------------------------------------------------------------------
template<class T>
struct GeoParams
{
    T lo[3];
    T half[3]; // 0.5 * (1 / 2^L) * box length, rounded in T as the reference does
};

template<class K, class T, int Kind>
__global__ void geoCentersKernel(const K* __restrict__ prefixes, int Nhost, const int* Ldev, T* __restrict__ centers,
                                 T* __restrict__ sizes, GeoParams<T> g)
{
    int i       = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = Ldev ? linkSizes(Ldev, 0).N : Nhost;
    if (i >= N) return;
    K prefix          = prefixes[i];
    K start           = decodePlaceholderBit<K>(prefix);
    unsigned level    = decodePrefixLength<K>(prefix) / 3;
    unsigned maxCoord = 1u << KeyTraits<K>::maxLevel;
    unsigned cube     = maxCoord >> level;
    unsigned ix, iy, iz;
    if (Kind == CS_HILBERT)
    {
        decodeHilbert<K>(start, ix, iy, iz);
        unsigned mask = ~(cube - 1u);
        ix &= mask;
        iy &= mask;
        iz &= mask;
    }
    else { decodeMorton<K>(start, ix, iy, iz); }
    unsigned imin[3] = {ix, iy, iz};
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int a                = int(imin[k]);
        int b                = a + int(cube);
        centers[3 * i + k]   = RN<T>::add(g.lo[k], RN<T>::mul(T(b + a), g.half[k]));
        sizes[3 * i + k]     = RN<T>::mul(T(b - a), g.half[k]);
    }
}

template<class K, class T>
int geoCenters(cudaStream_t s, const K* prefixes, int N, T* centers, T* sizes, const cs_box& box, int kind,
               const int* Ldev)
{
    if (N <= 0) return CS_OK;
    auto bp = makeBoxParams<T>(box);
    GeoParams<T> g;
    const T uL = T(1) / T(int(1u << KeyTraits<K>::maxLevel));
    for (int k = 0; k < 3; ++k)
    {
        g.lo[k]   = bp.lo[k];
        g.half[k] = T(0.5) * uL * bp.len[k];
    }
    if (kind == CS_HILBERT)
        geoCentersKernel<K, T, CS_HILBERT><<<iceil(N, 256), 256, 0, s>>>(prefixes, N, Ldev, centers, sizes, g);
    else geoCentersKernel<K, T, CS_MORTON><<<iceil(N, 256), 256, 0, s>>>(prefixes, N, Ldev, centers, sizes, g);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

// batched sets in one 64-bit tree: node key = (set << 30) | the set's 32-bit key, set roots at level rootLevel; every
// node at or below a set root gets the geometry the set's own 32-bit tree gives it (its box, its levels); the nodes
// above the set roots and the empty filler nodes get a zero box (never traversed)
template<class T, int Kind>
__global__ void geoCentersBatchKernel(const uint64_t* __restrict__ prefixes, int N, T* __restrict__ centers,
                                      T* __restrict__ sizes, const GeoParams<T>* __restrict__ sets, int numSets,
                                      unsigned rootLevel)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    uint64_t prefix = prefixes[i];
    uint64_t start  = decodePlaceholderBit<uint64_t>(prefix);
    unsigned level  = decodePrefixLength<uint64_t>(prefix) / 3;
    uint64_t set    = start >> 30;
    if (level < rootLevel || set >= uint64_t(numSets))
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
            centers[3 * size_t(i) + k] = sizes[3 * size_t(i) + k] = T(0);
        return;
    }
    const uint32_t rel = uint32_t(start & ((uint64_t(1) << 30) - 1));
    unsigned cube      = (1u << KeyTraits<uint32_t>::maxLevel) >> (level - rootLevel);
    unsigned ix, iy, iz;
    if (Kind == CS_HILBERT)
    {
        decodeHilbert<uint32_t>(rel, ix, iy, iz);
        unsigned mask = ~(cube - 1u);
        ix &= mask;
        iy &= mask;
        iz &= mask;
    }
    else { decodeMorton<uint32_t>(rel, ix, iy, iz); }
    const GeoParams<T> g = sets[set];
    unsigned imin[3]     = {ix, iy, iz};
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int a0                     = int(imin[k]);
        int b0                     = a0 + int(cube);
        centers[3 * size_t(i) + k] = RN<T>::add(g.lo[k], RN<T>::mul(T(b0 + a0), g.half[k]));
        sizes[3 * size_t(i) + k]   = RN<T>::mul(T(b0 - a0), g.half[k]);
    }
}

template<class T>
size_t geoParamsBytes(int numSets)
{
    return size_t(numSets) * sizeof(GeoParams<T>) + 256;
}

template<class T>
int geoCentersBatched(cudaStream_t s, const uint64_t* prefixes, int N, T* centers, T* sizes, const cs_box* boxes,
                      int numSets, int kind, void* paramsDev, unsigned rootLevel)
{
    if (N <= 0) return CS_OK;
    std::vector<GeoParams<T>> g(numSets);
    const T uL = T(1) / T(int(1u << KeyTraits<uint32_t>::maxLevel));
    for (int j = 0; j < numSets; ++j)
    {
        auto bp = makeBoxParams<T>(boxes[j]);
        for (int k = 0; k < 3; ++k)
        {
            g[j].lo[k]   = bp.lo[k];
            g[j].half[k] = T(0.5) * uL * bp.len[k];
        }
    }
    auto* gd = static_cast<GeoParams<T>*>(paramsDev);
    CSG_CUDA_TRY(cudaMemcpyAsync(gd, g.data(), g.size() * sizeof(GeoParams<T>), cudaMemcpyHostToDevice, s));
    if (kind == CS_HILBERT)
        geoCentersBatchKernel<T, CS_HILBERT><<<iceil(N, 256), 256, 0, s>>>(prefixes, N, centers, sizes, gd, numSets,
                                                                           rootLevel);
    else
        geoCentersBatchKernel<T, CS_MORTON><<<iceil(N, 256), 256, 0, s>>>(prefixes, N, centers, sizes, gd, numSets,
                                                                          rootLevel);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template size_t geoParamsBytes<float>(int);
template size_t geoParamsBytes<double>(int);
template int geoCentersBatched<float>(cudaStream_t, const uint64_t*, int, float*, float*, const cs_box*, int, int,
                                      void*, unsigned);
template int geoCentersBatched<double>(cudaStream_t, const uint64_t*, int, double*, double*, const cs_box*, int, int,
                                       void*, unsigned);

template int geoCenters<uint32_t, float>(cudaStream_t, const uint32_t*, int, float*, float*, const cs_box&, int,
                                         const int*);
template int geoCenters<uint32_t, double>(cudaStream_t, const uint32_t*, int, double*, double*, const cs_box&, int,
                                          const int*);
template int geoCenters<uint64_t, float>(cudaStream_t, const uint64_t*, int, float*, float*, const cs_box&, int,
                                         const int*);
template int geoCenters<uint64_t, double>(cudaStream_t, const uint64_t*, int, double*, double*, const cs_box&, int,
                                          const int*);

} // namespace csg

using namespace csg;

extern "C" size_t cs_build_octree_workspace_bytes(int32_t num_leaves, int key_bits)
{
    return key_bits == 32 ? buildLinkWorkspaceBytes<uint32_t>(num_leaves) : buildLinkWorkspaceBytes<uint64_t>(num_leaves);
}

template<class K>
static int buildOctreeEntry(cs_stream_t stream, const K* leaves, int32_t L, const cs_octree_view* view,
                            int32_t* levelRangeHost, void* ws, size_t wsb)
{
    if (!leaves || !view || !view->prefixes || !view->child_offsets || !view->parents || !view->level_range ||
        !view->internal_to_leaf || !view->leaf_to_internal)
    {
        setLastError("build octree: null pointer");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    Workspace w;
    size_t need = buildLinkWorkspaceBytes<K>(L);
    int rc      = w.acquire(ws, wsb, need, s);
    if (rc) return rc;
    rc = buildLink<K>(s, leaves, L, *view, 0, w.ptr, need, nullptr);
    if (rc) return rc;
    if (levelRangeHost)
    {
        CSG_CUDA_TRY(cudaMemcpyAsync(levelRangeHost, view->level_range, (KeyTraits<K>::maxLevel + 2) * sizeof(int32_t),
                                     cudaMemcpyDeviceToHost, s));
        CSG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return CS_OK;
}

extern "C" int cs_build_octree_u32(cs_stream_t stream, const uint32_t* leaves, int32_t L, const cs_octree_view* view,
                                   int32_t* lr, void* ws, size_t wsb)
{
    return buildOctreeEntry<uint32_t>(stream, leaves, L, view, lr, ws, wsb);
}
extern "C" int cs_build_octree_u64(cs_stream_t stream, const uint64_t* leaves, int32_t L, const cs_octree_view* view,
                                   int32_t* lr, void* ws, size_t wsb)
{
    return buildOctreeEntry<uint64_t>(stream, leaves, L, view, lr, ws, wsb);
}

#define CS_GEO_ENTRY(kb, K, tb, T)                                                                                     \
    extern "C" int cs_geo_centers_##kb##_##tb(cs_stream_t stream, const K* prefixes, int32_t n, T* c, T* sz,           \
                                              const cs_box* box, int kind)                                             \
    {                                                                                                                  \
        if (!box || (n > 0 && (!prefixes || !c || !sz)))                                                               \
        {                                                                                                              \
            setLastError("geo centers: null pointer");                                                                 \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        return geoCenters<K, T>(cudaStream_t(stream), prefixes, n, c, sz, *box, kind);                                \
    }
CS_GEO_ENTRY(u32, uint32_t, f32, float)
CS_GEO_ENTRY(u32, uint32_t, f64, double)
CS_GEO_ENTRY(u64, uint64_t, f32, float)
CS_GEO_ENTRY(u64, uint64_t, f64, double)
