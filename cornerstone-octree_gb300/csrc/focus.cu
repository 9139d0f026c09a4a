// Focus (locally essential) tree helpers around findHalos: rebalance decisions that combine particle counts with
// multipole-acceptance flags, refinement by MAC alone, ancestor protection, mandatory keys, counts of focus leaves
// from a coarser global tree, and the particle layout of the present (assigned + halo) focus leaves.
//
// All of it is integer work and equals the reference bit for bit:
//  - rebalanceDecisionEssential    mergeCountAndMacOp per node          (focus/rebalance.hpp:31-73, rebalance_gpu.cu:30-70)
//  - macRefineDecision             macRefineOp per leaf outside the focus (focus/rebalance.hpp:76-82, rebalance_gpu.cu:72-98)
//  - protectAncestors              nzAncestorOp per node, in place       (focus/rebalance.hpp:96-181, rebalance_gpu.cu:100-145)
//  - enforceKeys                   enforceKeySingle per mandatory key    (focus/rebalance.hpp:183-261, rebalance_gpu.cu:147-185)
//  - rangeCount                    counts summed over global leaves      (focus/rebalance.hpp:263-286, rebalance_gpu.cu:187-225)
//  - computeNodeLayout             masked counts + exclusive scan        (domain/layout.hpp:154-186)
//
// Differences in structure: protectAncestors counts the changed nodes with a warp reduction and one atomic per
// warp into a caller-visible word instead of a module-global device variable (so concurrent calls on different
// streams do not share state); enforceKeys processes the keys in their given order in one warp, each key's sibling
// loops spread over the lanes, which gives the reference's sequential result (the reference's one-block-per-key
// kernel lets two keys that touch the same node race).
#include "cs_common.cuh"

namespace csg
{

int exclusiveScanI32(cudaStream_t s, const int32_t* in, int32_t* out, size_t n, int32_t init, void* ws, size_t wsb);
size_t exclusiveScanWorkspaceBytes(size_t n);

template<class K>
__device__ int mergeCountAndMacOp(int i, const K* prefixes, const int32_t* childOffsets, const int32_t* parents,
                                  const uint32_t* counts, const uint8_t* macs, K focusStart, K focusEnd,
                                  unsigned bucket)
{
    constexpr unsigned ML = KeyTraits<K>::maxLevel;
    const K key           = prefixes[i];
    const unsigned level  = decodePrefixLength<K>(key) / 3;
    if (i)
    {
        int parent      = parents[(i - 1) / 8];
        bool countMerge = counts[parent] <= bucket;
        bool macMerge   = macs[parent] == 0;
        K firstKey      = decodePlaceholderBit<K>(prefixes[parent]);
        K lastKey       = firstKey + 8 * nodeRange<K>(level);
        bool inFringe   = lastKey > focusStart && focusEnd > firstKey;
        if (countMerge || (macMerge && !inFringe)) return 0;
    }
    K start      = decodePlaceholderBit<K>(key);
    bool isLeaf  = childOffsets[i] == 0;
    bool inFocus = start >= focusStart && start < focusEnd;
    if (isLeaf && (macs[i] || inFocus))
    {
        uint32_t c = counts[i];
        if (level + 3 < ML && c > 4096u * bucket) return 4096;
        if (level + 2 < ML && c > 512u * bucket) return 512;
        if (level + 1 < ML && c > 64u * bucket) return 64;
        if (level < ML && c > bucket) return 8;
    }
    return 1;
}

template<class K>
__global__ void essentialKernel(const K* prefixes, const int32_t* childOffsets, const int32_t* parents,
                                const uint32_t* counts, const uint8_t* macs, K f0, K f1, unsigned bucket,
                                int32_t* ops, int numNodes)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < numNodes) ops[i] = mergeCountAndMacOp<K>(i, prefixes, childOffsets, parents, counts, macs, f0, f1, bucket);
}

template<class K>
__global__ void macRefineKernel(const K* prefixes, const uint8_t* macs, const int32_t* l2i, int numLeaves, int f0,
                                int f1, int32_t* ops)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numLeaves) return;
    if (i < f0 || i >= f1)
    {
        int n          = l2i[i];
        unsigned level = decodePrefixLength<K>(prefixes[n]) / 3;
        ops[i]         = (level < unsigned(KeyTraits<K>::maxLevel) && macs[n]) ? 8 : 1;
    }
    else ops[i] = 1;
}

// nzAncestorOp: in place; another thread may rewrite an ancestor's op meanwhile, but every outcome is the same (an
// ancestor becomes nonzero only when it starts where its closest nonzero ancestor starts)
template<class K>
__global__ void protectKernel(const K* prefixes, const int32_t* parents, int32_t* ops, int numNodes, int* changed)
{
    int i  = blockIdx.x * blockDim.x + threadIdx.x;
    int op = 1;
    if (i < numNodes)
    {
        if (i == 0) op = ops[0];
        else
        {
            volatile int32_t* vo = ops;
            int a                = i;
            while (vo[a] == 0)
                a = parents[(a - 1) / 8];
            op = decodePlaceholderBit<K>(prefixes[i]) == decodePlaceholderBit<K>(prefixes[a]) ? vo[a] : 0;
        }
        ops[i] = op;
    }
    unsigned m = __ballot_sync(0xffffffffu, op != 1);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(changed, __popc(m));
}

// containingNode (tree/octree.hpp:199-215)
template<class K>
__device__ int containingNode(K nodeKey, const K* prefixes, const int32_t* childOffsets)
{
    int level = int(decodePrefixLength<K>(nodeKey)) / 3;
    K key     = decodePlaceholderBit<K>(nodeKey);
    int ret   = 0;
    for (int i = 1; i <= level; ++i)
    {
        if (childOffsets[ret] == 0 || nodeKey == prefixes[ret]) break;
        ret = childOffsets[ret] + int(octalDigit<K>(key, unsigned(i)));
    }
    return ret;
}

template<class K>
__device__ __forceinline__ int lastNzPlaceF(K x)
{
    return x ? KeyTraits<K>::maxLevel - ctzKey<K>(x) / 3 : KeyTraits<K>::maxLevel;
}

// one warp, the keys in order (the reference's sequential semantics); status: max over keys of
// 0 converged, 1 cancelMerge, 2 rebalance, 3 failed
template<class K>
__global__ void enforceKeysKernel(const K* keys, int numKeys, const K* prefixes, const int32_t* childOffsets,
                                  const int32_t* parents, int32_t* ops, int* status)
{
    const int lane = threadIdx.x;
    int worst      = 0;
    for (int k = 0; k < numKeys; ++k)
    {
        K key = keys[k];
        int st = 0;
        if (!(key == 0 || key == nodeRange<K>(0)))
        {
            K want       = key ? encodePlaceholderBit<K>(key, 3 * lastNzPlaceF<K>(key)) : K(1);
            int idx      = containingNode<K>(want, prefixes, childOffsets);
            K have       = prefixes[idx];
            int lvHave   = int(decodePrefixLength<K>(have)) / 3;
            bool trySplit = have != want && lvHave < KeyTraits<K>::maxLevel;
            bool undo     = ops[idx] == 0 || trySplit;
            __syncwarp();
            if (undo && idx > 0)
            {
                st         = 1;
                int parent = idx;
                do
                {
                    parent    = parents[(parent - 1) / 8];
                    int first = childOffsets[parent];
                    if (lane < 8 && ops[first + lane] == 0) ops[first + lane] = 1;
                    __syncwarp();
                } while (parent != 0);
            }
            if (trySplit)
            {
                int diff = lastNzPlaceF<K>(key) - lvHave;
                st       = diff > 1 ? 3 : 2;
                diff     = diff > 1 ? 1 : diff;
                int want_op = 1 << (3 * diff);
                if (lane == 0 && ops[idx] < want_op) ops[idx] = want_op;
                __syncwarp();
            }
        }
        worst = st > worst ? st : worst;
    }
    if (lane == 0) *status = worst;
}

template<class K>
__global__ void rangeCountKernel(const K* leaves, int numLeafKeys, const uint32_t* counts, const K* focus,
                                 const int32_t* idx, int nIdx, uint32_t* out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nIdx) return;
    int li  = idx[i];
    K start = focus[li], end = focus[li + 1];
    // findNodeBelow: upper_bound - 1; findNodeAbove: lower_bound
    int lo = 0, hi = numLeafKeys;
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (leaves[mid] <= start) lo = mid + 1;
        else hi = mid;
    }
    int s = lo - 1;
    lo = 0, hi = numLeafKeys;
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (leaves[mid] < end) lo = mid + 1;
        else hi = mid;
    }
    int e                  = lo;
    unsigned long long sum = 0;
    for (int j = max(s, 0); j < e; ++j)
        sum += counts[j];
    out[li] = uint32_t(min(sum, 0xFFFFFFFFull));
}

__global__ void layoutMaskKernel(const uint32_t* counts, int numLeaves, const uint8_t* flags, const int32_t* l2i,
                                 int first, int last, int32_t* masked)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < numLeaves)
    {
        bool have = (first <= i && i < last) || flags[l2i[i]];
        masked[i] = have ? int32_t(counts[i]) : 0;
    }
    else if (i == numLeaves) masked[i] = 0;
}

} // namespace csg

using namespace csg;

#define CS_FOCUS_ENTRIES(SUF, K)                                                                                       \
    extern "C" int cs_rebalance_decision_essential_##SUF(                                                              \
        cs_stream_t stream, const K* prefixes, const int32_t* child_offsets, const int32_t* parents,                   \
        const uint32_t* counts, const uint8_t* macs, K focus_start, K focus_end, unsigned bucket, int32_t* node_ops,   \
        int32_t num_nodes)                                                                                             \
    {                                                                                                                  \
        if (num_nodes <= 0) return CS_OK;                                                                              \
        if (!prefixes || !child_offsets || (!parents && num_nodes > 1) || !counts || !macs || !node_ops)              \
        {                                                                                                              \
            setLastError("rebalance decision essential: null pointer");                                                \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        essentialKernel<K><<<iceil(size_t(num_nodes), 256), 256, 0, cudaStream_t(stream)>>>(                          \
            prefixes, child_offsets, parents, counts, macs, focus_start, focus_end, bucket, node_ops, num_nodes);      \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }                                                                                                                  \
    extern "C" int cs_mac_refine_decision_##SUF(cs_stream_t stream, const K* prefixes, const uint8_t* macs,           \
                                               const int32_t* leaf_to_internal, int32_t num_leaves,                   \
                                               int32_t focus_first, int32_t focus_last, int32_t* node_ops)            \
    {                                                                                                                  \
        if (num_leaves <= 0) return CS_OK;                                                                             \
        if (!prefixes || !macs || !leaf_to_internal || !node_ops)                                                      \
        {                                                                                                              \
            setLastError("mac refine decision: null pointer");                                                         \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        macRefineKernel<K><<<iceil(size_t(num_leaves), 256), 256, 0, cudaStream_t(stream)>>>(                         \
            prefixes, macs, leaf_to_internal, num_leaves, focus_first, focus_last, node_ops);                          \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }                                                                                                                  \
    extern "C" int cs_protect_ancestors_##SUF(cs_stream_t stream, const K* prefixes, const int32_t* parents,          \
                                             int32_t* node_ops, int32_t num_nodes, int* changed_dev,                  \
                                             int* converged_host)                                                      \
    {                                                                                                                  \
        if (num_nodes <= 0)                                                                                            \
        {                                                                                                              \
            if (converged_host) *converged_host = 1;                                                                   \
            return CS_OK;                                                                                              \
        }                                                                                                              \
        if (!prefixes || (!parents && num_nodes > 1) || !node_ops || !changed_dev)                                     \
        {                                                                                                              \
            setLastError("protect ancestors: null pointer");                                                           \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        cudaStream_t s = cudaStream_t(stream);                                                                         \
        CSG_CUDA_TRY(cudaMemsetAsync(changed_dev, 0, sizeof(int), s));                                                 \
        protectKernel<K><<<iceil(size_t(num_nodes), 256), 256, 0, s>>>(prefixes, parents, node_ops, num_nodes,        \
                                                                        changed_dev);                                  \
        CSG_CHECK_LAUNCH();                                                                                            \
        if (converged_host)                                                                                            \
        {                                                                                                              \
            int h = 0;                                                                                                 \
            CSG_CUDA_TRY(cudaMemcpyAsync(&h, changed_dev, sizeof(int), cudaMemcpyDeviceToHost, s));                    \
            CSG_CUDA_TRY(cudaStreamSynchronize(s));                                                                    \
            *converged_host = h == 0;                                                                                  \
        }                                                                                                              \
        return CS_OK;                                                                                                  \
    }                                                                                                                  \
    extern "C" int cs_enforce_keys_##SUF(cs_stream_t stream, const K* forced_keys, int32_t num_forced,                \
                                        const K* prefixes, const int32_t* child_offsets, const int32_t* parents,      \
                                        int32_t* node_ops, int* status_dev, int* status_host)                         \
    {                                                                                                                  \
        if (num_forced < 0 || (num_forced && (!forced_keys || !prefixes || !child_offsets || !parents || !node_ops)) || \
            !status_dev)                                                                                               \
        {                                                                                                              \
            setLastError("enforce keys: invalid arguments");                                                           \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        cudaStream_t s = cudaStream_t(stream);                                                                         \
        enforceKeysKernel<K><<<1, 32, 0, s>>>(forced_keys, num_forced, prefixes, child_offsets, parents, node_ops,    \
                                              status_dev);                                                             \
        CSG_CHECK_LAUNCH();                                                                                            \
        if (status_host)                                                                                               \
        {                                                                                                              \
            CSG_CUDA_TRY(cudaMemcpyAsync(status_host, status_dev, sizeof(int), cudaMemcpyDeviceToHost, s));            \
            CSG_CUDA_TRY(cudaStreamSynchronize(s));                                                                    \
        }                                                                                                              \
        return CS_OK;                                                                                                  \
    }                                                                                                                  \
    extern "C" int cs_range_count_##SUF(cs_stream_t stream, const K* leaves, int32_t num_leaf_keys,                   \
                                       const uint32_t* counts, const K* leaves_focus, const int32_t* focus_idx,       \
                                       int32_t num_idx, uint32_t* counts_focus)                                       \
    {                                                                                                                  \
        if (num_idx <= 0) return CS_OK;                                                                                \
        if (!leaves || !counts || !leaves_focus || !focus_idx || !counts_focus || num_leaf_keys < 2)                  \
        {                                                                                                              \
            setLastError("range count: invalid arguments");                                                            \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        rangeCountKernel<K><<<iceil(size_t(num_idx), 64), 64, 0, cudaStream_t(stream)>>>(                             \
            leaves, num_leaf_keys, counts, leaves_focus, focus_idx, num_idx, counts_focus);                            \
        CSG_CHECK_LAUNCH();                                                                                            \
        return CS_OK;                                                                                                  \
    }

CS_FOCUS_ENTRIES(u32, uint32_t)
CS_FOCUS_ENTRIES(u64, uint64_t)

extern "C" size_t cs_node_layout_workspace_bytes(int32_t num_leaves)
{
    return (size_t(num_leaves) + 1) * 4 + exclusiveScanWorkspaceBytes(size_t(num_leaves) + 1) + 512;
}

extern "C" int cs_node_layout(cs_stream_t stream, const uint32_t* focus_leaf_counts, int32_t num_leaves,
                              const uint8_t* flags, const int32_t* leaf_to_internal, int32_t first, int32_t last,
                              uint32_t* layout, void* ws, size_t wsb)
{
    if (num_leaves < 0 || !layout || (num_leaves && (!focus_leaf_counts || !flags || !leaf_to_internal)))
    {
        setLastError("node layout: invalid arguments");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    size_t need    = cs_node_layout_workspace_bytes(num_leaves);
    Workspace w;
    int rc = w.acquire(ws, wsb, need, s);
    if (rc) return rc;
    Arena ar{static_cast<char*>(w.ptr), 0, need};
    int32_t* masked  = ar.take<int32_t>(size_t(num_leaves) + 1);
    size_t scanBytes = exclusiveScanWorkspaceBytes(size_t(num_leaves) + 1);
    void* sws        = ar.take<char>(scanBytes);
    layoutMaskKernel<<<iceil(size_t(num_leaves) + 1, 256), 256, 0, s>>>(focus_leaf_counts, num_leaves, flags,
                                                                        leaf_to_internal, first, last, masked);
    CSG_CHECK_LAUNCH();
    return exclusiveScanI32(s, masked, reinterpret_cast<int32_t*>(layout), size_t(num_leaves) + 1, 0, sws, scanBytes);
}
