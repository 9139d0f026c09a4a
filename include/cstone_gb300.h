/*
 * cstone_gb300 — C ABI of the GB300 (sm_103a) implementation of cornerstone-octree's single-GPU octree path:
 * SFC keys -> stable key sort -> cornerstone leaf build/update -> internal-tree link -> node geometry ->
 * findHalos -> findNeighbors.
 *
 * Conventions
 *  - Every entry point is stream-ordered on `stream` (a cudaStream_t passed as void*, NULL = legacy default stream)
 *    and returns a status code (CS_OK = 0). cs_last_error() describes the last failure of the calling thread.
 *  - All array arguments are device pointers owned by the caller, except where a name ends in `_host`.
 *  - No entry point keeps global device state, so calls on different streams may run concurrently.
 *  - Entry points that need temporary device memory take (workspace, workspace_bytes) and have a *_workspace_bytes
 *    query; passing workspace == NULL makes the call allocate stream-ordered memory (cudaMallocAsync) itself.
 *  - Key arrays hold 32-bit (u32) or 64-bit (u64) SFC keys, coordinates are float (f32) or double (f64).
 *  - Node arrays follow cstone::OctreeView (tree/octree.hpp:233-283): level-sorted node order, placeholder-bit
 *    prefixes, childOffsets (0 = leaf), parents per group of 8 siblings, levelRange of maxTreeLevel + 2 entries.
 *
 * Each declaration cites the reference interface it replaces (path:line within the reference project).
 */
#ifndef CSTONE_GB300_H
#define CSTONE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* cs_stream_t;

enum cs_status
{
    CS_OK           = 0,
    CS_ERR_INVALID  = 1, /* bad argument (size, pointer, bucket size ...) */
    CS_ERR_CAPACITY = 2, /* an output buffer is too small; the required size is reported */
    CS_ERR_CUDA     = 3, /* a CUDA runtime call failed */
    CS_ERR_TIMEOUT  = 4, /* a bounded device-side wait gave up (look-back or grid barrier) */
    CS_ERR_DEVICE   = 5  /* a device-side consistency check failed */
};

/* SFC kind: cstone::MortonKey / cstone::HilbertKey (sfc/sfc.hpp:31-40) */
enum cs_sfc_kind
{
    CS_MORTON  = 0,
    CS_HILBERT = 1
};

/* cstone::BoundaryType (sfc/box.hpp:77-83) */
enum cs_boundary
{
    CS_OPEN       = 0,
    CS_PERIODIC   = 1,
    CS_FIXED      = 2,
    CS_CUBIC_OPEN = 3
};

/* cstone::Box<T> (sfc/box.hpp:96-175). Limits are given in double; f32 entry points convert them to float and derive
 * lengths and inverse lengths in float, as Box<float> does. */
typedef struct
{
    double lo[3];
    double hi[3];
    int boundary[3];
} cs_box;

/* cstone::OctreeView<KeyType> (tree/octree.hpp:233-253), device pointers, sized as OctreeData::resize
 * (tree/octree.hpp:293-308): num_internal_nodes = (L-1)/7, num_nodes = L + num_internal_nodes,
 * prefixes/internal_to_leaf/leaf_to_internal: num_nodes, child_offsets: num_nodes + 1,
 * parents: max(1, (num_nodes-1)/8), level_range: maxTreeLevel + 2 (12 for u32, 23 for u64). */
typedef struct
{
    int32_t num_leaf_nodes;
    int32_t num_internal_nodes;
    int32_t num_nodes;
    void* prefixes; /* uint32_t* or uint64_t* */
    int32_t* child_offsets;
    int32_t* parents;
    int32_t* level_range;
    int32_t* internal_to_leaf;
    int32_t* leaf_to_internal;
} cs_octree_view;

/* cstone::OctreeNsView<T, KeyType> (tree/octree.hpp:255-283): what findNeighbors reads */
typedef struct
{
    int32_t num_leaf_nodes;
    int32_t num_nodes;
    const int32_t* child_offsets;
    const int32_t* parents;
    const int32_t* internal_to_leaf;
    const uint32_t* layout; /* first particle of each leaf, num_leaf_nodes + 1 entries */
    const void* centers;    /* 3 * num_nodes of T (node geometric centres) */
    const void* sizes;      /* 3 * num_nodes of T (node half sizes) */
    float search_ext_factor;
} cs_ns_view;

const char* cs_last_error(void);
int cs_version(void);

/* ---- bounded device-side waits --------------------------------------------------------------------------------
 * No counterpart in the reference (its CUB look-back and host-synchronised build loop never give up). The sort's
 * decoupled look-back and the cooperative build's grid barrier spin on flags that other blocks publish; each wait
 * gives up after a bounded number of polls, sets an error bit, and the call returns CS_ERR_TIMEOUT without writing
 * outside its buffers (the results of that call are then unspecified). cs_set_wait_limits sets the bounds for the
 * whole process (0 = default: 2^22 look-back rounds, 2^24 barrier polls) and, for tests, makes one wait stall on a
 * flag that nothing sets: CS_WAIT_STALL_SORT (tile 1 of every sort pass waits for its predecessor),
 * CS_WAIT_STALL_BARRIER (block 0 of every cooperative build never arrives at the first barrier). Kernels read the
 * values when they are launched; CUDA graphs keep the values they were captured with. */
#define CS_WAIT_STALL_SORT 1
#define CS_WAIT_STALL_BARRIER 2
int cs_set_wait_limits(uint32_t sort_spins, uint32_t barrier_spins, int stall);

/* ---- SFC keys ----------------------------------------------------------------------------------------------
 * replaces computeSfcKeys(execution::Gpu, x, y, z, keys, n, box) (sfc/sfc_gpu.h:24-26, kernel sfc/sfc_gpu.cu:23-44).
 * respect_remove_key = 1 keeps keys that equal removeKey (2^30 / 2^63) untouched, as the reference kernel does;
 * 0 writes every key without reading the key array first. */
int cs_sfc_keys_hilbert_u32_f32(cs_stream_t stream, const float* x, const float* y, const float* z, uint32_t* keys,
                                size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_hilbert_u32_f64(cs_stream_t stream, const double* x, const double* y, const double* z, uint32_t* keys,
                                size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_hilbert_u64_f32(cs_stream_t stream, const float* x, const float* y, const float* z, uint64_t* keys,
                                size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_hilbert_u64_f64(cs_stream_t stream, const double* x, const double* y, const double* z, uint64_t* keys,
                                size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_morton_u32_f32(cs_stream_t stream, const float* x, const float* y, const float* z, uint32_t* keys,
                               size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_morton_u32_f64(cs_stream_t stream, const double* x, const double* y, const double* z, uint32_t* keys,
                               size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_morton_u64_f32(cs_stream_t stream, const float* x, const float* y, const float* z, uint64_t* keys,
                               size_t n, const cs_box* box, int respect_remove_key);
int cs_sfc_keys_morton_u64_f64(cs_stream_t stream, const double* x, const double* y, const double* z, uint64_t* keys,
                               size_t n, const cs_box* box, int respect_remove_key);

/* ---- stable key sort ----------------------------------------------------------------------------------------
 * replaces sortByKeyTempStorage / sortByKey(exec, keys, values, keyBuf, valueBuf) (primitives/primitives_gpu.h:118-155,
 * CUB SortPairs in primitives/primitives_gpu.cu:310-356). Stable LSD radix sort (onesweep, decoupled look-back) of
 * bits [begin_bit, end_bit); keys_alt/values_alt are ping-pong buffers of n elements. The sorted result is left in
 * keys/values. values_are_iota = 1 ignores the input values and sorts the permutation 0..n-1 (the `sequence` +
 * sortByKey idiom of the reference's callers). n must be below 2^30. */
size_t cs_sort_pairs_workspace_bytes(size_t n, int key_bits);
int cs_sort_pairs_u32(cs_stream_t stream, uint32_t* keys, uint32_t* values, size_t n, uint32_t* keys_alt,
                      uint32_t* values_alt, int begin_bit, int end_bit, int values_are_iota, void* workspace,
                      size_t workspace_bytes);
int cs_sort_pairs_u64(cs_stream_t stream, uint64_t* keys, uint32_t* values, size_t n, uint64_t* keys_alt,
                      uint32_t* values_alt, int begin_bit, int end_bit, int values_are_iota, void* workspace,
                      size_t workspace_bytes);

/* No counterpart in the reference. The same stable sort of u64 keys for callers that cannot allocate device memory
 * when they sort (all device memory reserved up front by the host application's own pool, or a time-step loop that
 * cannot afford cudaMalloc/cudaFree's implicit device synchronisation). Every temporary lives in one fixed
 * file-scope device array, held by each device that loads the library until the process exits; the caller passes
 * only keys and values, sorted in place. At most CS_SORT_NOALLOC_MAX_N keys (larger n: CS_ERR_INVALID). All calls
 * share that array: calls that overlap on the GPU race, so serialise them. CUDA loads modules lazily by default, so
 * the array and the sort kernels reach device memory on first use: call once with n = 0 per device, with that device
 * current, before reserving the pool (or run with CUDA_MODULE_LOADING=EAGER). Every call reads the sort's error word
 * back and synchronises the stream before it returns, so it cannot be recorded into a CUDA graph; a call on a stream
 * that is being captured returns CS_ERR_INVALID. */
#define CS_SORT_NOALLOC_MAX_N 262144
int cs_sort_pairs_noalloc_u64(cs_stream_t stream, uint64_t* keys, uint32_t* values, size_t n, int begin_bit,
                              int end_bit, int values_are_iota);

/* ---- permutation gather --------------------------------------------------------------------------------------
 * replaces gather(exec, ordering, in, out) / gatherArrays (primitives/primitives_gpu.cu:74-90, domain/layout.hpp:231).
 * out[i] = in[perm[i]] for i < n. The 4-array form gathers x, y, z, h in one pass. */
int cs_gather_f32(cs_stream_t stream, const uint32_t* perm, const float* in, float* out, size_t n);
int cs_gather_f64(cs_stream_t stream, const uint32_t* perm, const double* in, double* out, size_t n);
int cs_gather4_f64(cs_stream_t stream, const uint32_t* perm, size_t n, const double* in0, const double* in1,
                   const double* in2, const double* in3, double* out0, double* out1, double* out2, double* out3);
int cs_gather4_f32(cs_stream_t stream, const uint32_t* perm, size_t n, const float* in0, const float* in1,
                   const float* in2, const float* in3, float* out0, float* out1, float* out2, float* out3);

/* ---- cornerstone leaf array -----------------------------------------------------------------------------------
 * cs_node_counts replaces computeNodeCountsGpu(exec, tree, counts, numNodes, keys, maxCount, useCountsAsGuess)
 * (tree/csarray_gpu.h:41-47, tree/csarray_gpu.cu:86-122): counts[i] = min(#keys in [tree[i], tree[i+1]), max_count).
 * With use_counts_as_guess the input counts seed an exponential search, as updateNodeCount does. */
size_t cs_node_counts_workspace_bytes(int32_t num_nodes);
int cs_node_counts_u32(cs_stream_t stream, const uint32_t* tree, uint32_t* counts, int32_t num_nodes,
                       const uint32_t* keys, size_t n, uint32_t max_count, int use_counts_as_guess, void* workspace,
                       size_t workspace_bytes);
int cs_node_counts_u64(cs_stream_t stream, const uint64_t* tree, uint32_t* counts, int32_t num_nodes,
                       const uint64_t* keys, size_t n, uint32_t max_count, int use_counts_as_guess, void* workspace,
                       size_t workspace_bytes);

/* cs_rebalance_decision replaces computeNodeOpsGpu's decision half (rebalanceDecisionKernel,
 * tree/csarray_gpu.cu:151-162): ops[i] in {0,1,8,64,512,4096} for i < num_nodes; *converged_dev (device int) is
 * set to 1 if every op is 1, else 0. */
int cs_rebalance_decision_u32(cs_stream_t stream, const uint32_t* tree, const uint32_t* counts, int32_t num_nodes,
                              unsigned bucket_size, int32_t* ops, int* converged_dev);
int cs_rebalance_decision_u64(cs_stream_t stream, const uint64_t* tree, const uint32_t* counts, int32_t num_nodes,
                              unsigned bucket_size, int32_t* ops, int* converged_dev);

/* cs_exclusive_scan_i32 replaces exclusiveScan(exec, first, last, output, init) (primitives/primitives_gpu.h:158-160)
 * for int32: out[i] = init + in[0] + ... + in[i-1] for i < n; out == in is allowed. workspace may be NULL (then
 * it is allocated stream-ordered). With the decision ops of cs_rebalance_decision (num_nodes + 1 entries, the last
 * one ignored) it gives computeNodeOpsGpu's scanned ops (tree/csarray_gpu.cu:172-196), whose last entry is the new
 * leaf count.
 * cs_rebalance_tree replaces rebalanceTreeGpu's emission (processNodes, tree/csarray_gpu.cu:166-231): new_tree
 * receives node_ops[num_nodes] + 1 keys, the last one the end key 8^maxLevel. */
size_t cs_exclusive_scan_workspace_bytes(size_t n);
int cs_exclusive_scan_i32(cs_stream_t stream, const int32_t* in, int32_t* out, size_t n, int32_t init, void* workspace,
                          size_t workspace_bytes);
int cs_rebalance_tree_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes, const int32_t* node_ops,
                          uint32_t* new_tree);
int cs_rebalance_tree_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes, const int32_t* node_ops,
                          uint64_t* new_tree);

/* cs_compute_octree replaces computeOctree / the `while(!updateOctreeGpu(...))` build loop (tree/csarray.hpp:429-440,
 * tree/update_gpu.cuh:43-68). Builds the converged cornerstone leaf array of the sorted keys from the root in one
 * cooperative launch (no host round trip per iteration). tree must hold capacity+1 keys, counts capacity entries,
 * layout (optional, may be NULL) capacity+1 entries = first particle of each leaf. *num_leaves_host receives L; on
 * CS_ERR_CAPACITY it receives the number of leaves that did not fit. *iterations_host (may be NULL) receives the
 * number of updateOctree steps the reference loop would take. */
size_t cs_compute_octree_workspace_bytes(int32_t capacity);
int cs_compute_octree_u32(cs_stream_t stream, const uint32_t* keys, size_t n, unsigned bucket_size,
                          uint32_t max_count, uint32_t* tree, uint32_t* counts, uint32_t* layout, int32_t capacity,
                          int32_t* num_leaves_host, int* iterations_host, void* workspace, size_t workspace_bytes);
int cs_compute_octree_u64(cs_stream_t stream, const uint64_t* keys, size_t n, unsigned bucket_size,
                          uint32_t max_count, uint64_t* tree, uint32_t* counts, uint32_t* layout, int32_t capacity,
                          int32_t* num_leaves_host, int* iterations_host, void* workspace, size_t workspace_bytes);

/* cs_update_octree replaces one updateOctree / updateOctreeGpu step (tree/csarray.hpp:408-426,
 * tree/update_gpu.cuh:43-68): decision on counts_in, rebalance, recount of tree_out against keys (guessed search).
 * *num_leaves_out_host receives the new leaf count, *converged_host whether the decision changed nothing. */
size_t cs_update_octree_workspace_bytes(int32_t num_leaves_in, int32_t capacity);
int cs_update_octree_u32(cs_stream_t stream, const uint32_t* keys, size_t n, unsigned bucket_size, uint32_t max_count,
                         const uint32_t* tree_in, const uint32_t* counts_in, int32_t num_leaves_in, uint32_t* tree_out,
                         uint32_t* counts_out, int32_t capacity, int32_t* num_leaves_out_host, int* converged_host,
                         void* workspace, size_t workspace_bytes);
int cs_update_octree_u64(cs_stream_t stream, const uint64_t* keys, size_t n, unsigned bucket_size, uint32_t max_count,
                         const uint64_t* tree_in, const uint32_t* counts_in, int32_t num_leaves_in, uint64_t* tree_out,
                         uint32_t* counts_out, int32_t capacity, int32_t* num_leaves_out_host, int* converged_host,
                         void* workspace, size_t workspace_bytes);

/* ---- internal tree ------------------------------------------------------------------------------------------------
 * replaces buildOctreeGpu(exec, leaves, OctreeView) (tree/octree_gpu.h:35-45, tree/octree_gpu.cu:138-203) and
 * updateInternalTree (tree/octree.hpp:362-369): placeholder prefixes in (level, key) order, childOffsets, parents,
 * levelRange (written to device memory), internalToLeaf, leafToInternal. level_range_host (may be NULL) receives a
 * host copy of levelRange (the call then synchronises the stream). */
size_t cs_build_octree_workspace_bytes(int32_t num_leaves, int key_bits);
int cs_build_octree_u32(cs_stream_t stream, const uint32_t* leaves, int32_t num_leaves, const cs_octree_view* view,
                        int32_t* level_range_host, void* workspace, size_t workspace_bytes);
int cs_build_octree_u64(cs_stream_t stream, const uint64_t* leaves, int32_t num_leaves, const cs_octree_view* view,
                        int32_t* level_range_host, void* workspace, size_t workspace_bytes);

/* ---- node geometry ----------------------------------------------------------------------------------------------
 * replaces computeGeoCentersGpu(exec, prefixes, numNodes, centers, sizes, box) (focus/source_center_gpu.cu:212-240,
 * CPU nodeFpCenters focus/source_center.hpp:145-158). centers/sizes hold 3*num_nodes values (x,y,z per node).
 * kind = CS_HILBERT decodes node boxes as the reference always does; CS_MORTON decodes them as Morton boxes, for
 * trees built from Morton keys (an extension: the reference has no Morton geometry). */
int cs_geo_centers_u32_f32(cs_stream_t stream, const uint32_t* prefixes, int32_t num_nodes, float* centers,
                           float* sizes, const cs_box* box, int kind);
int cs_geo_centers_u32_f64(cs_stream_t stream, const uint32_t* prefixes, int32_t num_nodes, double* centers,
                           double* sizes, const cs_box* box, int kind);
int cs_geo_centers_u64_f32(cs_stream_t stream, const uint64_t* prefixes, int32_t num_nodes, float* centers,
                           float* sizes, const cs_box* box, int kind);
int cs_geo_centers_u64_f64(cs_stream_t stream, const uint64_t* prefixes, int32_t num_nodes, double* centers,
                           double* sizes, const cs_box* box, int kind);

/* ---- halo discovery -----------------------------------------------------------------------------------------------
 * cs_search_boxes replaces computeBoundingBoxGpu (focus/source_center_gpu.cu:23-92) as called by discoverHalos
 * (focus/octree_focus_mpi.hpp:534-544): for leaves [first_leaf, last_leaf), the box around p -/+ h*scale of the
 * leaf's particles, initialised with the leaf's geometric centre centers[leaf_to_internal[leaf]]
 * (leaf_to_internal = OctreeView.leafToInternal + numInternalNodes). search_centers/sizes hold 3 values per leaf.
 * With leaf_to_internal = NULL the initial value is read from search_centers[leaf] instead (in/out, node_centers
 * unused), which is computeBoundingBoxGpu's own contract (the caller fills the centres first).
 * cs_find_halos replaces findHalosGpu (traversal/collisions_gpu.h:46-59, traversal/collisions_gpu.cu:23-77): flags
 * (num_nodes bytes, zeroed by the caller) are set to 1 for every node outside [leaves[first], leaves[last]) that
 * overlaps a search box of a focus leaf. */
int cs_search_boxes_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                        const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, float scale,
                        const int32_t* leaf_to_internal, const float* node_centers, float* search_centers,
                        float* search_sizes);
int cs_search_boxes_f64(cs_stream_t stream, const double* x, const double* y, const double* z, const double* h,
                        const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, double scale,
                        const int32_t* leaf_to_internal, const double* node_centers, double* search_centers,
                        double* search_sizes);
/* computeBoundingBoxGpu<double, float> (focus/source_center_gpu.cu:95-101): double coordinates, float h; the radius
 * h * scale is rounded to float */
int cs_search_boxes_f64_hf32(cs_stream_t stream, const double* x, const double* y, const double* z, const float* h,
                             const uint32_t* layout, int32_t first, int32_t last, float scale, const int32_t* l2i,
                             const double* node_centers, double* search_centers, double* search_sizes);
int cs_find_halos_u32_f32(cs_stream_t stream, const uint32_t* prefixes, const int32_t* child_offsets,
                          const int32_t* parents, const float* node_centers, const float* node_sizes,
                          const uint32_t* leaves, const float* search_centers, const float* search_sizes,
                          const cs_box* box, int32_t first_node, int32_t last_node, uint8_t* flags);
int cs_find_halos_u64_f32(cs_stream_t stream, const uint64_t* prefixes, const int32_t* child_offsets,
                          const int32_t* parents, const float* node_centers, const float* node_sizes,
                          const uint64_t* leaves, const float* search_centers, const float* search_sizes,
                          const cs_box* box, int32_t first_node, int32_t last_node, uint8_t* flags);
int cs_find_halos_u64_f64(cs_stream_t stream, const uint64_t* prefixes, const int32_t* child_offsets,
                          const int32_t* parents, const double* node_centers, const double* node_sizes,
                          const uint64_t* leaves, const double* search_centers, const double* search_sizes,
                          const cs_box* box, int32_t first_node, int32_t last_node, uint8_t* flags);

/* ---- neighbour search ---------------------------------------------------------------------------------------------
 * replaces findNeighbors(x, y, z, h, firstId, lastId, box, OctreeNsView, ngmax, neighbors, neighborsCount)
 * (findneighbors.hpp:156-177) and the GPU builder GpuAlwaysTraverseNeighborhoodBuilder
 * (traversal/ijloop/gpu_alwaystraverse.cuh:174-204). Particles are in SFC order; for each i in [first, last)
 * counts[i-first] receives the uncapped number of j != i with |x_j - x_i|^2 < (2 h_i)^2 among the leaves whose
 * boxes pass the reference's pruning test, and neighbors[(i-first)*ngmax + k] the k-th such j in ascending order
 * for k < min(count, ngmax) — exactly the CPU reference's result. */
int cs_find_neighbors_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                          uint32_t first, uint32_t last, const cs_box* box, const cs_ns_view* tree, unsigned ngmax,
                          uint32_t* neighbors, uint32_t* counts);
int cs_find_neighbors_f64(cs_stream_t stream, const double* x, const double* y, const double* z, const double* h,
                          uint32_t first, uint32_t last, const cs_box* box, const cs_ns_view* tree, unsigned ngmax,
                          uint32_t* neighbors, uint32_t* counts);
/* The reference's findNeighbors with double coordinates and float smoothing lengths (Tc = double, ThP = const float*,
 * findneighbors.hpp:77-177): radiusSq = 4 h h and the cell radius are rounded to float, distances are double. */
int cs_find_neighbors_f64_hf32(cs_stream_t stream, const double* x, const double* y, const double* z, const float* h,
                               uint32_t first, uint32_t last, const cs_box* box, const cs_ns_view* tree,
                               unsigned ngmax, uint32_t* neighbors, uint32_t* counts);

/* No call counterpart in the reference (its findNeighbors leaves the ngmax-strided rows to the caller): compaction of
 * the rows written by cs_find_neighbors_* into CSR form. offsets (u64, n + 1 entries, offsets[n] = total) and list
 * (list_capacity entries) may be device or pinned host memory; row i's min(neighbor_counts[i], ngmax) entries go to
 * list[offsets[i] ..). Entries at or past list_capacity are skipped; compare offsets[n] with it. */
size_t cs_neighbors_csr_workspace_bytes(size_t n);
int cs_neighbors_csr(cs_stream_t stream, const uint32_t* neighbors, const uint32_t* neighbor_counts, size_t n,
                     unsigned ngmax, uint64_t* offsets, uint32_t* list, size_t list_capacity, void* workspace,
                     size_t workspace_bytes);

/* ---- upsweeps and source centres ------------------------------------------------------------------------------
 * cs_upsweep_sum replaces upsweepSumGpu(exec, numLevels, levelRange, childOffsets, nodeCounts)
 * (tree/octree_gpu.cu:218-236, NodeCount tree/octree.hpp:603-615): counts of nodes with children become
 * min(2^32 - 1, sum of their 8 children); leaf counts are inputs. With `parents` (the OctreeView array) the whole
 * upsweep is one launch (arrival counters per node, workspace cs_upsweep_workspace_bytes); with parents = NULL it runs
 * level by level from level_range_host (num_levels + 1 host entries), as the reference does.
 * cs_leaf_source_centers_* replace computeLeafSourceCenterGpu (focus/source_center_gpu.cu:103-170): per leaf the mass
 * centre (x, y, z, sum |m|) written to centers[4 * leafToInternal[leaf]], evaluated in the order of the reference's
 * CPU massCenter (focus/source_center.hpp:70-81). cs_upsweep_source_centers_* replace upsweepCentersGpu
 * (focus/source_center_gpu.cu:173-205) with CombineSourceCenter (focus/source_center.hpp:84-98). */
size_t cs_upsweep_workspace_bytes(int32_t num_nodes);
int cs_upsweep_sum(cs_stream_t stream, int num_levels, const int32_t* level_range_host, const int32_t* child_offsets,
                   const int32_t* parents, int32_t num_nodes, uint32_t* node_counts, void* workspace,
                   size_t workspace_bytes);
int cs_leaf_source_centers_f64(cs_stream_t stream, const double* x, const double* y, const double* z,
                               const double* m, const int32_t* leaf_to_internal, int32_t num_leaves,
                               const uint32_t* layout, double* centers);
int cs_leaf_source_centers_f64_m32(cs_stream_t stream, const double* x, const double* y, const double* z,
                                   const float* m, const int32_t* leaf_to_internal, int32_t num_leaves,
                                   const uint32_t* layout, double* centers);
int cs_leaf_source_centers_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* m,
                               const int32_t* leaf_to_internal, int32_t num_leaves, const uint32_t* layout,
                               float* centers);
int cs_upsweep_source_centers_f64(cs_stream_t stream, int num_levels, const int32_t* level_range_host,
                                  const int32_t* child_offsets, const int32_t* parents, int32_t num_nodes,
                                  double* centers, void* workspace, size_t workspace_bytes);
int cs_upsweep_source_centers_f32(cs_stream_t stream, int num_levels, const int32_t* level_range_host,
                                  const int32_t* child_offsets, const int32_t* parents, int32_t num_nodes,
                                  float* centers, void* workspace, size_t workspace_bytes);

/* ---- target groups ----------------------------------------------------------------------------------------------
 * replaces computeGroupSplits(exec, first, last, x, y, z, h, leaves, numLeaves, layout, box, groupSize, tolFactor,
 * numSplitsPerGroup, groups) (traversal/groups_gpu.h:63-78, traversal/groups_gpu.cu, groupSplitsKernel in
 * traversal/groups_gpu.cuh): fixed groups of group_size (32 or 64) particles from `first`, cut after particle j where
 * |X_{j+1} - X_j|^2 > min(distCrit^2, (2 h_j / minExtent)^2) in unit-box coordinates; distCrit = tol times the edge of
 * the smallest leaf among the group's first 32 particles. h may be NULL. groups receives the group starts and `last`
 * (num_groups + 1 entries); *num_groups is set (host) and CS_ERR_CAPACITY returned if groups_capacity is too small.
 * Synchronises the stream, as the reference does. */
size_t cs_group_splits_workspace_bytes(uint32_t num_particles, unsigned group_size);
int cs_group_splits_f64(cs_stream_t stream, uint32_t first, uint32_t last, const double* x, const double* y,
                        const double* z, const double* h, const uint64_t* leaves, int32_t num_leaves,
                        const uint32_t* layout, const cs_box* box, unsigned group_size, float tol, uint32_t* groups,
                        size_t groups_capacity, uint32_t* num_groups, void* workspace, size_t workspace_bytes);
int cs_group_splits_f32(cs_stream_t stream, uint32_t first, uint32_t last, const float* x, const float* y,
                        const float* z, const float* h, const uint64_t* leaves, int32_t num_leaves,
                        const uint32_t* layout, const cs_box* box, unsigned group_size, float tol, uint32_t* groups,
                        size_t groups_capacity, uint32_t* num_groups, void* workspace, size_t workspace_bytes);

/* ---- SFC gaps and spanning trees ------------------------------------------------------------------------------
 * cs_count_sfc_gaps / cs_fill_sfc_gaps replace countSfcGapsGpu / fillSfcGapsGpu (tree/csarray_gpu.h:73-82,
 * tree/csarray_gpu.cu:238-270): node_ops[i] = spanSfcRange(tree[i], tree[i+1]) (sfc/common.hpp:422-460); after an
 * exclusive scan of node_ops (num_nodes + 1 entries), the fill writes the keys of every interval and the last key.
 * cs_spanning_tree replaces computeSpanningTree (tree/csarray.hpp:482-506): the smallest cornerstone leaf array that
 * contains the given sorted keys (first 0, last nodeRange(0)); *out_size = its number of keys (host, synchronised). */
int cs_count_sfc_gaps_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes, int32_t* node_ops);
int cs_count_sfc_gaps_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes, int32_t* node_ops);
int cs_fill_sfc_gaps_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes, const int32_t* node_ops,
                         uint32_t* new_tree);
int cs_fill_sfc_gaps_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes, const int32_t* node_ops,
                         uint64_t* new_tree);
size_t cs_spanning_tree_workspace_bytes(int32_t num_keys);
int cs_spanning_tree_u32(cs_stream_t stream, const uint32_t* keys, int32_t num_keys, uint32_t* out, int32_t capacity,
                         int32_t* out_size, void* workspace, size_t workspace_bytes);
int cs_spanning_tree_u64(cs_stream_t stream, const uint64_t* keys, int32_t num_keys, uint64_t* out, int32_t capacity,
                         int32_t* out_size, void* workspace, size_t workspace_bytes);

/* ---- focus (locally essential) tree ---------------------------------------------------------------------------
 * cs_rebalance_decision_essential replaces rebalanceDecisionEssentialGpu (focus/rebalance_gpu.h:21-33,
 * mergeCountAndMacOp focus/rebalance.hpp:31-73): node_ops[i] in {0 merge, 1 keep, 8, 64, 512, 4096 split} per node.
 * cs_mac_refine_decision replaces macRefineDecisionGpu (focus/rebalance_gpu.h:35-48): per leaf, 8 where the leaf's
 * MAC fails outside [focus_first, focus_last), else 1. cs_protect_ancestors replaces protectAncestorsGpu
 * (focus/rebalance_gpu.h:50-52, nzAncestorOp focus/rebalance.hpp:96-118), in place; changed_dev (one device int) counts
 * the ops that differ from 1, *converged_host (if not NULL, synchronised) = that count is zero. cs_enforce_keys replaces
 * enforceKeysGpu (focus/rebalance_gpu.h:54-61, enforceKeySingle focus/rebalance.hpp:183-236): keys processed in order;
 * status 0 converged, 1 cancelMerge, 2 rebalance, 3 failed in status_dev (and *status_host, synchronised, if not
 * NULL). cs_range_count replaces rangeCountGpu (focus/rebalance_gpu.h:63-70, focus/rebalance.hpp:263-286).
 * cs_node_layout replaces computeNodeLayout (domain/layout.hpp:154-186): layout (num_leaves + 1) = exclusive scan of
 * the counts of the leaves in [first, last) or flagged (flags indexed by node) through leaf_to_internal. */
int cs_rebalance_decision_essential_u32(cs_stream_t stream, const uint32_t* prefixes, const int32_t* child_offsets,
                                        const int32_t* parents, const uint32_t* counts, const uint8_t* macs,
                                        uint32_t focus_start, uint32_t focus_end, unsigned bucket, int32_t* node_ops,
                                        int32_t num_nodes);
int cs_rebalance_decision_essential_u64(cs_stream_t stream, const uint64_t* prefixes, const int32_t* child_offsets,
                                        const int32_t* parents, const uint32_t* counts, const uint8_t* macs,
                                        uint64_t focus_start, uint64_t focus_end, unsigned bucket, int32_t* node_ops,
                                        int32_t num_nodes);
int cs_mac_refine_decision_u32(cs_stream_t stream, const uint32_t* prefixes, const uint8_t* macs,
                               const int32_t* leaf_to_internal, int32_t num_leaves, int32_t focus_first,
                               int32_t focus_last, int32_t* node_ops);
int cs_mac_refine_decision_u64(cs_stream_t stream, const uint64_t* prefixes, const uint8_t* macs,
                               const int32_t* leaf_to_internal, int32_t num_leaves, int32_t focus_first,
                               int32_t focus_last, int32_t* node_ops);
int cs_protect_ancestors_u32(cs_stream_t stream, const uint32_t* prefixes, const int32_t* parents, int32_t* node_ops,
                             int32_t num_nodes, int* changed_dev, int* converged_host);
int cs_protect_ancestors_u64(cs_stream_t stream, const uint64_t* prefixes, const int32_t* parents, int32_t* node_ops,
                             int32_t num_nodes, int* changed_dev, int* converged_host);
int cs_enforce_keys_u32(cs_stream_t stream, const uint32_t* forced_keys, int32_t num_forced, const uint32_t* prefixes,
                        const int32_t* child_offsets, const int32_t* parents, int32_t* node_ops, int* status_dev,
                        int* status_host);
int cs_enforce_keys_u64(cs_stream_t stream, const uint64_t* forced_keys, int32_t num_forced, const uint64_t* prefixes,
                        const int32_t* child_offsets, const int32_t* parents, int32_t* node_ops, int* status_dev,
                        int* status_host);
int cs_range_count_u32(cs_stream_t stream, const uint32_t* leaves, int32_t num_leaf_keys, const uint32_t* counts,
                       const uint32_t* leaves_focus, const int32_t* focus_idx, int32_t num_idx,
                       uint32_t* counts_focus);
int cs_range_count_u64(cs_stream_t stream, const uint64_t* leaves, int32_t num_leaf_keys, const uint32_t* counts,
                       const uint64_t* leaves_focus, const int32_t* focus_idx, int32_t num_idx,
                       uint32_t* counts_focus);
size_t cs_node_layout_workspace_bytes(int32_t num_leaves);
int cs_node_layout(cs_stream_t stream, const uint32_t* focus_leaf_counts, int32_t num_leaves, const uint8_t* flags,
                   const int32_t* leaf_to_internal, int32_t first, int32_t last, uint32_t* layout, void* workspace,
                   size_t workspace_bytes);

/* ---- neighbour-list consumers (ijLoop) ------------------------------------------------------------------------
 * An SPH density interaction over neighbours: rho_i = hinv^3 (m_i w(0) + sum_j m_j w(|x_i - x_j| hinv)), hinv = 1/h_i,
 * w(q) = (1 - 1.5 q^2) + 0.75 q^3 for q < 1, else 0.25 (2 - q)^3, over j != i with |x_i - x_j|^2 < (2 h_i)^2, summed in
 * ascending j with round-to-nearest arithmetic (no fused multiply-add).
 * cs_ijloop_density_list_* replaces the loop of CpuFullNbListNeighborhood (traversal/ijloop/cpu_fullnblist.hpp:94-112)
 * over the ngmax-strided rows of cs_find_neighbors_* (results equal it bit for bit; periodic boxes folded as
 * posDiffAndDistSq does, traversal/ijloop/common.hpp:154-172).
 * cs_cluster_nblist_build_* / cs_ijloop_density_clusters_* take the role of GpuSuperclusterNbListNeighborhoodBuilder
 * (traversal/ijloop/gpu_superclusternblist.cuh:248-360): clusters of 8 consecutive particles; lists holds, per
 * i-cluster i (n/8 rounded up of them), counts[i] j-cluster indices at lists[i * ncmax ..], ascending, covering every
 * j within 2 h of the cluster's particles (open boxes only). key_bits is the key width the tree was built with. If an
 * i-cluster needs more than ncmax j-clusters the build returns CS_ERR_CAPACITY and *max_count_host (if not NULL) the
 * largest count. The build synchronises the stream. The cluster loop's results equal the sum over all pairs within
 * 2 h_i in ascending j, bit for bit. */
int cs_ijloop_density_list_f64(cs_stream_t stream, const double* x, const double* y, const double* z, const double* h,
                               const double* m, uint32_t first, uint32_t last, const cs_box* box,
                               const uint32_t* neighbors, const uint32_t* neighbor_counts, unsigned ngmax,
                               double* rho);
int cs_ijloop_density_list_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                               const float* m, uint32_t first, uint32_t last, const cs_box* box,
                               const uint32_t* neighbors, const uint32_t* neighbor_counts, unsigned ngmax,
                               float* rho);
size_t cs_cluster_nblist_workspace_bytes(size_t n);
int cs_cluster_nblist_build_f64(cs_stream_t stream, const double* x, const double* y, const double* z,
                                const double* h, size_t n, const cs_ns_view* tree, const cs_box* box, int key_bits,
                                unsigned ncmax, uint32_t* lists, uint32_t* counts, void* workspace,
                                size_t workspace_bytes, int* max_count_host);
int cs_cluster_nblist_build_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                                size_t n, const cs_ns_view* tree, const cs_box* box, int key_bits, unsigned ncmax,
                                uint32_t* lists, uint32_t* counts, void* workspace, size_t workspace_bytes,
                                int* max_count_host);
int cs_ijloop_density_clusters_f64(cs_stream_t stream, const double* x, const double* y, const double* z,
                                   const double* h, const double* m, size_t n, const uint32_t* lists,
                                   const uint32_t* counts, unsigned ncmax, double* rho);
int cs_ijloop_density_clusters_f32(cs_stream_t stream, const float* x, const float* y, const float* z, const float* h,
                                   const float* m, size_t n, const uint32_t* lists, const uint32_t* counts,
                                   unsigned ncmax, float* rho);

/* ---- whole path: keys -> sort -> gather -> computeOctree -> link -> geometry -> findHalos -> findNeighbors ---------
 * The single-rank inner part of the reference's Domain::sync + discoverHalos + neighbour search
 * (domain/assignment.hpp:105-120, focus/octree_focus_mpi.hpp:512-568, findneighbors.hpp:156-177), as one object that
 * keeps its device buffers between calls (no allocation once sized). Coordinates and h are f32 or f64 (coord_bits),
 * keys u32 or u64 (key_bits). */
typedef struct cs_pipeline_s* cs_pipeline;

typedef struct
{
    int sfc_kind;           /* CS_HILBERT (the reference's SfcKind) or CS_MORTON */
    unsigned bucket_size;   /* computeOctree bucketSize */
    uint32_t max_count;     /* computeOctree maxCount (0xffffffff = uncapped) */
    unsigned ngmax;         /* findNeighbors ngmax; 0 = counts only */
    float search_ext;       /* OctreeNsView::searchExtFactor */
    float halo_search_ext;  /* discoverHalos searchExtFact: search box = p +- 2 h halo_search_ext */
    int do_halos;           /* run findHalos for the leaves in [focus_start, focus_end) of the key space */
    int do_neighbors;       /* run findNeighbors for all particles */
} cs_pipeline_config;

typedef struct
{
    int32_t num_leaves;
    int32_t num_nodes;
    int32_t iterations; /* updateOctree steps of the build */
    int32_t focus_first;
    int32_t focus_last;
    int32_t max_depth;  /* deepest leaf level */
} cs_pipeline_result;

/* device pointers to the results of the last cs_pipeline_run (valid until the next run or destroy) */
typedef struct
{
    void* sorted_keys;      /* n keys, SFC order */
    uint32_t* order;        /* n: sorted position -> input index (sort_by_key permutation) */
    void *x, *y, *z, *h;    /* n each, SFC order */
    void* leaves;           /* num_leaves + 1 */
    uint32_t* counts;       /* num_leaves */
    uint32_t* layout;       /* num_leaves + 1 */
    cs_octree_view octree;  /* linked internal tree */
    void* centers;          /* 3 * num_nodes */
    void* sizes;            /* 3 * num_nodes */
    uint8_t* halo_flags;    /* num_nodes */
    uint32_t* neighbors;    /* n * ngmax */
    uint32_t* neighbor_counts; /* n */
    void* search_centers;   /* 3 * num_leaves; leaves [focus_first, focus_last) hold the halo search boxes */
    void* search_sizes;     /* 3 * num_leaves, as search_centers */
} cs_pipeline_outputs;

int cs_pipeline_create(cs_pipeline* out, int coord_bits, int key_bits, const cs_pipeline_config* config);
int cs_pipeline_destroy(cs_pipeline p);
/* inputs are device arrays of n particles (any order); box as for cs_sfc_keys */
int cs_pipeline_run(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z, const void* h,
                    size_t n, const cs_box* box, uint64_t focus_start, uint64_t focus_end, cs_pipeline_result* result);
/* same from host arrays (pinned for full speed): copies the inputs in, runs, and copies the neighbour counts
 * (n uint32, may be NULL) and halo flags (num_nodes bytes, may be NULL; call with NULL first to learn num_nodes)
 * back; synchronises the stream. */
int cs_pipeline_run_host(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                         const void* h, size_t n, const cs_box* box, uint64_t focus_start, uint64_t focus_end,
                         uint32_t* neighbor_counts_host, uint8_t* halo_flags_host, size_t halo_flags_capacity,
                         cs_pipeline_result* result);
/* Pipelined form of cs_pipeline_run_host: returns once the run and the copy of its results are enqueued. Input copies go
 * to one of two device input sets in turn and wait only for the last reader of that set, so the next call's input
 * copies overlap this run's computation; results travel back on a stream of their own. The host arrays of a call must
 * stay unchanged, and its outputs unread, until cs_pipeline_wait returns; the device outputs of cs_pipeline_get_outputs
 * are those of the last call. */
int cs_pipeline_run_host_async(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                               const void* h, size_t n, const cs_box* box, uint64_t focus_start, uint64_t focus_end,
                               uint32_t* neighbor_counts_host, uint8_t* halo_flags_host, size_t halo_flags_capacity,
                               cs_pipeline_result* result);
/* waits for the results of the last cs_pipeline_run_host_async; returns the first device error (sort look-back
 * timeout, traversal stack overflow) of the runs since the previous wait */
int cs_pipeline_wait(cs_pipeline p);
/* The host-buffer runs above with the neighbour lists returned as well, in compressed sparse row form: row i's first
 * min(nc_i, ngmax) neighbours (ascending, as findNeighbors stores them into its ngmax-strided `neighbors` argument,
 * findneighbors.hpp:156-177) are list_host[offsets_host[i] .. offsets_host[i+1]), offsets_host has n + 1 entries and
 * offsets_host[n] is the total. Pinned host buffers (cudaHostAlloc / cudaHostRegister) give the full host-link rate.
 * The lists are compacted on the device right after the run (on `stream`); the offsets, counts and flags are copied
 * at once, and the list itself by the copy engine once its length is known on the host: at the pipeline's next call
 * (run, step or wait), which has already waited for that compaction. Entries past list_capacity are not written and
 * the wait reports CS_ERR_CAPACITY (offsets_host[n] = entries needed). The _async form follows
 * cs_pipeline_run_host_async (results valid after cs_pipeline_wait). */
int cs_pipeline_run_host_csr(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                             const void* h, size_t n, const cs_box* box, uint64_t focus_start, uint64_t focus_end,
                             uint32_t* neighbor_counts_host, uint8_t* halo_flags_host, size_t halo_flags_capacity,
                             uint64_t* offsets_host, uint32_t* list_host, size_t list_capacity,
                             cs_pipeline_result* result);
int cs_pipeline_run_host_csr_async(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                                   const void* h, size_t n, const cs_box* box, uint64_t focus_start,
                                   uint64_t focus_end, uint32_t* neighbor_counts_host, uint8_t* halo_flags_host,
                                   size_t halo_flags_capacity, uint64_t* offsets_host, uint32_t* list_host,
                                   size_t list_capacity, cs_pipeline_result* result);
int cs_pipeline_get_outputs(cs_pipeline p, cs_pipeline_outputs* out);
/* bytes of device memory the pipeline holds */
size_t cs_pipeline_device_bytes(cs_pipeline p);
/* Incremental time steps: the reference's per-step path with one updateOctree step from the previous tree instead of
 * a build from the root (updateOctreeGpu, tree/update_gpu.cuh:43-68, as driven by Domain::sync each time step).
 * The first call of a sequence (or a call with a different n) builds from the root like cs_pipeline_run; every later
 * call recomputes keys, re-sorts, applies one rebalance decision to the previous leaf array using the previous
 * counts, recounts the new leaves against the new keys, relinks, recomputes node geometry and the neighbours.
 * Halos are not part of a step. Inputs are device pointers. With use_graph = 1 the step is captured once into a CUDA
 * graph (one per direction of the leaf ping-pong; recaptured when the input pointers, n or the box change) and
 * replayed; every launch of a step is sized by a leaf capacity and reads the current leaf count from device memory,
 * so a step synchronises the host once, at its end. A step whose new tree outgrows the capacity is redone uncaptured
 * with larger buffers. Results (cs_pipeline_get_outputs) are those of the last step. */
int cs_pipeline_step(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z, const void* h,
                     size_t n, const cs_box* box, int use_graph, cs_pipeline_result* result);
/* the next cs_pipeline_step builds from the root again (drops the captured graphs) */
int cs_pipeline_reset_steps(cs_pipeline p);
/* steps of the current sequence that were replayed from a captured graph */
int cs_pipeline_graph_replays(cs_pipeline p);

/* ---- tuning: knobs that change the speed of a pipeline, never its results -----------------------------------------
 * nb_group: targets per warp of the neighbour traversal (32, 16 or 8; 1, 2 or 4 lanes per target).
 * nb_by_target_cost: with one target per lane, a candidate batch that few lanes need runs the by-target loop (lanes
 * hold the candidates, the warp loops over the needing targets) when 19 x (needing lanes) < nb_by_target_cost x (the
 * per-lane loop's candidate steps); 0 never.
 * sort_items: the key sort's tile shape, keys per thread (16 with 3 blocks of 256 threads per SM, or 12 with 4; 0
 * means 16). Default {32, 7, 16}. Setting a tuning ends a step sequence (the next cs_pipeline_step builds from the
 * root). The reference has no counterpart: its traversal shape is the compile-time TravConfig
 * (traversal/find_neighbors.cuh:29-58), and its sort's tiles are CUB's compile-time policy
 * (primitives/primitives_gpu.cu:322-356). */
typedef struct
{
    int nb_group;
    int nb_by_target_cost;
    int sort_items;
} cs_tuning;

int cs_pipeline_set_tuning(cs_pipeline p, const cs_tuning* tuning);
int cs_pipeline_get_tuning(cs_pipeline p, cs_tuning* tuning);
/* Autotuner: reruns the inputs of the last cs_pipeline_run / cs_pipeline_run_host, when no cs_pipeline_step came
 * after it (device input arrays must still be valid), reps times for each candidate tuning: first the traversal
 * ({32, 7}, {32, 0}, {32, 5}, {32, 10}, {16, 7}, {8, 7}, scored by the mean device time of the neighbour stage), then,
 * with the fastest of those, the sort's tile shapes (16 and 12 keys per thread, scored by the sort stage). Keeps the
 * fastest as the pipeline's tuning. Writes the best, and up to capacity candidates with their mean ms of the stage
 * that scored them (tried / ms may be NULL); *count = candidates run (8). The outputs afterwards are those of the
 * last candidate's run (identical for every tuning). */
int cs_pipeline_autotune(cs_pipeline p, cs_stream_t stream, int reps, cs_tuning* best, cs_tuning* tried, float* ms,
                         int capacity, int* count);

/* device time in ms of each stage of the last run: keys, sort, gather, build, link, geometry, float node boxes
 * (node preparation of the halo and neighbour searches), halos, neighbours (count <= 9 values); waits for the last
 * run to finish */
int cs_pipeline_stage_times(cs_pipeline p, float* ms, int count);
/* device times in ms of the last copy-back that returned neighbour lists (cs_pipeline_run_host_csr*), waiting for it:
 * the list compaction, the list's copy to host memory, how long the compacted list waited for the previous call's
 * copy, and the time from the start of the run (its keys) to the end of its list copy (count <= 4 values) */
int cs_pipeline_copy_times(cs_pipeline p, float* ms, int count);

/* ---- batched independent sets ----------------------------------------------------------------------------------
 * No counterpart call in the reference, which builds one tree per call: many independent particle sets of uneven size
 * go through keys -> sort -> build -> link -> geometry -> neighbours in one sequence of launches, with results equal
 * to running each set on its own through cs_pipeline_run (same coordinate type, 32-bit keys of the given curve, the
 * set's bucket size, ngmax, no halos). Each set's 32-bit key is combined with its index into one 64-bit key
 * (set << 30) | key, so one stable sort orders every set and keeps them apart, and one cooperative cornerstone build
 * over the combined keys builds every set's tree at once: each set is the subtree rooted at level 11, with its own
 * bucket size and no merge at or above that level; the neighbour traversal of a particle starts at its set's root.
 * Sets may be empty; the total is below 2^30 particles. Inputs are device arrays of all sets concatenated; the set
 * offsets (num_sets + 1), boxes and bucket sizes are host arrays. */
typedef struct cs_batch_s* cs_batch;
typedef struct
{
    int coord_bits;   /* 32 or 64 */
    int sfc_kind;     /* CS_MORTON or CS_HILBERT (32-bit keys per set; geometry decoded with the same curve) */
    unsigned ngmax;   /* stored neighbours per particle */
    float search_ext; /* searchExtFactor of the neighbour search */
    int do_neighbors;
} cs_batch_config;
typedef struct
{
    int32_t num_sets;
    int32_t num_leaves; /* of the combined tree, over all sets (+ a few empty filler leaves) */
    int32_t num_nodes;
    int32_t iterations; /* rebalance iterations until every set converged */
    uint64_t num_particles;
} cs_batch_result;
typedef struct
{
    const uint32_t* order;           /* sorted position -> input position (over all sets) */
    const void *x, *y, *z, *h;       /* sorted coordinates and h; set s occupies [set_offsets[s], set_offsets[s+1]) */
    const uint64_t* leaves;          /* combined leaf keys, num_leaves + 1 */
    const uint32_t* counts;          /* particles per leaf */
    const uint32_t* layout;          /* first sorted particle of each leaf, num_leaves + 1 */
    const int32_t* set_leaf_begin;   /* set s owns leaves [set_leaf_begin[s], set_leaf_begin[s+1]), num_sets + 1 */
    const int32_t* set_roots;        /* node index of each set's root in the combined tree */
    const uint32_t* set_offsets;     /* device copy of the set offsets */
    cs_octree_view octree;           /* the combined tree (uint64_t prefixes) */
    const void *centers, *sizes;     /* per node, with each set's box */
    const uint32_t* neighbors;       /* num_particles x ngmax, sorted positions over all sets */
    const uint32_t* neighbor_counts; /* uncapped counts */
} cs_batch_outputs;
int cs_batch_create(cs_batch* out, const cs_batch_config* cfg);
int cs_batch_destroy(cs_batch b);
/* the neighbour traversal's tuning for later runs (as cs_pipeline_set_tuning; results do not change) */
int cs_batch_set_tuning(cs_batch b, const cs_tuning* tuning);
int cs_batch_run(cs_batch b, cs_stream_t stream, const void* x, const void* y, const void* z, const void* h,
                 const uint32_t* set_offsets_host, int32_t num_sets, const cs_box* boxes_host,
                 const uint32_t* buckets_host, cs_batch_result* result);
int cs_batch_get_outputs(cs_batch b, cs_batch_outputs* out);
size_t cs_batch_device_bytes(cs_batch b);

/* ---- request server --------------------------------------------------------------------------------------------
 * No counterpart in the reference. Continuous batching of requests on one GPU: a BUILD request runs the whole path
 * (keys -> neighbours, no halos) on a particle set from host arrays; with tree >= 0 the tree stays resident on the
 * device, and an UPDATE request of that tree applies one updateOctree step to new positions of its particles
 * (cs_pipeline_step). num_slots requests run at once, each on its own stream and host worker; a request is admitted
 * when a slot is free and its device memory fits hbm_budget_bytes (idle resident trees are released least recently
 * used first to make room); requests of one tree run in submission order. Every result depends only on its own
 * inputs: the same alone and in any mix. The host arrays of a request must stay valid until it completes. */
enum cs_request_kind
{
    CS_REQ_BUILD  = 0,
    CS_REQ_UPDATE = 1
};
typedef struct cs_server_s* cs_server;
typedef struct
{
    int num_slots;               /* requests on the device at once */
    uint64_t hbm_budget_bytes;   /* device memory all requests and resident trees may hold */
    int coord_bits;              /* 32 or 64 */
    int key_bits;                /* 32 or 64 */
    cs_pipeline_config pipeline; /* curve, bucket size, ngmax, search extent (halos are not run) */
} cs_server_config;
typedef struct
{
    int kind;     /* cs_request_kind */
    int32_t tree; /* resident tree id (>= 0), or -1 for a one-off build */
    const void *x, *y, *z, *h;
    size_t n;
    cs_box box;
} cs_request;
typedef struct
{
    uint64_t id;
    int status;                 /* CS_OK or the failure (cs_last_error of the waiting thread has no detail) */
    int32_t num_leaves;
    uint64_t neighbor_checksum; /* order-independent hash of every particle's count and stored neighbour list */
    double queued_ms;           /* submission -> start */
    double run_ms;              /* start -> result on the host */
    double latency_ms;          /* submission -> result on the host */
} cs_request_result;
typedef struct
{
    uint64_t completed;
    uint64_t failed;
    uint64_t particles; /* of the completed requests */
    double p50_ms;      /* latency percentiles of the completed requests */
    double p99_ms;
    double elapsed_s;   /* first submission -> last completion */
    uint64_t device_bytes;
    int resident_trees;
} cs_server_stats;
int cs_server_create(cs_server* out, const cs_server_config* cfg);
/* finishes the queued requests, then stops the workers and frees the device memory */
int cs_server_destroy(cs_server s);
int cs_server_submit(cs_server s, const cs_request* request, uint64_t* id);
/* blocks until request id is done; copies its n neighbour counts into neighbor_counts_host (may be NULL); returns the
 * request's status */
int cs_server_wait(cs_server s, uint64_t id, cs_request_result* result, uint32_t* neighbor_counts_host);
int cs_server_release_tree(cs_server s, int32_t tree);
int cs_server_get_stats(cs_server s, cs_server_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* CSTONE_GB300_H */
