// Header-only C++ layer that defines the reference's GPU hot-path templates (namespace cstone) on top of the C ABI of
// libcstone_gb300 (cstone_gb300.h), with the reference's explicit instantiations.
//
// Use: compile exactly ONE translation unit that includes this header against the reference's include directory
// (it includes the reference's own declarations, so the signatures are checked against them) and link it with
// libcstone_gb300.so instead of the reference's object libraries for these symbols:
//
//   computeSfcKeys              sfc/sfc_gpu.h:24-26              -> cs_sfc_keys_{hilbert,morton}_{u32,u64}_{f32,f64}
//   sortByKeyTempStorage,
//   sortByKey (raw pointers)    primitives/primitives_gpu.h:118-130 -> cs_sort_pairs_{u32,u64}
//   exclusiveScan (int, uint)   primitives/primitives_gpu.h:158-160 -> cs_exclusive_scan_i32
//   computeNodeCountsGpu        tree/csarray_gpu.h:41-47         -> cs_node_counts_{u32,u64}
//   computeNodeOpsGpu           tree/csarray_gpu.h:59-65         -> cs_rebalance_decision + cs_exclusive_scan_i32
//   rebalanceTreeGpu            tree/csarray_gpu.h:67-73         -> cs_rebalance_tree_{u32,u64}
//   buildOctreeGpu (both)       tree/octree_gpu.h:35-45          -> cs_build_octree_{u32,u64}
//   computeGeoCentersGpu        focus/source_center_gpu.h:93-99  -> cs_geo_centers_*
//   computeBoundingBoxGpu       focus/source_center_gpu.h:40-51  -> cs_search_boxes_{f32,f64} (in/out init mode)
//   findHalosGpu                traversal/collisions_gpu.h:46-59 -> cs_find_halos_*
//
//   gather                      primitives/primitives_gpu.h:48-49 -> cs_gather_{f32,f64}
//   updateOctreeGpu             tree/update_gpu.cuh:43-68        (the reference's header template runs on the
//                                                                 functions above; standalone builds get the same
//                                                                 step defined here)
//
// Instantiations the C ABI does not cover fail to compile here (static_assert) instead of linking silently:
// sortByKey with 64-bit values or float keys, exclusiveScan into 64-bit sums, gather between different types. Those
// stay with the reference's own library.
//
// Two ways to build: against the reference's include directory (the default; its declarations check these
// definitions), or with -DCSTONE_GB300_STANDALONE and no reference headers at all, where cstone_types.hpp restates the
// interface types (Box, OctreeView, OctreeNsView, key types, execution::Gpu, DeviceVector) so that code written for
// the reference compiles against this library alone.
//
// Errors: the reference prints and exits on a CUDA error (cuda/errorcheck.cuh:15-27); here every failing call throws
// std::runtime_error with cs_last_error(). Synchronisation: calls that return host values (computeNodeOpsGpu,
// rebalanceTreeGpu, buildOctreeGpu's host levelRange) synchronise the stream, as the reference's do.
#pragma once

#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <cuda_runtime.h>

#ifdef CSTONE_GB300_STANDALONE
// no reference headers: the interface types restated in cstone_types.hpp
#include "cstone_gb300/cstone_types.hpp"
#else
#include "cstone/execution.hpp"
#include "cstone/focus/source_center_gpu.h"
#include "cstone/primitives/primitives_gpu.h"
#include "cstone/sfc/box.hpp"
#include "cstone/sfc/sfc.hpp"
#include "cstone/sfc/sfc_gpu.h"
#include "cstone/traversal/collisions_gpu.h"
#include "cstone/tree/csarray_gpu.h"
#include "cstone/tree/definitions.h"
#include "cstone/tree/octree.hpp"
#include "cstone/tree/octree_gpu.h"
#endif

#include "cstone_gb300.h"

namespace cstone
{
namespace gb300
{

inline void check(int rc, const char* what)
{
    if (rc != CS_OK) { throw std::runtime_error(std::string(what) + ": " + cs_last_error()); }
}

inline cs_stream_t stream(execution::Gpu exec) { return static_cast<cs_stream_t>(static_cast<cudaStream_t>(exec)); }

template<class T>
cs_box toBox(const Box<T>& b)
{
    cs_box c;
    c.lo[0]       = double(b.xmin());
    c.lo[1]       = double(b.ymin());
    c.lo[2]       = double(b.zmin());
    c.hi[0]       = double(b.xmax());
    c.hi[1]       = double(b.ymax());
    c.hi[2]       = double(b.zmax());
    c.boundary[0] = int(b.boundaryX());
    c.boundary[1] = int(b.boundaryY());
    c.boundary[2] = int(b.boundaryZ());
    return c;
}

//! whether the decision of the last computeNodeOpsGpu on this thread changed nothing (rebalanceTreeGpu's result;
//! the reference keeps the same state in a device global, tree/csarray_gpu.cu:130)
inline thread_local bool lastDecisionConverged = true;

template<class T>
constexpr bool isU32 = std::is_same_v<T, uint32_t> || std::is_same_v<T, unsigned>;

} // namespace gb300

static_assert(sizeof(Vec3<float>) == 3 * sizeof(float) && sizeof(Vec3<double>) == 3 * sizeof(double),
              "Vec3 must be three packed coordinates");
static_assert(std::is_same_v<TreeNodeIndex, int32_t> && std::is_same_v<LocalIndex, uint32_t>, "index types");

// ---- keys -------------------------------------------------------------------------------------------------------
template<class KeyType, class T>
void computeSfcKeys(execution::Gpu exec, const T* x, const T* y, const T* z, KeyType* keys, size_t numKeys,
                    const Box<T>& box)
{
    using I                = typename KeyType::ValueType;
    constexpr bool hilbert = std::is_same_v<KeyType, HilbertKey<I>>;
    static_assert(hilbert || std::is_same_v<KeyType, MortonKey<I>>, "Hilbert or Morton keys");
    cs_box cb = gb300::toBox(box);
    auto s    = gb300::stream(exec);
    auto* k   = reinterpret_cast<I*>(keys);
    int rc;
    // the reference kernel leaves keys equal to removeKey untouched (sfc/sfc_gpu.cu:23-44)
    if constexpr (gb300::isU32<I>)
    {
        if constexpr (std::is_same_v<T, double>)
            rc = hilbert ? cs_sfc_keys_hilbert_u32_f64(s, x, y, z, k, numKeys, &cb, 1)
                         : cs_sfc_keys_morton_u32_f64(s, x, y, z, k, numKeys, &cb, 1);
        else
            rc = hilbert ? cs_sfc_keys_hilbert_u32_f32(s, x, y, z, k, numKeys, &cb, 1)
                         : cs_sfc_keys_morton_u32_f32(s, x, y, z, k, numKeys, &cb, 1);
    }
    else
    {
        if constexpr (std::is_same_v<T, double>)
            rc = hilbert ? cs_sfc_keys_hilbert_u64_f64(s, x, y, z, k, numKeys, &cb, 1)
                         : cs_sfc_keys_morton_u64_f64(s, x, y, z, k, numKeys, &cb, 1);
        else
            rc = hilbert ? cs_sfc_keys_hilbert_u64_f32(s, x, y, z, k, numKeys, &cb, 1)
                         : cs_sfc_keys_morton_u64_f32(s, x, y, z, k, numKeys, &cb, 1);
    }
    gb300::check(rc, "computeSfcKeys");
}

template void computeSfcKeys(execution::Gpu, const float*, const float*, const float*, MortonKey<unsigned>*, size_t,
                             const Box<float>&);
template void computeSfcKeys(execution::Gpu, const double*, const double*, const double*, MortonKey<unsigned>*,
                             size_t, const Box<double>&);
template void computeSfcKeys(execution::Gpu, const float*, const float*, const float*, MortonKey<uint64_t>*, size_t,
                             const Box<float>&);
template void computeSfcKeys(execution::Gpu, const double*, const double*, const double*, MortonKey<uint64_t>*,
                             size_t, const Box<double>&);
template void computeSfcKeys(execution::Gpu, const float*, const float*, const float*, HilbertKey<unsigned>*, size_t,
                             const Box<float>&);
template void computeSfcKeys(execution::Gpu, const double*, const double*, const double*, HilbertKey<unsigned>*,
                             size_t, const Box<double>&);
template void computeSfcKeys(execution::Gpu, const float*, const float*, const float*, HilbertKey<uint64_t>*, size_t,
                             const Box<float>&);
template void computeSfcKeys(execution::Gpu, const double*, const double*, const double*, HilbertKey<uint64_t>*,
                             size_t, const Box<double>&);

// ---- stable key sort ------------------------------------------------------------------------------------------
template<class KeyType, class ValueType>
uint64_t sortByKeyTempStorage(uint64_t numElements)
{
    static_assert(gb300::isU32<KeyType> || std::is_same_v<KeyType, uint64_t>, "u32 or u64 keys");
    static_assert(sizeof(ValueType) == 4, "32-bit values");
    return cs_sort_pairs_workspace_bytes(size_t(numElements), int(8 * sizeof(KeyType)));
}

template<class KeyType, class ValueType>
void sortByKey(execution::Gpu exec, KeyType* first, KeyType* last, ValueType* values, KeyType* keyBuf,
               ValueType* valueBuf, void* tmp, uint64_t tmpBytes)
{
    static_assert(gb300::isU32<KeyType> || std::is_same_v<KeyType, uint64_t>, "u32 or u64 keys");
    static_assert(sizeof(ValueType) == 4, "32-bit values");
    size_t n = size_t(last - first);
    if (tmpBytes < sortByKeyTempStorage<KeyType, ValueType>(n)) { throw std::runtime_error("temp storage too small\n"); }
    auto* v  = reinterpret_cast<uint32_t*>(values);
    auto* vb = reinterpret_cast<uint32_t*>(valueBuf);
    int rc;
    // all key bits, the result left in (first, values) as the reference copies it back
    if constexpr (gb300::isU32<KeyType>)
        rc = cs_sort_pairs_u32(gb300::stream(exec), reinterpret_cast<uint32_t*>(first), v, n,
                               reinterpret_cast<uint32_t*>(keyBuf), vb, 0, 32, 0, tmp, size_t(tmpBytes));
    else
        rc = cs_sort_pairs_u64(gb300::stream(exec), first, v, n, keyBuf, vb, 0, 64, 0, tmp, size_t(tmpBytes));
    gb300::check(rc, "sortByKey");
}

template uint64_t sortByKeyTempStorage<unsigned, unsigned>(uint64_t);
template uint64_t sortByKeyTempStorage<unsigned, int>(uint64_t);
template uint64_t sortByKeyTempStorage<uint64_t, unsigned>(uint64_t);
template uint64_t sortByKeyTempStorage<uint64_t, int>(uint64_t);
template void sortByKey(execution::Gpu, unsigned*, unsigned*, unsigned*, unsigned*, unsigned*, void*, uint64_t);
template void sortByKey(execution::Gpu, unsigned*, unsigned*, int*, unsigned*, int*, void*, uint64_t);
template void sortByKey(execution::Gpu, uint64_t*, uint64_t*, unsigned*, uint64_t*, unsigned*, void*, uint64_t);
template void sortByKey(execution::Gpu, uint64_t*, uint64_t*, int*, uint64_t*, int*, void*, uint64_t);

template<class IndexType, class SumType>
void exclusiveScan(execution::Gpu exec, const IndexType* first, const IndexType* last, SumType* output, SumType init)
{
    static_assert(sizeof(IndexType) == 4 && sizeof(SumType) == 4, "32-bit scans (two's complement sums)");
    gb300::check(cs_exclusive_scan_i32(gb300::stream(exec), reinterpret_cast<const int32_t*>(first),
                                       reinterpret_cast<int32_t*>(output), size_t(last - first), int32_t(init),
                                       nullptr, 0),
                 "exclusiveScan");
}

template void exclusiveScan(execution::Gpu, const int*, const int*, int*, int);
template void exclusiveScan(execution::Gpu, const int*, const int*, unsigned*, unsigned);
template void exclusiveScan(execution::Gpu, const unsigned*, const unsigned*, unsigned*, unsigned);

// ---- permutation gather -----------------------------------------------------------------------------------------
// a bit copy out[i] = in[perm[i]]: any 4- or 8-byte element type maps onto the float or double gather
template<class TS, class TD, class IndexType>
void gather(execution::Gpu exec, const IndexType* ordering, size_t numElements, const TS* src, TD* buffer)
{
    static_assert(sizeof(IndexType) == 4, "32-bit permutation");
    static_assert(std::is_same_v<TS, TD> && (sizeof(TS) == 4 || sizeof(TS) == 8),
                  "the same 4- or 8-byte element type on both sides");
    auto* perm = reinterpret_cast<const uint32_t*>(ordering);
    int rc;
    if constexpr (sizeof(TS) == 8)
        rc = cs_gather_f64(gb300::stream(exec), perm, reinterpret_cast<const double*>(src),
                           reinterpret_cast<double*>(buffer), numElements);
    else
        rc = cs_gather_f32(gb300::stream(exec), perm, reinterpret_cast<const float*>(src),
                           reinterpret_cast<float*>(buffer), numElements);
    gb300::check(rc, "gather");
}

template void gather(execution::Gpu, const unsigned*, size_t, const double*, double*);
template void gather(execution::Gpu, const unsigned*, size_t, const float*, float*);
template void gather(execution::Gpu, const unsigned*, size_t, const int*, int*);
template void gather(execution::Gpu, const unsigned*, size_t, const unsigned*, unsigned*);
template void gather(execution::Gpu, const unsigned*, size_t, const unsigned long*, unsigned long*);
template void gather(execution::Gpu, const int*, size_t, const int*, int*);
template void gather(execution::Gpu, const int*, size_t, const uint32_t*, uint32_t*);
template void gather(execution::Gpu, const int*, size_t, const uint64_t*, uint64_t*);

// ---- cornerstone leaf array -----------------------------------------------------------------------------------
template<class KeyType>
void computeNodeCountsGpu(execution::Gpu exec, const KeyType* tree, unsigned* counts, TreeNodeIndex numNodes,
                          std::span<const KeyType> keys, unsigned maxCount, bool useCountsAsGuess)
{
    int rc;
    if constexpr (gb300::isU32<KeyType>)
        rc = cs_node_counts_u32(gb300::stream(exec), tree, counts, numNodes, keys.data(), keys.size(), maxCount,
                                useCountsAsGuess, nullptr, 0);
    else
        rc = cs_node_counts_u64(gb300::stream(exec), tree, counts, numNodes, keys.data(), keys.size(), maxCount,
                                useCountsAsGuess, nullptr, 0);
    gb300::check(rc, "computeNodeCountsGpu");
}

template void computeNodeCountsGpu(execution::Gpu, const unsigned*, unsigned*, TreeNodeIndex,
                                   std::span<const unsigned>, unsigned, bool);
template void computeNodeCountsGpu(execution::Gpu, const uint64_t*, unsigned*, TreeNodeIndex,
                                   std::span<const uint64_t>, unsigned, bool);

template<class KeyType>
TreeNodeIndex computeNodeOpsGpu(execution::Gpu exec, const KeyType* tree, TreeNodeIndex numNodes,
                                const unsigned* counts, unsigned bucketSize, TreeNodeIndex* nodeOps)
{
    cudaStream_t cs = exec;
    auto s          = gb300::stream(exec);
    int* convergedDev;
    if (cudaMallocAsync(&convergedDev, sizeof(int), cs) != cudaSuccess) { gb300::check(CS_ERR_CUDA, "cudaMallocAsync"); }
    int rc = gb300::isU32<KeyType>
                 ? cs_rebalance_decision_u32(s, reinterpret_cast<const uint32_t*>(tree), counts, numNodes, bucketSize,
                                             nodeOps, convergedDev)
                 : cs_rebalance_decision_u64(s, reinterpret_cast<const uint64_t*>(tree), counts, numNodes, bucketSize,
                                             nodeOps, convergedDev);
    if (rc == CS_OK) rc = cs_exclusive_scan_i32(s, nodeOps, nodeOps, size_t(numNodes) + 1, 0, nullptr, 0);
    int host[2] = {0, 1};
    if (rc == CS_OK)
    {
        cudaMemcpyAsync(&host[0], nodeOps + numNodes, sizeof(int), cudaMemcpyDeviceToHost, cs);
        cudaMemcpyAsync(&host[1], convergedDev, sizeof(int), cudaMemcpyDeviceToHost, cs);
    }
    cudaFreeAsync(convergedDev, cs);
    if (cudaStreamSynchronize(cs) != cudaSuccess && rc == CS_OK) rc = CS_ERR_CUDA;
    gb300::check(rc, "computeNodeOpsGpu");
    gb300::lastDecisionConverged = host[1] != 0;
    return host[0];
}

template<class KeyType>
bool rebalanceTreeGpu(execution::Gpu exec, const KeyType* tree, TreeNodeIndex numNodes, TreeNodeIndex /*newNumNodes*/,
                      const TreeNodeIndex* nodeOps, KeyType* newTree)
{
    int rc;
    if constexpr (gb300::isU32<KeyType>)
        rc = cs_rebalance_tree_u32(gb300::stream(exec), tree, numNodes, nodeOps, newTree);
    else
        rc = cs_rebalance_tree_u64(gb300::stream(exec), tree, numNodes, nodeOps, newTree);
    if (rc == CS_OK && cudaStreamSynchronize(static_cast<cudaStream_t>(exec)) != cudaSuccess) rc = CS_ERR_CUDA;
    gb300::check(rc, "rebalanceTreeGpu");
    return gb300::lastDecisionConverged;
}

template TreeNodeIndex computeNodeOpsGpu(execution::Gpu, const unsigned*, TreeNodeIndex, const unsigned*, unsigned,
                                         TreeNodeIndex*);
template TreeNodeIndex computeNodeOpsGpu(execution::Gpu, const uint64_t*, TreeNodeIndex, const unsigned*, unsigned,
                                         TreeNodeIndex*);
template bool rebalanceTreeGpu(execution::Gpu, const unsigned*, TreeNodeIndex, TreeNodeIndex, const TreeNodeIndex*,
                               unsigned*);
template bool rebalanceTreeGpu(execution::Gpu, const uint64_t*, TreeNodeIndex, TreeNodeIndex, const TreeNodeIndex*,
                               uint64_t*);

// ---- internal tree ----------------------------------------------------------------------------------------------
template<class KeyType>
void buildOctreeGpu(execution::Gpu exec, const KeyType* cstoneTree, OctreeView<KeyType> d, std::span<KeyType>,
                    std::span<TreeNodeIndex>, std::span<char> cubTmp)
{
    cs_octree_view v{d.numLeafNodes, d.numInternalNodes, d.numNodes,    d.prefixes,      d.childOffsets,
                     d.parents,      d.d_levelRange,     d.internalToLeaf, d.leafToInternal};
    constexpr int bits = int(8 * sizeof(KeyType));
    size_t need        = cs_build_octree_workspace_bytes(d.numLeafNodes, bits);
    // the caller's sort scratch serves as workspace when it is large enough
    void* ws   = cubTmp.size() >= need ? static_cast<void*>(cubTmp.data()) : nullptr;
    size_t wsb = ws ? cubTmp.size() : 0;
    int rc;
    if constexpr (gb300::isU32<KeyType>)
        rc = cs_build_octree_u32(gb300::stream(exec), cstoneTree, d.numLeafNodes, &v, d.levelRange, ws, wsb);
    else
        rc = cs_build_octree_u64(gb300::stream(exec), cstoneTree, d.numLeafNodes, &v, d.levelRange, ws, wsb);
    gb300::check(rc, "buildOctreeGpu");
}

template<class KeyType>
void buildOctreeGpu(execution::Gpu exec, const KeyType* cstoneTree, OctreeView<KeyType> d)
{
    buildOctreeGpu(exec, cstoneTree, d, std::span<KeyType>{}, std::span<TreeNodeIndex>{}, std::span<char>{});
}

template void buildOctreeGpu(execution::Gpu, const uint32_t*, OctreeView<uint32_t>, std::span<uint32_t>,
                             std::span<TreeNodeIndex>, std::span<char>);
template void buildOctreeGpu(execution::Gpu, const uint64_t*, OctreeView<uint64_t>, std::span<uint64_t>,
                             std::span<TreeNodeIndex>, std::span<char>);
template void buildOctreeGpu(execution::Gpu, const uint32_t*, OctreeView<uint32_t>);
template void buildOctreeGpu(execution::Gpu, const uint64_t*, OctreeView<uint64_t>);

// ---- node geometry and halos ------------------------------------------------------------------------------------
template<class KeyType, class T>
void computeGeoCentersGpu(execution::Gpu exec, const KeyType* prefixes, TreeNodeIndex numNodes, Vec3<T>* centers,
                          Vec3<T>* sizes, const Box<T>& box)
{
    cs_box cb = gb300::toBox(box);
    auto s    = gb300::stream(exec);
    auto* c   = reinterpret_cast<T*>(centers);
    auto* z   = reinterpret_cast<T*>(sizes);
    int rc;
    if constexpr (gb300::isU32<KeyType>)
    {
        if constexpr (std::is_same_v<T, double>) rc = cs_geo_centers_u32_f64(s, prefixes, numNodes, c, z, &cb, CS_HILBERT);
        else rc = cs_geo_centers_u32_f32(s, prefixes, numNodes, c, z, &cb, CS_HILBERT);
    }
    else
    {
        if constexpr (std::is_same_v<T, double>) rc = cs_geo_centers_u64_f64(s, prefixes, numNodes, c, z, &cb, CS_HILBERT);
        else rc = cs_geo_centers_u64_f32(s, prefixes, numNodes, c, z, &cb, CS_HILBERT);
    }
    gb300::check(rc, "computeGeoCentersGpu");
}

template void computeGeoCentersGpu(execution::Gpu, const uint32_t*, TreeNodeIndex, Vec3<float>*, Vec3<float>*,
                                   const Box<float>&);
template void computeGeoCentersGpu(execution::Gpu, const uint32_t*, TreeNodeIndex, Vec3<double>*, Vec3<double>*,
                                   const Box<double>&);
template void computeGeoCentersGpu(execution::Gpu, const uint64_t*, TreeNodeIndex, Vec3<float>*, Vec3<float>*,
                                   const Box<float>&);
template void computeGeoCentersGpu(execution::Gpu, const uint64_t*, TreeNodeIndex, Vec3<double>*, Vec3<double>*,
                                   const Box<double>&);

template<class Tc, class Th>
void computeBoundingBoxGpu(execution::Gpu exec, const Tc* x, const Tc* y, const Tc* z, const Th* h,
                           const LocalIndex* layout, TreeNodeIndex first, TreeNodeIndex last, Th scale,
                           Vec3<Tc>* centers, Vec3<Tc>* sizes)
{
    static_assert(std::is_same_v<Tc, Th> || (std::is_same_v<Tc, double> && std::is_same_v<Th, float>),
                  "h in the coordinate type, or float h with double coordinates");
    auto* c = reinterpret_cast<Tc*>(centers);
    auto* s = reinterpret_cast<Tc*>(sizes);
    int rc;
    // NULL leaf-to-node map: initialised from the caller's centres[leaf], as the reference kernel reads them
    if constexpr (std::is_same_v<Tc, double> && std::is_same_v<Th, float>)
        rc = cs_search_boxes_f64_hf32(gb300::stream(exec), x, y, z, h, layout, first, last, scale, nullptr, nullptr, c,
                                      s);
    else if constexpr (std::is_same_v<Tc, double>)
        rc = cs_search_boxes_f64(gb300::stream(exec), x, y, z, h, layout, first, last, scale, nullptr, nullptr, c, s);
    else
        rc = cs_search_boxes_f32(gb300::stream(exec), x, y, z, h, layout, first, last, scale, nullptr, nullptr, c, s);
    gb300::check(rc, "computeBoundingBoxGpu");
}

template void computeBoundingBoxGpu(execution::Gpu, const double*, const double*, const double*, const double*,
                                    const LocalIndex*, TreeNodeIndex, TreeNodeIndex, double, Vec3<double>*,
                                    Vec3<double>*);
template void computeBoundingBoxGpu(execution::Gpu, const double*, const double*, const double*, const float*,
                                    const LocalIndex*, TreeNodeIndex, TreeNodeIndex, float, Vec3<double>*,
                                    Vec3<double>*);
template void computeBoundingBoxGpu(execution::Gpu, const float*, const float*, const float*, const float*,
                                    const LocalIndex*, TreeNodeIndex, TreeNodeIndex, float, Vec3<float>*,
                                    Vec3<float>*);

template<class KeyType, class T>
void findHalosGpu(execution::Gpu exec, const KeyType* prefixes, const TreeNodeIndex* childOffsets,
                  const TreeNodeIndex* parents, const Vec3<T>* nodeCenters, const Vec3<T>* nodeSizes,
                  const KeyType* leaves, const Vec3<T>* searchCenters, const Vec3<T>* searchSizes, const Box<T>& box,
                  TreeNodeIndex firstNode, TreeNodeIndex lastNode, uint8_t* collisionFlags)
{
    cs_box cb = gb300::toBox(box);
    auto s    = gb300::stream(exec);
    auto nc   = reinterpret_cast<const T*>(nodeCenters);
    auto ns   = reinterpret_cast<const T*>(nodeSizes);
    auto sc   = reinterpret_cast<const T*>(searchCenters);
    auto ss   = reinterpret_cast<const T*>(searchSizes);
    int rc;
    if constexpr (gb300::isU32<KeyType>)
    {
        static_assert(std::is_same_v<T, float>, "the reference instantiates 32-bit keys with float only");
        rc = cs_find_halos_u32_f32(s, prefixes, childOffsets, parents, nc, ns, leaves, sc, ss, &cb, firstNode,
                                   lastNode, collisionFlags);
    }
    else if constexpr (std::is_same_v<T, double>)
        rc = cs_find_halos_u64_f64(s, prefixes, childOffsets, parents, nc, ns, leaves, sc, ss, &cb, firstNode,
                                   lastNode, collisionFlags);
    else
        rc = cs_find_halos_u64_f32(s, prefixes, childOffsets, parents, nc, ns, leaves, sc, ss, &cb, firstNode,
                                   lastNode, collisionFlags);
    gb300::check(rc, "findHalosGpu");
}

template void findHalosGpu(execution::Gpu, const uint32_t*, const TreeNodeIndex*, const TreeNodeIndex*,
                           const Vec3<float>*, const Vec3<float>*, const uint32_t*, const Vec3<float>*,
                           const Vec3<float>*, const Box<float>&, TreeNodeIndex, TreeNodeIndex, uint8_t*);
template void findHalosGpu(execution::Gpu, const uint64_t*, const TreeNodeIndex*, const TreeNodeIndex*,
                           const Vec3<float>*, const Vec3<float>*, const uint64_t*, const Vec3<float>*,
                           const Vec3<float>*, const Box<float>&, TreeNodeIndex, TreeNodeIndex, uint8_t*);
template void findHalosGpu(execution::Gpu, const uint64_t*, const TreeNodeIndex*, const TreeNodeIndex*,
                           const Vec3<double>*, const Vec3<double>*, const uint64_t*, const Vec3<double>*,
                           const Vec3<double>*, const Box<double>&, TreeNodeIndex, TreeNodeIndex, uint8_t*);

#ifdef CSTONE_GB300_STANDALONE
// ---- one rebalance/count step (tree/update_gpu.cuh:43-68 is a header template in the reference) ----------------
template<class KeyType, class DevKeyVec, class DevCountVec, class DevIdxVec>
bool updateOctreeGpu(execution::Gpu exec, std::span<const KeyType> keys, unsigned bucketSize, DevKeyVec& tree,
                     DevCountVec& counts, DevKeyVec& tmpTree, DevIdxVec& workArray,
                     unsigned maxCount = 0xFFFFFFFFu)
{
    workArray.resize(tree.size());
    TreeNodeIndex newNumNodes =
        computeNodeOpsGpu(exec, rawPtr(tree), nNodes(tree), rawPtr(counts), bucketSize, rawPtr(workArray));
    tmpTree.resize(newNumNodes + 1);
    bool converged = rebalanceTreeGpu(exec, rawPtr(tree), nNodes(tree), newNumNodes, rawPtr(workArray),
                                      rawPtr(tmpTree));
    swap(tree, tmpTree);
    counts.resize(nNodes(tree));
    computeNodeCountsGpu(exec, rawPtr(tree), rawPtr(counts), nNodes(tree), keys, maxCount, true);
    return converged;
}
#endif

} // namespace cstone
