/*
 * Thin C wrapper around the reference's own header-only CPU implementation, compiled in place from the reference
 * sources (see oracle/Makefile, target `ref`). Output goes to oracle/_ref/ only; nothing here is copied from the
 * reference. TEST INFRASTRUCTURE ONLY: used to pin the C restatement (cs_oracle.c) and to generate the golden
 * fixtures under tests/golden/.
 *
 * Entry points mirror cs_oracle.h (prefix csr_ instead of cso_), so the two can be compared call by call.
 */
#include <cstdint>
#include <span>
#include <vector>

#include "cstone/domain/layout.hpp"
#include "cstone/findneighbors.hpp"
#include "cstone/focus/rebalance.hpp"
#include "cstone/focus/source_center.hpp"
#include "cstone/sfc/sfc.hpp"
#include "cstone/traversal/collisions.hpp"
#include "cstone/tree/csarray.hpp"
#include "cstone/tree/octree.hpp"

using namespace cstone;

namespace
{
template<class T>
Box<T> makeBox(const double* lo, const double* hi, const int* bnd)
{
    return Box<T>(T(lo[0]), T(hi[0]), T(lo[1]), T(hi[1]), T(lo[2]), T(hi[2]), BoundaryType(bnd[0]),
                  BoundaryType(bnd[1]), BoundaryType(bnd[2]));
}

template<class T, class K, template<class> class Kind>
void keysImpl(const T* x, const T* y, const T* z, uint64_t* keys, size_t n, const Box<T>& box)
{
    std::vector<K> k(n);
    for (size_t i = 0; i < n; ++i)
        k[i] = K(keys[i]);
    computeSfcKeys(x, y, z, reinterpret_cast<Kind<K>*>(k.data()), n, box);
    for (size_t i = 0; i < n; ++i)
        keys[i] = k[i];
}

template<class T>
void keysDispatch(const T* x, const T* y, const T* z, uint64_t* keys, size_t n, const Box<T>& box, int kind,
                  int bits)
{
    if (kind == 1 && bits == 64) keysImpl<T, uint64_t, HilbertKey>(x, y, z, keys, n, box);
    if (kind == 1 && bits == 32) keysImpl<T, unsigned, HilbertKey>(x, y, z, keys, n, box);
    if (kind == 0 && bits == 64) keysImpl<T, uint64_t, MortonKey>(x, y, z, keys, n, box);
    if (kind == 0 && bits == 32) keysImpl<T, unsigned, MortonKey>(x, y, z, keys, n, box);
}

template<class K>
std::vector<K> narrow(const uint64_t* a, size_t n)
{
    return std::vector<K>(a, a + n);
}

template<class K>
int32_t computeOctreeImpl(const uint64_t* keys64, size_t n, unsigned bucket, uint32_t maxCount, uint64_t* tree,
                          uint32_t* counts, int32_t capacity, int* iterations)
{
    auto keys = narrow<K>(keys64, n);
    std::vector<K> t{0, nodeRange<K>(0)};
    std::vector<unsigned> c{unsigned(n)};
    int it = 0;
    while (true)
    {
        ++it;
        if (updateOctree<K>(std::span<const K>(keys), bucket, t, c, maxCount)) break;
    }
    if (iterations) *iterations = it;
    int32_t L = int32_t(nNodes(t));
    if (L > capacity) return -L;
    for (int32_t i = 0; i <= L; ++i)
        tree[i] = t[i];
    for (int32_t i = 0; i < L; ++i)
        counts[i] = c[i];
    return L;
}

template<class K>
int updateOctreeImpl(const uint64_t* keys64, size_t n, unsigned bucket, uint32_t maxCount, uint64_t* tree,
                     uint32_t* counts, int32_t* numNodes, int32_t capacity)
{
    auto keys = narrow<K>(keys64, n);
    std::vector<K> t(tree, tree + *numNodes + 1);
    std::vector<unsigned> c(counts, counts + *numNodes);
    bool conv = updateOctree<K>(std::span<const K>(keys), bucket, t, c, maxCount);
    int32_t L = int32_t(nNodes(t));
    if (L > capacity)
    {
        *numNodes = L;
        return -1;
    }
    for (int32_t i = 0; i <= L; ++i)
        tree[i] = t[i];
    for (int32_t i = 0; i < L; ++i)
        counts[i] = c[i];
    *numNodes = L;
    return conv ? 1 : 0;
}

template<class K>
void buildOctreeImpl(const uint64_t* leaves64, int32_t L, uint64_t* prefixes, int32_t* childOffsets,
                     int32_t* parents, int32_t* levelRange, int32_t* i2l, int32_t* l2i)
{
    auto leaves = narrow<K>(leaves64, size_t(L) + 1);
    OctreeData<K, execution::Cpu> o;
    o.resize(L);
    updateInternalTree<K>(std::span<const K>(leaves), o.data());
    for (int32_t i = 0; i < o.numNodes; ++i)
    {
        prefixes[i]     = o.prefixes[i];
        childOffsets[i] = o.childOffsets[i];
        i2l[i]          = o.internalToLeaf[i];
        l2i[i]          = o.leafToInternal[i];
    }
    for (size_t i = 0; i < o.parents.size(); ++i)
        parents[i] = o.parents[i];
    for (size_t i = 0; i < o.levelRange.size(); ++i)
        levelRange[i] = o.levelRange[i];
}

template<class K, class T>
void centersImpl(const uint64_t* prefixes64, int32_t numNodes, const Box<T>& box, T* centers, T* sizes)
{
    auto p = narrow<K>(prefixes64, size_t(numNodes));
    nodeFpCenters<K>(std::span<const K>(p), reinterpret_cast<Vec3<T>*>(centers), reinterpret_cast<Vec3<T>*>(sizes),
                     box);
}

template<class T, class Th = T>
void searchBoxesImpl(const T* x, const T* y, const T* z, const Th* h, const uint32_t* layout, int32_t first,
                     int32_t last, Th scale, const int32_t* l2i, const T* nodeCenters, T* sc, T* ss)
{
    for (int32_t leaf = first; leaf < last; ++leaf)
    {
        const T* c = nodeCenters + 3 * size_t(l2i[leaf]);
        Vec3<T> init{c[0], c[1], c[2]};
        auto [center, size] = computeBoundingBox(x, y, z, h, layout[leaf], layout[leaf + 1], scale, init);
        for (int k = 0; k < 3; ++k)
        {
            sc[3 * size_t(leaf) + k] = center[k];
            ss[3 * size_t(leaf) + k] = size[k];
        }
    }
}

template<class K, class T>
void findHalosImpl(const uint64_t* prefixes64, const int32_t* childOffsets, const int32_t* parents,
                   const T* nodeCenters, const T* nodeSizes, const uint64_t* leaves64, int32_t numNodes,
                   int32_t numLeaves, const T* sc, const T* ss, const Box<T>& box, int32_t first, int32_t last,
                   uint8_t* flags)
{
    auto p = narrow<K>(prefixes64, size_t(numNodes));
    auto l = narrow<K>(leaves64, size_t(numLeaves) + 1);
    findHalos(p.data(), childOffsets, parents, reinterpret_cast<const Vec3<T>*>(nodeCenters),
              reinterpret_cast<const Vec3<T>*>(nodeSizes), l.data(), reinterpret_cast<const Vec3<T>*>(sc),
              reinterpret_cast<const Vec3<T>*>(ss), box, first, last, flags);
}

template<class K, class T, class Th = T>
void findNeighborsImpl(const T* x, const T* y, const T* z, const Th* h, uint32_t first, uint32_t last,
                       const Box<T>& box, int32_t numLeaves, int32_t numNodes, const int32_t* childOffsets,
                       const int32_t* parents, const int32_t* i2l, const uint32_t* layout, const T* centers,
                       const T* sizes, float ext, unsigned ngmax, uint32_t* nb, uint32_t* nc)
{
    OctreeNsView<T, K> v{numLeaves,
                         numNodes,
                         nullptr,
                         childOffsets,
                         parents,
                         i2l,
                         nullptr,
                         nullptr,
                         nullptr,
                         layout,
                         reinterpret_cast<const Vec3<T>*>(centers),
                         reinterpret_cast<const Vec3<T>*>(sizes),
                         ext};
    findNeighbors(x, y, z, h, first, last, box, v, ngmax, nb, nc);
}
} // namespace

extern "C"
{
    uint64_t csr_imorton(unsigned ix, unsigned iy, unsigned iz, int bits)
    {
        return bits == 32 ? uint64_t(iMorton<unsigned>(ix, iy, iz)) : iMorton<uint64_t>(ix, iy, iz);
    }
    uint64_t csr_ihilbert(unsigned ix, unsigned iy, unsigned iz, int bits)
    {
        return bits == 32 ? uint64_t(iHilbert<unsigned>(ix, iy, iz)) : iHilbert<uint64_t>(ix, iy, iz);
    }
    void csr_decode_hilbert(uint64_t key, int bits, unsigned* ixyz)
    {
        auto t = bits == 32 ? decodeHilbert<unsigned>(unsigned(key)) : decodeHilbert<uint64_t>(key);
        ixyz[0] = util::get<0>(t);
        ixyz[1] = util::get<1>(t);
        ixyz[2] = util::get<2>(t);
    }
    void csr_sfc_keys_f64(const double* x, const double* y, const double* z, uint64_t* keys, size_t n,
                          const double* lo, const double* hi, const int* bnd, int kind, int bits)
    {
        keysDispatch<double>(x, y, z, keys, n, makeBox<double>(lo, hi, bnd), kind, bits);
    }
    void csr_sfc_keys_f32(const float* x, const float* y, const float* z, uint64_t* keys, size_t n,
                          const double* lo, const double* hi, const int* bnd, int kind, int bits)
    {
        keysDispatch<float>(x, y, z, keys, n, makeBox<float>(lo, hi, bnd), kind, bits);
    }
    void csr_sort_by_key(uint64_t* keys, uint32_t* values, size_t n)
    {
        std::vector<uint64_t> k(keys, keys + n);
        std::vector<uint32_t> v(values, values + n);
        sort_by_key(k.begin(), k.end(), v.begin());
        for (size_t i = 0; i < n; ++i)
        {
            keys[i]   = k[i];
            values[i] = v[i];
        }
    }
    void csr_find_search_bounds(int64_t guess, uint64_t target, const uint64_t* codes, int64_t n, int64_t* lo,
                                int64_t* hi)
    {
        auto r = findSearchBounds<uint64_t>(guess, target, codes, codes + n);
        *lo    = r[0] - codes;
        *hi    = r[1] - codes;
    }
    void csr_node_counts(const uint64_t* tree, uint32_t* counts, int32_t numNodes, const uint64_t* keys, size_t n,
                         uint32_t maxCount, int useGuess, int bits)
    {
        if (bits == 64)
        {
            computeNodeCounts<uint64_t>(tree, counts, numNodes, std::span<const uint64_t>(keys, n), maxCount,
                                        useGuess != 0);
        }
        else
        {
            auto t = narrow<unsigned>(tree, size_t(numNodes) + 1);
            auto k = narrow<unsigned>(keys, n);
            computeNodeCounts<unsigned>(t.data(), counts, numNodes, std::span<const unsigned>(k), maxCount,
                                        useGuess != 0);
        }
    }
    int csr_rebalance_decision(const uint64_t* tree, const uint32_t* counts, int32_t numNodes, unsigned bucket,
                               int32_t* ops, int bits)
    {
        if (bits == 64) return rebalanceDecision(tree, counts, numNodes, bucket, ops);
        auto t = narrow<unsigned>(tree, size_t(numNodes) + 1);
        return rebalanceDecision(t.data(), counts, numNodes, bucket, ops);
    }
    int32_t csr_compute_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t maxCount, uint64_t* tree,
                               uint32_t* counts, int32_t capacity, int bits, int* iterations)
    {
        if (bits == 64) return computeOctreeImpl<uint64_t>(keys, n, bucket, maxCount, tree, counts, capacity, iterations);
        return computeOctreeImpl<unsigned>(keys, n, bucket, maxCount, tree, counts, capacity, iterations);
    }
    int csr_update_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t maxCount, uint64_t* tree,
                          uint32_t* counts, int32_t* numNodes, int32_t capacity, int bits)
    {
        if (bits == 64) return updateOctreeImpl<uint64_t>(keys, n, bucket, maxCount, tree, counts, numNodes, capacity);
        return updateOctreeImpl<unsigned>(keys, n, bucket, maxCount, tree, counts, numNodes, capacity);
    }
    int32_t csr_binary_key_weight(uint64_t key, unsigned level, int bits)
    {
        return bits == 64 ? binaryKeyWeight<uint64_t>(key, level) : binaryKeyWeight<unsigned>(unsigned(key), level);
    }
    void csr_build_octree(const uint64_t* leaves, int32_t L, int bits, uint64_t* prefixes, int32_t* childOffsets,
                          int32_t* parents, int32_t* levelRange, int32_t* i2l, int32_t* l2i)
    {
        if (bits == 64) buildOctreeImpl<uint64_t>(leaves, L, prefixes, childOffsets, parents, levelRange, i2l, l2i);
        else buildOctreeImpl<unsigned>(leaves, L, prefixes, childOffsets, parents, levelRange, i2l, l2i);
    }
    void csr_node_fp_centers_f64(const uint64_t* prefixes, int32_t numNodes, int bits, const double* lo,
                                 const double* hi, const int* bnd, double* centers, double* sizes)
    {
        auto box = makeBox<double>(lo, hi, bnd);
        if (bits == 64) centersImpl<uint64_t, double>(prefixes, numNodes, box, centers, sizes);
        else centersImpl<unsigned, double>(prefixes, numNodes, box, centers, sizes);
    }
    void csr_node_fp_centers_f32(const uint64_t* prefixes, int32_t numNodes, int bits, const double* lo,
                                 const double* hi, const int* bnd, float* centers, float* sizes)
    {
        auto box = makeBox<float>(lo, hi, bnd);
        if (bits == 64) centersImpl<uint64_t, float>(prefixes, numNodes, box, centers, sizes);
        else centersImpl<unsigned, float>(prefixes, numNodes, box, centers, sizes);
    }
    void csr_search_boxes_f64(const double* x, const double* y, const double* z, const double* h,
                              const uint32_t* layout, int32_t first, int32_t last, double scale, const int32_t* l2i,
                              const double* nodeCenters, double* sc, double* ss)
    {
        searchBoxesImpl<double>(x, y, z, h, layout, first, last, scale, l2i, nodeCenters, sc, ss);
    }
    void csr_search_boxes_f64_hf32(const double* x, const double* y, const double* z, const float* h,
                                   const uint32_t* layout, int32_t first, int32_t last, float scale,
                                   const int32_t* l2i, const double* nodeCenters, double* sc, double* ss)
    {
        searchBoxesImpl<double, float>(x, y, z, h, layout, first, last, scale, l2i, nodeCenters, sc, ss);
    }
    void csr_find_neighbors_f64_hf32(const double* x, const double* y, const double* z, const float* h,
                                     uint32_t first, uint32_t last, const double* lo, const double* hi,
                                     const int* bnd, int32_t numLeaves, int32_t numNodes,
                                     const int32_t* childOffsets, const int32_t* parents, const int32_t* i2l,
                                     const uint32_t* layout, const double* centers, const double* sizes, float ext,
                                     unsigned ngmax, uint32_t* nb, uint32_t* nc)
    {
        auto box = makeBox<double>(lo, hi, bnd);
        findNeighborsImpl<uint64_t, double, float>(x, y, z, h, first, last, box, numLeaves, numNodes, childOffsets,
                                                   parents, i2l, layout, centers, sizes, ext, ngmax, nb, nc);
    }
    void csr_search_boxes_f32(const float* x, const float* y, const float* z, const float* h,
                              const uint32_t* layout, int32_t first, int32_t last, float scale, const int32_t* l2i,
                              const float* nodeCenters, float* sc, float* ss)
    {
        searchBoxesImpl<float>(x, y, z, h, layout, first, last, scale, l2i, nodeCenters, sc, ss);
    }
    void csr_find_halos_f64(const uint64_t* prefixes, const int32_t* childOffsets, const int32_t* parents,
                            const double* nc, const double* ns, const uint64_t* leaves, int32_t numNodes,
                            int32_t numLeaves, const double* sc, const double* ss, const double* lo,
                            const double* hi, const int* bnd, int32_t first, int32_t last, int bits, uint8_t* flags)
    {
        auto box = makeBox<double>(lo, hi, bnd);
        if (bits == 64)
            findHalosImpl<uint64_t, double>(prefixes, childOffsets, parents, nc, ns, leaves, numNodes, numLeaves, sc,
                                            ss, box, first, last, flags);
        else
            findHalosImpl<unsigned, double>(prefixes, childOffsets, parents, nc, ns, leaves, numNodes, numLeaves, sc,
                                            ss, box, first, last, flags);
    }
    void csr_find_halos_f32(const uint64_t* prefixes, const int32_t* childOffsets, const int32_t* parents,
                            const float* nc, const float* ns, const uint64_t* leaves, int32_t numNodes,
                            int32_t numLeaves, const float* sc, const float* ss, const double* lo, const double* hi,
                            const int* bnd, int32_t first, int32_t last, int bits, uint8_t* flags)
    {
        auto box = makeBox<float>(lo, hi, bnd);
        if (bits == 64)
            findHalosImpl<uint64_t, float>(prefixes, childOffsets, parents, nc, ns, leaves, numNodes, numLeaves, sc,
                                           ss, box, first, last, flags);
        else
            findHalosImpl<unsigned, float>(prefixes, childOffsets, parents, nc, ns, leaves, numNodes, numLeaves, sc,
                                           ss, box, first, last, flags);
    }
    void csr_find_neighbors_f64(const double* x, const double* y, const double* z, const double* h, uint32_t first,
                                uint32_t last, const double* lo, const double* hi, const int* bnd, int32_t numLeaves,
                                int32_t numNodes, const int32_t* childOffsets, const int32_t* parents,
                                const int32_t* i2l, const uint32_t* layout, const double* centers,
                                const double* sizes, float ext, unsigned ngmax, uint32_t* nb, uint32_t* nc)
    {
        auto box = makeBox<double>(lo, hi, bnd);
        findNeighborsImpl<uint64_t, double>(x, y, z, h, first, last, box, numLeaves, numNodes, childOffsets, parents,
                                            i2l, layout, centers, sizes, ext, ngmax, nb, nc);
    }
    void csr_find_neighbors_f32(const float* x, const float* y, const float* z, const float* h, uint32_t first,
                                uint32_t last, const double* lo, const double* hi, const int* bnd, int32_t numLeaves,
                                int32_t numNodes, const int32_t* childOffsets, const int32_t* parents,
                                const int32_t* i2l, const uint32_t* layout, const float* centers, const float* sizes,
                                float ext, unsigned ngmax, uint32_t* nb, uint32_t* nc)
    {
        auto box = makeBox<float>(lo, hi, bnd);
        findNeighborsImpl<uint64_t, float>(x, y, z, h, first, last, box, numLeaves, numNodes, childOffsets, parents,
                                           i2l, layout, centers, sizes, ext, ngmax, nb, nc);
    }
}

// ---- around the path: upsweeps, source centres, SFC gaps, focus rebalance ----
namespace
{
template<class K>
int32_t spanningTreeImpl(const uint64_t* keys64, int32_t nKeys, uint64_t* out, int32_t cap)
{
    auto keys = narrow<K>(keys64, size_t(nKeys));
    auto t    = computeSpanningTree<K>(std::span<const K>(keys));
    if (int32_t(t.size()) > cap) return -int32_t(t.size());
    for (size_t i = 0; i < t.size(); ++i)
        out[i] = t[i];
    return int32_t(t.size());
}

template<class K>
void essentialImpl(const uint64_t* prefixes64, const int32_t* childOffsets, const int32_t* parents,
                   const uint32_t* counts, const uint8_t* macs, int32_t numNodes, uint64_t f0, uint64_t f1,
                   unsigned bucket, int32_t* ops)
{
    auto prefixes = narrow<K>(prefixes64, size_t(numNodes));
    rebalanceDecisionEssential<K>(std::span<const K>(prefixes), childOffsets, parents, counts, macs, K(f0), K(f1),
                                  bucket, ops);
}

template<class K>
int protectImpl(const uint64_t* prefixes64, const int32_t* parents, int32_t* ops, int32_t numNodes)
{
    auto prefixes = narrow<K>(prefixes64, size_t(numNodes));
    return protectAncestors<K>(std::span<const K>(prefixes), parents, ops) ? 1 : 0;
}

template<class K>
int enforceImpl(const uint64_t* keys64, int32_t nKeys, const uint64_t* prefixes64, int32_t numNodes,
                const int32_t* childOffsets, const int32_t* parents, int32_t* ops)
{
    auto keys     = narrow<K>(keys64, size_t(nKeys));
    auto prefixes = narrow<K>(prefixes64, size_t(numNodes));
    return int(enforceKeys<K>(std::span<const K>(keys), prefixes.data(), childOffsets, parents, ops));
}

template<class K>
void rangeCountImpl(const uint64_t* leaves64, int32_t nLeafKeys, const uint32_t* counts, const uint64_t* focus64,
                    int32_t nFocusKeys, const int32_t* idx, int32_t nIdx, uint32_t* countsFocus)
{
    auto leaves = narrow<K>(leaves64, size_t(nLeafKeys));
    auto focus  = narrow<K>(focus64, size_t(nFocusKeys));
    rangeCount<K>(std::span<const K>(leaves), std::span<const unsigned>(counts, size_t(nLeafKeys - 1)),
                  std::span<const K>(focus), std::span<const TreeNodeIndex>(idx, size_t(nIdx)),
                  std::span<unsigned>(countsFocus, size_t(nFocusKeys - 1)));
}
} // namespace

extern "C"
{
    int32_t csr_spanning_tree(const uint64_t* keys, int32_t nKeys, uint64_t* out, int32_t cap, int bits)
    {
        return bits == 64 ? spanningTreeImpl<uint64_t>(keys, nKeys, out, cap)
                          : spanningTreeImpl<unsigned>(keys, nKeys, out, cap);
    }
    void csr_upsweep_sum(const int32_t* levelRange, int numLevels, const int32_t* childOffsets, uint32_t* counts)
    {
        std::vector<TreeNodeIndex> lr(levelRange, levelRange + numLevels + 1);
        upsweep(std::span<const TreeNodeIndex>(lr), childOffsets, counts, NodeCount<unsigned>{});
    }
    void csr_leaf_mass_centers_f64(const double* x, const double* y, const double* z, const double* m,
                                   const int32_t* l2i, int32_t numLeaves, const uint32_t* layout, double* centers,
                                   size_t n)
    {
        computeLeafMassCenter<double, double, double>(
            std::span<const double>(x, n), std::span<const double>(y, n), std::span<const double>(z, n),
            std::span<const double>(m, n), std::span<const TreeNodeIndex>(l2i, size_t(numLeaves)), layout,
            reinterpret_cast<SourceCenterType<double>*>(centers));
    }
    void csr_leaf_mass_centers_f32(const float* x, const float* y, const float* z, const float* m, const int32_t* l2i,
                                   int32_t numLeaves, const uint32_t* layout, float* centers, size_t n)
    {
        computeLeafMassCenter<float, float, float>(
            std::span<const float>(x, n), std::span<const float>(y, n), std::span<const float>(z, n),
            std::span<const float>(m, n), std::span<const TreeNodeIndex>(l2i, size_t(numLeaves)), layout,
            reinterpret_cast<SourceCenterType<float>*>(centers));
    }
    void csr_upsweep_centers_f64(const int32_t* levelRange, int numLevels, const int32_t* childOffsets,
                                 double* centers)
    {
        std::vector<TreeNodeIndex> lr(levelRange, levelRange + numLevels + 1);
        upsweep(std::span<const TreeNodeIndex>(lr), childOffsets, reinterpret_cast<SourceCenterType<double>*>(centers),
                CombineSourceCenter<double>{});
    }
    void csr_upsweep_centers_f32(const int32_t* levelRange, int numLevels, const int32_t* childOffsets,
                                 float* centers)
    {
        std::vector<TreeNodeIndex> lr(levelRange, levelRange + numLevels + 1);
        upsweep(std::span<const TreeNodeIndex>(lr), childOffsets, reinterpret_cast<SourceCenterType<float>*>(centers),
                CombineSourceCenter<float>{});
    }
    void csr_rebalance_decision_essential(const uint64_t* prefixes, const int32_t* childOffsets,
                                          const int32_t* parents, const uint32_t* counts, const uint8_t* macs,
                                          int32_t numNodes, uint64_t f0, uint64_t f1, unsigned bucket, int32_t* ops,
                                          int bits)
    {
        if (bits == 64) essentialImpl<uint64_t>(prefixes, childOffsets, parents, counts, macs, numNodes, f0, f1, bucket, ops);
        else essentialImpl<unsigned>(prefixes, childOffsets, parents, counts, macs, numNodes, f0, f1, bucket, ops);
    }
    int csr_mac_refine_op(uint64_t prefix, int mac, int bits)
    {
        return bits == 64 ? macRefineOp<uint64_t>(prefix, char(mac)) : macRefineOp<unsigned>(unsigned(prefix), char(mac));
    }
    int csr_protect_ancestors(const uint64_t* prefixes, const int32_t* parents, int32_t* ops, int32_t numNodes,
                              int bits)
    {
        return bits == 64 ? protectImpl<uint64_t>(prefixes, parents, ops, numNodes)
                          : protectImpl<unsigned>(prefixes, parents, ops, numNodes);
    }
    int csr_enforce_keys(const uint64_t* keys, int32_t nKeys, const uint64_t* prefixes, int32_t numNodes,
                         const int32_t* childOffsets, const int32_t* parents, int32_t* ops, int bits)
    {
        return bits == 64 ? enforceImpl<uint64_t>(keys, nKeys, prefixes, numNodes, childOffsets, parents, ops)
                          : enforceImpl<unsigned>(keys, nKeys, prefixes, numNodes, childOffsets, parents, ops);
    }
    void csr_range_count(const uint64_t* leaves, int32_t nLeafKeys, const uint32_t* counts, const uint64_t* focus,
                         int32_t nFocusKeys, const int32_t* idx, int32_t nIdx, uint32_t* countsFocus, int bits)
    {
        if (bits == 64) rangeCountImpl<uint64_t>(leaves, nLeafKeys, counts, focus, nFocusKeys, idx, nIdx, countsFocus);
        else rangeCountImpl<unsigned>(leaves, nLeafKeys, counts, focus, nFocusKeys, idx, nIdx, countsFocus);
    }
    void csr_node_layout(const uint32_t* counts, int32_t numLeaves, const uint8_t* flags, int32_t numNodes,
                         const int32_t* l2i, int32_t first, int32_t last, uint32_t* layout)
    {
        computeNodeLayout(execution::Cpu{}, std::span<const unsigned>(counts, size_t(numLeaves)),
                          std::span<const uint8_t>(flags, size_t(numNodes)),
                          std::span<const TreeNodeIndex>(l2i, size_t(numLeaves)), TreeIndexPair(first, last),
                          std::span<LocalIndex>(layout, size_t(numLeaves) + 1));
    }
}
