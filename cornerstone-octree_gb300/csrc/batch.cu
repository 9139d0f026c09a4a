// Batched independent sets (cs_batch_*): many particle sets of uneven size through keys -> sort -> build -> link ->
// geometry -> neighbours in one sequence of launches, each set's results equal to its own single-set pipeline run.
//
// Set s of S keeps its own box and bucket size. Its 32-bit SFC key k (10 levels) becomes the 64-bit key (s << 30) | k,
// so the key range of set s is the aligned node of level 11 at s << 30, and the 10 levels of the set's own tree are
// levels 11..21 of the combined one. Then:
//   keys     one kernel over all particles (the set of a particle by binary search in the offsets)
//   sort     one stable radix sort of the combined keys over 30 + ceil(log2 S) bits: every set sorted by its own
//            key, the sets in order (the segmented sort)
//   build    one cooperative cornerstone build from the leaf array {set roots, empty fillers up to 2^63}: the
//            decision of a leaf uses its set's bucket size, and no node at or above level 11 merges, so each set's
//            leaves go through exactly the iterations of its own build from its root (a converged set stays fixed
//            while others still change)
//   link     the usual internal-tree link of the combined leaves
//   geometry each node decoded with its set's box and its level inside the set's tree
//   roots    the node of each set's root (level 11) and the first leaf of each set
//   search   the neighbour traversal of a particle starts at its set's root; exact path checks stop there
#include "cs_common.cuh"
#include "neighbors.cuh"
#include "octree_build.cuh"
#include "octree_link.cuh"
#include "radix_sort.cuh"
#include "sfc_keys.cuh"

#include <algorithm>
#include <memory>
#include <vector>

namespace csg
{

constexpr int SET_SHIFT  = 30; // bits of a set's own key
constexpr int ROOT_LEVEL = 11; // level of a set root in the combined 64-bit tree: 63 - 3 * 11 = 30

// per set: its root node (the level-11 node of key s << 30) and its first leaf
__global__ void setRootsKernel(const uint64_t* __restrict__ prefixes, const int32_t* __restrict__ levelRange,
                               const uint64_t* __restrict__ leaves, int L, int numSets, int32_t* __restrict__ roots,
                               int32_t* __restrict__ leafBegin)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > numSets) return;
    const uint64_t key = uint64_t(s) << SET_SHIFT;
    int lo = 0, hi = L + 1;
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (leaves[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    leafBegin[s] = lo;
    if (s == numSets) return;
    const uint64_t want = encodePlaceholderBit<uint64_t>(key, 3 * ROOT_LEVEL);
    lo = levelRange[ROOT_LEVEL];
    hi = levelRange[ROOT_LEVEL + 1];
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (prefixes[mid] < want) lo = mid + 1;
        else hi = mid;
    }
    roots[s] = lo; // a set root is never merged away, so it is always present at level 11
}

struct BatchBase
{
    cs_batch_config cfg{};
    cs_tuning tuning{32, 7, 16};
    virtual ~BatchBase() = default;
    virtual int run(cudaStream_t s, const void* x, const void* y, const void* z, const void* h, const uint32_t* off,
                    int S, const cs_box* boxes, const uint32_t* buckets, cs_batch_result* res) = 0;
    virtual int outputs(cs_batch_outputs* o) = 0;
    virtual size_t deviceBytes() const       = 0;
};

template<class T>
struct Batch final : BatchBase
{
    DevBuf keys, keysAlt, order, orderAlt, packed, xs, ys, zs, hs, shadowHi, shadowLo, sortWs, errWords;
    DevBuf setOff, keyParams, geoParams, buckets, initTree, initOff, roots, leafBegin;
    DevBuf buildWs, leaves, counts, layout;
    DevBuf prefixes, childOffsets, parents, levelRange, i2l, l2i, linkWs, centers, sizes;
    DevBuf nbPrepWs, pout, nb, nc;
    int capacity = 0;
    size_t n     = 0;
    cs_batch_result last{};
    bool haveRun          = false;
    uint64_t* sortedKeys  = nullptr;
    uint32_t* sortedOrder = nullptr;

    size_t deviceBytes() const override
    {
        size_t t = 0;
        for (const DevBuf* b : {&keys, &keysAlt, &order, &orderAlt, &packed, &xs, &ys, &zs, &hs, &shadowHi, &shadowLo,
                                &sortWs, &errWords,
                                &setOff, &keyParams, &geoParams, &buckets, &initTree, &initOff, &roots, &leafBegin,
                                &buildWs, &leaves, &counts, &layout, &prefixes, &childOffsets, &parents, &levelRange,
                                &i2l, &l2i, &linkWs, &centers, &sizes, &nbPrepWs, &pout, &nb, &nc})
            t += b->bytes;
        return t;
    }

    int run(cudaStream_t s, const void* xv, const void* yv, const void* zv, const void* hv, const uint32_t* off,
            int S, const cs_box* boxes, const uint32_t* bk, cs_batch_result* res) override
    {
        int rc;
        if (S < 1 || S > (1 << 24) || !off || !boxes || !bk)
        {
            setLastError("batch: %d sets (1 .. 2^24) with offsets, boxes and bucket sizes needed", S);
            return CS_ERR_INVALID;
        }
        if (off[0] != 0)
        {
            setLastError("batch: the first set offset must be 0");
            return CS_ERR_INVALID;
        }
        for (int j = 0; j < S; ++j)
            if (off[j + 1] < off[j] || bk[j] == 0)
            {
                setLastError("batch: set %d has decreasing offsets or a zero bucket size", j);
                return CS_ERR_INVALID;
            }
        n = off[S];
        if (n == 0 || n >= (size_t(1) << 30))
        {
            setLastError("batch: %zu particles outside [1, 2^30)", n);
            return CS_ERR_INVALID;
        }
        const T *x = static_cast<const T*>(xv), *y = static_cast<const T*>(yv), *z = static_cast<const T*>(zv),
                *h = static_cast<const T*>(hv);
        int setBits = 0;
        while ((1 << setBits) < S)
            ++setBits;
        const int keyBits = SET_SHIFT + setBits;

        for (DevBuf* b : {&keys, &keysAlt})
            if ((rc = b->ensure(n * sizeof(uint64_t)))) return rc;
        for (DevBuf* b : {&order, &orderAlt, &nc})
            if ((rc = b->ensure(n * sizeof(uint32_t)))) return rc;
        for (DevBuf* b : {&xs, &ys, &zs, &hs})
            if ((rc = b->ensure(n * sizeof(T)))) return rc;
        if ((rc = packed.ensure(n * sizeof(PackedT<T>)))) return rc;
        constexpr bool F64 = std::is_same_v<T, double>;
        const bool shadows = F64 && cfg.do_neighbors;
        if (shadows)
            for (DevBuf* b : {&shadowHi, &shadowLo})
                if ((rc = b->ensure(n * sizeof(float4)))) return rc;
        if ((rc = sortWs.ensure(radixSortWorkspaceBytes<uint64_t>(n, 0, keyBits)))) return rc;
        if ((rc = errWords.ensure(64))) return rc;
        if ((rc = setOff.ensure((size_t(S) + 1) * sizeof(uint32_t)))) return rc;
        if ((rc = keyParams.ensure(size_t(S) * sizeof(KeyParams<T, uint32_t>)))) return rc;
        if ((rc = geoParams.ensure(geoParamsBytes<T>(S)))) return rc;
        if ((rc = buckets.ensure(size_t(S) * sizeof(uint32_t)))) return rc;
        if ((rc = roots.ensure(size_t(S) * sizeof(int32_t)))) return rc;
        if ((rc = leafBegin.ensure((size_t(S) + 1) * sizeof(int32_t)))) return rc;
        uint32_t* err = errWords.as<uint32_t>();
        float* cmax   = reinterpret_cast<float*>(err + 8);
        CSG_CUDA_TRY(cudaMemsetAsync(err, 0, 64, s));

        // per-set parameters (pageable host sources: each copy returns once its source is staged)
        std::vector<KeyParams<T, uint32_t>> kp(S);
        for (int j = 0; j < S; ++j)
            kp[j] = makeKeyParams<T, uint32_t>(makeBoxParams<T>(boxes[j]));
        CSG_CUDA_TRY(cudaMemcpyAsync(setOff.p, off, (size_t(S) + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CSG_CUDA_TRY(cudaMemcpyAsync(keyParams.p, kp.data(), kp.size() * sizeof(kp[0]), cudaMemcpyHostToDevice, s));
        CSG_CUDA_TRY(cudaMemcpyAsync(buckets.p, bk, size_t(S) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));

        // ---- keys, the segmented sort, gather ----
        if ((rc = sfcKeysBatched<T>(s, x, y, z, h, n, setOff.as<uint32_t>(), S, keyParams.as<KeyParams<T, uint32_t>>(),
                                    cfg.sfc_kind, keys.as<uint64_t>(), packed.as<PackedT<T>>())))
            return rc;
        bool inAlt = false;
        rc = radixSortPairs<uint64_t>(s, keys.as<uint64_t>(), order.as<uint32_t>(), keysAlt.as<uint64_t>(),
                                      orderAlt.as<uint32_t>(), n, 0, keyBits, true, sortWs.p, sortWs.bytes, err,
                                      &inAlt, tuning.sort_items);
        if (rc) return rc;
        sortedKeys  = inAlt ? keysAlt.as<uint64_t>() : keys.as<uint64_t>();
        sortedOrder = inAlt ? orderAlt.as<uint32_t>() : order.as<uint32_t>();
        if ((rc = gatherPacked<T>(s, sortedOrder, n, packed.as<PackedT<T>>(), xs.as<T>(), ys.as<T>(), zs.as<T>(),
                                  hs.as<T>(), shadows ? shadowHi.as<float4>() : nullptr,
                                  shadows ? shadowLo.as<float4>() : nullptr, cmax)))
            return rc;

        // ---- the starting leaf array: set roots, then the empty nodes that span [S << 30, 2^63) ----
        std::vector<uint64_t> t0;
        std::vector<uint32_t> o0;
        for (int j = 0; j < S; ++j)
        {
            t0.push_back(uint64_t(j) << SET_SHIFT);
            o0.push_back(off[j]);
        }
        const uint64_t end = nodeRange<uint64_t>(0);
        for (uint64_t k = uint64_t(S) << SET_SHIFT; k < end;)
        {
            uint64_t r = nodeRange<uint64_t>(ROOT_LEVEL);
            while (k % (r * 8) == 0 && k + r * 8 <= end && r * 8 <= nodeRange<uint64_t>(1))
                r *= 8;
            t0.push_back(k);
            o0.push_back(uint32_t(n));
            k += r;
        }
        t0.push_back(end);
        o0.push_back(uint32_t(n));
        const int L0 = int(t0.size()) - 1;
        if ((rc = initTree.ensure(t0.size() * sizeof(uint64_t)))) return rc;
        if ((rc = initOff.ensure(o0.size() * sizeof(uint32_t)))) return rc;
        CSG_CUDA_TRY(cudaMemcpyAsync(initTree.p, t0.data(), t0.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        CSG_CUDA_TRY(cudaMemcpyAsync(initOff.p, o0.data(), o0.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));

        // ---- one cooperative build of every set ----
        BatchTree<uint64_t> bt;
        bt.initTree      = initTree.as<uint64_t>();
        bt.initOff       = initOff.as<uint32_t>();
        bt.initL         = L0;
        bt.setBucket     = buckets.as<uint32_t>();
        bt.setShift      = SET_SHIFT;
        bt.numSets       = S;
        bt.minMergeLevel = ROOT_LEVEL;
        uint32_t minBucket = *std::min_element(bk, bk + S);
        if (capacity == 0)
            capacity = int(std::min<size_t>(size_t(1) << 30, n / std::max(1u, minBucket) * 4 + size_t(L0) + 4096));
        BuildResult br;
        for (;;)
        {
            if ((rc = buildWs.ensure(octreeBuildWorkspaceBytes<uint64_t>(capacity, false)))) return rc;
            if ((rc = leaves.ensure((size_t(capacity) + 1) * sizeof(uint64_t)))) return rc;
            if ((rc = counts.ensure(size_t(capacity) * sizeof(uint32_t)))) return rc;
            if ((rc = layout.ensure((size_t(capacity) + 1) * sizeof(uint32_t)))) return rc;
            br = BuildResult{};
            rc = octreeBuild<uint64_t>(s, sortedKeys, n, 64, 0xffffffffu, nullptr, nullptr, 0, leaves.as<uint64_t>(),
                                       counts.as<uint32_t>(), layout.as<uint32_t>(), capacity, buildWs.p,
                                       buildWs.bytes, &br, true, FocusQuery<uint64_t>{}, nullptr, &bt, err);
            if (rc == CS_ERR_CAPACITY)
            {
                capacity = std::max(2 * capacity, br.needed + br.needed / 4);
                continue;
            }
            if (rc) return rc;
            break;
        }
        const int L = br.numLeaves, I = (L - 1) / 7, N = L + I;

        // ---- link, geometry, set roots ----
        if ((rc = prefixes.ensure(size_t(N) * sizeof(uint64_t)))) return rc;
        if ((rc = childOffsets.ensure((size_t(N) + 1) * sizeof(int32_t)))) return rc;
        if ((rc = parents.ensure(size_t(std::max(1, (N - 1) / 8)) * sizeof(int32_t)))) return rc;
        if ((rc = levelRange.ensure(size_t(KeyTraits<uint64_t>::maxLevel + 2) * sizeof(int32_t)))) return rc;
        if ((rc = i2l.ensure(size_t(N) * sizeof(int32_t)))) return rc;
        if ((rc = l2i.ensure(size_t(N) * sizeof(int32_t)))) return rc;
        if ((rc = linkWs.ensure(buildLinkWorkspaceBytes<uint64_t>(L)))) return rc;
        cs_octree_view v{L, I, N, prefixes.p, childOffsets.as<int32_t>(), parents.as<int32_t>(),
                         levelRange.as<int32_t>(), i2l.as<int32_t>(), l2i.as<int32_t>()};
        int prefixBits = std::min(64, 3 * br.maxDepth + 1);
        if ((rc = buildLink<uint64_t>(s, leaves.as<uint64_t>(), L, v, prefixBits, linkWs.p, linkWs.bytes, err + 1)))
            return rc;
        if ((rc = centers.ensure(3 * size_t(N) * sizeof(T)))) return rc;
        if ((rc = sizes.ensure(3 * size_t(N) * sizeof(T)))) return rc;
        if ((rc = geoCentersBatched<T>(s, prefixes.as<uint64_t>(), N, centers.as<T>(), sizes.as<T>(), boxes, S,
                                       cfg.sfc_kind, geoParams.p, ROOT_LEVEL)))
            return rc;
        setRootsKernel<<<iceil(size_t(S) + 1, 256), 256, 0, s>>>(prefixes.as<uint64_t>(), levelRange.as<int32_t>(),
                                                                 leaves.as<uint64_t>(), L, S, roots.as<int32_t>(),
                                                                 leafBegin.as<int32_t>());
        CSG_CHECK_LAUNCH();

        // ---- neighbours, each particle from its set's root ----
        if (cfg.do_neighbors)
        {
            if ((rc = nb.ensure(std::max<size_t>(1, n * cfg.ngmax) * sizeof(uint32_t)))) return rc;
            if ((rc = nbPrepWs.ensure(nbPrepBytes(0, N)))) return rc;
            if ((rc = pout.ensure(n))) return rc;
            NbPrep prep{};
            prep.cmax = cmax;
            prep.phi  = shadows ? shadowHi.as<float4>() : nullptr;
            prep.plo  = shadows ? shadowLo.as<float4>() : nullptr;
            if ((rc = nbPrepareNodes<T>(s, centers.as<T>(), sizes.as<T>(), childOffsets.as<int32_t>(),
                                        i2l.as<int32_t>(), layout.as<uint32_t>(), N, nbPrepWs.p, nbPrepWs.bytes,
                                        &prep)))
                return rc;
            if ((rc = nbMarkOutside<T>(s, xs.as<T>(), ys.as<T>(), zs.as<T>(), prep.phi, centers.as<T>(), sizes.as<T>(),
                                       childOffsets.as<int32_t>(), i2l.as<int32_t>(), layout.as<uint32_t>(), N, prep,
                                       pout.as<uint8_t>())))
                return rc;
            prep.pout = pout.as<uint8_t>();
            cs_box open{{0, 0, 0}, {1, 1, 1}, {CS_OPEN, CS_OPEN, CS_OPEN}};
            cs_ns_view nv{L, N, childOffsets.as<int32_t>(), parents.as<int32_t>(), i2l.as<int32_t>(),
                          layout.as<uint32_t>(), centers.p, sizes.p, cfg.search_ext};
            NbArgs<T> a  = makeNbArgs<T>(xs.as<T>(), ys.as<T>(), zs.as<T>(), hs.as<T>(), 0, uint32_t(n), open, nv,
                                         cfg.ngmax, nb.as<uint32_t>(), nc.as<uint32_t>());
            a.errWord      = err + 3;
            a.groupSize    = tuning.nb_group;
            a.byTargetCost = tuning.nb_by_target_cost;
            a.setOffsets   = setOff.as<uint32_t>();
            a.setRoots   = roots.as<int32_t>();
            a.numSets    = S;
            if ((rc = findNeighbors<T>(s, a, prep))) return rc;
        }

        uint32_t herr[4] = {0, 0, 0, 0};
        CSG_CUDA_TRY(cudaMemcpyAsync(herr, errWords.p, sizeof(herr), cudaMemcpyDeviceToHost, s));
        CSG_CUDA_TRY(cudaStreamSynchronize(s));
        if (herr[0] | herr[1])
        {
            setLastError("batch: a bounded device wait timed out (sort look-back)");
            return CS_ERR_TIMEOUT;
        }
        if (herr[3])
        {
            setLastError("batch: neighbour traversal stack overflow");
            return CS_ERR_DEVICE;
        }
        last    = cs_batch_result{S, L, N, br.iterations, uint64_t(n)};
        haveRun = true;
        if (res) *res = last;
        return CS_OK;
    }

    int outputs(cs_batch_outputs* o) override
    {
        if (!haveRun)
        {
            setLastError("batch: no run yet");
            return CS_ERR_INVALID;
        }
        const int L = last.num_leaves, N = last.num_nodes;
        o->order           = sortedOrder;
        o->x               = xs.p;
        o->y               = ys.p;
        o->z               = zs.p;
        o->h               = hs.p;
        o->leaves          = leaves.as<uint64_t>();
        o->counts          = counts.as<uint32_t>();
        o->layout          = layout.as<uint32_t>();
        o->set_leaf_begin  = leafBegin.as<int32_t>();
        o->set_roots       = roots.as<int32_t>();
        o->set_offsets     = setOff.as<uint32_t>();
        o->octree          = cs_octree_view{L, N - L, N, prefixes.p, childOffsets.as<int32_t>(), parents.as<int32_t>(),
                                   levelRange.as<int32_t>(), i2l.as<int32_t>(), l2i.as<int32_t>()};
        o->centers         = centers.p;
        o->sizes           = sizes.p;
        o->neighbors       = cfg.do_neighbors ? nb.as<uint32_t>() : nullptr;
        o->neighbor_counts = nc.as<uint32_t>();
        return CS_OK;
    }
};

} // namespace csg

using namespace csg;

struct cs_batch_s
{
    std::unique_ptr<BatchBase> impl;
};

extern "C" int cs_batch_create(cs_batch* out, const cs_batch_config* cfg)
{
    if (!out || !cfg || (cfg->coord_bits != 32 && cfg->coord_bits != 64) ||
        (cfg->sfc_kind != CS_MORTON && cfg->sfc_kind != CS_HILBERT))
    {
        setLastError("batch create: invalid arguments");
        return CS_ERR_INVALID;
    }
    auto* b = new cs_batch_s;
    if (cfg->coord_bits == 64) b->impl = std::make_unique<Batch<double>>();
    else b->impl = std::make_unique<Batch<float>>();
    b->impl->cfg = *cfg;
    *out         = b;
    return CS_OK;
}

extern "C" int cs_batch_destroy(cs_batch b)
{
    delete b;
    return CS_OK;
}

extern "C" int cs_batch_set_tuning(cs_batch b, const cs_tuning* t)
{
    if (!b || !t || !(t->nb_group == 8 || t->nb_group == 16 || t->nb_group == 32) || t->nb_by_target_cost < 0 ||
        t->nb_by_target_cost > 64 || !(t->sort_items == 0 || t->sort_items == 12 || t->sort_items == 16))
    {
        setLastError("batch set tuning: nb_group must be 8, 16 or 32, nb_by_target_cost in [0, 64], sort_items 0, 12 or 16");
        return CS_ERR_INVALID;
    }
    b->impl->tuning = *t;
    return CS_OK;
}

extern "C" int cs_batch_run(cs_batch b, cs_stream_t stream, const void* x, const void* y, const void* z, const void* h,
                            const uint32_t* off, int32_t numSets, const cs_box* boxes, const uint32_t* buckets,
                            cs_batch_result* res)
{
    if (!b || !x || !y || !z || !h)
    {
        setLastError("batch run: null argument");
        return CS_ERR_INVALID;
    }
    return b->impl->run(cudaStream_t(stream), x, y, z, h, off, numSets, boxes, buckets, res);
}

extern "C" int cs_batch_get_outputs(cs_batch b, cs_batch_outputs* out)
{
    if (!b || !out)
    {
        setLastError("batch outputs: null argument");
        return CS_ERR_INVALID;
    }
    return b->impl->outputs(out);
}

extern "C" size_t cs_batch_device_bytes(cs_batch b) { return b ? b->impl->deviceBytes() : 0; }
