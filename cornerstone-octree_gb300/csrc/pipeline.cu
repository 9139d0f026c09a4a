// The whole single-GPU path behind one C-ABI object: keys -> stable sort -> gather -> computeOctree -> link ->
// node geometry -> search boxes + findHalos -> findNeighbors. The object owns its device buffers and only grows
// them, so repeated runs (time steps, requests) allocate nothing once sized. The only host synchronisation per run
// is the one that returns the leaf count of the build (the reference's updateOctreeGpu synchronises three times per
// rebalance iteration; here the whole rebalance loop is one cooperative launch).
// Host inputs are copied in chunks on a copy stream into one of two device input sets in turn, so a run's copies
// overlap the previous run; results go back on a stream of their own (run_host_async / wait). The neighbour
// traversal's tuning is set per object and can be chosen by timing candidates on the last run's inputs (autotune).
#include "cs_common.cuh"
#include "halos.cuh"
#include "pipeline.cuh"
#include "neighbor_csr.cuh"
#include "neighbors.cuh"
#include "octree_build.cuh"
#include "octree_link.cuh"
#include "radix_sort.cuh"
#include "sfc_keys.cuh"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <type_traits>

namespace csg
{

template<class T, class K>
struct Pipeline final : PipelineBase
{
    // device copies of host inputs: two sets used in turn, so that a run's input copies overlap the previous run
    DevBuf inBuf[2][4];
    int inSet = 0;
    DevBuf keys, keysAlt, order, orderAlt;
    DevBuf xs, ys, zs, hs;
    DevBuf packed, shadowHi, shadowLo; // x,y,z,h records of the keys pass; float shadows made by the gather
    DevBuf pout;                       // per particle: outside its leaf's box (neighbour search)
    DevBuf sortWs, errWords;
    DevBuf buildWs, leaves, counts, layout;
    DevBuf prefixes, childOffsets, parents, levelRange, i2l, l2i, linkWs;
    DevBuf centers, sizes, sc, ss, flags, haloList;
    DevBuf nbPrepWs, nb, nc, nbStats;
    // the other set of per-run outputs copied back to the host (counts, halo flags): a pipelined host run writes one
    // set while the previous run's copy-back still reads the other, so it never waits for that copy (outSlot: the set
    // in nc / flags now)
    DevBuf ncAlt, flagsAlt;
    int outSlot = 0;
    // incremental time steps (step()): the current and the next leaf array with their counts, the current leaf
    // count in device memory, the leaf capacity every buffer of a step is sized for, and one captured graph per
    // direction of the leaf ping-pong
    DevBuf incLeaves[2], incCounts[2], incL;
    int incCur = -1, incCap = 0, incLhost = 0;
    size_t incN = 0;
    struct GraphKey
    {
        const void *x = nullptr, *y = nullptr, *z = nullptr, *h = nullptr;
        size_t n      = 0;
        cs_box box{};
        int cap       = 0;
        bool valid    = false;
        bool operator==(const GraphKey& o) const
        {
            return valid && o.valid && x == o.x && y == o.y && z == o.z && h == o.h && n == o.n && cap == o.cap &&
                   std::memcmp(&box, &o.box, sizeof(cs_box)) == 0;
        }
    };
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    GraphKey gkey[2];
    // graph steps run on this stream, ordered after the caller's (which may be the legacy default stream, on which
    // no capture is possible)
    cudaStream_t gstream = nullptr;
    cudaEvent_t joinEv   = nullptr;
    // host inputs: the copy stream, one event per chunk copied, and the fork point
    static constexpr int kCopyChunks = 4;
    cudaStream_t copyStream          = nullptr;
    cudaEvent_t copyEv[kCopyChunks]  = {};
    cudaEvent_t inUsed[2]            = {}; // on the compute stream after the keys of the last run that read the set
    bool inUsedRec[2]                = {false, false};
    // results to host: with lists, the compaction first, on the compute stream (outReady after it); then the error
    // words (errCopied), counts and flags (reuse[s]: a later run may overwrite output set s) on d2hStream, and the
    // offsets and compacted lists (from one of two device buffer sets in turn) on listStream (outDone). The two
    // streams do not wait for each other (a list copy never queues behind counts); wait() waits for both
    // (outDone and reuse[lastOutSlot])
    cudaStream_t d2hStream = nullptr, listStream = nullptr;
    cudaEvent_t outReady = nullptr, errCopied = nullptr, outDone = nullptr;
    cudaEvent_t reuse[2] = {};  // on d2hStream after the copy of output set s (counts, flags) to the host
    bool reuseRec[2]     = {false, false};
    int lastOutSlot      = 0; // the output set of the last copy-back
    cudaEvent_t listCopied[2]  = {};  // on listStream after the copy out of compaction buffer b
    cudaEvent_t cbEv[4]        = {};  // timing: compaction start / end, list copy start / end (cs_pipeline_copy_times)
    bool cbTimed               = false;
    bool listCopiedRec[2]      = {false, false};
    int csrCur                 = 0;
    uint32_t* herrHost         = nullptr; // pinned and mapped, the last copied error words (herrDev: device view)
    uint32_t* herrDev          = nullptr;
    uint32_t* listTotalHost    = nullptr; // pinned and mapped: the list total of compaction buffer set b at [2 b]
    uint32_t* listTotalDev     = nullptr;
    uint32_t* listOverflowHost = nullptr; // pinned, set when a list buffer was too small
    struct PendingList
    {
        bool on      = false;
        int b        = 0;
        uint32_t* dst = nullptr;
        size_t cap   = 0;
    } pendingList; // a copy-back whose list copy is not yet enqueued
    DevBuf csrWs, csrOff[2], csrList[2]; // the compacted lists on the device (two sets in turn), copied to the host
    bool outPending      = false;   // a copy-back whose errors are not yet reported
    int stickyRc         = CS_OK;   // an earlier run's device error, reported by the next wait
    char stickyMsg[160]  = {};
    const void* outLeaves      = nullptr;
    const uint32_t* outCounts  = nullptr;
    // opt-in traversal statistics of the neighbour search, printed to stderr (CSTONE_GB300_NB_STATS=1)
    bool statsOn = std::getenv("CSTONE_GB300_NB_STATS") != nullptr;
    int capacity = 0;
    size_t n     = 0;
    cs_pipeline_result last{};
    K* sortedKeys = nullptr;
    uint32_t* sortedOrder = nullptr;

    Pipeline()
    {
        for (auto& e : ev)
            cudaEventCreate(&e);
    }
    ~Pipeline() override
    {
        dropGraphs();
        if (gstream) cudaStreamDestroy(gstream);
        if (joinEv) cudaEventDestroy(joinEv);
        if (copyStream) cudaStreamDestroy(copyStream);
        for (auto& e : copyEv)
            if (e) cudaEventDestroy(e);
        for (auto& e : inUsed)
            if (e) cudaEventDestroy(e);
        if (d2hStream) cudaStreamDestroy(d2hStream);
        if (listStream) cudaStreamDestroy(listStream);
        for (cudaEvent_t e : {outReady, errCopied, reuse[0], reuse[1], outDone, listCopied[0], listCopied[1], cbEv[0], cbEv[1],
                              cbEv[2], cbEv[3]})
            if (e) cudaEventDestroy(e);
        if (herrHost) cudaFreeHost(herrHost);
        if (listTotalHost) cudaFreeHost(listTotalHost);
        if (listOverflowHost) cudaFreeHost(listOverflowHost);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }

    void dropGraphs()
    {
        for (int c = 0; c < 2; ++c)
        {
            if (gexec[c]) cudaGraphExecDestroy(gexec[c]);
            gexec[c]       = nullptr;
            gkey[c].valid  = false;
        }
    }

    void resetSteps() override
    {
        dropGraphs();
        incCur = -1;
    }

    const void* lastIn[4] = {};
    size_t lastNIn        = 0;
    cs_box lastBox{};
    uint64_t lastF0 = 0, lastF1 = 0;

    // Each candidate reruns the last run's inputs (device arrays, or the device copies of host inputs) reps times and
    // is scored by the mean device time of the neighbour stage. The results do not depend on the tuning.
    int autotune(cudaStream_t s, int reps, cs_tuning* best, cs_tuning* tried, float* ms, int capacity,
                 int* count) override
    {
        if (!lastNIn || !cfg.do_neighbors)
        {
            setLastError("autotune: needs a previous run with neighbours");
            return CS_ERR_INVALID;
        }
        static constexpr cs_tuning candidates[] = {{32, 7, 0}, {32, 0, 0}, {32, 5, 0}, {32, 10, 0}, {16, 7, 0},
                                                   {8, 7, 0}};
        static constexpr int sortCandidates[] = {16, 12};
        const void* in[4] = {lastIn[0], lastIn[1], lastIn[2], lastIn[3]};
        const size_t n0   = lastNIn;
        const cs_box box0 = lastBox;
        const uint64_t f0 = lastF0, f1 = lastF1;
        const cs_tuning keep = tuning;
        cs_tuning win        = keep;
        float winMs          = 0.f;
        int k                = 0;
        // mean device time of one stage [first, last) over reps runs with tuning c
        auto score = [&](const cs_tuning& c, int first, int last, float& mean) -> int {
            tuning    = c;
            float acc = 0.f;
            for (int r = 0; r < std::max(1, reps); ++r)
            {
                int rc = run(s, in[0], in[1], in[2], in[3], n0, box0, f0, f1, nullptr, false);
                if (rc) return rc;
                float t = 0.f;
                CSG_CUDA_TRY(cudaEventSynchronize(ev[ST_COUNT]));
                CSG_CUDA_TRY(cudaEventElapsedTime(&t, ev[first], ev[last]));
                acc += t;
            }
            mean = acc / float(std::max(1, reps));
            if (k < capacity)
            {
                if (tried) tried[k] = c;
                if (ms) ms[k] = mean;
            }
            ++k;
            return CS_OK;
        };
        for (cs_tuning c : candidates)
        {
            c.sort_items = keep.sort_items;
            float t      = 0.f;
            if (int rc = score(c, ST_NEIGHBORS, ST_COUNT, t))
            {
                tuning = keep;
                return rc;
            }
            if (k == 1 || t < winMs) win = c, winMs = t;
        }
        float sortWin = 0.f;
        for (int items : sortCandidates)
        {
            cs_tuning c  = win;
            c.sort_items = items;
            float t      = 0.f;
            if (int rc = score(c, ST_SORT, ST_GATHER, t))
            {
                tuning = keep;
                return rc;
            }
            if (items == sortCandidates[0] || t < sortWin) sortWin = t, win.sort_items = items;
        }
        tuning = win;
        if (best) *best = win;
        if (count) *count = k;
        return CS_OK;
    }

    // grow a buffer keeping its first keep bytes (stream-ordered copy, then the old buffer is released)
    static int growKeep(DevBuf& b, size_t need, size_t keep, cudaStream_t s)
    {
        if (need <= b.bytes) return CS_OK;
        DevBuf nb;
        int rc = nb.ensure(need);
        if (rc) return rc;
        if (keep && b.p) CSG_CUDA_TRY(cudaMemcpyAsync(nb.p, b.p, std::min(keep, b.bytes), cudaMemcpyDeviceToDevice, s));
        CSG_CUDA_TRY(cudaStreamSynchronize(s));
        std::swap(b.p, nb.p);
        std::swap(b.bytes, nb.bytes);
        return CS_OK;
    }

    // every buffer of an incremental step, sized for cap leaves: nothing is allocated inside a graph capture
    int allocSteps(cudaStream_t s, size_t nIn, int cap)
    {
        int rc;
        const int keyBits = 3 * KeyTraits<K>::maxLevel;
        const int Ncap    = cap + (cap - 1) / 7;
        for (DevBuf* b : {&keys, &keysAlt})
            if ((rc = b->ensure(nIn * sizeof(K)))) return rc;
        for (DevBuf* b : {&order, &orderAlt, &nc})
            if ((rc = b->ensure(nIn * sizeof(uint32_t)))) return rc;
        for (DevBuf* b : {&xs, &ys, &zs, &hs})
            if ((rc = b->ensure(nIn * sizeof(T)))) return rc;
        if ((rc = packed.ensure(nIn * sizeof(PackedT<T>)))) return rc;
        if (std::is_same_v<T, double> && cfg.do_neighbors)
            for (DevBuf* b : {&shadowHi, &shadowLo})
                if ((rc = b->ensure(nIn * sizeof(float4)))) return rc;
        if ((rc = sortWs.ensure(radixSortWorkspaceBytes<K>(nIn, 0, keyBits)))) return rc;
        if ((rc = errWords.ensure(64))) return rc;
        for (int c = 0; c < 2; ++c)
        {
            size_t keepL = incCur >= 0 ? (size_t(incLhost) + 1) * sizeof(K) : 0;
            size_t keepC = incCur >= 0 ? size_t(incLhost) * sizeof(uint32_t) : 0;
            if ((rc = growKeep(incLeaves[c], (size_t(cap) + 1) * sizeof(K), keepL, s))) return rc;
            if ((rc = growKeep(incCounts[c], size_t(cap) * sizeof(uint32_t), keepC, s))) return rc;
        }
        if ((rc = incL.ensure(sizeof(int)))) return rc;
        if ((rc = layout.ensure((size_t(cap) + 1) * sizeof(uint32_t)))) return rc;
        if ((rc = buildWs.ensure(octreeBuildWorkspaceBytes<K>(cap, true)))) return rc;
        if ((rc = prefixes.ensure(size_t(Ncap) * sizeof(K)))) return rc;
        if ((rc = childOffsets.ensure((size_t(Ncap) + 1) * sizeof(int32_t)))) return rc;
        if ((rc = parents.ensure(size_t(std::max(1, (Ncap - 1) / 8)) * sizeof(int32_t)))) return rc;
        if ((rc = levelRange.ensure(size_t(KeyTraits<K>::maxLevel + 2) * sizeof(int32_t)))) return rc;
        if ((rc = i2l.ensure(size_t(Ncap) * sizeof(int32_t)))) return rc;
        if ((rc = l2i.ensure(size_t(Ncap) * sizeof(int32_t)))) return rc;
        if ((rc = linkWs.ensure(buildLinkWorkspaceBytes<K>(cap)))) return rc;
        if ((rc = centers.ensure(3 * size_t(Ncap) * sizeof(T)))) return rc;
        if ((rc = sizes.ensure(3 * size_t(Ncap) * sizeof(T)))) return rc;
        if ((rc = nbPrepWs.ensure(nbPrepBytes(0, Ncap)))) return rc;
        if ((rc = flags.ensure(size_t(Ncap)))) return rc;
        if (cfg.do_neighbors)
        {
            if ((rc = nb.ensure(std::max<size_t>(1, nIn * cfg.ngmax) * sizeof(uint32_t)))) return rc;
            if ((rc = pout.ensure(nIn))) return rc;
        }
        return CS_OK;
    }

    // one incremental step from leaf array cur, every launch sized by the capacity and every count read from device
    // memory: no host synchronisation and no allocation, so the whole step can be captured into a CUDA graph
    int enqueueStep(cudaStream_t s, int cur, const T* x, const T* y, const T* z, const T* h, size_t nIn,
                    const cs_box& box, bool capturing)
    {
        // inside a capture a stage event must be an external record node to be recorded at replay
        auto rec = [&](cudaEvent_t e) {
            return capturing ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
        };
        int rc;
        const int nxt      = cur ^ 1;
        const int keyBits  = 3 * KeyTraits<K>::maxLevel;
        const int cap      = incCap;
        const int Icap     = (cap - 1) / 7, Ncap = cap + Icap;
        constexpr bool F64 = std::is_same_v<T, double>;
        const bool shadows = F64 && cfg.do_neighbors;
        uint32_t* err      = errWords.as<uint32_t>();
        float* cmax        = reinterpret_cast<float*>(err + 8);
        int* Ldev          = incL.as<int>();
        CSG_CUDA_TRY(cudaMemsetAsync(err, 0, 64, s));

        CSG_CUDA_TRY(rec(ev[ST_KEYS]));
        if ((rc = sfcKeysPacked<T, K>(s, x, y, z, h, keys.as<K>(), packed.as<PackedT<T>>(), nIn, box, cfg.sfc_kind)))
            return rc;
        CSG_CUDA_TRY(rec(ev[ST_SORT]));
        bool inAlt = false;
        rc = radixSortPairs<K>(s, keys.as<K>(), order.as<uint32_t>(), keysAlt.as<K>(), orderAlt.as<uint32_t>(), nIn,
                               0, keyBits, true, sortWs.p, sortWs.bytes, err, &inAlt, tuning.sort_items);
        if (rc) return rc;
        sortedKeys  = inAlt ? keysAlt.as<K>() : keys.as<K>();
        sortedOrder = inAlt ? orderAlt.as<uint32_t>() : order.as<uint32_t>();
        CSG_CUDA_TRY(rec(ev[ST_GATHER]));
        if ((rc = gatherPacked<T>(s, sortedOrder, nIn, packed.as<PackedT<T>>(), xs.as<T>(), ys.as<T>(), zs.as<T>(),
                                  hs.as<T>(), shadows ? shadowHi.as<float4>() : nullptr,
                                  shadows ? shadowLo.as<float4>() : nullptr, cmax)))
            return rc;

        // one updateOctree step: decision on the previous counts, rebalance, recount against the new keys
        CSG_CUDA_TRY(rec(ev[ST_BUILD]));
        BuildResult br;
        rc = octreeBuild<K>(s, sortedKeys, nIn, cfg.bucket_size, cfg.max_count, incLeaves[cur].as<K>(),
                            incCounts[cur].as<uint32_t>(), 0, incLeaves[nxt].as<K>(), incCounts[nxt].as<uint32_t>(),
                            layout.as<uint32_t>(), cap, buildWs.p, buildWs.bytes, &br, false, FocusQuery<K>{}, Ldev,
                            nullptr, err);
        if (rc) return rc;
        if ((rc = commitLeafCount<K>(s, buildWs.p, buildWs.bytes, cap, Ldev))) return rc;

        CSG_CUDA_TRY(rec(ev[ST_LINK]));
        cs_octree_view v{cap, Icap, Ncap, prefixes.p, childOffsets.as<int32_t>(), parents.as<int32_t>(),
                         levelRange.as<int32_t>(), i2l.as<int32_t>(), l2i.as<int32_t>()};
        if ((rc = buildLink<K>(s, incLeaves[nxt].as<K>(), cap, v, 0, linkWs.p, linkWs.bytes, err + 1, Ldev)))
            return rc;
        CSG_CUDA_TRY(rec(ev[ST_GEO]));
        if ((rc = geoCenters<K, T>(s, prefixes.as<K>(), Ncap, centers.as<T>(), sizes.as<T>(), box, cfg.sfc_kind,
                                   Ldev)))
            return rc;

        CSG_CUDA_TRY(rec(ev[ST_NBPREP]));
        NbPrep prep{};
        if (cfg.do_neighbors)
        {
            prep.phi  = shadows ? shadowHi.as<float4>() : nullptr;
            prep.plo  = shadows ? shadowLo.as<float4>() : nullptr;
            prep.cmax = cmax;
            if ((rc = nbPrepareNodes<T>(s, centers.as<T>(), sizes.as<T>(), childOffsets.as<int32_t>(),
                                        i2l.as<int32_t>(), layout.as<uint32_t>(), Ncap, nbPrepWs.p, nbPrepWs.bytes,
                                        &prep, Ldev)))
                return rc;
            if ((rc = nbMarkOutside<T>(s, xs.as<T>(), ys.as<T>(), zs.as<T>(), prep.phi, centers.as<T>(),
                                       sizes.as<T>(), childOffsets.as<int32_t>(), i2l.as<int32_t>(),
                                       layout.as<uint32_t>(), Ncap, prep, pout.as<uint8_t>(), Ldev)))
                return rc;
            prep.pout = pout.as<uint8_t>();
        }
        CSG_CUDA_TRY(rec(ev[ST_HALOS]));
        CSG_CUDA_TRY(rec(ev[ST_NEIGHBORS]));
        if (cfg.do_neighbors)
        {
            cs_ns_view nv{cap, Ncap, childOffsets.as<int32_t>(), parents.as<int32_t>(), i2l.as<int32_t>(),
                          layout.as<uint32_t>(), centers.p, sizes.p, cfg.search_ext};
            NbArgs<T> a = makeNbArgs<T>(xs.as<T>(), ys.as<T>(), zs.as<T>(), hs.as<T>(), 0, uint32_t(nIn), box, nv,
                                        cfg.ngmax, nb.as<uint32_t>(), nc.as<uint32_t>());
            a.errWord   = err + 3;
            a.groupSize    = tuning.nb_group;
            a.byTargetCost = tuning.nb_by_target_cost;
            if ((rc = findNeighbors<T>(s, a, prep))) return rc;
        }
        CSG_CUDA_TRY(rec(ev[ST_COUNT]));
        return CS_OK;
    }

    int step(cudaStream_t s, const void* xv, const void* yv, const void* zv, const void* hv, size_t nIn,
             const cs_box& box, bool useGraph, cs_pipeline_result* res) override
    {
        int rc;
        if ((rc = flushListCopy())) return rc;
        if (reuseRec[outSlot]) CSG_CUDA_TRY(cudaStreamWaitEvent(s, reuse[outSlot], 0)); // a copy-back reads them
        lastNIn = 0; // autotune reruns plain runs only (a step's inputs need not outlive it)
        if (incCur < 0 || nIn != incN)
        {
            // the first step of a sequence builds from the root and becomes the current tree; the step buffers are
            // sized first (from an estimate), so that the root build's outputs are not moved afterwards
            dropGraphs();
            graphReplays = 0;
            incCur       = -1; // nothing to keep yet
            incCap = std::max(incCap, int(std::min<size_t>(size_t(1) << 29,
                                                           nIn / std::max(1u, cfg.bucket_size) * 2 + 4096)));
            if ((rc = allocSteps(s, nIn, incCap))) return rc;
            if ((rc = run(s, xv, yv, zv, hv, nIn, box, 0, 0, res, false))) return rc;
            if (last.num_leaves + last.num_leaves / 4 + 4096 > incCap)
            {
                incCap = last.num_leaves + last.num_leaves / 4 + 4096;
                if ((rc = allocSteps(s, nIn, incCap))) return rc;
                if ((rc = run(s, xv, yv, zv, hv, nIn, box, 0, 0, res, false))) return rc;
            }
            incCur      = -1;
            const int L = last.num_leaves;
            CSG_CUDA_TRY(cudaMemcpyAsync(incLeaves[0].p, leaves.p, (size_t(L) + 1) * sizeof(K),
                                         cudaMemcpyDeviceToDevice, s));
            CSG_CUDA_TRY(cudaMemcpyAsync(incCounts[0].p, counts.p, size_t(L) * sizeof(uint32_t),
                                         cudaMemcpyDeviceToDevice, s));
            incLhost = L;
            CSG_CUDA_TRY(cudaMemcpyAsync(incL.p, &incLhost, sizeof(int), cudaMemcpyHostToDevice, s));
            CSG_CUDA_TRY(cudaStreamSynchronize(s));
            incCur = 0;
            incN   = nIn;
            return CS_OK;
        }
        const T *x = static_cast<const T*>(xv), *y = static_cast<const T*>(yv), *z = static_cast<const T*>(zv),
                *h = static_cast<const T*>(hv);
        n = nIn;
        if ((rc = allocSteps(s, nIn, incCap))) return rc;
        const int cur = incCur;
        // the step's cooperative build runs between here and octreeBuildFinish (graph or not)
        std::lock_guard<std::mutex> coop(cooperativeBuildMutex());
        if (useGraph)
        {
            if (!gstream) CSG_CUDA_TRY(cudaStreamCreateWithFlags(&gstream, cudaStreamNonBlocking));
            if (!joinEv) CSG_CUDA_TRY(cudaEventCreateWithFlags(&joinEv, cudaEventDisableTiming));
            CSG_CUDA_TRY(cudaEventRecord(joinEv, s));
            CSG_CUDA_TRY(cudaStreamWaitEvent(gstream, joinEv, 0));
            s = gstream; // the rest of the step, including its final synchronisation, runs there
            GraphKey k;
            k.x = xv, k.y = yv, k.z = zv, k.h = hv, k.n = nIn, k.box = box, k.cap = incCap, k.valid = true;
            if (!gexec[cur] || !(gkey[cur] == k))
            {
                if (gexec[cur]) cudaGraphExecDestroy(gexec[cur]);
                gexec[cur] = nullptr;
                CSG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                int erc = enqueueStep(s, cur, x, y, z, h, nIn, box, true);
                cudaGraph_t g = nullptr;
                cudaError_t ce = cudaStreamEndCapture(s, &g);
                if (erc || ce != cudaSuccess)
                {
                    if (g) cudaGraphDestroy(g);
                    cudaGetLastError();
                    if (!erc) setLastError("pipeline step: graph capture failed: %s", cudaGetErrorString(ce));
                    return erc ? erc : CS_ERR_CUDA;
                }
                cudaError_t ie = cudaGraphInstantiate(&gexec[cur], g, 0);
                cudaGraphDestroy(g);
                if (ie != cudaSuccess)
                {
                    gexec[cur] = nullptr;
                    setLastError("pipeline step: graph instantiation failed: %s", cudaGetErrorString(ie));
                    return CS_ERR_CUDA;
                }
                gkey[cur] = k;
            }
            CSG_CUDA_TRY(cudaGraphLaunch(gexec[cur], s));
            graphReplays++;
        }
        else if ((rc = enqueueStep(s, cur, x, y, z, h, nIn, box, false)))
            return rc;

        BuildResult br;
        rc = octreeBuildFinish<K>(s, buildWs.p, buildWs.bytes, incCap, true, &br);
        if (rc == CS_ERR_CAPACITY)
        {
            // the new leaf array did not fit: grow every buffer of the step and redo it from the same input
            incCap = br.numLeaves + br.numLeaves / 4 + 4096;
            dropGraphs();
            if ((rc = allocSteps(s, nIn, incCap))) return rc;
            CSG_CUDA_TRY(cudaMemcpyAsync(incL.p, &incLhost, sizeof(int), cudaMemcpyHostToDevice, s));
            if ((rc = enqueueStep(s, cur, x, y, z, h, nIn, box, false))) return rc;
            rc = octreeBuildFinish<K>(s, buildWs.p, buildWs.bytes, incCap, true, &br);
        }
        if (rc) return rc;
        uint32_t herr[4] = {0, 0, 0, 0};
        CSG_CUDA_TRY(cudaMemcpyAsync(herr, errWords.p, sizeof(herr), cudaMemcpyDeviceToHost, s));
        CSG_CUDA_TRY(cudaStreamSynchronize(s));
        if (herr[0] | herr[1])
        {
            setLastError("pipeline step: a bounded device wait timed out (sort look-back)");
            return CS_ERR_TIMEOUT;
        }
        if (herr[3])
        {
            setLastError("pipeline step: neighbour traversal stack overflow (malformed tree)");
            return CS_ERR_DEVICE;
        }
        incCur   = cur ^ 1;
        incLhost = br.numLeaves;
        const int L = br.numLeaves, N = L + (L - 1) / 7;
        last        = cs_pipeline_result{L, N, 1, 0, 0, br.maxDepth};
        lastN       = 1;
        outLeaves   = incLeaves[incCur].p;
        outCounts   = incCounts[incCur].as<uint32_t>();
        if (res) *res = last;
        return CS_OK;
    }

    size_t deviceBytes() const override
    {
        size_t t = 0;
        for (const DevBuf* b : {&inBuf[0][0], &inBuf[0][1], &inBuf[0][2], &inBuf[0][3], &inBuf[1][0], &inBuf[1][1],
                                &inBuf[1][2], &inBuf[1][3], &keys, &keysAlt, &order, &orderAlt, &xs, &ys, &zs, &hs,
                                &packed, &shadowHi, &shadowLo, &pout, &sortWs, &errWords, &buildWs, &leaves, &counts,
                                &layout, &prefixes, &childOffsets, &haloList,
                                &parents, &levelRange, &i2l, &l2i, &linkWs, &centers, &sizes, &sc, &ss, &flags,
                                &nbPrepWs, &nb, &nc, &ncAlt, &flagsAlt})
            t += b->bytes;
        return t;
    }

    int run(cudaStream_t s, const void* xv, const void* yv, const void* zv, const void* hv, size_t nIn,
            const cs_box& box, uint64_t f0, uint64_t f1, cs_pipeline_result* res, bool hostIn) override
    {
        n  = nIn;
        int rc;
        const T* hostSrc[4] = {};
        constexpr int KB = 8 * sizeof(K);
        if (n == 0 || n >= (size_t(1) << 30))
        {
            setLastError("pipeline: n = %zu outside [1, 2^30)", n);
            return CS_ERR_INVALID;
        }
        const T *x = static_cast<const T*>(xv), *y = static_cast<const T*>(yv), *z = static_cast<const T*>(zv),
                *h = static_cast<const T*>(hv);
        if (hostIn && outPending)
        {
            // the previous run's counts and flags may still be on their way to the host: this run writes the other
            // set (the graphs of time steps hold the old set's addresses, so a later step captures again)
            std::swap(nc.p, ncAlt.p);
            std::swap(nc.bytes, ncAlt.bytes);
            std::swap(flags.p, flagsAlt.p);
            std::swap(flags.bytes, flagsAlt.bytes);
            outSlot ^= 1;
            dropGraphs();
        }
        if (hostIn)
        {
            for (DevBuf& b : inBuf[inSet])
                if ((rc = b.ensure(n * sizeof(T)))) return rc;
            // the host arrays arrive in chunks on a copy stream, the keys of chunk c computed while chunk c + 1
            // travels (the keys are per particle); concurrent copies would share the host link and gain nothing
            if (!copyStream)
            {
                CSG_CUDA_TRY(cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking));
                for (auto& e : copyEv)
                    CSG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                for (auto& e : inUsed)
                    CSG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            }
            hostSrc[0] = x, hostSrc[1] = y, hostSrc[2] = z, hostSrc[3] = h;
            x = inBuf[inSet][0].as<T>();
            y = inBuf[inSet][1].as<T>();
            z = inBuf[inSet][2].as<T>();
            h = inBuf[inSet][3].as<T>();
        }
        // device inputs of this run (the copies of host inputs), for autotune
        lastIn[0] = x, lastIn[1] = y, lastIn[2] = z, lastIn[3] = h;
        lastNIn = n, lastBox = box, lastF0 = f0, lastF1 = f1;
        for (DevBuf* b : {&keys, &keysAlt})
            if ((rc = b->ensure(n * sizeof(K)))) return rc;
        for (DevBuf* b : {&order, &orderAlt})
            if ((rc = b->ensure(n * sizeof(uint32_t)))) return rc;
        for (DevBuf* b : {&xs, &ys, &zs, &hs})
            if ((rc = b->ensure(n * sizeof(T)))) return rc;
        if ((rc = packed.ensure(n * sizeof(PackedT<T>)))) return rc;
        constexpr bool F64 = std::is_same_v<T, double>;
        const bool shadows = F64 && cfg.do_neighbors;
        if (shadows)
            for (DevBuf* b : {&shadowHi, &shadowLo})
                if ((rc = b->ensure(n * sizeof(float4)))) return rc;
        // keys have 3*maxLevel significant bits (no removeKey entries: they are computed here)
        const int keyBits = 3 * KeyTraits<K>::maxLevel;
        if ((rc = sortWs.ensure(radixSortWorkspaceBytes<K>(n, 0, keyBits)))) return rc;
        if ((rc = errWords.ensure(64))) return rc;
        // error words [0] sort, [1] link sort, [2] halo stack, [3] neighbour stack; [8] the neighbour search's
        // coordinate bound (float, atomic max from 0)
        uint32_t* err = errWords.as<uint32_t>();
        float* cmax   = reinterpret_cast<float*>(err + 8);
        if (outPending) CSG_CUDA_TRY(cudaStreamWaitEvent(s, errCopied, 0)); // the previous copy-back read them
        CSG_CUDA_TRY(cudaMemsetAsync(err, 0, 64, s));

        if (hostIn)
        {
            // chunk c: four copies on the copy stream, then its keys on s; the keys stage of a host run begins when
            // the first chunk has arrived and so includes the copies of the others
            // the copies wait only for the last reader of this input set (the keys of the run before the previous
            // one), so that they overlap the previous run's computation
            const size_t chunk = ((n + kCopyChunks - 1) / kCopyChunks + 255) & ~size_t(255);
            if (inUsedRec[inSet]) CSG_CUDA_TRY(cudaStreamWaitEvent(copyStream, inUsed[inSet], 0));
            T* dst[4] = {inBuf[inSet][0].as<T>(), inBuf[inSet][1].as<T>(), inBuf[inSet][2].as<T>(),
                         inBuf[inSet][3].as<T>()};
            for (int c = 0; c < kCopyChunks && size_t(c) * chunk < n; ++c)
            {
                const size_t a = size_t(c) * chunk, m = std::min(chunk, n - a);
                for (int k = 0; k < 4; ++k)
                    CSG_CUDA_TRY(cudaMemcpyAsync(dst[k] + a, hostSrc[k] + a, m * sizeof(T), cudaMemcpyHostToDevice,
                                                 copyStream));
                CSG_CUDA_TRY(cudaEventRecord(copyEv[c], copyStream));
                CSG_CUDA_TRY(cudaStreamWaitEvent(s, copyEv[c], 0));
                if (c == 0) CSG_CUDA_TRY(cudaEventRecord(ev[ST_KEYS], s));
                if ((rc = sfcKeysPacked<T, K>(s, x + a, y + a, z + a, h + a, keys.as<K>() + a,
                                              packed.as<PackedT<T>>() + a, m, box, cfg.sfc_kind)))
                    return rc;
            }
            CSG_CUDA_TRY(cudaEventRecord(inUsed[inSet], s));
            inUsedRec[inSet] = true;
            inSet ^= 1;
        }
        else
        {
            CSG_CUDA_TRY(cudaEventRecord(ev[ST_KEYS], s));
            if ((rc = sfcKeysPacked<T, K>(s, x, y, z, h, keys.as<K>(), packed.as<PackedT<T>>(), n, box,
                                          cfg.sfc_kind)))
                return rc;
        }

        CSG_CUDA_TRY(cudaEventRecord(ev[ST_SORT], s));
        bool inAlt = false;
        rc = radixSortPairs<K>(s, keys.as<K>(), order.as<uint32_t>(), keysAlt.as<K>(), orderAlt.as<uint32_t>(), n, 0,
                               keyBits, true, sortWs.p, sortWs.bytes, err, &inAlt, tuning.sort_items);
        if (rc) return rc;
        sortedKeys  = inAlt ? keysAlt.as<K>() : keys.as<K>();
        sortedOrder = inAlt ? orderAlt.as<uint32_t>() : order.as<uint32_t>();

        CSG_CUDA_TRY(cudaEventRecord(ev[ST_GATHER], s));
        if ((rc = gatherPacked<T>(s, sortedOrder, n, packed.as<PackedT<T>>(), xs.as<T>(), ys.as<T>(), zs.as<T>(),
                                  hs.as<T>(), shadows ? shadowHi.as<float4>() : nullptr,
                                  shadows ? shadowLo.as<float4>() : nullptr, cmax)))
            return rc;

        // ---- cornerstone build: grow the capacity until the converged tree fits ----
        CSG_CUDA_TRY(cudaEventRecord(ev[ST_BUILD], s));
        if (capacity == 0) capacity = int(std::min<size_t>(size_t(1) << 30, n / std::max(1u, cfg.bucket_size) * 16 + 4096));
        BuildResult br;
        for (;;)
        {
            if ((rc = buildWs.ensure(octreeBuildWorkspaceBytes<K>(capacity, false)))) return rc;
            if ((rc = leaves.ensure((size_t(capacity) + 1) * sizeof(K)))) return rc;
            if ((rc = counts.ensure(size_t(capacity) * sizeof(uint32_t)))) return rc;
            if ((rc = layout.ensure((size_t(capacity) + 1) * sizeof(uint32_t)))) return rc;
            br = BuildResult{};
            rc = octreeBuild<K>(s, sortedKeys, n, cfg.bucket_size, cfg.max_count, nullptr, nullptr, 0, leaves.as<K>(),
                                counts.as<uint32_t>(), layout.as<uint32_t>(), capacity, buildWs.p, buildWs.bytes, &br,
                                true, FocusQuery<K>{K(f0), K(f1), cfg.do_halos != 0}, nullptr, nullptr, err);
            if (rc == CS_ERR_CAPACITY)
            {
                capacity = std::max(2 * capacity, br.needed + br.needed / 4);
                continue;
            }
            if (rc) return rc;
            break;
        }
        const int L = br.numLeaves, I = (L - 1) / 7, N = L + I;
        // the build's result was read on the host: everything before it on this stream is done, the previous call's
        // list compaction included, so its list copy can be sized and enqueued now
        if ((rc = flushListCopy())) return rc;

        // ---- internal tree ----
        CSG_CUDA_TRY(cudaEventRecord(ev[ST_LINK], s));
        if ((rc = prefixes.ensure(size_t(N) * sizeof(K)))) return rc;
        if ((rc = childOffsets.ensure((size_t(N) + 1) * sizeof(int32_t)))) return rc;
        if ((rc = parents.ensure(size_t(std::max(1, (N - 1) / 8)) * sizeof(int32_t)))) return rc;
        if ((rc = levelRange.ensure(size_t(KeyTraits<K>::maxLevel + 2) * sizeof(int32_t)))) return rc;
        if ((rc = i2l.ensure(size_t(N) * sizeof(int32_t)))) return rc;
        if ((rc = l2i.ensure(size_t(N) * sizeof(int32_t)))) return rc;
        if ((rc = linkWs.ensure(buildLinkWorkspaceBytes<K>(L)))) return rc;
        cs_octree_view v{L, I, N, prefixes.p, childOffsets.as<int32_t>(), parents.as<int32_t>(),
                         levelRange.as<int32_t>(), i2l.as<int32_t>(), l2i.as<int32_t>()};
        int prefixBits = std::min(KB, 3 * br.maxDepth + 1);
        if ((rc = buildLink<K>(s, leaves.as<K>(), L, v, prefixBits, linkWs.p, linkWs.bytes, err + 1))) return rc;

        CSG_CUDA_TRY(cudaEventRecord(ev[ST_GEO], s));
        if ((rc = centers.ensure(3 * size_t(N) * sizeof(T)))) return rc;
        if ((rc = sizes.ensure(3 * size_t(N) * sizeof(T)))) return rc;
        if ((rc = geoCenters<K, T>(s, prefixes.as<K>(), N, centers.as<T>(), sizes.as<T>(), box, cfg.sfc_kind))) return rc;

        // ---- float node boxes for the halo pre-filter and the neighbour search ----
        CSG_CUDA_TRY(cudaEventRecord(ev[ST_NBPREP], s));
        if ((rc = nc.ensure(n * sizeof(uint32_t)))) return rc;
        NbPrep prep{};
        const bool nodeShadows = cfg.do_neighbors || (F64 && cfg.do_halos);
        if (nodeShadows)
        {
            if ((rc = nbPrepWs.ensure(nbPrepBytes(0, N)))) return rc;
            prep.phi  = shadows ? shadowHi.as<float4>() : nullptr;
            prep.plo  = shadows ? shadowLo.as<float4>() : nullptr;
            prep.cmax = cmax;
            if ((rc = nbPrepareNodes<T>(s, centers.as<T>(), sizes.as<T>(), childOffsets.as<int32_t>(),
                                        i2l.as<int32_t>(), layout.as<uint32_t>(), N, nbPrepWs.p, nbPrepWs.bytes,
                                        &prep)))
                return rc;
        }
        if (cfg.do_neighbors)
        {
            const size_t nbNeed = std::max<size_t>(1, n * cfg.ngmax) * sizeof(uint32_t);
            if ((rc = nb.ensure(nbNeed))) return rc;
            if ((rc = pout.ensure(n))) return rc;
            if ((rc = nbMarkOutside<T>(s, xs.as<T>(), ys.as<T>(), zs.as<T>(), prep.phi, centers.as<T>(),
                                       sizes.as<T>(), childOffsets.as<int32_t>(), i2l.as<int32_t>(),
                                       layout.as<uint32_t>(), N, prep, pout.as<uint8_t>())))
                return rc;
            prep.pout = pout.as<uint8_t>();
        }

        // ---- halos for the focus leaves ----
        CSG_CUDA_TRY(cudaEventRecord(ev[ST_HALOS], s));
        if ((rc = flags.ensure(size_t(N)))) return rc;
        if (reuseRec[outSlot]) CSG_CUDA_TRY(cudaStreamWaitEvent(s, reuse[outSlot], 0)); // the set's last copy-back
        CSG_CUDA_TRY(cudaMemsetAsync(flags.p, 0, size_t(N), s));
        if (cfg.do_halos && br.focusLast > br.focusFirst)
        {
            if ((rc = sc.ensure(3 * size_t(L) * sizeof(T)))) return rc;
            if ((rc = ss.ensure(3 * size_t(L) * sizeof(T)))) return rc;
            T scale = T(2.0f * cfg.halo_search_ext);
            if ((rc = searchBoxes<T, T>(s, xs.as<T>(), ys.as<T>(), zs.as<T>(), hs.as<T>(), layout.as<uint32_t>(),
                                     br.focusFirst, br.focusLast, scale, l2i.as<int32_t>() + I, centers.as<T>(),
                                     sc.as<T>(), ss.as<T>(), prep.phi)))
                return rc;
            if constexpr (!(std::is_same_v<K, uint32_t> && std::is_same_v<T, double>))
            {
                if ((rc = haloList.ensure((size_t(br.focusLast - br.focusFirst) + 2) * sizeof(int32_t)))) return rc;
                if ((rc = findHalos<K, T>(s, prefixes.as<K>(), childOffsets.as<int32_t>(), parents.as<int32_t>(),
                                          centers.as<T>(), sizes.as<T>(), leaves.as<K>(), sc.as<T>(), ss.as<T>(), box,
                                          br.focusFirst, br.focusLast, flags.as<uint8_t>(), err + 2, prep.nrec,
                                          haloList.as<int32_t>())))
                    return rc;
            }
        }

        CSG_CUDA_TRY(cudaEventRecord(ev[ST_NEIGHBORS], s));
        if (cfg.do_neighbors)
        {
            cs_ns_view nv{L, N, childOffsets.as<int32_t>(), parents.as<int32_t>(), i2l.as<int32_t>(),
                          layout.as<uint32_t>(), centers.p, sizes.p, cfg.search_ext};
            NbArgs<T> a = makeNbArgs<T>(xs.as<T>(), ys.as<T>(), zs.as<T>(), hs.as<T>(), 0, uint32_t(n), box, nv,
                                        cfg.ngmax, nb.as<uint32_t>(), nc.as<uint32_t>());
            a.errWord   = err + 3;
            a.groupSize    = tuning.nb_group;
            a.byTargetCost = tuning.nb_by_target_cost;
            if (statsOn)
            {
                if ((rc = nbStats.ensure(32 * sizeof(unsigned long long)))) return rc;
                CSG_CUDA_TRY(cudaMemsetAsync(nbStats.p, 0, 32 * sizeof(unsigned long long), s));
                a.stats = nbStats.as<unsigned long long>();
            }
            if ((rc = findNeighbors<T>(s, a, prep))) return rc;
            if (statsOn)
            {
                unsigned long long h[32];
                CSG_CUDA_TRY(cudaMemcpyAsync(h, nbStats.p, sizeof(h), cudaMemcpyDeviceToHost, s));
                CSG_CUDA_TRY(cudaStreamSynchronize(s));
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] warps %llu | per warp: node expansions %.1f leaves %.1f "
                             "candidates %.1f | lane cell tests %llu (fp64 %llu) | lane pair tests %llu "
                             "(exact %llu)\n",
                             h[7], double(h[6]) / h[7], double(h[4]) / h[7], double(h[5]) / h[7], h[0], h[1], h[2],
                             h[3]);
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] slowest warp: %llu cycles, expansions %llu leaves %llu "
                             "candidates %llu loose %llu first target %llu | loose warps %llu\n",
                             h[8], h[9], h[10], h[11], h[12], h[13], h[14]);
                auto asf = [](unsigned long long v) {
                    unsigned u = unsigned(v);
                    float f;
                    std::memcpy(&f, &u, 4);
                    return double(f);
                };
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] slowest warp geometry: rmax %g rmin %g group radius %g "
                             "box half %g C %g\n",
                             asf(h[15]), asf(h[18]), asf(h[16]), asf(h[17]), asf(h[19]));
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] candidate batches %.1f per warp, steps %.1f, needing "
                             "lanes %.1f, min-cost/step-cost %.3f | cycles in batches %.1f%% of warp cycles\n",
                             double(h[23]) / h[7], double(h[20]) / h[23], double(h[21]) / h[23],
                             double(h[22]) / (11.0 * double(h[20])), 100.0 * double(h[24]) / double(h[25]));
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] cycles in leaf visits %.1f%% | leaf visits no lane "
                             "needed %.1f per warp\n",
                             100.0 * double(h[26]) / double(h[25]), double(h[27]) / h[7]);
                std::fprintf(stderr,
                             "[cstone_gb300 neighbour stats] output per warp: sum of the most hits of a lane per "
                             "batch %.1f, lanes with hits %.1f, rounds of 32 hits %.1f | exact path walks %.2f\n",
                             double(h[28]) / h[7], double(h[29]) / h[7], double(h[30]) / h[7], double(h[31]) / h[7]);
            }
        }
        CSG_CUDA_TRY(cudaEventRecord(ev[ST_COUNT], s));

        last             = cs_pipeline_result{L, N, br.iterations, br.focusFirst, br.focusLast, br.maxDepth};
        lastN            = 1;
        outLeaves        = leaves.p;
        outCounts        = counts.as<uint32_t>();
        incCur           = -1; // a plain run ends any step sequence
        if (res) *res    = last;
        return CS_OK;
    }

    // the error words of a finished copy-back as a status (and message)
    static int deviceErrors(const uint32_t* herr)
    {
        if (herr[0] | herr[1])
        {
            setLastError("pipeline: a bounded device wait timed out (sort look-back)");
            return CS_ERR_TIMEOUT;
        }
        if (herr[3])
        {
            setLastError("pipeline: neighbour traversal stack overflow (malformed tree)");
            return CS_ERR_DEVICE;
        }
        if (herr[2])
        {
            setLastError("pipeline: halo traversal stack overflow (malformed tree)");
            return CS_ERR_DEVICE;
        }
        return CS_OK;
    }

    // Enqueue the copy of the last run's results to host memory on the copy-back stream, after the run's work.
    int copyBackAsync(cudaStream_t s, uint32_t* ncHost, uint8_t* flagsHost, size_t flagsCap, uint64_t* listOffsets,
                      uint32_t* listHost, size_t listCap) override
    {
        if (flagsHost && flagsCap < size_t(last.num_nodes))
        {
            setLastError("pipeline: halo flag buffer holds %zu, %d needed", flagsCap, last.num_nodes);
            return CS_ERR_CAPACITY;
        }
        if (listOffsets && !cfg.do_neighbors)
        {
            setLastError("pipeline: neighbour lists requested from a pipeline without neighbour search");
            return CS_ERR_INVALID;
        }
        if (!d2hStream)
        {
            // the highest priority: the one-warp copies of error words run as soon as a slot frees
            int lowPrio = 0, highPrio = 0;
            CSG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lowPrio, &highPrio));
            CSG_CUDA_TRY(cudaStreamCreateWithPriority(&d2hStream, cudaStreamNonBlocking, highPrio));
            CSG_CUDA_TRY(cudaStreamCreateWithPriority(&listStream, cudaStreamNonBlocking, highPrio));
            for (cudaEvent_t* e : {&outReady, &errCopied, &reuse[0], &reuse[1], &outDone, &listCopied[0], &listCopied[1]})
                CSG_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
            for (cudaEvent_t& e : cbEv)
                CSG_CUDA_TRY(cudaEventCreate(&e));
            CSG_CUDA_TRY(cudaHostAlloc(&herrHost, 4 * sizeof(uint32_t), cudaHostAllocPortable | cudaHostAllocMapped));
            CSG_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&herrDev), herrHost, 0));
            CSG_CUDA_TRY(
                cudaHostAlloc(&listTotalHost, 4 * sizeof(uint32_t), cudaHostAllocPortable | cudaHostAllocMapped));
            CSG_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&listTotalDev), listTotalHost, 0));
            CSG_CUDA_TRY(cudaHostAlloc(&listOverflowHost, sizeof(uint32_t), cudaHostAllocDefault));
            *listOverflowHost = 0;
        }
        if (outPending)
        {
            // the previous copy-back's error words (copied long ago) before they are overwritten
            CSG_CUDA_TRY(cudaEventSynchronize(errCopied));
            int rc = deviceErrors(herrHost);
            if (rc && stickyRc == CS_OK)
            {
                stickyRc = rc;
                std::snprintf(stickyMsg, sizeof(stickyMsg), "%s", cs_last_error());
            }
        }
        if (int rc = flushListCopy()) return rc; // a previous call's list (normally already enqueued by run)
        const size_t devCap = listOffsets ? std::min(listCap, n * size_t(cfg.ngmax)) : 0;
        const int b         = csrCur;
        if (listOffsets)
        {
            // the stored neighbour indices compacted on the compute stream, right after the run (a full-bandwidth
            // pass of about 2 ms at 16M; beside the next run it would slow that run's sort), into buffer set b once
            // the copy out of it two calls ago has finished (a buffer that grows is freed first: wait on the host for
            // its last reader); the total goes to mapped host memory for the list copy's size
            const size_t wsNeed = neighborCsrWorkspaceBytes(n), offNeed = (n + 1) * sizeof(uint64_t);
            const size_t listNeed = std::max<size_t>(devCap, 1) * sizeof(uint32_t);
            if (listCopiedRec[b] && (offNeed > csrOff[b].bytes || listNeed > csrList[b].bytes))
                CSG_CUDA_TRY(cudaEventSynchronize(listCopied[b]));
            int rc = csrWs.ensure(wsNeed);
            if (!rc) rc = csrOff[b].ensure(offNeed);
            if (!rc) rc = csrList[b].ensure(listNeed);
            if (rc) return rc;
            if (listCopiedRec[b]) CSG_CUDA_TRY(cudaStreamWaitEvent(s, listCopied[b], 0));
            CSG_CUDA_TRY(cudaEventRecord(cbEv[0], s));
            if ((rc = neighborCsr(s, nb.as<uint32_t>(), nc.as<uint32_t>(), n, cfg.ngmax, csrOff[b].as<uint64_t>(),
                                  csrList[b].as<uint32_t>(), devCap, csrWs.p, csrWs.bytes, nullptr)))
                return rc;
            copyWordsKernel<<<1, 32, 0, s>>>(reinterpret_cast<const uint32_t*>(csrOff[b].as<uint64_t>() + n),
                                             listTotalDev + 2 * b, 2);
            CSG_CHECK_LAUNCH();
            CSG_CUDA_TRY(cudaEventRecord(cbEv[1], s));
        }
        CSG_CUDA_TRY(cudaEventRecord(outReady, s));
        CSG_CUDA_TRY(cudaStreamWaitEvent(d2hStream, outReady, 0));
        // the error words by a one-warp kernel into mapped memory: no copy engine, so they never queue behind lists
        copyWordsKernel<<<1, 32, 0, d2hStream>>>(errWords.as<uint32_t>(), herrDev, 4);
        CSG_CHECK_LAUNCH();
        CSG_CUDA_TRY(cudaEventRecord(errCopied, d2hStream));
        // counts and flags: the run after next writes this output set again and waits for them (reuse[outSlot]), so
        // they must not queue behind a list copy on the copy engines; pinned destinations are written by a small
        // kernel instead
        if (ncHost)
            if (int rc = copyToHostAsync(d2hStream, ncHost, nc.p, n * sizeof(uint32_t))) return rc;
        if (flagsHost)
            if (int rc = copyToHostAsync(d2hStream, flagsHost, flags.p, size_t(last.num_nodes))) return rc;
        CSG_CUDA_TRY(cudaEventRecord(reuse[outSlot], d2hStream));
        reuseRec[outSlot] = true;
        CSG_CUDA_TRY(cudaStreamWaitEvent(listStream, outReady, 0));
        if (listOffsets)
        {
            // the offsets now; the list itself by the copy engine once its length is known on the host, which is
            // when the next call (run, step or wait) has seen this compaction finish (flushListCopy)
            if (int rc = copyToHostInPieces(listStream, listOffsets, csrOff[b].p, (n + 1) * sizeof(uint64_t)))
                return rc;
            pendingList = PendingList{true, b, listHost, listHost ? listCap : 0};
            csrCur      = 1 - b;
        }
        CSG_CUDA_TRY(cudaEventRecord(outDone, listStream));
        lastOutSlot = outSlot;
        outPending  = true;
        return CS_OK;
    }

    // A large device-to-host copy issued as one cudaMemcpyAsync and the kernels running beside it slowed each other
    // down (measured on a GB300 host: a 6.9 GB copy beside two 16M runs, both done after 432 ms, against 37 and 45 ms
    // alone); issued in pieces of 64 MB the two overlap (58 ms for both). So every copy of the lists and offsets goes
    // in such pieces.
    static int copyToHostInPieces(cudaStream_t st, void* dst, const void* src, size_t bytes)
    {
        constexpr size_t kPiece = size_t(64) << 20;
        for (size_t off = 0; off < bytes; off += kPiece)
            CSG_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off,
                                         std::min(kPiece, bytes - off), cudaMemcpyDeviceToHost, st));
        return CS_OK;
    }

    // Enqueue the list copy of the last copy-back that returned lists, if not done yet: waits (on the host) for that
    // run's compaction, reads the total from mapped memory and copies min(total, capacity) entries on listStream.
    int flushListCopy()
    {
        if (!pendingList.on) return CS_OK;
        const PendingList pl = pendingList;
        pendingList.on       = false;
        CSG_CUDA_TRY(cudaEventSynchronize(cbEv[1]));
        uint64_t total = 0;
        std::memcpy(&total, const_cast<const uint32_t*>(listTotalHost) + 2 * pl.b, sizeof(total));
        const size_t m = size_t(std::min<uint64_t>(total, pl.cap));
        if (total > pl.cap) *listOverflowHost = 1;
        CSG_CUDA_TRY(cudaEventRecord(cbEv[2], listStream));
        if (int rc = copyToHostInPieces(listStream, pl.dst, csrList[pl.b].p, m * sizeof(uint32_t))) return rc;
        CSG_CUDA_TRY(cudaEventRecord(cbEv[3], listStream));
        CSG_CUDA_TRY(cudaEventRecord(listCopied[pl.b], listStream));
        listCopiedRec[pl.b] = true;
        cbTimed             = true;
        CSG_CUDA_TRY(cudaEventRecord(outDone, listStream));
        return CS_OK;
    }

    int copyTimes(float* ms, int count) override
    {
        if (int rc = flushListCopy()) return rc;
        if (!cbTimed)
        {
            setLastError("copy times: no copy-back with neighbour lists yet");
            return CS_ERR_INVALID;
        }
        CSG_CUDA_TRY(cudaEventSynchronize(cbEv[3]));
        const cudaEvent_t from[4] = {cbEv[0], cbEv[2], cbEv[1], ev[ST_KEYS]};
        const cudaEvent_t to[4]   = {cbEv[1], cbEv[3], cbEv[2], cbEv[3]};
        for (int i = 0; i < count && i < 4; ++i)
            CSG_CUDA_TRY(cudaEventElapsedTime(&ms[i], from[i], to[i]));
        return CS_OK;
    }

    // Wait for the last copy-back; report the first device error of the runs since the previous wait.
    int wait() override
    {
        int rc = flushListCopy();
        if (rc) return rc;
        if (outPending)
        {
            CSG_CUDA_TRY(cudaEventSynchronize(outDone));
            CSG_CUDA_TRY(cudaEventSynchronize(reuse[lastOutSlot]));
            outPending = false;
            rc         = deviceErrors(herrHost);
            if (rc == CS_OK && listOverflowHost && *listOverflowHost)
            {
                setLastError("pipeline: a neighbour list buffer was too small (offsets[n] holds the entries needed)");
                rc = CS_ERR_CAPACITY;
            }
            if (listOverflowHost) *listOverflowHost = 0;
        }
        if (stickyRc != CS_OK)
        {
            rc = stickyRc;
            setLastError("%s", stickyMsg);
            stickyRc = CS_OK;
        }
        return rc;
    }

    int outputs(cs_pipeline_outputs* o) override
    {
        if (!lastN)
        {
            setLastError("pipeline: no run yet");
            return CS_ERR_INVALID;
        }
        int L = last.num_leaves, N = last.num_nodes, I = N - L;
        o->sorted_keys     = sortedKeys;
        o->order           = sortedOrder;
        o->x               = xs.p;
        o->y               = ys.p;
        o->z               = zs.p;
        o->h               = hs.p;
        o->leaves          = const_cast<void*>(outLeaves);
        o->counts          = const_cast<uint32_t*>(outCounts);
        o->layout          = layout.as<uint32_t>();
        o->octree          = cs_octree_view{L, I, N, prefixes.p, childOffsets.as<int32_t>(), parents.as<int32_t>(),
                                   levelRange.as<int32_t>(), i2l.as<int32_t>(), l2i.as<int32_t>()};
        o->centers         = centers.p;
        o->sizes           = sizes.p;
        o->halo_flags      = flags.as<uint8_t>();
        o->neighbors       = cfg.do_neighbors ? nb.as<uint32_t>() : nullptr;
        o->neighbor_counts = nc.as<uint32_t>();
        o->search_centers  = sc.p;
        o->search_sizes    = ss.p;
        return CS_OK;
    }
};

// splitmix64's finaliser (Steele, Lea, Flood 2014) as the mixing step of the neighbour checksum
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void neighborChecksumKernel(const uint32_t* __restrict__ nb, const uint32_t* __restrict__ nc, size_t n,
                                       unsigned ngmax, unsigned long long* out)
{
    unsigned long long acc = 0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        uint32_t c = nc[i];
        unsigned m = c < ngmax ? c : ngmax;
        uint64_t h = mix64(uint64_t(i) * 0x9e3779b97f4a7c15ull ^ c);
        for (unsigned k = 0; k < m; ++k)
            h = mix64(h ^ nb[i * ngmax + k]);
        acc += h;
    }
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

uint64_t neighborChecksum(cudaStream_t s, const uint32_t* nb, const uint32_t* nc, size_t n, unsigned ngmax,
                          uint64_t* scratchDev)
{
    uint64_t h = 0;
    if (cudaMemsetAsync(scratchDev, 0, sizeof(uint64_t), s) != cudaSuccess) return 0;
    unsigned g = unsigned(std::min<size_t>((n + 255) / 256, size_t(smCount()) * 8));
    if (n && ngmax) neighborChecksumKernel<<<std::max(1u, g), 256, 0, s>>>(nb, nc, n, ngmax,
                                                                           reinterpret_cast<unsigned long long*>(scratchDev));
    cudaMemcpyAsync(&h, scratchDev, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return h;
}

std::unique_ptr<PipelineBase> makePipeline(int coordBits, int keyBits, const cs_pipeline_config& cfg)
{
    std::unique_ptr<PipelineBase> p;
    if (coordBits == 64 && keyBits == 64) p = std::make_unique<Pipeline<double, uint64_t>>();
    else if (coordBits == 64) p = std::make_unique<Pipeline<double, uint32_t>>();
    else if (keyBits == 64) p = std::make_unique<Pipeline<float, uint64_t>>();
    else p = std::make_unique<Pipeline<float, uint32_t>>();
    p->cfg = cfg;
    return p;
}

} // namespace csg

using namespace csg;

struct cs_pipeline_s
{
    std::unique_ptr<PipelineBase> impl;
};

extern "C" int cs_pipeline_create(cs_pipeline* out, int coord_bits, int key_bits, const cs_pipeline_config* cfg)
{
    if (!out || !cfg || (coord_bits != 32 && coord_bits != 64) || (key_bits != 32 && key_bits != 64) ||
        cfg->bucket_size == 0)
    {
        setLastError("pipeline create: invalid arguments");
        return CS_ERR_INVALID;
    }
    auto* p = new cs_pipeline_s;
    p->impl = makePipeline(coord_bits, key_bits, *cfg);
    *out    = p;
    return CS_OK;
}

extern "C" int cs_pipeline_destroy(cs_pipeline p)
{
    delete p;
    return CS_OK;
}

extern "C" int cs_pipeline_run(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                               const void* h, size_t n, const cs_box* box, uint64_t f0, uint64_t f1,
                               cs_pipeline_result* res)
{
    if (!p || !box || !x || !y || !z || !h)
    {
        setLastError("pipeline run: null argument");
        return CS_ERR_INVALID;
    }
    return p->impl->run(cudaStream_t(stream), x, y, z, h, n, *box, f0, f1, res, false);
}

extern "C" int cs_pipeline_run_host(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                                    const void* h, size_t n, const cs_box* box, uint64_t f0, uint64_t f1,
                                    uint32_t* ncHost, uint8_t* flagsHost, size_t flagsCap, cs_pipeline_result* res)
{
    if (!p || !box || !x || !y || !z || !h)
    {
        setLastError("pipeline run: null argument");
        return CS_ERR_INVALID;
    }
    int rc = p->impl->run(cudaStream_t(stream), x, y, z, h, n, *box, f0, f1, res, true);
    if (rc) return rc;
    if ((rc = p->impl->copyBackAsync(cudaStream_t(stream), ncHost, flagsHost, flagsCap))) return rc;
    return p->impl->wait();
}

extern "C" int cs_pipeline_run_host_async(cs_pipeline p, cs_stream_t stream, const void* x, const void* y,
                                          const void* z, const void* h, size_t n, const cs_box* box, uint64_t f0,
                                          uint64_t f1, uint32_t* ncHost, uint8_t* flagsHost, size_t flagsCap,
                                          cs_pipeline_result* res)
{
    if (!p || !box || !x || !y || !z || !h)
    {
        setLastError("pipeline run: null argument");
        return CS_ERR_INVALID;
    }
    int rc = p->impl->run(cudaStream_t(stream), x, y, z, h, n, *box, f0, f1, res, true);
    if (rc) return rc;
    return p->impl->copyBackAsync(cudaStream_t(stream), ncHost, flagsHost, flagsCap);
}

extern "C" int cs_pipeline_run_host_csr_async(cs_pipeline p, cs_stream_t stream, const void* x, const void* y,
                                              const void* z, const void* h, size_t n, const cs_box* box, uint64_t f0,
                                              uint64_t f1, uint32_t* ncHost, uint8_t* flagsHost, size_t flagsCap,
                                              uint64_t* offsetsHost, uint32_t* listHost, size_t listCap,
                                              cs_pipeline_result* res)
{
    if (!p || !box || !x || !y || !z || !h || !offsetsHost || (!listHost && listCap))
    {
        setLastError("pipeline run: null argument");
        return CS_ERR_INVALID;
    }
    int rc = p->impl->run(cudaStream_t(stream), x, y, z, h, n, *box, f0, f1, res, true);
    if (rc) return rc;
    return p->impl->copyBackAsync(cudaStream_t(stream), ncHost, flagsHost, flagsCap, offsetsHost, listHost, listCap);
}

extern "C" int cs_pipeline_run_host_csr(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                                        const void* h, size_t n, const cs_box* box, uint64_t f0, uint64_t f1,
                                        uint32_t* ncHost, uint8_t* flagsHost, size_t flagsCap, uint64_t* offsetsHost,
                                        uint32_t* listHost, size_t listCap, cs_pipeline_result* res)
{
    int rc = cs_pipeline_run_host_csr_async(p, stream, x, y, z, h, n, box, f0, f1, ncHost, flagsHost, flagsCap,
                                            offsetsHost, listHost, listCap, res);
    if (rc) return rc;
    return p->impl->wait();
}

extern "C" int cs_pipeline_wait(cs_pipeline p)
{
    if (!p)
    {
        setLastError("pipeline wait: null argument");
        return CS_ERR_INVALID;
    }
    return p->impl->wait();
}

extern "C" int cs_pipeline_set_tuning(cs_pipeline p, const cs_tuning* t)
{
    if (!p || !t || !(t->nb_group == 8 || t->nb_group == 16 || t->nb_group == 32) || t->nb_by_target_cost < 0 ||
        t->nb_by_target_cost > 64 || !(t->sort_items == 0 || t->sort_items == 12 || t->sort_items == 16))
    {
        setLastError("set tuning: nb_group must be 8, 16 or 32, nb_by_target_cost in [0, 64], sort_items 0, 12 or 16");
        return CS_ERR_INVALID;
    }
    p->impl->tuning = *t;
    p->impl->resetSteps(); // captured step graphs hold the old launch arguments
    return CS_OK;
}

extern "C" int cs_pipeline_get_tuning(cs_pipeline p, cs_tuning* t)
{
    if (!p || !t)
    {
        setLastError("get tuning: null argument");
        return CS_ERR_INVALID;
    }
    *t = p->impl->tuning;
    return CS_OK;
}

extern "C" int cs_pipeline_autotune(cs_pipeline p, cs_stream_t stream, int reps, cs_tuning* best, cs_tuning* tried,
                                    float* ms, int capacity, int* count)
{
    if (!p || reps < 1 || capacity < 0)
    {
        setLastError("autotune: invalid argument");
        return CS_ERR_INVALID;
    }
    return p->impl->autotune(cudaStream_t(stream), reps, best, tried, ms, capacity, count);
}

extern "C" int cs_pipeline_step(cs_pipeline p, cs_stream_t stream, const void* x, const void* y, const void* z,
                                const void* h, size_t n, const cs_box* box, int use_graph, cs_pipeline_result* res)
{
    if (!p || !box || !x || !y || !z || !h)
    {
        setLastError("pipeline step: null argument");
        return CS_ERR_INVALID;
    }
    if (n == 0 || n >= (size_t(1) << 30))
    {
        setLastError("pipeline step: n = %zu outside [1, 2^30)", n);
        return CS_ERR_INVALID;
    }
    return p->impl->step(cudaStream_t(stream), x, y, z, h, n, *box, use_graph != 0, res);
}

extern "C" int cs_pipeline_reset_steps(cs_pipeline p)
{
    if (!p)
    {
        setLastError("pipeline reset: null argument");
        return CS_ERR_INVALID;
    }
    p->impl->resetSteps();
    return CS_OK;
}

extern "C" int cs_pipeline_graph_replays(cs_pipeline p) { return p ? p->impl->graphReplays : 0; }

extern "C" int cs_pipeline_get_outputs(cs_pipeline p, cs_pipeline_outputs* out)
{
    if (!p || !out)
    {
        setLastError("pipeline outputs: null argument");
        return CS_ERR_INVALID;
    }
    return p->impl->outputs(out);
}

extern "C" size_t cs_pipeline_device_bytes(cs_pipeline p) { return p ? p->impl->deviceBytes() : 0; }

extern "C" int cs_pipeline_copy_times(cs_pipeline p, float* ms, int count)
{
    if (!p || !ms || count < 0)
    {
        setLastError("pipeline copy times: invalid argument");
        return CS_ERR_INVALID;
    }
    return p->impl->copyTimes(ms, count);
}

/* per-stage device time of the last run in ms (keys, sort, gather, build, link, geometry, node prep, halos,
 * neighbours) */
extern "C" int cs_pipeline_stage_times(cs_pipeline p, float* ms, int count)
{
    if (!p || !ms)
    {
        setLastError("pipeline stage times: null argument");
        return CS_ERR_INVALID;
    }
    CSG_CUDA_TRY(cudaEventSynchronize(p->impl->ev[ST_COUNT]));
    for (int i = 0; i < count && i < ST_COUNT; ++i)
    {
        float t = 0;
        CSG_CUDA_TRY(cudaEventElapsedTime(&t, p->impl->ev[i], p->impl->ev[i + 1]));
        ms[i] = t;
    }
    return CS_OK;
}
