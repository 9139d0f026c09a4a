// Internal interface of the cornerstone leaf-array build (octree_build.cu).
#pragma once
#include "cs_common.cuh"

#include <mutex>

namespace csg
{

constexpr uint32_t ERRBIT_BARRIER_TIMEOUT = 2u;
constexpr uint32_t ERRBIT_CAPACITY        = 4u;
constexpr uint32_t ERRBIT_NO_CONVERGENCE  = 8u;
constexpr uint32_t ERRBIT_UPSTREAM        = 16u; // the key sort before the build reported a timeout

struct BuildResult
{
    int numLeaves  = 0;
    int iterations = 0;
    int converged  = 0;
    int needed     = 0;
    int maxDepth   = 0; // deepest leaf level
    int focusFirst = 0; // lower_bound(leaves, focus.start)
    int focusLast  = 0; // lower_bound(leaves, focus.end)
    int* stateDev  = nullptr; // device address of the state block (numLeaves, iterations, needed, err, converged)
};

//! optional: leaf range [lower_bound(start), lower_bound(end)) of a key range, computed by the build's last phase
template<class K>
struct FocusQuery
{
    K start     = 0;
    K end       = 0;
    bool enable = false;
};

template<class K>
size_t octreeBuildWorkspaceBytes(int capacity, bool update);

/*! Build (treeIn == nullptr: computeOctree from the root) or update (one updateOctree step from treeIn/countsIn).
 *  With sync == false the call only enqueues work; the state block (see BuildResult::stateDev) holds the outcome.
 *  upstreamErr (device, may be null): the error word of the sort that produced `keys`; if it is set when the build
 *  starts, the build does nothing and reports CS_ERR_TIMEOUT (keys from a sort that gave up may be unordered). */
//! many independent sets in one tree: set s owns the key range [s << setShift, (s + 1) << setShift) (an aligned
//! subtree rooted at level minMergeLevel), uses bucket size setBucket[s], and no node at or above minMergeLevel is
//! merged; the build starts from initTree (set roots and empty filler nodes, initL leaves) with particle offsets
//! initOff instead of the root
template<class K>
struct BatchTree
{
    const K* initTree           = nullptr;
    const uint32_t* initOff     = nullptr;
    int initL                   = 0;
    const uint32_t* setBucket   = nullptr;
    int setShift                = 0;
    int numSets                 = 0;
    int minMergeLevel           = 0;
};

template<class K>
int octreeBuild(cudaStream_t s, const K* keys, size_t n, unsigned bucket, uint32_t maxCount, const K* treeIn,
                const uint32_t* countsIn, int Lin, K* treeOut, uint32_t* countsOut, uint32_t* layoutOut, int capacity,
                void* ws, size_t wsBytes, BuildResult* res, bool sync, FocusQuery<K> focus = FocusQuery<K>{},
                const int* LinDev = nullptr, const BatchTree<K>* batch = nullptr,
                const uint32_t* upstreamErr = nullptr);

/*! after an octreeBuild with sync = false (e.g. replayed from a CUDA graph): read its state block from the same
 *  workspace, synchronise, fill res and map the device error bits to a status, as the sync path does */
template<class K>
int octreeBuildFinish(cudaStream_t s, void* ws, size_t wsBytes, int capacity, bool update, BuildResult* res);

//! after an update octreeBuild with sync = false: *Ldev = the new leaf count if the build succeeded (else unchanged)
template<class K>
int commitLeafCount(cudaStream_t s, void* ws, size_t wsBytes, int capacity, int* Ldev);

//! cooperative builds launched by concurrent host threads must not overlap on the device (each grid is sized for the
//! whole GPU and waits at grid barriers for all its blocks): octreeBuild with sync holds this lock from its launch
//! until the build has finished; a caller that launches without sync and finishes later holds it over both
std::mutex& cooperativeBuildMutex();

template<class K>
int nodeCounts(cudaStream_t s, const K* tree, uint32_t* counts, int numNodes, const K* keys, size_t n,
               uint32_t maxCount, void* ws, size_t wsBytes);

} // namespace csg
