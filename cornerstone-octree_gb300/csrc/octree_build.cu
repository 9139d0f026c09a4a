// Cornerstone leaf-array construction (tree/csarray.hpp:76-440, tree/csarray_gpu.cu:35-231, tree/update_gpu.cuh).
//
// computeOctree runs the reference's `while (!updateOctree(...))` loop inside ONE cooperative launch. Per iteration:
//   A  rebalance decision per leaf (calculateNodeOp, tree/csarray.hpp:267-290) + per-block sums of the ops
//   C  exclusive scan of the ops (block sums scanned redundantly by every block, then a block-local scan)
//   D  emit the new leaves (processNode, tree/csarray.hpp:339-366) - one thread per NEW leaf, which finds its parent
//      leaf by binary search in the scanned ops - together with the new leaf's first-particle offset.
// Counts are exact (count = min(#keys in the leaf, maxCount)) in the reference whatever guess it searches from, so
// instead of re-searching all keys each iteration this keeps every leaf boundary's particle offset: unchanged and
// merged leaves keep their boundary's offset, split leaves binary-search only inside their parent's particle range.
// Phases are separated by a grid barrier whose spin is bounded (timeout -> CS_ERR_TIMEOUT, no hang).
//
// updateOctree (one step against possibly new keys) uses the same kernel in UPDATE mode: the decision reads the
// caller's counts, and the new leaves are recounted by exponential search around the previous layout.
#include "cs_common.cuh"
#include "octree_build.cuh"

#include <algorithm>
#include <atomic>

namespace csg
{

constexpr int BUILD_THREADS   = 256;
constexpr int BUILD_MAX_ITERS = 256;

struct BuildState
{
    unsigned barCount;
    unsigned barGen;
    int L;
    int iterations;
    int needed;
    uint32_t err;
    int converged;
    int maxDepth;
    int focusFirst;
    int focusLast;
    int changed[BUILD_MAX_ITERS];
};

// grid-wide barrier for a cooperative launch; returns false if the wait gave up. With `stall` set (test mode, first
// barrier only) block 0 does not arrive and gives up at once, so that every other block's wait runs out.
__device__ bool gridBarrier(BuildState* st, unsigned nblocks, unsigned spinLimit, bool stall = false)
{
    __shared__ int sFail;
    __syncthreads();
    if (threadIdx.x == 0 && stall && blockIdx.x == 0)
    {
        atomicOr(&st->err, ERRBIT_BARRIER_TIMEOUT);
        sFail = 1;
    }
    else if (threadIdx.x == 0)
    {
        sFail                  = 0;
        volatile unsigned* gen = &st->barGen;
        unsigned g             = *gen;
        __threadfence();
        unsigned arrived = atomicAdd(&st->barCount, 1u);
        if (arrived == nblocks - 1)
        {
            atomicExch(&st->barCount, 0u);
            __threadfence();
            atomicAdd(&st->barGen, 1u);
        }
        else
        {
            unsigned spins = 0;
            while (*gen == g)
            {
                if (++spins > spinLimit)
                {
                    atomicOr(&st->err, ERRBIT_BARRIER_TIMEOUT);
                    sFail = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return sFail == 0;
}

template<class T>
__device__ __forceinline__ T ldcg(const T* p)
{
    return __ldcg(p);
}

template<class K>
__device__ __forceinline__ size_t lowerBound(const K* __restrict__ a, size_t lo, size_t hi, K v)
{
    while (lo < hi)
    {
        size_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// findSearchBounds (tree/csarray.hpp:100-133) + lower_bound: exact lower bound of `target` searched outward from a
// guessed index
template<class K>
__device__ size_t guessedLowerBound(const K* __restrict__ keys, size_t n, long long guess, K target)
{
    using SI = long long;
    SI nCodes = SI(n);
    if (nCodes == 0) return 0;
    if (target >= nodeRange<K>(0)) return lowerBound(keys, 0, n, target);
    guess   = max(SI(0), min(nCodes - 1, guess));
    SI d    = (__ldg(keys + guess) < target) ? 1 : -1;
    SI step = 1;
    SI sec  = guess + d;
    while (0 <= sec && sec < nCodes && d * SI(__ldg(keys + sec)) <= d * SI(target))
    {
        step *= 2;
        sec = guess + step * d;
    }
    sec = max(SI(0), min(nCodes, sec));
    return lowerBound(keys, size_t(min(guess, sec)), size_t(max(guess, sec)), target);
}

__device__ __forceinline__ unsigned log8ceil32(unsigned v)
{
    // log8ceil<unsigned> of the reference for v in {8, 64, 512, 4096}
    unsigned lz = __clz(v - 1);
    return 10u - (lz - 2u) / 3u;
}

// per-set buckets and the merge floor of a batched tree (BatchTree); numSets = 0: one tree, the build's bucket
struct SetRules
{
    const uint32_t* setBucket = nullptr;
    int setShift              = 0;
    int numSets               = 0;
    unsigned minMergeLevel    = 0;
};

// calculateNodeOp with siblingAndLevel (tree/csarray.hpp:250-290); cnt(i) gives the (capped) leaf count
template<class K, class CountFn>
__device__ __forceinline__ int nodeOp(const K* tree, int i, unsigned bucketAll, CountFn cnt, const SetRules& sr = {})
{
    K node         = ldcg(tree + i);
    unsigned level = treeLevel<K>(ldcg(tree + i + 1) - node);
    unsigned long long bucket = bucketAll;
    if (sr.numSets)
    {
        // the set's own bucket; filler nodes past the last set never change (empty, never merged)
        K set  = node >> sr.setShift;
        bucket = set < K(sr.numSets) ? (unsigned long long)__ldg(sr.setBucket + set) : ~0ull;
    }
    int sib = -1;
    if (level > sr.minMergeLevel)
    {
        sib = int(octalDigit<K>(node, level));
        if (ldcg(tree + i - sib + 8) != ldcg(tree + i - sib) + nodeRange<K>(level - 1)) sib = -1;
    }
    if (sib > 0)
    {
        unsigned long long parent = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s)
            parent += cnt(i - sib + s);
        if (parent <= bucket) return 0;
    }
    constexpr unsigned L = KeyTraits<K>::maxLevel;
    unsigned long long c = cnt(i);
    if (c > bucket * 512u && level + 3 < L) return 4096;
    if (c > bucket * 64u && level + 2 < L) return 512;
    if (c > bucket * 8u && level + 1 < L) return 64;
    if (c > bucket && level < L) return 8;
    return 1;
}

__device__ __forceinline__ int blockReduceSum(int v, int* sRed)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sRed[warp] = v;
    __syncthreads();
    int r = 0;
    if (threadIdx.x < 32)
    {
        r = threadIdx.x < (blockDim.x >> 5) ? sRed[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1)
            r += __shfl_down_sync(0xffffffffu, r, o);
        if (threadIdx.x == 0) sRed[0] = r;
    }
    __syncthreads();
    r = sRed[0];
    __syncthreads();
    return r;
}

// exclusive block scan of one int per thread, returns the block total in *total
__device__ __forceinline__ int blockExclusiveScan(int v, int* sScan, int* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) sScan[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        int w = lane < nw ? sScan[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) sScan[lane] = w;
    }
    __syncthreads();
    int pre = warp > 0 ? sScan[warp - 1] : 0;
    *total  = sScan[nw - 1];
    return pre + x - v;
}

template<class K>
struct BuildArgs
{
    const K* keys;
    size_t n;
    unsigned bucket;
    uint32_t maxCount;
    K* tree[2];
    uint32_t* off[2];
    int* ops;      // capacity + 1
    long long* gscan; // UPDATE: exclusive scan of input counts (guesses), capacity + 1
    int* blockSums;   // gridDim.x
    long long* blockCnt; // gridDim.x (UPDATE)
    int capacity;
    int updateMode;
    const uint32_t* countsIn; // UPDATE
    int Lin;                  // UPDATE
    const int* LinDev;        // UPDATE: the input leaf count in device memory (replaces Lin when set)
    int initL;                // BUILD from a given leaf array (batched sets): its leaf count, 0 = from the root
    SetRules rules;
    // outputs
    K* treeOut;
    uint32_t* countsOut;
    uint32_t* layoutOut;
    BuildState* st;
    FocusQuery<K> focus;
    const uint32_t* upstreamErr; // the key sort's error word (may be null): set means the keys may be unordered
    unsigned spinLimit;    // polls of a grid barrier before it gives up
    int stallFirstBarrier; // test mode: block 0 never arrives at the first barrier
};

template<class K>
__global__ void __launch_bounds__(BUILD_THREADS) octreeBuildKernel(BuildArgs<K> a)
{
    __shared__ int sRed[32];
    __shared__ long long sRedLL[32];
    const unsigned G   = gridDim.x;
    const unsigned b   = blockIdx.x;
    const unsigned tid = threadIdx.x;
    BuildState* st     = a.st;

    // keys from a sort whose look-back gave up may be unordered: every block leaves before touching them (all blocks
    // read the same word, written before this launch, so none waits at a barrier for the others)
    if (a.upstreamErr && *a.upstreamErr)
    {
        if (b == 0 && tid == 0) atomicOr(&st->err, ERRBIT_UPSTREAM);
        return;
    }

    int L   = a.updateMode ? (a.LinDev ? *a.LinDev : a.Lin) : (a.initL ? a.initL : 1);
    int cur = 0;
    if (!a.updateMode && !a.initL && b == 0 && tid == 0)
    {
        a.tree[0][0] = 0;
        a.tree[0][1] = nodeRange<K>(0);
        a.off[0][0]  = 0;
        a.off[0][1]  = uint32_t(a.n);
    }
    if (!gridBarrier(st, G, a.spinLimit, a.stallFirstBarrier != 0)) return;

    int iter = 0;
    bool converged = false;
    for (; iter < (a.updateMode ? 1 : BUILD_MAX_ITERS); ++iter)
    {
        const K* tr        = a.tree[cur];
        const uint32_t* of = a.off[cur];
        K* ntr             = a.tree[cur ^ 1];
        uint32_t* nof      = a.off[cur ^ 1];

        // ---------------- phase A: decisions ----------------
        int chunk = (L + int(G) - 1) / int(G);
        int cs    = min(L, int(b) * chunk);
        int ce    = min(L, cs + chunk);
        int sum   = 0;
        long long csum = 0;
        bool changed = false;
        for (int i = cs + int(tid); i < ce; i += BUILD_THREADS)
        {
            int op;
            if (a.updateMode)
            {
                const uint32_t* cin = a.countsIn;
                op = nodeOp<K>(tr, i, a.bucket, [cin](int j) { return __ldg(cin + j); }, a.rules);
                csum += __ldg(cin + i);
            }
            else
            {
                // computeOctree seeds the root with the uncapped key count (tree/csarray.hpp:433-434); every later
                // count is capped at maxCount as computeNodeCounts does
                uint32_t mc = iter == 0 ? 0xffffffffu : a.maxCount;
                op = nodeOp<K>(
                    tr, i, a.bucket,
                    [of, mc](int j) {
                        uint32_t c = ldcg(of + j + 1) - ldcg(of + j);
                        return c < mc ? c : mc;
                    },
                    a.rules);
            }
            a.ops[i] = op;
            sum += op;
            changed |= (op != 1);
        }
        int bsum = blockReduceSum(sum, sRed);
        long long bcnt = 0;
        if (a.updateMode)
        {
            // reduce csum (long long) over the block
            long long v = csum;
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_down_sync(0xffffffffu, v, o);
            if ((tid & 31) == 0) sRedLL[tid >> 5] = v;
            __syncthreads();
            if (tid == 0)
            {
                long long r = 0;
                for (int w = 0; w < BUILD_THREADS / 32; ++w)
                    r += sRedLL[w];
                sRedLL[0] = r;
            }
            __syncthreads();
            bcnt = sRedLL[0];
            __syncthreads();
        }
        if (__syncthreads_or(changed) && tid == 0) atomicOr(&st->changed[iter], 1);
        if (tid == 0)
        {
            a.blockSums[b] = bsum;
            if (a.updateMode) a.blockCnt[b] = bcnt;
        }
        if (!gridBarrier(st, G, a.spinLimit)) return;

        if (!a.updateMode && ldcg(&st->changed[iter]) == 0)
        {
            converged = true;
            break;
        }

        // ---------------- phase C: scan ----------------
        int pre = 0, tot = 0;
        long long preC = 0;
        for (unsigned j = tid; j < G; j += BUILD_THREADS)
        {
            int v = ldcg(a.blockSums + j);
            tot += v;
            if (j < b) pre += v;
            if (a.updateMode && j < b) preC += ldcg(a.blockCnt + j);
        }
        pre = blockReduceSum(pre, sRed);
        tot = blockReduceSum(tot, sRed);
        if (a.updateMode)
        {
            long long v = preC;
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_down_sync(0xffffffffu, v, o);
            if ((tid & 31) == 0) sRedLL[tid >> 5] = v;
            __syncthreads();
            if (tid == 0)
            {
                long long r = 0;
                for (int w = 0; w < BUILD_THREADS / 32; ++w)
                    r += sRedLL[w];
                sRedLL[0] = r;
            }
            __syncthreads();
            preC = sRedLL[0];
            __syncthreads();
        }
        if (tot > a.capacity)
        {
            if (b == 0 && tid == 0)
            {
                st->needed = tot;
                atomicOr(&st->err, ERRBIT_CAPACITY);
                st->L = L;
            }
            return; // every block computed the same total and leaves here
        }
        int carry = pre;
        long long carryC = preC;
        for (int t0 = cs; t0 < ce; t0 += BUILD_THREADS)
        {
            int i   = t0 + int(tid);
            int v   = i < ce ? a.ops[i] : 0;
            int tt  = 0;
            int ex  = blockExclusiveScan(v, sRed, &tt);
            if (i < ce) a.ops[i] = carry + ex;
            carry += tt;
            if (a.updateMode)
            {
                // guesses: exclusive scan of the input counts, in long long to be safe
                long long c = i < ce ? (long long)__ldg(a.countsIn + i) : 0;
                long long x = c;
                const int lane = tid & 31, warp = tid >> 5;
                for (int o = 1; o < 32; o <<= 1)
                {
                    long long y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                __syncthreads();
                if (lane == 31) sRedLL[warp] = x;
                __syncthreads();
                long long wp = 0;
                for (int w = 0; w < warp; ++w)
                    wp += sRedLL[w];
                long long blockTot = 0;
                for (int w = 0; w < BUILD_THREADS / 32; ++w)
                    blockTot += sRedLL[w];
                if (i < ce) a.gscan[i] = carryC + wp + x - c;
                carryC += blockTot;
                __syncthreads();
            }
        }
        if (b == 0 && tid == 0)
        {
            a.ops[L] = tot;
            if (a.updateMode) a.gscan[L] = (long long)a.n;
        }
        if (!gridBarrier(st, G, a.spinLimit)) return;

        // ---------------- phase D: emit new leaves ----------------
        const int newL = tot;
        for (int j = int(b * BUILD_THREADS + tid); j <= newL; j += int(G * BUILD_THREADS))
        {
            if (j == newL)
            {
                ntr[newL] = ldcg(tr + L);
                nof[newL] = uint32_t(a.n);
                continue;
            }
            // parent leaf: last i with ops[i] <= j (leaves with op 0 have ops[i] == ops[i+1] and are skipped)
            int lo = 0, hi = L + 1;
            while (lo < hi)
            {
                int mid = (lo + hi) >> 1;
                if (ldcg(a.ops + mid) <= j) lo = mid + 1;
                else hi = mid;
            }
            int i      = lo - 1;
            int first  = ldcg(a.ops + i);
            int op     = ldcg(a.ops + i + 1) - first;
            int s      = j - first;
            K node     = ldcg(tr + i);
            K key;
            if (op == 1) { key = node; }
            else
            {
                unsigned level = treeLevel<K>(ldcg(tr + i + 1) - node);
                unsigned ld    = log8ceil32(unsigned(op));
                key            = node + K(s) * nodeRange<K>(level + ld);
            }
            ntr[j] = key;
            if (a.updateMode)
            {
                // guess: the previous layout position of the parent leaf
                a.gscan[size_t(a.capacity) + 1 + j] = ldcg(a.gscan + i);
            }
            else
            {
                uint32_t o;
                if (s == 0) o = ldcg(of + i);
                else o = uint32_t(lowerBound<K>(a.keys, ldcg(of + i), ldcg(of + i + 1), key));
                nof[j] = o;
            }
        }
        if (!gridBarrier(st, G, a.spinLimit)) return;
        L   = newL;
        cur ^= 1;
    }

    if (a.updateMode)
    {
        // recount the new leaves against the keys (exact lower bounds from guessed positions)
        K* tr         = a.tree[cur];
        uint32_t* of  = a.off[cur];
        for (int j = int(b * BUILD_THREADS + tid); j <= L; j += int(G * BUILD_THREADS))
        {
            long long g = j < L ? ldcg(a.gscan + size_t(a.capacity) + 1 + j) : (long long)a.n;
            of[j]       = uint32_t(guessedLowerBound<K>(a.keys, a.n, g, ldcg(tr + j)));
        }
        if (!gridBarrier(st, G, a.spinLimit)) return;
        converged = ldcg(&st->changed[0]) == 0;
    }
    else if (!converged)
    {
        if (b == 0 && tid == 0) atomicOr(&st->err, ERRBIT_NO_CONVERGENCE);
    }

    // ---------------- outputs ----------------
    const K* tr        = a.tree[cur];
    const uint32_t* of = a.off[cur];
    int depth          = 0;
    for (int j = int(b * BUILD_THREADS + tid); j <= L; j += int(G * BUILD_THREADS))
    {
        K kj = ldcg(tr + j);
        if (a.treeOut) a.treeOut[j] = kj;
        if (a.layoutOut) a.layoutOut[j] = ldcg(of + j);
        if (j < L)
        {
            uint32_t c     = ldcg(of + j + 1) - ldcg(of + j);
            a.countsOut[j] = c < a.maxCount ? c : a.maxCount;
            depth          = max(depth, int(treeLevel<K>(ldcg(tr + j + 1) - kj)));
        }
    }
    depth = __reduce_max_sync(0xffffffffu, depth);
    if ((tid & 31) == 0 && depth > 0) atomicMax(&st->maxDepth, depth);
    if (a.focus.enable && b == 0 && tid < 2)
    {
        K key  = tid == 0 ? a.focus.start : a.focus.end;
        int lo = 0, hi = L + 1;
        while (lo < hi)
        {
            int mid = (lo + hi) >> 1;
            if (ldcg(tr + mid) < key) lo = mid + 1;
            else hi = mid;
        }
        lo = min(lo, L);
        if (tid == 0) st->focusFirst = lo;
        else st->focusLast = lo;
    }
    if (b == 0 && tid == 0)
    {
        st->L          = L;
        st->iterations = a.updateMode ? 1 : iter + 1;
        st->converged  = converged ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------------------

template<class K>
struct BuildLayout
{
    K* tree[2];
    uint32_t* off[2];
    int* ops;
    long long* gscan;
    int* blockSums;
    long long* blockCnt;
    BuildState* st;
};

// blocks of the cooperative build on the current device: all resident at once (at most 4 per SM), computed once per
// device ordinal since devices may differ in SM count
static int buildGridSize()
{
    constexpr int MAX_DEVICES = 64;
    static std::atomic<int> cached[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < MAX_DEVICES && cached[dev].load() > 0) return cached[dev].load();
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, octreeBuildKernel<uint64_t>, BUILD_THREADS, 0);
    int perSm32 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm32, octreeBuildKernel<uint32_t>, BUILD_THREADS, 0);
    perSm     = std::max(1, std::min(std::min(perSm, perSm32), 4));
    const int g = perSm * smCount();
    if (dev >= 0 && dev < MAX_DEVICES) cached[dev].store(g);
    return g;
}

template<class K>
static BuildLayout<K> buildLayout(Arena& ar, int capacity, bool update)
{
    BuildLayout<K> l;
    size_t c1   = size_t(capacity) + 1;
    l.tree[0]   = ar.take<K>(c1);
    l.tree[1]   = ar.take<K>(c1);
    l.off[0]    = ar.take<uint32_t>(c1);
    l.off[1]    = ar.take<uint32_t>(c1);
    l.ops       = ar.take<int>(c1);
    l.gscan     = update ? ar.take<long long>(2 * c1) : nullptr;
    l.blockSums = ar.take<int>(4096);
    l.blockCnt  = ar.take<long long>(4096);
    l.st        = ar.take<BuildState>(1);
    return l;
}

std::mutex& cooperativeBuildMutex()
{
    static std::mutex m;
    return m;
}

template<class K>
size_t octreeBuildWorkspaceBytes(int capacity, bool update)
{
    Arena ar;
    buildLayout<K>(ar, capacity, update);
    return ar.size + 256;
}

template<class K>
int octreeBuild(cudaStream_t s, const K* keys, size_t n, unsigned bucket, uint32_t maxCount, const K* treeIn,
                const uint32_t* countsIn, int Lin, K* treeOut, uint32_t* countsOut, uint32_t* layoutOut, int capacity,
                void* ws, size_t wsBytes, BuildResult* res, bool sync, FocusQuery<K> focus, const int* LinDev,
                const BatchTree<K>* batch, const uint32_t* upstreamErr)
{
    bool update = treeIn != nullptr;
    if (batch && (update || batch->initL < 1 || batch->initL > capacity || !batch->initTree || !batch->initOff))
    {
        setLastError("octree: invalid batched start (leaves %d, capacity %d)", batch ? batch->initL : 0, capacity);
        return CS_ERR_INVALID;
    }
    if (bucket == 0)
    {
        setLastError("octree: bucket size must be positive");
        return CS_ERR_INVALID;
    }
    if (capacity < 1 || (update && !LinDev && Lin > capacity))
    {
        setLastError("octree: capacity %d too small", capacity);
        return CS_ERR_INVALID;
    }
    if (n >= (size_t(1) << 32))
    {
        setLastError("octree: too many keys");
        return CS_ERR_INVALID;
    }
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    BuildLayout<K> l = buildLayout<K>(ar, capacity, update);
    if (!ar.ok())
    {
        setLastError("octree: workspace too small");
        return CS_ERR_INVALID;
    }
    CSG_CUDA_TRY(cudaMemsetAsync(l.st, 0, sizeof(BuildState), s));
    if (update)
    {
        // with the count in device memory the whole capacity is copied (the host does not know Lin)
        size_t keysIn = LinDev ? size_t(capacity) + 1 : size_t(Lin) + 1;
        CSG_CUDA_TRY(cudaMemcpyAsync(l.tree[0], treeIn, keysIn * sizeof(K), cudaMemcpyDeviceToDevice, s));
    }

    if (batch)
    {
        CSG_CUDA_TRY(cudaMemcpyAsync(l.tree[0], batch->initTree, (size_t(batch->initL) + 1) * sizeof(K),
                                     cudaMemcpyDeviceToDevice, s));
        CSG_CUDA_TRY(cudaMemcpyAsync(l.off[0], batch->initOff, (size_t(batch->initL) + 1) * sizeof(uint32_t),
                                     cudaMemcpyDeviceToDevice, s));
    }

    std::unique_lock<std::mutex> coop(cooperativeBuildMutex(), std::defer_lock);
    if (sync) coop.lock(); // held until octreeBuildFinish below has synchronised

    int G = buildGridSize();
    BuildArgs<K> a;
    a.keys       = keys;
    a.n          = n;
    a.bucket     = bucket;
    a.maxCount   = maxCount;
    a.tree[0]    = l.tree[0];
    a.tree[1]    = l.tree[1];
    a.off[0]     = l.off[0];
    a.off[1]     = l.off[1];
    a.ops        = l.ops;
    a.gscan      = l.gscan;
    a.blockSums  = l.blockSums;
    a.blockCnt   = l.blockCnt;
    a.capacity   = capacity;
    a.updateMode = update ? 1 : 0;
    a.countsIn   = countsIn;
    a.Lin        = Lin;
    a.LinDev     = LinDev;
    a.initL      = batch ? batch->initL : 0;
    a.rules      = batch ? SetRules{batch->setBucket, batch->setShift, batch->numSets, unsigned(batch->minMergeLevel)}
                         : SetRules{};
    a.treeOut    = treeOut;
    a.countsOut  = countsOut;
    a.layoutOut  = layoutOut;
    a.st         = l.st;
    a.focus      = focus;
    a.upstreamErr = upstreamErr;
    const WaitLimits wl = waitLimits();
    a.spinLimit         = wl.barrierSpins;
    a.stallFirstBarrier = (wl.stall & CS_WAIT_STALL_BARRIER) ? 1 : 0;
    void* params[] = {&a};
    CSG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)octreeBuildKernel<K>, dim3(G), dim3(BUILD_THREADS), params,
                                             0, s));
    if (res) res->stateDev = &l.st->L;
    if (!sync) return CS_OK;
    return octreeBuildFinish<K>(s, ws, wsBytes, capacity, update, res);
}

template<class K>
int octreeBuildFinish(cudaStream_t s, void* ws, size_t wsBytes, int capacity, bool update, BuildResult* res)
{
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    BuildLayout<K> l = buildLayout<K>(ar, capacity, update);
    if (!ar.ok())
    {
        setLastError("octree: workspace too small");
        return CS_ERR_INVALID;
    }
    BuildState h;
    static_assert(sizeof(BuildState) % 4 == 0 && sizeof(BuildState) <= 4096, "read as at most 4 KB of 32-bit words");
    if (int rc = readSmallToHost(s, &h, l.st, sizeof(BuildState))) return rc;
    if (res)
    {
        res->numLeaves  = h.L;
        res->iterations = h.iterations;
        res->converged  = h.converged;
        res->needed     = h.needed;
        res->maxDepth   = h.maxDepth;
        res->focusFirst = h.focusFirst;
        res->focusLast  = h.focusLast;
    }
    if (h.err & ERRBIT_UPSTREAM)
    {
        setLastError("octree: the key sort's look-back timed out; the build did not run");
        return CS_ERR_TIMEOUT;
    }
    if (h.err & ERRBIT_BARRIER_TIMEOUT)
    {
        setLastError("octree: grid barrier timed out");
        return CS_ERR_TIMEOUT;
    }
    if (h.err & ERRBIT_CAPACITY)
    {
        setLastError("octree: %d leaves needed, capacity %d", h.needed, capacity);
        if (res) res->numLeaves = h.needed;
        return CS_ERR_CAPACITY;
    }
    if (h.err & ERRBIT_NO_CONVERGENCE)
    {
        setLastError("octree: no convergence after %d iterations", BUILD_MAX_ITERS);
        return CS_ERR_DEVICE;
    }
    return CS_OK;
}

// after an update build without host synchronisation: the new leaf count becomes the current one only if the build
// succeeded; on failure (capacity) the input count stays, so every later kernel of the step stays within its buffers
__global__ void commitLeafCountKernel(const BuildState* st, int* Ldev)
{
    if (st->err == 0) *Ldev = st->L;
}

template<class K>
int commitLeafCount(cudaStream_t s, void* ws, size_t wsBytes, int capacity, int* Ldev)
{
    Arena ar{static_cast<char*>(ws), 0, wsBytes};
    BuildLayout<K> l = buildLayout<K>(ar, capacity, true);
    if (!ar.ok())
    {
        setLastError("octree: workspace too small");
        return CS_ERR_INVALID;
    }
    commitLeafCountKernel<<<1, 1, 0, s>>>(l.st, Ldev);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int commitLeafCount<uint32_t>(cudaStream_t, void*, size_t, int, int*);
template int commitLeafCount<uint64_t>(cudaStream_t, void*, size_t, int, int*);
template int octreeBuildFinish<uint32_t>(cudaStream_t, void*, size_t, int, bool, BuildResult*);
template int octreeBuildFinish<uint64_t>(cudaStream_t, void*, size_t, int, bool, BuildResult*);
template size_t octreeBuildWorkspaceBytes<uint32_t>(int, bool);
template size_t octreeBuildWorkspaceBytes<uint64_t>(int, bool);
template int octreeBuild<uint32_t>(cudaStream_t, const uint32_t*, size_t, unsigned, uint32_t, const uint32_t*,
                                   const uint32_t*, int, uint32_t*, uint32_t*, uint32_t*, int, void*, size_t,
                                   BuildResult*, bool, FocusQuery<uint32_t>, const int*, const BatchTree<uint32_t>*,
                                   const uint32_t*);
template int octreeBuild<uint64_t>(cudaStream_t, const uint64_t*, size_t, unsigned, uint32_t, const uint64_t*,
                                   const uint32_t*, int, uint64_t*, uint32_t*, uint32_t*, int, void*, size_t,
                                   BuildResult*, bool, FocusQuery<uint64_t>, const int*, const BatchTree<uint64_t>*,
                                   const uint32_t*);

// ---------------------------------------------------------------------------------------------------------------
// standalone counts and decisions
// ---------------------------------------------------------------------------------------------------------------

template<class K>
__global__ void boundaryOffsetsKernel(const K* __restrict__ tree, int numNodes, const K* __restrict__ keys, size_t n,
                                      uint32_t* __restrict__ off)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j <= numNodes) off[j] = uint32_t(lowerBound<K>(keys, 0, n, tree[j]));
}

__global__ void countsFromOffsetsKernel(const uint32_t* __restrict__ off, int numNodes, uint32_t maxCount,
                                        uint32_t* __restrict__ counts)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < numNodes)
    {
        uint32_t c = off[j + 1] - off[j];
        counts[j]  = c < maxCount ? c : maxCount;
    }
}

template<class K>
int nodeCounts(cudaStream_t s, const K* tree, uint32_t* counts, int numNodes, const K* keys, size_t n,
               uint32_t maxCount, void* ws, size_t wsBytes)
{
    if (numNodes <= 0) return CS_OK;
    Workspace w;
    int rc = w.acquire(ws, wsBytes, (size_t(numNodes) + 1) * sizeof(uint32_t) + 256, s);
    if (rc) return rc;
    uint32_t* off = static_cast<uint32_t*>(w.ptr);
    boundaryOffsetsKernel<K><<<iceil(size_t(numNodes) + 1, 256), 256, 0, s>>>(tree, numNodes, keys, n, off);
    CSG_CHECK_LAUNCH();
    countsFromOffsetsKernel<<<iceil(size_t(numNodes), 256), 256, 0, s>>>(off, numNodes, maxCount, counts);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template<class K>
__global__ void decisionKernel(const K* __restrict__ tree, const uint32_t* __restrict__ counts, int numNodes,
                               unsigned bucket, int* __restrict__ ops, int* convergedDev)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool changed = false;
    if (i < numNodes)
    {
        int op = nodeOp<K>(tree, i, bucket, [counts](int j) { return __ldg(counts + j); });
        ops[i] = op;
        changed = op != 1;
    }
    if (__syncthreads_or(changed) && threadIdx.x == 0) atomicExch(convergedDev, 0);
}

template<class K>
int rebalanceDecision(cudaStream_t s, const K* tree, const uint32_t* counts, int numNodes, unsigned bucket, int* ops,
                      int* convergedDev)
{
    int one = 1;
    CSG_CUDA_TRY(cudaMemcpyAsync(convergedDev, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    if (numNodes <= 0) return CS_OK;
    decisionKernel<K><<<iceil(size_t(numNodes), 256), 256, 0, s>>>(tree, counts, numNodes, bucket, ops, convergedDev);
    CSG_CHECK_LAUNCH();
    // the host value `one` must outlive the copy
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    return CS_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// exclusive scan of int32 (in place allowed) and the emission of a rebalanced leaf array from scanned ops
// ---------------------------------------------------------------------------------------------------------------
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS   = 4;
constexpr int SCAN_TILE    = SCAN_THREADS * SCAN_ITEMS;

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ __forceinline__ int scanBlockExclusive(int v, int* sWarp, int* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        int w = lane < SCAN_THREADS / 32 ? sWarp[lane] : 0;
        int wi = w;
        for (int o = 1; o < 32; o <<= 1)
        {
            int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < SCAN_THREADS / 32) sWarp[lane] = wi - w;
        if (lane == 31) sWarp[SCAN_THREADS / 32] = wi;
    }
    __syncthreads();
    int r  = sWarp[warp] + incl - v;
    *total = sWarp[SCAN_THREADS / 32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) scanTileSumsKernel(const int32_t* __restrict__ in, size_t n,
                                                                   int32_t* __restrict__ tileSums)
{
    __shared__ int sWarp[SCAN_THREADS / 32 + 1];
    size_t base = size_t(blockIdx.x) * SCAN_TILE + size_t(threadIdx.x) * SCAN_ITEMS;
    int v       = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) v += in[base + k];
    int total;
    scanBlockExclusive(v, sWarp, &total);
    if (threadIdx.x == 0) tileSums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums (plus init), in place
__global__ void __launch_bounds__(SCAN_THREADS) scanTileOffsetsKernel(int32_t* tileSums, int numTiles, int32_t init)
{
    __shared__ int sWarp[SCAN_THREADS / 32 + 1];
    int carry = init;
    for (int b = 0; b < numTiles; b += SCAN_THREADS)
    {
        int i = b + threadIdx.x;
        int v = i < numTiles ? tileSums[i] : 0;
        int total;
        int e = scanBlockExclusive(v, sWarp, &total);
        if (i < numTiles) tileSums[i] = carry + e;
        carry += total;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) scanApplyKernel(const int32_t* in, int32_t* out, size_t n,
                                                                const int32_t* __restrict__ tileOffsets)
{
    __shared__ int sWarp[SCAN_THREADS / 32 + 1];
    size_t base = size_t(blockIdx.x) * SCAN_TILE + size_t(threadIdx.x) * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        v[k] = base + k < n ? in[base + k] : 0;
        sum += v[k];
    }
    int total;
    int e = scanBlockExclusive(sum, sWarp, &total) + tileOffsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
}

size_t exclusiveScanWorkspaceBytes(size_t n) { return (n / SCAN_TILE + 1) * sizeof(int32_t) + 256; }

int exclusiveScanI32(cudaStream_t s, const int32_t* in, int32_t* out, size_t n, int32_t init, void* ws, size_t wsb)
{
    if (n == 0) return CS_OK;
    if (!in || !out || n >= (size_t(1) << 31))
    {
        setLastError("exclusive scan: null pointer or n >= 2^31");
        return CS_ERR_INVALID;
    }
    Workspace w;
    int rc = w.acquire(ws, wsb, exclusiveScanWorkspaceBytes(n), s);
    if (rc) return rc;
    int32_t* tiles = static_cast<int32_t*>(w.ptr);
    unsigned nt    = unsigned((n + SCAN_TILE - 1) / SCAN_TILE);
    scanTileSumsKernel<<<nt, SCAN_THREADS, 0, s>>>(in, n, tiles);
    CSG_CHECK_LAUNCH();
    scanTileOffsetsKernel<<<1, SCAN_THREADS, 0, s>>>(tiles, int(nt), init);
    CSG_CHECK_LAUNCH();
    scanApplyKernel<<<nt, SCAN_THREADS, 0, s>>>(in, out, n, tiles);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

// processNode (tree/csarray.hpp:339-366): node i with ops[i+1] - ops[i] = 8^k new nodes emits its 8^k descendants
// k levels down in key order (k = 0: the node itself; 0 new nodes: merged into its first sibling)
template<class K>
__global__ void rebalanceTreeKernel(const K* __restrict__ tree, int numNodes, const int32_t* __restrict__ ops,
                                    K* __restrict__ newTree)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numNodes) return;
    int off  = ops[i];
    int cnt  = ops[i + 1] - off;
    K key    = tree[i];
    K range  = tree[i + 1] - key;
    K step   = cnt > 0 ? range / K(cnt) : range;
    for (int j = 0; j < cnt; ++j)
        newTree[off + j] = key + K(j) * step;
    if (i == numNodes - 1) newTree[ops[numNodes]] = nodeRange<K>(0);
}

template<class K>
int rebalanceTree(cudaStream_t s, const K* tree, int numNodes, const int32_t* ops, K* newTree)
{
    if (numNodes <= 0) return CS_OK;
    if (!tree || !ops || !newTree)
    {
        setLastError("rebalance tree: null pointer");
        return CS_ERR_INVALID;
    }
    rebalanceTreeKernel<K><<<iceil(size_t(numNodes), 256), 256, 0, s>>>(tree, numNodes, ops, newTree);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int nodeCounts<uint32_t>(cudaStream_t, const uint32_t*, uint32_t*, int, const uint32_t*, size_t, uint32_t,
                                  void*, size_t);
template int nodeCounts<uint64_t>(cudaStream_t, const uint64_t*, uint32_t*, int, const uint64_t*, size_t, uint32_t,
                                  void*, size_t);

} // namespace csg

using namespace csg;

extern "C" size_t cs_node_counts_workspace_bytes(int32_t num_nodes) { return (size_t(num_nodes) + 1) * 4 + 256; }

extern "C" int cs_node_counts_u32(cs_stream_t stream, const uint32_t* tree, uint32_t* counts, int32_t num_nodes,
                                  const uint32_t* keys, size_t n, uint32_t max_count, int, void* ws, size_t wsb)
{
    return nodeCounts<uint32_t>(cudaStream_t(stream), tree, counts, num_nodes, keys, n, max_count, ws, wsb);
}
extern "C" int cs_node_counts_u64(cs_stream_t stream, const uint64_t* tree, uint32_t* counts, int32_t num_nodes,
                                  const uint64_t* keys, size_t n, uint32_t max_count, int, void* ws, size_t wsb)
{
    return nodeCounts<uint64_t>(cudaStream_t(stream), tree, counts, num_nodes, keys, n, max_count, ws, wsb);
}

extern "C" int cs_rebalance_decision_u32(cs_stream_t stream, const uint32_t* tree, const uint32_t* counts,
                                         int32_t num_nodes, unsigned bucket, int32_t* ops, int* converged_dev)
{
    return rebalanceDecision<uint32_t>(cudaStream_t(stream), tree, counts, num_nodes, bucket, ops, converged_dev);
}
extern "C" int cs_rebalance_decision_u64(cs_stream_t stream, const uint64_t* tree, const uint32_t* counts,
                                         int32_t num_nodes, unsigned bucket, int32_t* ops, int* converged_dev)
{
    return rebalanceDecision<uint64_t>(cudaStream_t(stream), tree, counts, num_nodes, bucket, ops, converged_dev);
}

extern "C" size_t cs_exclusive_scan_workspace_bytes(size_t n) { return exclusiveScanWorkspaceBytes(n); }
extern "C" int cs_exclusive_scan_i32(cs_stream_t stream, const int32_t* in, int32_t* out, size_t n, int32_t init,
                                     void* ws, size_t wsb)
{
    return exclusiveScanI32(cudaStream_t(stream), in, out, n, init, ws, wsb);
}
extern "C" int cs_rebalance_tree_u32(cs_stream_t stream, const uint32_t* tree, int32_t num_nodes,
                                     const int32_t* node_ops, uint32_t* new_tree)
{
    return rebalanceTree<uint32_t>(cudaStream_t(stream), tree, num_nodes, node_ops, new_tree);
}
extern "C" int cs_rebalance_tree_u64(cs_stream_t stream, const uint64_t* tree, int32_t num_nodes,
                                     const int32_t* node_ops, uint64_t* new_tree)
{
    return rebalanceTree<uint64_t>(cudaStream_t(stream), tree, num_nodes, node_ops, new_tree);
}

extern "C" size_t cs_compute_octree_workspace_bytes(int32_t capacity)
{
    return octreeBuildWorkspaceBytes<uint64_t>(capacity, false);
}

template<class K>
static int computeOctreeEntry(cs_stream_t stream, const K* keys, size_t n, unsigned bucket, uint32_t maxCount,
                              K* tree, uint32_t* counts, uint32_t* layout, int32_t capacity, int32_t* numLeaves,
                              int* iterations, void* ws, size_t wsb)
{
    if (!tree || !counts || (!keys && n))
    {
        setLastError("compute octree: null pointer");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    Workspace w;
    int rc = w.acquire(ws, wsb, octreeBuildWorkspaceBytes<K>(capacity, false), s);
    if (rc) return rc;
    BuildResult r{};
    rc = octreeBuild<K>(s, keys, n, bucket, maxCount, nullptr, nullptr, 0, tree, counts, layout, capacity, w.ptr,
                        octreeBuildWorkspaceBytes<K>(capacity, false), &r, true);
    if (numLeaves) *numLeaves = r.numLeaves;
    if (iterations) *iterations = r.iterations;
    return rc;
}

extern "C" int cs_compute_octree_u32(cs_stream_t stream, const uint32_t* keys, size_t n, unsigned bucket,
                                     uint32_t max_count, uint32_t* tree, uint32_t* counts, uint32_t* layout,
                                     int32_t capacity, int32_t* num_leaves, int* iterations, void* ws, size_t wsb)
{
    return computeOctreeEntry<uint32_t>(stream, keys, n, bucket, max_count, tree, counts, layout, capacity, num_leaves,
                                        iterations, ws, wsb);
}
extern "C" int cs_compute_octree_u64(cs_stream_t stream, const uint64_t* keys, size_t n, unsigned bucket,
                                     uint32_t max_count, uint64_t* tree, uint32_t* counts, uint32_t* layout,
                                     int32_t capacity, int32_t* num_leaves, int* iterations, void* ws, size_t wsb)
{
    return computeOctreeEntry<uint64_t>(stream, keys, n, bucket, max_count, tree, counts, layout, capacity, num_leaves,
                                        iterations, ws, wsb);
}

extern "C" size_t cs_update_octree_workspace_bytes(int32_t, int32_t capacity)
{
    return octreeBuildWorkspaceBytes<uint64_t>(capacity, true);
}

template<class K>
static int updateOctreeEntry(cs_stream_t stream, const K* keys, size_t n, unsigned bucket, uint32_t maxCount,
                             const K* treeIn, const uint32_t* countsIn, int32_t Lin, K* treeOut, uint32_t* countsOut,
                             int32_t capacity, int32_t* Lout, int* converged, void* ws, size_t wsb)
{
    if (!treeIn || !countsIn || !treeOut || !countsOut || (!keys && n) || Lin < 1)
    {
        setLastError("update octree: invalid arguments");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    Workspace w;
    size_t need = octreeBuildWorkspaceBytes<K>(capacity, true);
    int rc      = w.acquire(ws, wsb, need, s);
    if (rc) return rc;
    BuildResult r{};
    rc = octreeBuild<K>(s, keys, n, bucket, maxCount, treeIn, countsIn, Lin, treeOut, countsOut, nullptr, capacity,
                        w.ptr, need, &r, true);
    if (Lout) *Lout = r.numLeaves;
    if (converged) *converged = r.converged;
    return rc;
}

extern "C" int cs_update_octree_u32(cs_stream_t stream, const uint32_t* keys, size_t n, unsigned bucket,
                                    uint32_t max_count, const uint32_t* tree_in, const uint32_t* counts_in,
                                    int32_t L_in, uint32_t* tree_out, uint32_t* counts_out, int32_t capacity,
                                    int32_t* L_out, int* converged, void* ws, size_t wsb)
{
    return updateOctreeEntry<uint32_t>(stream, keys, n, bucket, max_count, tree_in, counts_in, L_in, tree_out,
                                       counts_out, capacity, L_out, converged, ws, wsb);
}
extern "C" int cs_update_octree_u64(cs_stream_t stream, const uint64_t* keys, size_t n, unsigned bucket,
                                    uint32_t max_count, const uint64_t* tree_in, const uint32_t* counts_in,
                                    int32_t L_in, uint64_t* tree_out, uint32_t* counts_out, int32_t capacity,
                                    int32_t* L_out, int* converged, void* ws, size_t wsb)
{
    return updateOctreeEntry<uint64_t>(stream, keys, n, bucket, max_count, tree_in, counts_in, L_in, tree_out,
                                       counts_out, capacity, L_out, converged, ws, wsb);
}
