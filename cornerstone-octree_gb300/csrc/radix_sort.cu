// Stable LSD radix sort of (key, uint32 value) pairs: one histogram kernel for all digit positions, then one
// "onesweep" kernel per 8-bit digit (Adinets & Merrill, "Onesweep: a faster least significant digit radix sort for
// GPUs", 2022). Each block takes the next tile (256 threads x 16 or 12 keys: a runtime choice, SortShape) from an
// atomic counter, ranks its keys by digit in input
// order (warp match + per-warp counters), publishes its per-digit counts and obtains the counts of all earlier tiles
// by decoupled look-back, then scatters through shared memory so that global writes are runs of consecutive
// addresses. Traffic per pass: 2 * (sizeof(K) + 4) bytes per pair; the histogram reads the keys once.
//
// Look-back waits spin on a flag that an earlier tile (which has already started, because tiles are handed out in
// order) will publish; every wait is bounded, and a wait that gives up sets ERRBIT_SORT_TIMEOUT and continues.
#include "radix_sort.cuh"

#include <algorithm>
#include <cstdio>

namespace csg
{

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS   = RS_THREADS / 32;
constexpr int RS_MIN_TILE = RS_THREADS * 12; // the smaller of the two tile shapes sizes the workspace
constexpr int RS_BINS    = 256;
constexpr int RS_MAXPASS = 8;

constexpr uint32_t ST_AGG   = 1u << 30;
constexpr uint32_t ST_INC   = 2u << 30;
constexpr uint32_t ST_FLAGS = 3u << 30;
constexpr uint32_t ST_COUNT = (1u << 30) - 1;


struct SortLayout
{
    uint32_t* hist;        // [passes][256]
    uint32_t* status;      // [passes][tiles][256]
    uint32_t* tileCounter; // [passes]
    size_t tiles;
    int passes;
};

static inline int numPasses(int beginBit, int endBit) { return (endBit - beginBit + 7) / 8; }

template<class K>
static SortLayout sortLayout(Arena& a, size_t n, int beginBit, int endBit, int tile)
{
    SortLayout L;
    L.passes      = numPasses(beginBit, endBit);
    L.tiles       = (n + tile - 1) / tile;
    L.hist        = a.take<uint32_t>(size_t(RS_MAXPASS) * RS_BINS);
    L.tileCounter = a.take<uint32_t>(RS_MAXPASS);
    L.status      = a.take<uint32_t>(size_t(L.passes) * L.tiles * RS_BINS + 1);
    return L;
}

template<class K>
size_t radixSortWorkspaceBytes(size_t n, int beginBit, int endBit)
{
    Arena a;
    sortLayout<K>(a, n, beginBit, endBit, RS_MIN_TILE);
    return a.size + 256;
}

template<class K>
__device__ __forceinline__ uint32_t digitOf(K key, int shift, uint32_t mask)
{
    return uint32_t(key >> shift) & mask;
}

// all digit histograms in one read of the keys
template<class K>
__global__ void __launch_bounds__(256) radixHistogramKernel(const K* __restrict__ keys, size_t n, int beginBit,
                                                            int endBit, int passes, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t sh[2][RS_MAXPASS][RS_BINS];
    for (int i = threadIdx.x; i < 2 * RS_MAXPASS * RS_BINS; i += blockDim.x)
        (&sh[0][0][0])[i] = 0;
    __syncthreads();

    const int copy = (threadIdx.x >> 5) & 1;
    const int lane = threadIdx.x & 31;
    size_t stride  = size_t(gridDim.x) * blockDim.x;
    for (size_t i0 = size_t(blockIdx.x) * blockDim.x; i0 < n; i0 += stride)
    {
        size_t i   = i0 + threadIdx.x;
        bool valid = i < n;
        K key      = valid ? keys[i] : K(0);
        for (int p = 0; p < passes; ++p)
        {
            int shift     = beginBit + 8 * p;
            int bitsHere  = min(8, endBit - shift);
            uint32_t mask = (1u << bitsHere) - 1u;
            uint32_t d    = digitOf(key, shift, mask);
            uint32_t d0   = __shfl_sync(0xffffffffu, d, 0);
            unsigned vmask = __ballot_sync(0xffffffffu, valid);
            bool uniform   = __all_sync(0xffffffffu, !valid || d == d0) && (vmask & 1u);
            if (uniform)
            {
                if (lane == 0) atomicAdd(&sh[copy][p][d0], __popc(vmask));
            }
            else if (valid) { atomicAdd(&sh[copy][p][d], 1u); }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * RS_BINS; i += blockDim.x)
    {
        uint32_t c = (&sh[0][0][0])[i] + (&sh[1][0][0])[i];
        if (c) atomicAdd(hist + i, c);
    }
}

// exclusive scan of 256 values held one per thread (blockDim.x == 256)
__device__ __forceinline__ uint32_t blockExclusiveScan256(uint32_t v, uint32_t* sWarpSums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x     = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sWarpSums[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = lane < RS_WARPS ? sWarpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < RS_WARPS; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < RS_WARPS) sWarpSums[lane] = w; // inclusive warp sums
    }
    __syncthreads();
    uint32_t warpPrefix = warp > 0 ? sWarpSums[warp - 1] : 0;
    return warpPrefix + x - v;
}

template<class K, bool Iota, int Items, int MinBlocks>
__global__ void __launch_bounds__(RS_THREADS, MinBlocks) onesweepKernel(const K* __restrict__ keysIn,
                                                             const uint32_t* __restrict__ valsIn,
                                                             K* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                             size_t n, int shift, uint32_t mask,
                                                             const uint32_t* __restrict__ passHist,
                                                             uint32_t* status, uint32_t* tileCounter,
                                                             uint32_t* errWord, uint32_t spinLimit, int stallTile1)
{
    constexpr int Tile = RS_THREADS * Items;
    extern __shared__ __align__(16) unsigned char smem[];
    K* sKeys        = reinterpret_cast<K*>(smem);
    uint32_t* sVals = reinterpret_cast<uint32_t*>(smem + Tile * sizeof(K));

    __shared__ uint32_t sWarpHist[RS_WARPS][RS_BINS];
    __shared__ uint32_t sTileOff[RS_BINS];
    __shared__ uint32_t sGlobalBase[RS_BINS];
    __shared__ uint32_t sWarpSums[RS_WARPS];
    __shared__ uint32_t sTile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) sTile = atomicAdd(tileCounter, 1u);
    for (int i = tid; i < RS_WARPS * RS_BINS; i += RS_THREADS)
        (&sWarpHist[0][0])[i] = 0;
    __syncthreads();

    const uint32_t tile   = sTile;
    const size_t tileBase = size_t(tile) * Tile;
    const size_t warpBase = tileBase + size_t(warp) * Items * 32;

    K k[Items];
    uint32_t v[Items];
#pragma unroll
    for (int j = 0; j < Items; ++j)
    {
        size_t idx = warpBase + j * 32 + lane;
        if (idx < n)
        {
            k[j] = keysIn[idx];
            v[j] = Iota ? uint32_t(idx) : valsIn[idx];
        }
        else
        {
            k[j] = ~K(0); // padding ranks after every real key in the last digit bucket, lands at positions >= n
            v[j] = 0;
        }
    }

    // rank within the warp's 512-key sub-tile, in input order
    uint32_t rank[Items];
    const unsigned ltMask = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < Items; ++j)
    {
        uint32_t d      = digitOf(k[j], shift, mask);
        unsigned peers  = __match_any_sync(0xffffffffu, d);
        int leader      = 31 - __clz(peers);
        uint32_t before = __popc(peers & ltMask);
        uint32_t base   = sWarpHist[warp][d];
        __syncwarp();
        if (lane == leader) sWarpHist[warp][d] = base + __popc(peers);
        __syncwarp();
        rank[j] = base + before;
    }
    __syncthreads();

    // per digit (one thread per digit): tile total and per-warp exclusive prefixes
    const uint32_t dg = tid;
    uint32_t total    = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w)
    {
        uint32_t c        = sWarpHist[w][dg];
        sWarpHist[w][dg]  = total;
        total            += c;
    }
    volatile uint32_t* vstatus = status;
    size_t myIdx               = size_t(tile) * RS_BINS + dg;
    if (tile == 0) { vstatus[myIdx] = ST_INC | total; }
    else { vstatus[myIdx] = ST_AGG | total; }

    uint32_t excl = blockExclusiveScan256(total, sWarpSums);
    sTileOff[dg]  = excl;

    // decoupled look-back for this digit
    uint32_t prefix = 0;
    if (tile > 0)
    {
        // four predecessors per round (independent loads), consumed in order down to the first inclusive entry;
        // an unpublished entry ends the round and is read again. Below tile 0 reads as an empty inclusive entry.
        constexpr int LB = 4;
        long t          = long(tile) - 1;
        uint32_t spins  = 0;
        bool timedOut   = false;
        while (true)
        {
            uint32_t st[LB];
#pragma unroll
            for (int u = 0; u < LB; ++u)
                st[u] = t - u >= 0 ? uint32_t(vstatus[size_t(t - u) * RS_BINS + dg]) : uint32_t(ST_INC);
            // test mode: tile 1 waits for an entry that is never published, until the spin limit
            if (stallTile1 && tile == 1) st[0] = 0;
            int used  = 0;
            bool done = false, wait = false;
#pragma unroll
            for (int u = 0; u < LB; ++u)
            {
                if (done || wait) continue;
                if ((st[u] & ST_FLAGS) == 0)
                {
                    wait = true;
                    continue;
                }
                prefix += st[u] & ST_COUNT;
                used++;
                if (st[u] & ST_INC) done = true;
            }
            if (done) break;
            t -= used;
            if (wait)
            {
                if (++spins > spinLimit)
                {
                    timedOut = true;
                    break;
                }
                __nanosleep(20);
            }
        }
        if (timedOut) atomicOr(errWord, ERRBIT_SORT_TIMEOUT);
        vstatus[myIdx] = ST_INC | (prefix + total);
    }
    sGlobalBase[dg] = passHist[dg] + prefix;
    __syncthreads();

    // scatter into shared memory in (digit, input order) order
#pragma unroll
    for (int j = 0; j < Items; ++j)
    {
        uint32_t d   = digitOf(k[j], shift, mask);
        uint32_t pos = sTileOff[d] + sWarpHist[warp][d] + rank[j];
        sKeys[pos]   = k[j];
        sVals[pos]   = v[j];
    }
    __syncthreads();

    // coalesced write-out: consecutive shared slots of one digit go to consecutive global positions
#pragma unroll 4
    for (int i = tid; i < Tile; i += RS_THREADS)
    {
        K key      = sKeys[i];
        uint32_t d = digitOf(key, shift, mask);
        size_t out = size_t(sGlobalBase[d]) + (i - sTileOff[d]);
        if (out < n)
        {
            keysOut[out] = key;
            valsOut[out] = sVals[i];
        }
    }
}

__global__ void iotaKernel(uint32_t* v, size_t n)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) v[i] = uint32_t(i);
}

// exclusive scan of each pass's 256-bin histogram, in place (one block per pass)
__global__ void histScanKernel(uint32_t* hist)
{
    __shared__ uint32_t sWarpSums[RS_WARPS];
    uint32_t* h = hist + size_t(blockIdx.x) * RS_BINS;
    uint32_t v  = h[threadIdx.x];
    uint32_t e  = blockExclusiveScan256(v, sWarpSums);
    h[threadIdx.x] = e;
}

// the onesweep passes with one tile shape (Items keys per thread, MinBlocks resident blocks per SM); on return kin /
// vin point at the buffers holding the result
template<class K, int Items, int MinBlocks>
static int onesweepPasses(cudaStream_t s, K*& kin, uint32_t*& vin, K* keysAlt, uint32_t* valsAlt, size_t n,
                          int beginBit, int endBit, bool iota, const SortLayout& L, uint32_t* err)
{
    const size_t smemBytes = size_t(RS_THREADS) * Items * (sizeof(K) + sizeof(uint32_t));
    CSG_CUDA_TRY(cudaFuncSetAttribute(onesweepKernel<K, true, Items, MinBlocks>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(smemBytes)));
    CSG_CUDA_TRY(cudaFuncSetAttribute(onesweepKernel<K, false, Items, MinBlocks>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(smemBytes)));
    const WaitLimits wl = waitLimits();
    const int stall     = (wl.stall & CS_WAIT_STALL_SORT) ? 1 : 0;
    K* kout             = keysAlt;
    uint32_t* vout      = valsAlt;
    for (int p = 0; p < L.passes; ++p)
    {
        int shift     = beginBit + 8 * p;
        int bitsHere  = std::min(8, endBit - shift);
        uint32_t mask = (1u << bitsHere) - 1u;
        uint32_t* st  = L.status + size_t(p) * L.tiles * RS_BINS;
        if (p == 0 && iota)
            onesweepKernel<K, true, Items, MinBlocks><<<unsigned(L.tiles), RS_THREADS, smemBytes, s>>>(
                kin, vin, kout, vout, n, shift, mask, L.hist + p * RS_BINS, st, L.tileCounter + p, err, wl.sortSpins,
                stall);
        else
            onesweepKernel<K, false, Items, MinBlocks><<<unsigned(L.tiles), RS_THREADS, smemBytes, s>>>(
                kin, vin, kout, vout, n, shift, mask, L.hist + p * RS_BINS, st, L.tileCounter + p, err, wl.sortSpins,
                stall);
        CSG_CHECK_LAUNCH();
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    return CS_OK;
}

template<class K>
int radixSortPairs(cudaStream_t s, K* keys, uint32_t* vals, K* keysAlt, uint32_t* valsAlt, size_t n, int beginBit,
                   int endBit, bool iota, void* ws, size_t wsBytes, uint32_t* errWord, bool* resultInAlt,
                   int sortItems)
{
    constexpr int KB = 8 * sizeof(K);
    if (beginBit < 0 || endBit > KB || beginBit > endBit)
    {
        setLastError("sort: invalid bit range [%d, %d)", beginBit, endBit);
        return CS_ERR_INVALID;
    }
    if (n >= (size_t(1) << 30))
    {
        setLastError("sort: n = %zu exceeds the 2^30 limit", n);
        return CS_ERR_INVALID;
    }
    if (resultInAlt) *resultInAlt = false;
    if (n == 0) return CS_OK;
    int passes = numPasses(beginBit, endBit);
    if (passes == 0 || n == 1)
    {
        // nothing to reorder; the values still become 0..n-1 when asked for
        if (iota)
        {
            iotaKernel<<<iceil(n, 256), 256, 0, s>>>(vals, n);
            CSG_CHECK_LAUNCH();
        }
        return CS_OK;
    }

    if (sortItems != 0 && sortItems != 12 && sortItems != 16)
    {
        setLastError("sort: keys per thread must be 12 or 16 (0: the default, 16)");
        return CS_ERR_INVALID;
    }
    Arena a{static_cast<char*>(ws), 0, wsBytes};
    SortLayout L = sortLayout<K>(a, n, beginBit, endBit, RS_THREADS * (sortItems == 12 ? 12 : 16));
    if (!a.ok())
    {
        setLastError("sort: workspace too small");
        return CS_ERR_INVALID;
    }
    if (!errWord)
    {
        setLastError("sort: internal error word missing");
        return CS_ERR_INVALID;
    }
    uint32_t* err = errWord;

    size_t zeroBytes = (reinterpret_cast<char*>(L.status + size_t(L.passes) * L.tiles * RS_BINS) -
                        reinterpret_cast<char*>(L.hist));
    CSG_CUDA_TRY(cudaMemsetAsync(L.hist, 0, zeroBytes, s));

    {
        unsigned grid = unsigned(std::min<size_t>((n + 255) / 256, size_t(smCount()) * 8));
        radixHistogramKernel<K><<<grid, 256, 0, s>>>(keys, n, beginBit, endBit, passes, L.hist);
        CSG_CHECK_LAUNCH();
        histScanKernel<<<passes, RS_BINS, 0, s>>>(L.hist);
        CSG_CHECK_LAUNCH();
    }

    K* kin        = keys;
    uint32_t* vin = vals;
    int rc        = sortItems == 12
                        ? onesweepPasses<K, 12, 4>(s, kin, vin, keysAlt, valsAlt, n, beginBit, endBit, iota, L, err)
                        : onesweepPasses<K, 16, 3>(s, kin, vin, keysAlt, valsAlt, n, beginBit, endBit, iota, L, err);
    if (rc) return rc;
    bool inAlt = (kin == keysAlt);
    if (resultInAlt) { *resultInAlt = inAlt; }
    else if (inAlt)
    {
        CSG_CUDA_TRY(cudaMemcpyAsync(keys, keysAlt, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
        CSG_CUDA_TRY(cudaMemcpyAsync(vals, valsAlt, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
    return CS_OK;
}

template<class K>
int radixSortPreload()
{
    cudaFuncAttributes fa;
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, radixHistogramKernel<K>));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, histScanKernel));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, iotaKernel));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, onesweepKernel<K, true, 16, 3>));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, onesweepKernel<K, false, 16, 3>));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, onesweepKernel<K, true, 12, 4>));
    CSG_CUDA_TRY(cudaFuncGetAttributes(&fa, onesweepKernel<K, false, 12, 4>));
    return CS_OK;
}

template int radixSortPreload<uint32_t>();
template int radixSortPreload<uint64_t>();
template size_t radixSortWorkspaceBytes<uint32_t>(size_t, int, int);
template size_t radixSortWorkspaceBytes<uint64_t>(size_t, int, int);
template int radixSortPairs<uint32_t>(cudaStream_t, uint32_t*, uint32_t*, uint32_t*, uint32_t*, size_t, int, int, bool,
                                      void*, size_t, uint32_t*, bool*, int);
template int radixSortPairs<uint64_t>(cudaStream_t, uint64_t*, uint32_t*, uint64_t*, uint32_t*, size_t, int, int, bool,
                                      void*, size_t, uint32_t*, bool*, int);

} // namespace csg

using namespace csg;

extern "C" size_t cs_sort_pairs_workspace_bytes(size_t n, int key_bits)
{
    size_t b = key_bits == 32 ? radixSortWorkspaceBytes<uint32_t>(n, 0, 32) : radixSortWorkspaceBytes<uint64_t>(n, 0, 64);
    return b + 512; // + error word
}

template<class K>
static int sortEntry(cs_stream_t stream, K* keys, uint32_t* values, size_t n, K* keysAlt, uint32_t* valuesAlt,
                     int beginBit, int endBit, int iota, void* ws, size_t wsBytes)
{
    if (n == 0) return CS_OK;
    if (!keys || !values || !keysAlt || !valuesAlt)
    {
        setLastError("sort: null pointer");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    size_t need    = radixSortWorkspaceBytes<K>(n, beginBit, endBit) + 512;
    Workspace w;
    int rc = w.acquire(ws, wsBytes, need, s);
    if (rc) return rc;
    char* base     = static_cast<char*>(w.ptr);
    uint32_t* err  = reinterpret_cast<uint32_t*>(base + need - 256);
    CSG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    rc = radixSortPairs<K>(s, keys, values, keysAlt, valuesAlt, n, beginBit, endBit, iota != 0, base, need - 512, err,
                           nullptr);
    if (rc) return rc;
    // the reference's sortByKey synchronises the stream on return (primitives/primitives_gpu.h:152); so does this
    uint32_t herr = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr)
    {
        setLastError("sort: a look-back wait timed out");
        return CS_ERR_TIMEOUT;
    }
    return CS_OK;
}

extern "C" int cs_sort_pairs_u32(cs_stream_t stream, uint32_t* keys, uint32_t* values, size_t n, uint32_t* keys_alt,
                                 uint32_t* values_alt, int begin_bit, int end_bit, int iota, void* ws, size_t wsb)
{
    return sortEntry<uint32_t>(stream, keys, values, n, keys_alt, values_alt, begin_bit, end_bit, iota, ws, wsb);
}
extern "C" int cs_sort_pairs_u64(cs_stream_t stream, uint64_t* keys, uint32_t* values, size_t n, uint64_t* keys_alt,
                                 uint32_t* values_alt, int begin_bit, int end_bit, int iota, void* ws, size_t wsb)
{
    return sortEntry<uint64_t>(stream, keys, values, n, keys_alt, values_alt, begin_bit, end_bit, iota, ws, wsb);
}
