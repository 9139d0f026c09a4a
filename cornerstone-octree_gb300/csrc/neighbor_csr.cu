// Compaction of ngmax-strided neighbour rows into a compressed sparse row (CSR) list.
//
// findNeighbors (findneighbors.hpp:156-177) writes particle i's first min(nc_i, ngmax) neighbours into row i of an
// array of n x ngmax entries; most rows are far from full (16M Plummer particles with 100 neighbours fill half of
// ngmax = 200). A caller that wants the lists in host memory copies only the stored entries: offsets[i] =
// sum_{k<i} min(nc_k, ngmax) (u64, n + 1 entries, offsets[n] = total) and list[offsets[i] .. offsets[i+1]) = row i.
//
// Three kernels: per tile of rows the sum of the stored counts; one block scans the tile sums; per tile a block scan
// gives each row's offset and the block's warps copy their rows (a null list: offsets only). Outputs may be device
// memory or pinned host memory (the kernels then write over the host link, with no host-side knowledge of the total).
// Entries past list_capacity are not written; offsets[n] always holds the total, so the caller can tell. The
// pipeline's host-buffer runs compact into device memory and copy the list to the host with the copy engine.
//
// Algorithmic bytes: reads 4 n (counts) + 4 total (stored entries), writes 8 (n + 1) + 4 total.
#include "cs_common.cuh"
#include "neighbor_csr.cuh"

namespace csg
{

constexpr int CSR_THREADS = 256;
constexpr int CSR_ROWS    = 8;                          // rows per thread in the scans
constexpr int CSR_TILE    = CSR_THREADS * CSR_ROWS;     // rows per block

__device__ __forceinline__ unsigned long long blockExclusiveScanU64(unsigned long long v, unsigned long long* sWarp,
                                                                    unsigned long long* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sWarp[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        constexpr int NW = CSR_THREADS / 32;
        unsigned long long w = lane < NW ? sWarp[lane] : 0;
#pragma unroll
        for (int o = 1; o < NW; o <<= 1)
        {
            unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NW) sWarp[lane] = w;
    }
    __syncthreads();
    unsigned long long pre = warp > 0 ? sWarp[warp - 1] : 0;
    *total                 = sWarp[CSR_THREADS / 32 - 1];
    __syncthreads();
    return pre + x - v;
}

__global__ void __launch_bounds__(CSR_THREADS) csrTileSumsKernel(const uint32_t* __restrict__ nc, size_t n,
                                                                  unsigned ngmax, unsigned long long* tileSums)
{
    __shared__ unsigned long long sWarp[CSR_THREADS / 32];
    size_t base = size_t(blockIdx.x) * CSR_TILE + size_t(threadIdx.x) * CSR_ROWS;
    unsigned long long v = 0;
#pragma unroll
    for (int k = 0; k < CSR_ROWS; ++k)
        if (base + k < n) v += min(__ldg(nc + base + k), ngmax);
    unsigned long long total;
    blockExclusiveScanU64(v, sWarp, &total);
    if (threadIdx.x == 0) tileSums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place; the grand total goes to offsets[n], and a total above the
// list capacity sets *overflow (when given)
__global__ void __launch_bounds__(CSR_THREADS) csrTileOffsetsKernel(unsigned long long* tileSums, int numTiles,
                                                                     uint64_t* offsetsN, size_t capacity,
                                                                     uint32_t* overflow)
{
    __shared__ unsigned long long sWarp[CSR_THREADS / 32];
    unsigned long long carry = 0;
    for (int b = 0; b < numTiles; b += CSR_THREADS)
    {
        int i                  = b + threadIdx.x;
        unsigned long long v   = i < numTiles ? tileSums[i] : 0;
        unsigned long long total;
        unsigned long long e = blockExclusiveScanU64(v, sWarp, &total);
        if (i < numTiles) tileSums[i] = carry + e;
        carry += total;
    }
    if (threadIdx.x == 0)
    {
        *offsetsN = carry;
        if (overflow && carry > capacity) *overflow = 1u;
    }
}

__global__ void __launch_bounds__(CSR_THREADS) csrWriteKernel(const uint32_t* __restrict__ nb,
                                                               const uint32_t* __restrict__ nc, size_t n,
                                                               unsigned ngmax,
                                                               const unsigned long long* __restrict__ tileOffsets,
                                                               uint64_t* offsets, uint32_t* list, size_t capacity)
{
    __shared__ unsigned long long sWarp[CSR_THREADS / 32];
    __shared__ unsigned long long sOff[CSR_TILE];
    __shared__ unsigned sCnt[CSR_TILE];
    const size_t tile0 = size_t(blockIdx.x) * CSR_TILE;
    const int t0       = threadIdx.x * CSR_ROWS;
    unsigned c[CSR_ROWS];
    unsigned long long sum = 0;
#pragma unroll
    for (int k = 0; k < CSR_ROWS; ++k)
    {
        size_t i = tile0 + t0 + k;
        c[k]     = i < n ? min(__ldg(nc + i), ngmax) : 0u;
        sum += c[k];
    }
    unsigned long long total;
    unsigned long long e = blockExclusiveScanU64(sum, sWarp, &total) + tileOffsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < CSR_ROWS; ++k)
    {
        sOff[t0 + k] = e;
        sCnt[t0 + k] = c[k];
        e += c[k];
    }
    __syncthreads();
    // offsets: consecutive threads write consecutive rows
    for (int r = threadIdx.x; r < CSR_TILE; r += CSR_THREADS)
    {
        size_t i = tile0 + r;
        if (i < n) offsets[i] = sOff[r];
    }
    if (!list) return; // offsets only
    // rows: warp w copies rows w, w + 8, ...; lanes copy 32 consecutive entries per round
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < CSR_TILE; r += CSR_THREADS / 32)
    {
        size_t i = tile0 + r;
        if (i >= n) break;
        const unsigned cnt           = sCnt[r];
        const unsigned long long dst = sOff[r];
        const uint32_t* src          = nb + i * size_t(ngmax);
        for (unsigned k = lane; k < cnt; k += 32)
            if (dst + k < capacity) list[dst + k] = __ldcs(src + k);
    }
}

size_t neighborCsrWorkspaceBytes(size_t n) { return ((n + CSR_TILE - 1) / CSR_TILE + 1) * 8 + 256; }

int neighborCsr(cudaStream_t s, const uint32_t* nb, const uint32_t* nc, size_t n, unsigned ngmax, uint64_t* offsets,
                uint32_t* list, size_t capacity, void* ws, size_t wsBytes, uint32_t* overflow)
{
    if (!offsets || (!nb && n) || (!nc && n) || (!list && capacity))
    {
        setLastError("neighbour csr: null pointer");
        return CS_ERR_INVALID;
    }
    if (n >= (size_t(1) << 32))
    {
        setLastError("neighbour csr: n = %zu too large", n);
        return CS_ERR_INVALID;
    }
    if (n == 0)
    {
        CSG_CUDA_TRY(cudaMemsetAsync(offsets, 0, sizeof(uint64_t), s));
        return CS_OK;
    }
    Workspace w;
    int rc = w.acquire(ws, wsBytes, neighborCsrWorkspaceBytes(n), s);
    if (rc) return rc;
    unsigned long long* tiles = static_cast<unsigned long long*>(w.ptr);
    const unsigned nt         = unsigned((n + CSR_TILE - 1) / CSR_TILE);
    csrTileSumsKernel<<<nt, CSR_THREADS, 0, s>>>(nc, n, ngmax, tiles);
    CSG_CHECK_LAUNCH();
    csrTileOffsetsKernel<<<1, CSR_THREADS, 0, s>>>(tiles, int(nt), offsets + n, capacity, overflow);
    CSG_CHECK_LAUNCH();
    csrWriteKernel<<<nt, CSR_THREADS, 0, s>>>(nb, nc, n, ngmax, tiles, offsets, list, capacity);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

} // namespace csg

using namespace csg;

extern "C" size_t cs_neighbors_csr_workspace_bytes(size_t n) { return neighborCsrWorkspaceBytes(n); }

extern "C" int cs_neighbors_csr(cs_stream_t stream, const uint32_t* neighbors, const uint32_t* neighbor_counts,
                                size_t n, unsigned ngmax, uint64_t* offsets, uint32_t* list, size_t list_capacity,
                                void* workspace, size_t workspace_bytes)
{
    return neighborCsr(cudaStream_t(stream), neighbors, neighbor_counts, n, ngmax, offsets, list, list_capacity,
                       workspace, workspace_bytes, nullptr);
}
