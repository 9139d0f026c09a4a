// Stable key sort that allocates no device memory.
//
// Some callers cannot allocate device memory at the point where they need a sort: a simulation code that reserves
// all device memory up front in its own pool (so cudaMalloc / cudaMallocAsync would fail or fragment it), or a
// time-step loop that must not pay the implicit device-wide synchronisation of cudaMalloc/cudaFree. For them,
// cs_sort_pairs_noalloc_u64 runs the same onesweep radix sort as cs_sort_pairs_u64, but takes every temporary
// buffer (ping-pong key/value copies, digit histograms, look-back status words, the error word) from one
// file-scope device array of fixed size. The array exists once per device that loads this library and stays
// allocated until the process exits.
//
// Limits and rules:
//  - at most CS_SORT_NOALLOC_MAX_N keys per call; larger calls are rejected with CS_ERR_INVALID;
//  - every call uses the same array, so two calls that overlap on the GPU (different streams, or different host
//    threads on the same device) race and corrupt each other: serialise them;
//  - the first call on a device looks up the array's device address (cudaGetSymbolAddress) with that device
//    current and caches it; make that first call before capturing any stream into a graph;
//  - the parts of the array that must start at zero are cleared by every call with cudaMemsetAsync.
#include "cs_common.cuh"
#include "radix_sort.cuh"

#include <mutex>

namespace csg
{
namespace
{

constexpr size_t NOALLOC_MAX_N = CS_SORT_NOALLOC_MAX_N;
// alt keys + alt values + error words + sort workspace (histograms, tile counters, status words) for MAX_N keys,
// with room for the 256-byte alignment of each piece
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_MAX_N * (sizeof(uint64_t) + sizeof(uint32_t)) + (1u << 20);

static __device__ __align__(256) unsigned char g_sortScratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static void* g_scratchAddr[NOALLOC_MAX_DEVICES] = {};
static std::mutex g_scratchMutex;

// device address of g_sortScratch on the current device (looked up once per device)
int scratchAddress(void** out)
{
    int dev = 0;
    CSG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    {
        setLastError("sort (no-alloc): device ordinal %d not supported", dev);
        return CS_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddr[dev])
    {
        void* p          = nullptr;
        cudaError_t err_ = cudaGetSymbolAddress(&p, g_sortScratch);
        if (err_ != cudaSuccess || p == nullptr)
        {
            setLastError("sort (no-alloc): cudaGetSymbolAddress failed: %s", cudaGetErrorString(err_));
            return CS_ERR_CUDA;
        }
        g_scratchAddr[dev] = p;
    }
    *out = g_scratchAddr[dev];
    return CS_OK;
}

} // namespace
} // namespace csg

using namespace csg;

extern "C" int cs_sort_pairs_noalloc_u64(cs_stream_t stream, uint64_t* keys, uint32_t* values, size_t n,
                                         int begin_bit, int end_bit, int values_are_iota)
{
    if (n > NOALLOC_MAX_N)
    {
        setLastError("sort (no-alloc): n = %zu exceeds the fixed scratch limit of %zu keys", n, NOALLOC_MAX_N);
        return CS_ERR_INVALID;
    }
    if (n == 0) return CS_OK;
    if (!keys || !values)
    {
        setLastError("sort (no-alloc): null pointer");
        return CS_ERR_INVALID;
    }
    cudaStream_t s = cudaStream_t(stream);
    void* base     = nullptr;
    int rc         = scratchAddress(&base);
    if (rc) return rc;

    Arena a{static_cast<char*>(base), 0, NOALLOC_SCRATCH_BYTES};
    uint64_t* keysAlt   = a.take<uint64_t>(n);
    uint32_t* valuesAlt = a.take<uint32_t>(n);
    uint32_t* err       = a.take<uint32_t>(64);
    size_t wsBytes      = radixSortWorkspaceBytes<uint64_t>(n, begin_bit, end_bit);
    void* ws            = a.take<char>(wsBytes);
    if (!a.ok())
    {
        setLastError("sort (no-alloc): internal scratch layout exceeds %zu bytes", NOALLOC_SCRATCH_BYTES);
        return CS_ERR_INVALID;
    }
    // the error word starts at zero; the sort clears its own histograms, tile counters and status words
    CSG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    rc = radixSortPairs<uint64_t>(s, keys, values, keysAlt, valuesAlt, n, begin_bit, end_bit, values_are_iota != 0,
                                  ws, wsBytes, err, nullptr);
    if (rc) return rc;
    uint32_t herr = 0;
    CSG_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr)
    {
        setLastError("sort (no-alloc): a look-back wait timed out");
        return CS_ERR_TIMEOUT;
    }
    return CS_OK;
}
