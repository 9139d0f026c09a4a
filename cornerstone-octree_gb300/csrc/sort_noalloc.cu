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
//  - CUDA loads modules lazily by default (CUDA_MODULE_LOADING=LAZY): the array and the sort kernels come into
//    device memory on first use. A call with n = 0 does that set-up (looks the array up with cudaGetSymbolAddress
//    and loads the kernels) without sorting; make it once per device, with that device current, before reserving
//    the memory pool. CUDA_MODULE_LOADING=EAGER loads everything when the library is loaded instead;
//  - each call reads the sort's error word back and synchronises its stream before returning, so it cannot be
//    recorded into a CUDA graph: a call made while its stream is being captured is refused with CS_ERR_INVALID;
//  - the array's address is looked up on every call (cheap next to the sort), so a device reset or a new context
//    needs nothing special;
//  - the parts of the array that must start at zero are cleared by every call with cudaMemsetAsync.
#include "cs_common.cuh"
#include "radix_sort.cuh"

namespace csg
{
namespace
{

constexpr size_t NOALLOC_MAX_N = CS_SORT_NOALLOC_MAX_N;
// alt keys + alt values + error words + sort workspace (histograms, tile counters, status words) for MAX_N keys,
// with room for the 256-byte alignment of each piece
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_MAX_N * (sizeof(uint64_t) + sizeof(uint32_t)) + (1u << 20);

static __device__ __align__(256) unsigned char g_sortScratch[NOALLOC_SCRATCH_BYTES];

// device address of g_sortScratch on the current device. In host code the name g_sortScratch is a host-side
// stand-in; only the address from cudaGetSymbolAddress may be passed to kernels.
int scratchAddress(void** out)
{
    void* p          = nullptr;
    cudaError_t err_ = cudaGetSymbolAddress(&p, g_sortScratch);
    if (err_ != cudaSuccess || p == nullptr)
    {
        setLastError("sort (no-alloc): cudaGetSymbolAddress failed: %s", cudaGetErrorString(err_));
        return CS_ERR_CUDA;
    }
    *out = p;
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
    cudaStream_t s = cudaStream_t(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CSG_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone)
    {
        setLastError("sort (no-alloc): the stream is being captured; this call synchronises its stream and cannot be "
                     "part of a CUDA graph");
        return CS_ERR_INVALID;
    }
    // set-up on every call, including n == 0 (the warm-up call): the array's address, which loads this file's
    // module and so the array itself, and the sort kernels
    void* base = nullptr;
    int rc     = scratchAddress(&base);
    if (rc) return rc;
    rc = radixSortPreload<uint64_t>();
    if (rc) return rc;
    if (n == 0) return CS_OK;
    if (!keys || !values)
    {
        setLastError("sort (no-alloc): null pointer");
        return CS_ERR_INVALID;
    }

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
