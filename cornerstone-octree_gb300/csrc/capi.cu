// Error reporting, device queries and version of the C ABI.
#include "cs_common.cuh"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

namespace csg
{

static thread_local char tlsError[512] = "";

void setLastError(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(tlsError, sizeof(tlsError), fmt, ap);
    va_end(ap);
}

int smCount()
{
    static thread_local int cachedDevice = -1;
    static thread_local int cachedCount  = 0;
    int dev                              = 0;
    cudaGetDevice(&dev);
    if (dev != cachedDevice)
    {
        int c = 0;
        cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
        cachedCount  = c > 0 ? c : 1;
        cachedDevice = dev;
    }
    return cachedCount;
}

__global__ void copyWordsKernel(const uint32_t* src, uint32_t* dst, unsigned words)
{
    for (unsigned k = threadIdx.x; k < words; k += blockDim.x)
        dst[k] = src[k];
}

int readSmallToHost(cudaStream_t s, void* hostDst, const void* devSrc, size_t bytes)
{
    constexpr size_t kMax = 4096;
    if (bytes % 4 || bytes > kMax)
    {
        setLastError("internal: small read of %zu bytes", bytes);
        return CS_ERR_INVALID;
    }
    // one staging buffer per host thread (calls on a thread are sequential: each ends with a synchronisation);
    // portable + mapped, so that kernels of any device reach it through its device address
    static thread_local uint32_t* staging = nullptr;
    static thread_local uint32_t* stagingDev = nullptr;
    if (!staging)
    {
        CSG_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&staging), kMax, cudaHostAllocPortable | cudaHostAllocMapped));
        CSG_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&stagingDev), staging, 0));
    }
    copyWordsKernel<<<1, 32, 0, s>>>(static_cast<const uint32_t*>(devSrc), stagingDev, unsigned(bytes / 4));
    CSG_CHECK_LAUNCH();
    CSG_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(hostDst, staging, bytes);
    return CS_OK;
}

// bytes [0, n) from src to dst; the 16-byte words where src and dst sit at the same offset within 16 bytes
__global__ void copyBytesKernel(const unsigned char* __restrict__ src, unsigned char* dst, size_t n)
{
    const size_t tid    = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const uintptr_t sa = reinterpret_cast<uintptr_t>(src), da = reinterpret_cast<uintptr_t>(dst);
    if ((sa & 15u) != (da & 15u))
    {
        for (size_t k = tid; k < n; k += stride)
            dst[k] = src[k];
        return;
    }
    const size_t head = min(size_t((16u - (da & 15u)) & 15u), n);
    const size_t nv   = (n - head) / 16;
    for (size_t k = tid; k < head; k += stride)
        dst[k] = src[k];
    const uint4* s4 = reinterpret_cast<const uint4*>(src + head);
    uint4* d4       = reinterpret_cast<uint4*>(dst + head);
    for (size_t v = tid; v < nv; v += stride)
        d4[v] = __ldcs(s4 + v);
    for (size_t k = head + 16 * nv + tid; k < n; k += stride)
        dst[k] = src[k];
}

int copyToHostAsync(cudaStream_t s, void* hostDst, const void* devSrc, size_t bytes)
{
    if (bytes == 0) return CS_OK;
    cudaPointerAttributes attr{};
    void* mapped = nullptr;
    if (cudaPointerGetAttributes(&attr, hostDst) == cudaSuccess)
    {
        if (attr.type == cudaMemoryTypeHost) mapped = attr.devicePointer;
    }
    else
        cudaGetLastError(); // the query's own error (a pointer the runtime does not know): fall back to the copy
    if (!mapped)
    {
        CSG_CUDA_TRY(cudaMemcpyAsync(hostDst, devSrc, bytes, cudaMemcpyDeviceToHost, s));
        return CS_OK;
    }
    // 64 blocks carry the host link's rate (about 190 GB/s) and leave the SMs to other work
    const unsigned blocks = unsigned(std::min<size_t>(64, (bytes + 4095) / 4096));
    copyBytesKernel<<<blocks, 256, 0, s>>>(static_cast<const unsigned char*>(devSrc),
                                           static_cast<unsigned char*>(mapped), bytes);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

static std::atomic<uint32_t> gSortSpins{WaitLimits{}.sortSpins};
static std::atomic<uint32_t> gBarrierSpins{WaitLimits{}.barrierSpins};
static std::atomic<int> gStall{0};

WaitLimits waitLimits()
{
    WaitLimits w;
    w.sortSpins    = gSortSpins.load();
    w.barrierSpins = gBarrierSpins.load();
    w.stall        = gStall.load();
    return w;
}

} // namespace csg

extern "C" const char* cs_last_error(void) { return csg::tlsError; }

extern "C" int cs_version(void) { return 100; }

extern "C" int cs_set_wait_limits(uint32_t sort_spins, uint32_t barrier_spins, int stall)
{
    if (stall < 0 || stall > (CS_WAIT_STALL_SORT | CS_WAIT_STALL_BARRIER))
    {
        csg::setLastError("wait limits: unknown stall mode %d", stall);
        return CS_ERR_INVALID;
    }
    const csg::WaitLimits d;
    csg::gSortSpins.store(sort_spins ? sort_spins : d.sortSpins);
    csg::gBarrierSpins.store(barrier_spins ? barrier_spins : d.barrierSpins);
    csg::gStall.store(stall);
    return CS_OK;
}
