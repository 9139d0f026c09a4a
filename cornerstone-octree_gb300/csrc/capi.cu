// Error reporting, device queries and version of the C ABI.
#include "cs_common.cuh"

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
