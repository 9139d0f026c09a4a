// Error reporting, device queries and version of the C ABI.
#include "cs_common.cuh"

#include <cstdarg>
#include <cstdio>

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
    static int cachedDevice = -1;
    static int cachedCount  = 0;
    int dev                 = 0;
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

} // namespace csg

extern "C" const char* cs_last_error(void) { return csg::tlsError; }

extern "C" int cs_version(void) { return 100; }
