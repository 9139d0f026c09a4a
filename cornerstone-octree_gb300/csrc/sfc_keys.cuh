// Internal interface of sfc_keys.cu (keys and gathers), used by the pipeline drivers.
#pragma once
#include "cs_common.cuh"

namespace csg
{

template<class T, class K>
int sfcKeys(cudaStream_t s, const T* x, const T* y, const T* z, K* keys, size_t n, const cs_box& box, int kind,
            bool respectRemove);

template<class T, int NA>
struct GatherArgs
{
    const T* in[NA];
    T* out[NA];
};

template<class T, int NA>
int gatherN(cudaStream_t s, const uint32_t* perm, size_t n, GatherArgs<T, NA> a);

} // namespace csg
