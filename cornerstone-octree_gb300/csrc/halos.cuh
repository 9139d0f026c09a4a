// Internal interface of halo discovery (halos.cu).
#pragma once
#include "cs_common.cuh"

namespace csg
{

//! Th: the type of h (T, or float with T = double as computeBoundingBoxGpu<double, float>). phi (may be null, used
//! with T = double): the coordinates rounded to nearest float as float4 (x, y, z, -), the neighbour search's shadows
//! of the same particles, read by the FP32 screen instead of estimates made from the doubles
template<class T, class Th>
int searchBoxes(cudaStream_t s, const T* x, const T* y, const T* z, const Th* h, const uint32_t* layout, int first,
                int last, Th scale, const int32_t* l2i, const T* nodeCenters, T* sc, T* ss,
                const float4* phi = nullptr);

//! nrec (may be null): the neighbour search's float node records (NbPrep::nrec: centre and half size rounded to
//! nearest at [3i] and [3i + 2]); with T = double and no periodic axis they enable the float pre-filter of the node
//! test. scratch (may be null): (last - first + 2) int32 of device memory for the list of leaves that need a
//! traversal; with it the traversals run on persistent warps over that list
template<class K, class T>
int findHalos(cudaStream_t s, const K* prefixes, const int32_t* childOffsets, const int32_t* parents, const T* nc,
              const T* ns, const K* leaves, const T* sc, const T* ss, const cs_box& box, int first, int last,
              uint8_t* flags, uint32_t* errWord, const float4* nrec, int32_t* scratch = nullptr);

} // namespace csg
