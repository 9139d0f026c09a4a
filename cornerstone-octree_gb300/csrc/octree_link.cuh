// Internal interface of the octree linkage and node geometry (octree_link.cu).
#pragma once
#include "cs_common.cuh"

namespace csg
{

template<class K>
size_t buildLinkWorkspaceBytes(int L);

/*! Link the internal tree of leaves[0..L] into `v`. prefixBits (0 = full key width) limits the radix sort of the
 *  placeholder prefixes to their significant bits (3 * deepest leaf level + 1). errWord: device word for sort
 *  timeouts (nullptr = internal). */
template<class K>
int buildLink(cudaStream_t s, const K* leaves, int L, const cs_octree_view& v, int prefixBits, void* ws,
              size_t wsBytes, uint32_t* errWord, const int* Ldev = nullptr);

//! with Ldev (device leaf count) L is a capacity: every launch covers it, the kernels use the device count, the
//! prefix sort runs over the capacity's node count with padding, and the host needs no synchronisation (graphs)

template<class K, class T>
int geoCenters(cudaStream_t s, const K* prefixes, int N, T* centers, T* sizes, const cs_box& box, int kind,
               const int* Ldev = nullptr);

//! node geometry of batched sets in one 64-bit tree (keys (s << 30) | 32-bit key of set s, set roots at rootLevel):
//! every node of a set's subtree gets the centre and half size its set's own 32-bit tree gives it, with the set's
//! box; paramsDev holds geoParamsBytes(numSets) of device memory
template<class T>
size_t geoParamsBytes(int numSets);
template<class T>
int geoCentersBatched(cudaStream_t s, const uint64_t* prefixes, int N, T* centers, T* sizes, const cs_box* boxes,
                      int numSets, int kind, void* paramsDev, unsigned rootLevel);

} // namespace csg
