// Internal interface of the stable LSD radix sort (radix_sort.cu).
#pragma once
#include "cs_common.cuh"

namespace csg
{

// device status word bits reported by the sort (OR-ed into the caller's error word)
constexpr uint32_t ERRBIT_SORT_TIMEOUT = 1u;

template<class K>
size_t radixSortWorkspaceBytes(size_t n, int beginBit, int endBit);

/*! Stable sort of (keys, vals) by bits [beginBit, endBit) of the keys.
 *  keysAlt/valsAlt are ping-pong buffers. If `resultInAlt` is non-null the result stays in whichever buffer the last
 *  pass wrote and *resultInAlt tells which; otherwise it is copied back into keys/vals.
 *  `errWord` (device, may be null) receives ERRBIT_SORT_TIMEOUT if a look-back wait gave up. No host sync.
 *  `iota` replaces the input values by 0..n-1. `sortItems` picks the tile shape: 16 keys per thread with 3 blocks per
 *  SM (0, the default) or 12 keys per thread with 4 blocks; the result does not depend on it. */
template<class K>
int radixSortPairs(cudaStream_t s, K* keys, uint32_t* vals, K* keysAlt, uint32_t* valsAlt, size_t n, int beginBit,
                   int endBit, bool iota, void* ws, size_t wsBytes, uint32_t* errWord, bool* resultInAlt,
                   int sortItems = 0);

/*! Loads the sort's kernels on the current device (cudaFuncGetAttributes), so that with lazy module loading the
 *  first sort does not load them. */
template<class K>
int radixSortPreload();

} // namespace csg
