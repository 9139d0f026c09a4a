// Internal interface of the neighbour-list compaction (neighbor_csr.cu).
#pragma once
#include "cs_common.cuh"

namespace csg
{

size_t neighborCsrWorkspaceBytes(size_t n);

/*! offsets[i] = sum_{k<i} min(nc[k], ngmax) for i <= n (offsets[n] = total), list[offsets[i] + j] = nb[i * ngmax + j]
 *  for j < min(nc[i], ngmax), entries at or past `capacity` skipped (and *overflow = 1 when overflow is given).
 *  Outputs may be device or pinned host memory. */
int neighborCsr(cudaStream_t s, const uint32_t* nb, const uint32_t* nc, size_t n, unsigned ngmax, uint64_t* offsets,
                uint32_t* list, size_t capacity, void* ws, size_t wsBytes, uint32_t* overflow);

} // namespace csg
