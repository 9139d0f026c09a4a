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

/*! dst[k] = src[k] for k < min(*totalDev, capacity) (device src; pinned host or device dst; both 4-byte aligned and
 *  at the same offset within 16 bytes, else CS_ERR_INVALID); *overflow = 1 when *totalDev > capacity (overflow may
 *  be null). No host synchronisation. */
int copyListToHost(cudaStream_t s, const uint32_t* src, uint32_t* dst, const uint64_t* totalDev, size_t capacity,
                   uint32_t* overflow);

} // namespace csg
