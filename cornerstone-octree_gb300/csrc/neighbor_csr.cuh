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

/*! Entries of the tile table that gatherListToHost needs for a list buffer of `capacity` entries. */
size_t listTileCount(size_t capacity);

/*! tileRows[k] = the row holding the first entry of output tile k (for the destination dst, whose alignment sets
 *  the tiles), from the offsets of neighborCsr (device). No host synchronisation. */
int listTileRows(cudaStream_t s, const uint64_t* offsets, size_t n, const uint32_t* dst, uint32_t* tileRows,
                 size_t maxTiles);

/*! dst[q] = the q-th stored entry of the ngmax-strided rows nb, for q < min(offsets[n], capacity) (dst: pinned host
 *  or device memory, 4-byte aligned); *overflow = 1 when offsets[n] > capacity (overflow may be null). Reads the
 *  offsets and tile table from device memory: no host synchronisation. */
int gatherListToHost(cudaStream_t s, const uint32_t* nb, unsigned ngmax, const uint64_t* offsets, size_t n,
                     uint32_t* dst, size_t capacity, const uint32_t* tileRows, size_t maxTiles, uint32_t* overflow);

} // namespace csg
