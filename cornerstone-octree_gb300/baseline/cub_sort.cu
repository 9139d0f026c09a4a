// Measurement baseline, not part of the library: CUB's DeviceRadixSort::SortPairs, the sort the reference's
// sortByKey calls (primitives/primitives_gpu.cu:322-356), compiled for sm_103a so that the benchmark can time it on the
// same keys as the library's own onesweep sort. Loaded only by the benchmark's sort workload.
#include <cstddef>
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>

extern "C" size_t cub_sort_pairs_u64_temp_bytes(size_t n, int begin_bit, int end_bit)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint64_t*)nullptr, (uint64_t*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, n, begin_bit, end_bit);
    return bytes;
}

extern "C" int cub_sort_pairs_u64(void* stream, const uint64_t* keys_in, uint64_t* keys_out, const uint32_t* vals_in,
                                  uint32_t* vals_out, size_t n, int begin_bit, int end_bit, void* temp,
                                  size_t temp_bytes)
{
    cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys_out, vals_in, vals_out, n,
                                                    begin_bit, end_bit, cudaStream_t(stream));
    return e == cudaSuccess ? 0 : int(e);
}
