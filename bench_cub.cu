// Same-box comparator for bench.py only: NVIDIA CUB's DeviceRadixSort (the
// CCCL that ships with the CUDA toolkit) on the benchmark's key-value input.
// Nothing in the library links or calls this; bench.py compiles it on first
// use and reports its time beside the library's, for information.
#include <cub/device/device_radix_sort.cuh>
#include <cstdint>

extern "C" int bench_cub_sort_pairs_u32(void* temp, size_t* temp_bytes, const uint32_t* keys_in,
  uint32_t* keys_out, const uint32_t* vals_in, uint32_t* vals_out, int64_t count, void* stream) {
  return (int)cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, keys_in, keys_out, vals_in,
    vals_out, count, 0, 32, (cudaStream_t)stream);
}
