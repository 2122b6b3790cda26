// k_checks.cu — the input scan of DrvTuning.check_inputs: a grid-stride pass
// over a float (or half) input that latches DRV_DEVERR_NUMERIC in the
// context's input-check word when any value is NaN or infinite. It stands in
// for a memory / value checker on inputs the reference reads unchecked (a NaN
// depth or flux would spread through its caches silently).
#include <cuda_fp16.h>

#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

__device__ __forceinline__ bool finite_bits(uint32_t b) { return (b & 0x7F800000u) != 0x7F800000u; }
__device__ __forceinline__ bool finite_half_bits(uint32_t h) { return (h & 0x7C00u) != 0x7C00u; }

__global__ void __launch_bounds__(256) scan_finite_kernel(const uint32_t* __restrict__ words, size_t n_words,
                                                          int half, uint32_t* word) {
  bool bad = false;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t w = __ldcs(words + i);
    bad |= half ? !(finite_half_bits(w) && finite_half_bits(w >> 16)) : !finite_bits(w);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) raise_error(word, DRV_DEVERR_NUMERIC);
}

// The last half of an odd-length half array (not covered by the word pass).
__global__ void scan_last_half_kernel(const uint16_t* __restrict__ h, uint32_t* word) {
  if (!((*h & 0x7C00u) != 0x7C00u)) raise_error(word, DRV_DEVERR_NUMERIC);
}

}  // namespace

cudaError_t launch_scan_finite(cudaStream_t s, const void* data, size_t n, int half, uint32_t* word) {
  if (n == 0) return cudaSuccess;
  // a half array is read as words of two halves (its base is 2-byte aligned:
  // an odd start is read half by half through the tail kernel instead)
  const uint32_t* w = static_cast<const uint32_t*>(data);
  size_t n_words = half ? n / 2 : n;
  const bool odd_base = half && (reinterpret_cast<uintptr_t>(data) & 3u);
  if (odd_base) {
    // first half alone, then the rest from the next 4-byte boundary
    scan_last_half_kernel<<<1, 1, 0, s>>>(static_cast<const uint16_t*>(data), word);
    w = reinterpret_cast<const uint32_t*>(static_cast<const uint16_t*>(data) + 1);
    n_words = (n - 1) / 2;
    if ((n - 1) % 2) scan_last_half_kernel<<<1, 1, 0, s>>>(static_cast<const uint16_t*>(data) + n - 1, word);
  } else if (half && n % 2) {
    scan_last_half_kernel<<<1, 1, 0, s>>>(static_cast<const uint16_t*>(data) + n - 1, word);
  }
  if (n_words) {
    const size_t blocks = (n_words + 255) / 256;
    scan_finite_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(w, n_words, half, word);
  }
  return cudaGetLastError();
}

}  // namespace drv
