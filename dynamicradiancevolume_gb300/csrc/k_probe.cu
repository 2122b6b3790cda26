// k_probe.cu — load throughput of this GPU's L1 and L2, the denominators of
// the cone pass's memory roofline (its voxel pyramid lives in L1/L2, not in
// HBM). No counterpart in the reference.
//
// L1: every CTA re-reads its own 32 KB window with 16-byte read-only loads
// (two CTAs per SM: 64 KB per SM, well inside L1), so after the first pass
// every load hits L1. L2: all CTAs sweep the caller's buffer with 16-byte
// loads that bypass L1 (ld.global.cg); a buffer that fits in L2 makes every
// load after the first sweep an L2 hit. Each thread folds what it reads into
// one word that it writes only if it matches a value no input produces, so
// the loads cannot be dropped.
#include "drv_internal.h"

namespace {

constexpr int kL1Threads = 512;
constexpr int kL1WindowVec = 32 * 1024 / 16;  // uint4 per 32 KB window

__global__ void __launch_bounds__(kL1Threads) l1_sweep_kernel(const uint4* __restrict__ buf, int reps,
                                                              uint32_t* sink) {
  const uint4* w = buf + (size_t)blockIdx.x * kL1WindowVec;
  uint32_t acc = 0;
  for (int r = 0; r < reps; ++r) {
    // each pass starts at another offset of the window (and depends on the
    // previous pass), so no pass's loads can be reused for another
    const int rot = (int)((acc & 1u) + (uint32_t)r * 97u) & (kL1WindowVec - 1);
#pragma unroll 4
    for (int i = threadIdx.x; i < kL1WindowVec; i += kL1Threads) {
      const uint4 q = __ldg(w + ((i + rot) & (kL1WindowVec - 1)));
      acc ^= q.x ^ q.y ^ q.z ^ q.w;
    }
    acc = acc * 2654435761u + (uint32_t)r;
  }
  if (acc == 0x9E3779B9u) sink[blockIdx.x * kL1Threads + threadIdx.x] = acc;
}

__global__ void __launch_bounds__(256) l2_sweep_kernel(const uint4* __restrict__ buf, size_t n_vec, int reps,
                                                       uint32_t* sink) {
  uint32_t acc = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r) {
    const size_t rot = ((size_t)(acc & 1u) + (size_t)r * 4099u) % n_vec;
#pragma unroll 4
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_vec; i += stride) {
      size_t j = i + rot;
      if (j >= n_vec) j -= n_vec;
      const uint4 q = __ldcg(buf + j);
      acc ^= q.x ^ q.y ^ q.z ^ q.w;
    }
    acc = acc * 2654435761u + (uint32_t)r;
  }
  if (acc == 0x9E3779B9u) sink[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace

extern "C" drv_status drv_measure_load_bandwidth(int32_t level, const void* buffer, size_t bytes, int32_t reps,
                                                 void* cuda_stream, float* out_gbs) {
  if (!buffer || !out_gbs || reps < 1 || (level != 1 && level != 2) || ((uintptr_t)buffer & 15u)) return DRV_ERR_INVALID_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return DRV_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const uint4* buf = static_cast<const uint4*>(buffer);
  // The sink is the buffer itself: nothing is ever written (see the file header).
  uint32_t* sink = static_cast<uint32_t*>(const_cast<void*>(buffer));
  int blocks = 0;
  double loaded = 0.0;
  if (level == 1) {
    blocks = 2 * sms;
    if (bytes < (size_t)blocks * kL1WindowVec * 16) return DRV_ERR_INVALID_ARG;
    loaded = (double)blocks * kL1WindowVec * 16.0 * reps;
  } else {
    blocks = 4 * sms;
    if (bytes < (size_t)blocks * 256 * 16) return DRV_ERR_INVALID_ARG;
    loaded = (double)(bytes / 16) * 16.0 * reps;
  }
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return DRV_ERR_CUDA;
  auto launch = [&](int r) {
    if (level == 1)
      l1_sweep_kernel<<<blocks, kL1Threads, 0, s>>>(buf, r, sink);
    else
      l2_sweep_kernel<<<blocks, 256, 0, s>>>(buf, bytes / 16, r, sink);
  };
  launch(1);  // warm: brings the windows into L1 / the buffer into L2
  cudaEventRecord(a, s);
  launch(reps);
  cudaEventRecord(b, s);
  float ms = 0.0f;
  cudaError_t e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess || !(ms > 0.0f)) return DRV_ERR_CUDA;
  *out_gbs = (float)(loaded / (ms * 1e-3) / 1e9);
  return DRV_OK;
}
