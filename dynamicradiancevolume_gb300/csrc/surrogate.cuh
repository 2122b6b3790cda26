// surrogate.cuh — the learned visibility surrogate that stands in for the
// indirect-shadow cone (cacheLightingRSM.comp:167-232): its input features,
// parameter layout and activation, shared by the pair generator, the trainer
// and the inference kernel.
//
// MLP: 32 inputs -> 64 -> 64 -> 64 -> 2, GELU (tanh form) between layers.
// Output 0 is the visibility logit (visibility = sigmoid), output 1 the
// confidence logit: pairs whose sigmoid(confidence) is below the threshold
// are re-traced with the cone.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "drv_device.cuh"
#include "voxel_sample.cuh"

namespace drv {

constexpr int kMlpIn = 32;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2;
constexpr int kMlpOutPad = 8;  // layer-4 rows padded to one n8 MMA tile
constexpr int kFeatures = 27;  // used inputs; the rest are zero

// Parameter offsets (floats) of the flat FP32 master copy; weights are
// [out][in] row-major (in contiguous), biases follow each weight matrix.
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden * kMlpHidden;
constexpr int kOffW4 = kOffB3 + kMlpHidden;
constexpr int kOffB4 = kOffW4 + kMlpOut * kMlpHidden;
constexpr int kMlpParams = kOffB4 + kMlpOut;  // 10562

// GELU, tanh approximation: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
__device__ __forceinline__ float gelu(float x) {
  const float u = 0.7978845608f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float u = 0.7978845608f * (x + 0.044715f * x2 * x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * 0.7978845608f * (1.0f + 3.0f * 0.044715f * x2);
}
__device__ __forceinline__ float sigmoidf(float x) { return 1.0f / (1.0f + __expf(-x)); }

// GELU for inference: the same tanh form with the hardware tanh
// approximation (MUFU.TANH), as the BF16 activations it feeds tolerate.
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_fast(float x) {
  const float u = 0.7978845608f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanh_fast(u));
}

// Two FP32 values -> bf16x2 (lo in the low half), round to nearest even.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// GELU of the inference MLP on two BF16 values at once, in bf16x2
// arithmetic with the hardware tanh: 0.5 x (1 + tanh(x (c0 + c1 x^2))) with
// c0 = sqrt(2/pi), c1 = 0.044715 c0 rounded to BF16 (0x3F4C, 0x3D12). The
// activations it produces are stored as BF16 anyway, and the error of BF16
// arithmetic here is of the order of that rounding.
__device__ __forceinline__ uint32_t gelu_bf16x2(uint32_t x) {
  uint32_t y;
  asm("{\n"
      ".reg .b32 x2, u, t, h;\n"
      "mul.rn.bf16x2 x2, %1, %1;\n"
      "fma.rn.bf16x2 u, x2, %2, %3;\n"
      "mul.rn.bf16x2 u, u, %1;\n"
      "tanh.approx.bf16x2 t, u;\n"
      "mul.rn.bf16x2 h, %1, %4;\n"
      "fma.rn.bf16x2 %0, h, t, h;\n"
      "}"
      : "=r"(y)
      : "r"(x), "r"(0x3D123D12u), "r"(0x3F4C3F4Cu), "r"(0x3F003F00u));
  return y;
}

// Distance (in voxels) the cone of cacheLightingRSM.comp:195-228 reaches
// before it stops: min(goal, the distance after max_steps steps). The step
// rule is stepSize = max(1, dist * dsr * 2 / (1 - dsr)); it is evaluated here
// in closed form (unit steps, then geometric growth), which is enough for a
// feature.
__device__ __forceinline__ float cone_reach(float goal, float dsr, int max_steps) {
  const float g = dsr * 2.0f / (1.0f - dsr);  // growth per step once steps exceed one voxel
  float dist = 0.0f;
  int s = 0;
  // unit steps while dist * g < 1
  const float unit_until = g > 0.0f ? 1.0f / g : 1e30f;
  const int n_unit = min(max_steps, (int)ceilf(fmaxf(unit_until, 0.0f)) + 1);
  dist = (float)n_unit;
  s = n_unit;
  if (s < max_steps) dist *= __powf(1.0f + g, (float)(max_steps - s));
  // the march starts 2 voxels out and stops once it passes the goal
  return fminf(dist, fmaxf(goal, 0.0f)) + 2.0f;
}

// Input features of one (cache, shadow block) pair. cache/target are world
// positions, (px, py, pz) the cache in normalised volume coordinates, n the
// first VPL's normal, dsr the cone aperture:
//   0-2 cache, 3-5 cone target (normalised volume coordinates), 6-8 normal,
//   9-16 eight mip-3 opacity samples along the part of the segment the cone
//   traces, 17 aperture, 18 length, 19-21 direction, 22-25 the cone's own
//   first four samples (same positions and LOD as cacheLightingRSM.comp:
//   211-225), 26 their composited occlusion.
__device__ __forceinline__ void surrogate_features(const VoxelView& v, float inv_extent, const float vol_min[3],
                                                   float voxel_size, int max_steps, float cx, float cy, float cz,
                                                   float tx, float ty, float tz, float nx, float ny, float nz,
                                                   float dsr, float* f) {
  const float px = (cx - vol_min[0]) * inv_extent, py = (cy - vol_min[1]) * inv_extent,
              pz = (cz - vol_min[2]) * inv_extent;
  const float qx = (tx - vol_min[0]) * inv_extent, qy = (ty - vol_min[1]) * inv_extent,
              qz = (tz - vol_min[2]) * inv_extent;
  const float dx = tx - cx, dy = ty - cy, dz = tz - cz;
  const float len = sqrtf(dx * dx + dy * dy + dz * dz);
  const float inv_len = 1.0f / fmaxf(len, 1e-20f);
  const float len_vox = len / voxel_size;
  const float reach = cone_reach(len_vox - 2.0f, dsr, max_steps);  // voxels from the cache
  f[0] = px;
  f[1] = py;
  f[2] = pz;
  f[3] = qx;
  f[4] = qy;
  f[5] = qz;
  f[6] = nx;
  f[7] = ny;
  f[8] = nz;
  // 8 opacity samples of mip level 3 along the traced part of the segment.
  const float reach_norm = fminf(reach * voxel_size * inv_len, 1.0f);
  const int level = min(3, v.max_level);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float t = (i + 0.5f) * 0.125f * reach_norm;
    f[9 + i] = level_any(v, level, px + (qx - px) * t, py + (qy - py) * t, pz + (qz - pz) * t);
  }
  f[17] = dsr * 8.0f;
  f[18] = len_vox * (1.0f / 64.0f);
  f[19] = dx * inv_len;
  f[20] = dy * inv_len;
  f[21] = dz * inv_len;
  // The cone's first four steps, exactly as the tracer takes them.
  {
    const float inv_n = 1.0f / (float)v.N;
    const float sx = dx * inv_len * inv_n, sy = dy * inv_len * inv_n, sz = dz * inv_len * inv_n;
    float ux = px + sx * 2.0f, uy = py + sy * 2.0f, uz = pz + sz * 2.0f;
    float step = 1.0f, dist = 0.0f, transmit = 1.0f;
    const float k = 2.0f / (1.0f - dsr);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      ux += sx * step;
      uy += sy * step;
      uz += sz * step;
      dist += step;
      const float radius = dist * dsr;
      const float occ = (dist - step < len_vox - 2.0f) ? sample_voxels(v, ux, uy, uz, __log2f(radius)) : 0.0f;
      f[22 + s] = occ;
      transmit *= 1.0f - occ;
      step = fmaxf(1.0f, radius * k);
    }
    f[26] = 1.0f - transmit;
  }
#pragma unroll
  for (int i = kFeatures; i < kMlpIn; ++i) f[i] = 0.0f;
}

}  // namespace drv
