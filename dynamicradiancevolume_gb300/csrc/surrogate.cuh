// surrogate.cuh — the learned visibility surrogate that stands in for the
// indirect-shadow cone (cacheLightingRSM.comp:167-232): its input features,
// parameter layout and activation, shared by the pair generator, the trainer
// and the inference kernel.
//
// MLP: 32 inputs -> 64 -> 64 -> 64 -> 2, GELU between layers in its
// sigmoid form x sigmoid(1.702 x) (Hendrycks & Gimpel 2016, section 2).
// Output 0 is the visibility logit (visibility = sigmoid), output 1 the
// confidence logit: pairs whose sigmoid(confidence) is below the threshold
// are re-traced with the cone. Input 31 is the constant 1 (it carries the
// first layer's bias on the tensor cores).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "drv_device.cuh"
#include "voxel_sample.cuh"

namespace drv {

constexpr int kMlpIn = 32;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2;
constexpr int kOneInput = kMlpIn - 1;  // the constant-1 input

// Feature sets (DRV_SURROGATE_FEATURES_*): the configuration's 17 inputs
// (cache, VPL position and normal, eight mip-3 opacities along the segment),
// or 27 inputs that add the cone's aperture, length, direction and its own
// first four samples.
constexpr int kFeatureSegment8 = 0;
constexpr int kFeatureCone4 = 1;
constexpr int kFeatureCone8 = 2;

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

// GELU, sigmoid form, and its derivative (training, FP32).
constexpr float kGeluK = 1.702f;
__device__ __forceinline__ float sigmoidf(float x) { return 1.0f / (1.0f + __expf(-x)); }
__device__ __forceinline__ float gelu(float x) { return x * sigmoidf(kGeluK * x); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float s = sigmoidf(kGeluK * x);
  return s + kGeluK * x * s * (1.0f - s);
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
  for (int i = 27; i < kOneInput; ++i) f[i] = 0.0f;
  f[kOneInput] = 1.0f;
}

// The configuration's 17 inputs of one (cache, shadow block) pair: 0-2 the
// cache and 3-5 the block's cone target (the VPL position) in normalised
// volume coordinates, 6-8 the VPL normal, 9-16 eight trilinear opacity
// samples of mip level 3 at the midpoints of eight equal parts of the
// segment from the cache to the target; 31 the constant 1.
__device__ __forceinline__ void segment_features(const VoxelView& v, float inv_extent, const float vol_min[3],
                                                 float cx, float cy, float cz, float tx, float ty, float tz, float nx,
                                                 float ny, float nz, float* f) {
  const float px = (cx - vol_min[0]) * inv_extent, py = (cy - vol_min[1]) * inv_extent,
              pz = (cz - vol_min[2]) * inv_extent;
  const float qx = (tx - vol_min[0]) * inv_extent, qy = (ty - vol_min[1]) * inv_extent,
              qz = (tz - vol_min[2]) * inv_extent;
  f[0] = px;
  f[1] = py;
  f[2] = pz;
  f[3] = qx;
  f[4] = qy;
  f[5] = qz;
  f[6] = nx;
  f[7] = ny;
  f[8] = nz;
  const int level = min(3, v.max_level);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float t = (i + 0.5f) * 0.125f;
    f[9 + i] = level_any(v, level, px + (qx - px) * t, py + (qy - py) * t, pz + (qz - pz) * t);
  }
#pragma unroll
  for (int i = 17; i < kOneInput; ++i) f[i] = 0.0f;
  f[kOneInput] = 1.0f;
}

// Inputs 0-8 as segment_features, then eight samples of the cone's own
// sampler (textureLod at the cone's level of detail, cacheLightingRSM.comp:
// 216-221) at marched distances goal^((j + 1) / 8), j = 0..7 (geometric, as
// the cone's steps grow), 17 their composited occlusion 1 - prod(1 - s),
// 18 the aperture (x 8), 19 the march length in voxels (/ 64), 20-22 the
// direction; 31 the constant 1.
__device__ __forceinline__ void cone8_features(const VoxelView& v, float inv_extent, const float vol_min[3],
                                               float voxel_size, float cx, float cy, float cz, float tx, float ty,
                                               float tz, float nx, float ny, float nz, float dsr, float* f) {
  const float px = (cx - vol_min[0]) * inv_extent, py = (cy - vol_min[1]) * inv_extent,
              pz = (cz - vol_min[2]) * inv_extent;
  const float qx = (tx - vol_min[0]) * inv_extent, qy = (ty - vol_min[1]) * inv_extent,
              qz = (tz - vol_min[2]) * inv_extent;
  f[0] = px;
  f[1] = py;
  f[2] = pz;
  f[3] = qx;
  f[4] = qy;
  f[5] = qz;
  f[6] = nx;
  f[7] = ny;
  f[8] = nz;
  const float dx = tx - cx, dy = ty - cy, dz = tz - cz;
  const float len = sqrtf(dx * dx + dy * dy + dz * dz);
  const float inv_len = 1.0f / fmaxf(len, 1e-20f);
  const float Dx = dx * inv_len, Dy = dy * inv_len, Dz = dz * inv_len;
  const float goal = fmaxf(len / voxel_size - 2.0f, 1.0f);  // voxels the cone marches
  const Coord P = voxel_pos(v, px, py, pz);
  const float lg = __log2f(goal) * 0.125f;
  float transmit = 1.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float d = exp2f(lg * (float)(j + 1));  // marched distance
    const float at = 2.0f + d;                   // from the cache: the march starts 2 voxels out
    const Coord U{P.x + Dx * at, P.y + Dy * at, P.z + Dz * at};
    const float s = sample_voxels_at(v, U, __log2f(d * dsr));
    f[9 + j] = s;
    transmit *= 1.0f - s;
  }
  f[17] = 1.0f - transmit;
  f[18] = dsr * 8.0f;
  f[19] = goal * (1.0f / 64.0f);
  f[20] = Dx;
  f[21] = Dy;
  f[22] = Dz;
#pragma unroll
  for (int i = 23; i < kOneInput; ++i) f[i] = 0.0f;
  f[kOneInput] = 1.0f;
}

// Features of a pair in feature set FS.
template <int FS>
__device__ __forceinline__ void pair_features(const VoxelView& v, float inv_extent, const float vol_min[3],
                                              float voxel_size, int max_steps, float cx, float cy, float cz,
                                              float tx, float ty, float tz, float nx, float ny, float nz, float dsr,
                                              float* f) {
  if (FS == kFeatureSegment8)
    segment_features(v, inv_extent, vol_min, cx, cy, cz, tx, ty, tz, nx, ny, nz, f);
  else if (FS == kFeatureCone8)
    cone8_features(v, inv_extent, vol_min, voxel_size, cx, cy, cz, tx, ty, tz, nx, ny, nz, dsr, f);
  else
    surrogate_features(v, inv_extent, vol_min, voxel_size, max_steps, cx, cy, cz, tx, ty, tz, nx, ny, nz, dsr, f);
}

}  // namespace drv
