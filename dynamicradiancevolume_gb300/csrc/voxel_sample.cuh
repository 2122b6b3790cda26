// voxel_sample.cuh — quadrilinear opacity lookups of the voxel pyramid on the
// GPU: textureLod(VoxelVolume, s, lod) with the LINEAR/LINEAR/LINEAR CLAMP
// sampler the reference binds for the cone trace (renderer.cpp:916-917),
// written in software (GL 4.5 §8.14: lod <= 0 magnifies level 0; otherwise
// LINEAR_MIPMAP_LINEAR between floor/ceil levels, clamped to the last level;
// texel centres at (i + 0.5) / n; CLAMP_TO_EDGE).
//
// Level 0 is read from the corner-packed byte grid: byte (x, y, z) holds the
// 8 voxels (x + dx, y + dy, z + dz), dx,dy,dz in {0,1}, with +1 clamped to the
// last voxel, stored in 4x4x4 bricks of 64 bytes, so one trilinear level-0
// sample is one byte load. Levels >= 1 are FP32 arrays (x fastest).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace drv {

struct VoxelView {
  const uint8_t* corners;  // level 0, N^3 bytes, bricked
  const void* mips;        // levels 1..L concatenated: float, or __half when half_mips
  uint32_t off[16];        // offset (floats) of level l in `mips`
  int N;                   // level-0 resolution (power of two)
  int log2n;
  int max_level;           // L = log2(N)
  int half_mips;
};

__device__ __forceinline__ float mip_texel(const VoxelView& v, uint32_t i) {
  return v.half_mips ? __half2float(__ldg(static_cast<const __half*>(v.mips) + i))
                     : __ldg(static_cast<const float*>(v.mips) + i);
}

// Byte offset of voxel (x, y, z) in the bricked level-0 corner grid.
__device__ __forceinline__ uint32_t corner_index(int x, int y, int z, int log2n) {
  const int lnb = log2n - 2;  // bricks per axis = N / 4
  uint32_t brick = ((uint32_t)((z >> 2) << lnb | (y >> 2)) << lnb) | (uint32_t)(x >> 2);
  return (brick << 6) | (uint32_t)((z & 3) << 4 | (y & 3) << 2 | (x & 3));
}

__device__ __forceinline__ float level0(const VoxelView& v, float sx, float sy, float sz) {
  const int n = v.N;
  float ux = sx * n - 0.5f, uy = sy * n - 0.5f, uz = sz * n - 0.5f;
  float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
  float ax = ux - fx, ay = uy - fy, az = uz - fz;
  int x = (int)fx, y = (int)fy, z = (int)fz;
  // Below 0 both taps clamp to voxel 0: keep the (0) corner only. At or above
  // n-1 both taps clamp to voxel n-1, which the packed byte already repeats.
  if (x < 0) { x = 0; ax = 0.0f; }
  if (y < 0) { y = 0; ay = 0.0f; }
  if (z < 0) { z = 0; az = 0.0f; }
  x = min(x, n - 1);
  y = min(y, n - 1);
  z = min(z, n - 1);
  const uint32_t b = __ldg(v.corners + corner_index(x, y, z, v.log2n));
  // Trilinear weights sum to one, so eight equal corners give that value
  // exactly: empty space (the common case) costs no interpolation.
  if (b == 0u) return 0.0f;
  if (b == 0xFFu) return 1.0f;
  const float t0 = (float)(b & 1u), t1 = (float)((b >> 1) & 1u), t2 = (float)((b >> 2) & 1u),
              t3 = (float)((b >> 3) & 1u), t4 = (float)((b >> 4) & 1u), t5 = (float)((b >> 5) & 1u),
              t6 = (float)((b >> 6) & 1u), t7 = (float)((b >> 7) & 1u);
  float c00 = t0 + (t1 - t0) * ax, c10 = t2 + (t3 - t2) * ax;
  float c01 = t4 + (t5 - t4) * ax, c11 = t6 + (t7 - t6) * ax;
  float c0 = c00 + (c10 - c00) * ay, c1 = c01 + (c11 - c01) * ay;
  return c0 + (c1 - c0) * az;
}

__device__ __forceinline__ float level_n(const VoxelView& v, int level, float sx, float sy, float sz) {
  const int ln = v.log2n - level, n = 1 << ln;
  float ux = sx * n - 0.5f, uy = sy * n - 0.5f, uz = sz * n - 0.5f;
  float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
  float ax = ux - fx, ay = uy - fy, az = uz - fz;
  int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
  const int xa = min(max(x0, 0), n - 1), xb = min(max(x0 + 1, 0), n - 1);
  const int ya = min(max(y0, 0), n - 1) << ln, yb = min(max(y0 + 1, 0), n - 1) << ln;
  const int za = min(max(z0, 0), n - 1) << (2 * ln), zb = min(max(z0 + 1, 0), n - 1) << (2 * ln);
  const uint32_t m = v.off[level];
  float t0 = mip_texel(v, m + (za | ya | xa)), t1 = mip_texel(v, m + (za | ya | xb));
  float t2 = mip_texel(v, m + (za | yb | xa)), t3 = mip_texel(v, m + (za | yb | xb));
  float t4 = mip_texel(v, m + (zb | ya | xa)), t5 = mip_texel(v, m + (zb | ya | xb));
  float t6 = mip_texel(v, m + (zb | yb | xa)), t7 = mip_texel(v, m + (zb | yb | xb));
  float c00 = t0 + (t1 - t0) * ax, c10 = t2 + (t3 - t2) * ax;
  float c01 = t4 + (t5 - t4) * ax, c11 = t6 + (t7 - t6) * ax;
  float c0 = c00 + (c10 - c00) * ay, c1 = c01 + (c11 - c01) * ay;
  return c0 + (c1 - c0) * az;
}

__device__ __forceinline__ float sample_voxels(const VoxelView& v, float sx, float sy, float sz, float lod) {
  if (!(lod > 0.0f)) return level0(v, sx, sy, sz);
  if (lod >= (float)v.max_level) return level_n(v, v.max_level, sx, sy, sz);
  const float fl = floorf(lod);
  const int d1 = (int)fl;
  const float fr = lod - fl;
  const float t1 = d1 == 0 ? level0(v, sx, sy, sz) : level_n(v, d1, sx, sy, sz);
  if (fr == 0.0f) return t1;
  const float t2 = level_n(v, d1 + 1, sx, sy, sz);
  return (1.0f - fr) * t1 + fr * t2;
}

// Indirect-shadow cone, cacheLightingRSM.comp:195-230: march from the cache
// toward the block's average VAL position, growing the sample sphere with the
// distance, front-to-back occlusion, at most max_steps samples. Once the
// occlusion reaches 1 a further step gives occlusion * (1 - s) + s >= 1 for
// any sample s in [0, 1], so the clamped result is 0 (to within one rounding)
// whatever is sampled: the march stops there (the reference marches on).
__device__ __forceinline__ float cone_shadow(const VoxelView& v, float voxel_size, int max_steps, float cx, float cy,
                                             float cz, float px, float py, float pz, float ax, float ay, float az,
                                             float dsr) {
  float tx = ax - cx, ty = ay - cy, tz = az - cz;
  const float light_dist = sqrtf(tx * tx + ty * ty + tz * tz);
  const float inv = 1.0f / light_dist;
  const float inv_n = 1.0f / (float)v.N;
  const float dx = tx * inv * inv_n, dy = ty * inv * inv_n, dz = tz * inv * inv_n;
  float qx = px + dx * 2.0f, qy = py + dy * 2.0f, qz = pz + dz * 2.0f;
  float occlusion = 0.0f, step = 1.0f, dist = 0.0f;
  const float goal = light_dist / voxel_size - 2.0f;
  const float k = 2.0f / (1.0f - dsr);
  for (int s = 0; s < max_steps; ++s) {
    qx += dx * step;
    qy += dy * step;
    qz += dz * step;
    dist += step;
    const float radius = dist * dsr;
    occlusion += (1.0f - occlusion) * sample_voxels(v, qx, qy, qz, __log2f(radius));
    if (dist >= goal || occlusion >= 1.0f) break;
    step = fmaxf(1.0f, radius * k);
  }
  return fminf(fmaxf(1.0f - occlusion, 0.0f), 1.0f);
}

}  // namespace drv
