// drv_device.cuh — device helpers shared by the sm_103a kernels.
//
// Functions marked "binary32 mirror" round every operation separately
// (__fmul_rn/__fadd_rn/__fdiv_rn, never contracted to FMA) in a fixed order:
// the integer decisions they feed (which cache cell a pixel lands in, which
// cascade it picks, which voxels a face covers) are part of the bit-exact
// contract of the allocation and voxelization stages.
#pragma once

#include <cmath>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/drv.h"
#include "f32x2.cuh"

namespace drv {

// utils.glsl:1 — the shaders' PI literal.
#define DRV_SHADER_PI 3.14159265358979f

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mkf3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 normalize3(f3 a) { return a * rsqrtf(dot3(a, a)); }
__device__ __forceinline__ float sat(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
__device__ __forceinline__ f3 ldf3(const float* p) { return {p[0], p[1], p[2]}; }


// ---- binary32 mirrors ------------------------------------------------------
// M-row * (x, y, z, 1), left to right.
__device__ __forceinline__ float mrow(const float* r, float x, float y, float z) {
  float a = __fmul_rn(r[0], x);
  float b = __fmul_rn(r[1], y);
  float s = __fadd_rn(a, b);
  float c = __fmul_rn(r[2], z);
  s = __fadd_rn(s, c);
  return __fadd_rn(s, r[3]);
}

// World position of the pixel at NDC (nx, ny) from its depth.
__device__ __forceinline__ void reconstruct_world_ndc(const DrvPerFrame& f, float nx, float ny, float depth,
                                                      float out[3]) {
  const float* M = f.inverse_view_projection;
  float X = mrow(M + 0, nx, ny, depth);
  float Y = mrow(M + 4, nx, ny, depth);
  float Z = mrow(M + 8, nx, ny, depth);
  float W = mrow(M + 12, nx, ny, depth);
  out[0] = __fdiv_rn(X, W);
  out[1] = __fdiv_rn(Y, W);
  out[2] = __fdiv_rn(Z, W);
}

// World position of pixel (px, py) from its depth (cacheGather.comp:113-119,
// cacheApply.frag:310-311).
__device__ __forceinline__ void reconstruct_world(const DrvPerFrame& f, int px, int py, int w, int h, float depth,
                                                  float out[3]) {
  float sx = __fadd_rn((float)px, 0.5f);
  float sy = __fadd_rn((float)py, 0.5f);
  float nx = __fdiv_rn(sx, (float)w);
  float ny = __fdiv_rn(sy, (float)h);
  nx = __fsub_rn(__fmul_rn(nx, 2.0f), 1.0f);
  ny = __fsub_rn(__fmul_rn(ny, 2.0f), 1.0f);
  const float* M = f.inverse_view_projection;
  float X = mrow(M + 0, nx, ny, depth);
  float Y = mrow(M + 4, nx, ny, depth);
  float Z = mrow(M + 8, nx, ny, depth);
  float W = mrow(M + 12, nx, ny, depth);
  out[0] = __fdiv_rn(X, W);
  out[1] = __fdiv_rn(Y, W);
  out[2] = __fdiv_rn(Z, W);
}

// ComputeAddressVolumeCascade, lightcache.glsl:109-122.
__device__ __forceinline__ int select_cascade(const DrvVolumeInfo& v, int n_cascades, const float p[3]) {
  int c = 0;
  for (; c < n_cascades - 1; ++c) {
    const DrvCascade& k = v.cascades[c];
    bool inside = p[0] <= k.decision_max[0] && p[1] <= k.decision_max[1] && p[2] <= k.decision_max[2] &&
                  p[0] >= k.decision_min[0] && p[1] >= k.decision_min[1] && p[2] >= k.decision_min[2];
    if (inside) break;
  }
  return c;
}

// ComputeAddressVolumeCascadeTransition, lightcache.glsl:125-134.
__device__ __forceinline__ float cascade_transition(const DrvVolumeInfo& v, int c, const float p[3]) {
  const DrvCascade& k = v.cascades[c];
  float a0 = __fsub_rn(k.decision_max[0], p[0]), a1 = __fsub_rn(k.decision_max[1], p[1]),
        a2 = __fsub_rn(k.decision_max[2], p[2]);
  float b0 = __fsub_rn(p[0], k.decision_min[0]), b1 = __fsub_rn(p[1], k.decision_min[1]),
        b2 = __fsub_rn(p[2], k.decision_min[2]);
  float m = fminf(fminf(fminf(a0, a1), a2), fminf(fminf(b0, b1), b2));
  float denom = __fmul_rn(k.world_voxel_size, v.cav_transition_zone_size);
  float t = __fsub_rn(1.0f, __fdiv_rn(m, denom));
  return fminf(fmaxf(t, 0.0f), 1.0f);
}

// clamp(ivec3(v), 0, res - 1), ivec3 truncating toward zero.
__device__ __forceinline__ int trunc_clamp(float v, int res) {
  if (!(v > 0.0f)) return 0;
  if (v >= (float)(res - 1)) return res - 1;
  return __float2int_rz(v);
}

// GetCache1DCoord, cacheGather.comp:20-30.
__device__ __forceinline__ int cache_1d_coord(const DrvVolumeInfo& v, int res, int c, const float p[3]) {
  const DrvCascade& k = v.cascades[c];
  int ix = trunc_clamp(__fdiv_rn(__fsub_rn(p[0], k.min[0]), k.world_voxel_size), res);
  int iy = trunc_clamp(__fdiv_rn(__fsub_rn(p[1], k.min[1]), k.world_voxel_size), res);
  int iz = trunc_clamp(__fdiv_rn(__fsub_rn(p[2], k.min[2]), k.world_voxel_size), res);
  return ix + iy * res + iz * res * res + c * res * res * res;
}

// Exact reciprocals of the divisors of the cascade arithmetic: where a
// cascade's cell size (or cell size x transition zone) is a power of two,
// x / d = x * (1 / d) exactly in binary32 (both are exact scalings), so the
// IEEE division can become one product; 0 marks a divisor that is not.
struct CellRecip {
  float inv_cell[DRV_MAX_CASCADES];
  float inv_zone[DRV_MAX_CASCADES];
};

// Host: 1 / d when d is a normal power of two (then exact), else 0.
inline float exact_reciprocal(float d) {
  int e = 0;
  const float m = frexpf(d, &e);
  return (m == 0.5f && e > -125 && e < 127) ? ldexpf(1.0f, 1 - e) : 0.0f;
}

inline CellRecip make_cell_recip(const DrvVolumeInfo& v) {
  CellRecip r{};
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) {
    const float d = v.cascades[c].world_voxel_size;
    r.inv_cell[c] = exact_reciprocal(d);
    const float zone = d * v.cav_transition_zone_size;  // the kernels' __fmul_rn of the same floats
    r.inv_zone[c] = exact_reciprocal(zone);
  }
  return r;
}

__device__ __forceinline__ float div_exact(float x, float d, float inv) {
  return inv != 0.0f ? __fmul_rn(x, inv) : __fdiv_rn(x, d);
}

__device__ __forceinline__ float cascade_transition(const DrvVolumeInfo& v, const CellRecip& r, int c,
                                                   const float p[3]) {
  const DrvCascade& k = v.cascades[c];
  float a0 = __fsub_rn(k.decision_max[0], p[0]), a1 = __fsub_rn(k.decision_max[1], p[1]),
        a2 = __fsub_rn(k.decision_max[2], p[2]);
  float b0 = __fsub_rn(p[0], k.decision_min[0]), b1 = __fsub_rn(p[1], k.decision_min[1]),
        b2 = __fsub_rn(p[2], k.decision_min[2]);
  float m = fminf(fminf(fminf(a0, a1), a2), fminf(fminf(b0, b1), b2));
  float denom = __fmul_rn(k.world_voxel_size, v.cav_transition_zone_size);
  float t = __fsub_rn(1.0f, div_exact(m, denom, r.inv_zone[c]));
  return fminf(fmaxf(t, 0.0f), 1.0f);
}

__device__ __forceinline__ int cache_1d_coord(const DrvVolumeInfo& v, const CellRecip& r, int res, int c,
                                              const float p[3]) {
  const DrvCascade& k = v.cascades[c];
  const float inv = r.inv_cell[c];
  int ix = trunc_clamp(div_exact(__fsub_rn(p[0], k.min[0]), k.world_voxel_size, inv), res);
  int iy = trunc_clamp(div_exact(__fsub_rn(p[1], k.min[1]), k.world_voxel_size, inv), res);
  int iz = trunc_clamp(div_exact(__fsub_rn(p[2], k.min[2]), k.world_voxel_size, inv), res);
  return ix + iy * res + iz * res * res + c * res * res * res;
}

// G-buffer diffuse of pixel i (drv_albedo_format): linear F32 RGB, or SRGB8
// bytes decoded through `srgb` (the GL decode of the 256 byte values).
__device__ __forceinline__ f3 load_albedo(const void* albedo, int format, const float* srgb, size_t i) {
  if (format == DRV_ALBEDO_SRGB8) {
    const uint8_t* a = static_cast<const uint8_t*>(albedo) + 3 * i;
    return mkf3(__ldg(srgb + __ldcs(a)), __ldg(srgb + __ldcs(a + 1)), __ldg(srgb + __ldcs(a + 2)));
  }
  const float* a = static_cast<const float*>(albedo) + 3 * i;
  return mkf3(__ldcs(a), __ldcs(a + 1), __ldcs(a + 2));
}

// ---- normal packing (utils.glsl:44-89) ----------------------------------
// Saturating conversion to int16 (GL leaves out-of-range integer writes
// undefined); the scale is applied as (x / PI) * 32768 so axis-aligned
// normals pack exactly.
__device__ __forceinline__ void pack_normal16i(f3 n, int16_t out[2]) {
  float px = n.x == 0.0f ? (float)((n.y > 0.0f) - (n.y < 0.0f)) * (DRV_SHADER_PI / 2.0f) : atan2f(n.y, n.x);
  float vx = truncf(__fmul_rn(__fdiv_rn(px, DRV_SHADER_PI), 32768.0f));
  float vy = truncf(__fmul_rn(n.z, 32768.0f));
  if (vx != vx) vx = 0.0f;
  if (vy != vy) vy = 0.0f;
  out[0] = (int16_t)fmaxf(-32768.0f, fminf(32767.0f, vx));
  out[1] = (int16_t)fmaxf(-32768.0f, fminf(32767.0f, vy));
}

__device__ __forceinline__ f3 unpack_normal16i(int16_t a, int16_t b) {
  float px = (float)a * (DRV_SHADER_PI / 32768.0f);
  float py = (float)b * (1.0f / 32768.0f);
  float sin_phi = sqrtf(1.0f - py * py);
  float s, c;
  sincosf(px, &s, &c);
  return normalize3(mkf3(c * sin_phi, s * sin_phi, py));
}

// cacheLightingRSM.comp:46-62.
__device__ __forceinline__ void morton_decode(uint32_t m, uint32_t& x, uint32_t& y) {
  uint32_t c0 = m, c1 = m >> 1;
  c0 &= 0x55555555u;
  c1 &= 0x55555555u;
  c0 = (c0 | (c0 >> 1)) & 0x33333333u;
  c1 = (c1 | (c1 >> 1)) & 0x33333333u;
  c0 = (c0 | (c0 >> 2)) & 0x0f0f0f0fu;
  c1 = (c1 | (c1 >> 2)) & 0x0f0f0f0fu;
  c0 = (c0 | (c0 >> 4)) & 0x00ff00ffu;
  c1 = (c1 | (c1 >> 4)) & 0x00ff00ffu;
  c0 = (c0 | (c0 >> 8)) & 0x0000ffffu;
  c1 = (c1 | (c1 >> 8)) & 0x0000ffffu;
  x = c0;
  y = c1;
}

// Float offsets of the SH fields inside a LightCacheEntry (lightcache.glsl:33-58),
// indexed by coefficient k (0 SH00, 1 SH1neg1, 2 SH10, 3 SH1pos1, 4 SH2neg2,
// 5 SH2neg1, 6 SH20, 7 SH2pos1, 8 SH2pos2) and channel.
__device__ __forceinline__ int sh_offset(int k, int ch) {
  switch (k) {
    case 0: return 7 + 4 * ch;
    case 1: return 4 + ch;
    case 2: return 8 + ch;
    case 3: return 12 + ch;
    case 4: return 16 + ch;
    case 5: return 20 + ch;
    case 6: return 19 + 4 * ch;
    case 7: return 24 + ch;
    default: return 28 + ch;
  }
}

// BF16 <-> FP32 (round to nearest even) as raw 16-bit storage.
__device__ __forceinline__ uint16_t to_bf16(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float from_bf16(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// Cell key of a BF16 cache entry: cascade-local corner coordinates (0..256,
// 9 bits each) + cascade.
__device__ __forceinline__ uint32_t pack_cell(int x, int y, int z, int c) {
  return (uint32_t)x | (uint32_t)y << 9 | (uint32_t)z << 18 | (uint32_t)c << 27;
}

// Atomic OR of device error bits.
__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bits) { atomicOr(err, bits); }

// Cull record of a VPL as the light stage stores it (normal n, position p,
// flux positive or not): the plane {n, -n . p + eps (1 + |p|_inf)}, or -inf in
// w when it has no flux (no cache can see it). A cache c passes when
// n . c + w > -eps |c|_inf (k_light.cu, cull_records_kernel).
constexpr float kCullRecordEps = 1e-5f;
__device__ __forceinline__ float4 make_cull_record(float nx, float ny, float nz, float px, float py, float pz,
                                                   bool flux) {
  const float pm = fmaxf(fmaxf(fabsf(px), fabsf(py)), fabsf(pz));
  return make_float4(nx, ny, nz, flux ? -(nx * px + ny * py + nz * pz) + kCullRecordEps * (1.0f + pm) : -INFINITY);
}

}  // namespace drv
