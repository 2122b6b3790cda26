// k_light.cu — Renderer::LightCachesRSM (renderer.cpp:899-933) /
// cacheLightingRSM.comp:80-374: per cache, gather every VPL of every light into
// RGB spherical harmonics, with the voxel cone-traced indirect shadow of
// cacheLightingRSM.comp:167-232.
//
// GB300 layout: a persistent grid (a multiple of the SM count) walks 64-cache
// tiles up to the device-side cache count (no indirect dispatch, so the launch
// is graph-capturable); VPL tiles of 64 (48 B each) and their shadow-cone
// sources are staged in shared memory once per CTA and broadcast to every
// thread; all lights accumulate in registers and the entry is read-modify-
// written once (`+=`, as the reference's per-light dispatches do).
#include <cmath>

#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

constexpr int kThreads = 64;  // LIGHTING_THREADS_PER_GROUP
constexpr int kVplTile = 64;

struct LightParams {
  LightLaunch ll;
  float vol_min[3];
  float voxel_size;
  int N;
  int max_level;
  const uint32_t* bits;
  const float* mips;
  size_t mip_off[kMaxVoxelLevels];
  int sh2;
  int shadow;
  int max_steps;
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  float* entries;
  int stride_floats;
  float ev[5];  // ShEvaFactor0, 1, 2n2_p1_n1, 20, 2p2 (renderer.cpp:302-306)
};

__device__ __forceinline__ float voxel0(const LightParams& p, int x, int y, int z) {
  size_t i = ((size_t)z * p.N + y) * p.N + x;
  return (float)((__ldg(p.bits + (i >> 5)) >> (i & 31)) & 1u);
}

// LINEAR sampling of one level with CLAMP_TO_EDGE (GL 4.5 §8.14.2).
__device__ float trilinear(const LightParams& p, int level, float sx, float sy, float sz) {
  const int n = p.N >> level;
  float ux = sx * n - 0.5f, uy = sy * n - 0.5f, uz = sz * n - 0.5f;
  float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
  float ax = ux - fx, ay = uy - fy, az = uz - fz;
  int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
  int xs[2] = {min(max(x0, 0), n - 1), min(max(x0 + 1, 0), n - 1)};
  int ys[2] = {min(max(y0, 0), n - 1), min(max(y0 + 1, 0), n - 1)};
  int zs[2] = {min(max(z0, 0), n - 1), min(max(z0 + 1, 0), n - 1)};
  float t[8];
  if (level == 0) {
#pragma unroll
    for (int k = 0; k < 8; ++k) t[k] = voxel0(p, xs[k & 1], ys[(k >> 1) & 1], zs[k >> 2]);
  } else {
    const float* m = p.mips + p.mip_off[level];
#pragma unroll
    for (int k = 0; k < 8; ++k) t[k] = __ldg(m + ((size_t)zs[k >> 2] * n + ys[(k >> 1) & 1]) * n + xs[k & 1]);
  }
  float c00 = t[0] + (t[1] - t[0]) * ax, c10 = t[2] + (t[3] - t[2]) * ax;
  float c01 = t[4] + (t[5] - t[4]) * ax, c11 = t[6] + (t[7] - t[6]) * ax;
  float c0 = c00 + (c10 - c00) * ay, c1 = c01 + (c11 - c01) * ay;
  return c0 + (c1 - c0) * az;
}

// textureLod with LINEAR_MIPMAP_LINEAR / LINEAR mag: lod <= 0 magnifies level 0.
__device__ __forceinline__ float sample_voxels(const LightParams& p, float sx, float sy, float sz, float lod) {
  if (!(lod > 0.0f)) return trilinear(p, 0, sx, sy, sz);
  if (lod >= (float)p.max_level) return trilinear(p, p.max_level, sx, sy, sz);
  float fl = floorf(lod);
  int d1 = (int)fl;
  float fr = lod - fl;
  float t1 = trilinear(p, d1, sx, sy, sz);
  if (fr == 0.0f) return t1;
  float t2 = trilinear(p, d1 + 1, sx, sy, sz);
  return (1.0f - fr) * t1 + fr * t2;
}

// cacheLightingRSM.comp:195-230.
__device__ float cone_shadow(const LightParams& p, f3 cache_pos, f3 voxel_pos, f3 avg, float dsr) {
  f3 to = avg - cache_pos;
  float light_dist = sqrtf(dot3(to, to));
  to = to * (1.0f / light_dist);
  const float inv_n = 1.0f / (float)p.N;
  f3 dir = to * inv_n;
  f3 cur = voxel_pos + dir * 2.0f;
  float occlusion = 0.0f, step = 1.0f, dist = 0.0f;
  const float goal = light_dist / p.voxel_size - 2.0f;
  const float k = 2.0f / (1.0f - dsr);
  for (int s = 0; s < p.max_steps; ++s) {
    cur = cur + dir * step;
    dist += step;
    float radius = dist * dsr;
    float occ = sample_voxels(p, cur.x, cur.y, cur.z, __log2f(radius));
    occlusion += (1.0f - occlusion) * occ;
    if (dist >= goal) break;
    step = fmaxf(1.0f, radius * k);
  }
  return sat(1.0f - occlusion);
}

__global__ void __launch_bounds__(kThreads) light_kernel(LightParams p) {
  __shared__ float4 s_vpl[kVplTile * 3];
  __shared__ float4 s_cone[kVplTile];
  const uint32_t count = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  const uint32_t n_tiles = (count + kThreads - 1) / kThreads;
  for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const uint32_t idx = tile * kThreads + threadIdx.x;
    const bool active = idx < count;
    f3 cp = mkf3(0.f, 0.f, 0.f);
    if (active) cp = ldf3(p.entries + (size_t)idx * p.stride_floats);
    const f3 voxel_pos = mkf3((cp.x - p.vol_min[0]) / (p.voxel_size * p.N), (cp.y - p.vol_min[1]) / (p.voxel_size * p.N),
                              (cp.z - p.vol_min[2]) / (p.voxel_size * p.N));
    float acc[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) acc[k] = 0.0f;
    for (int l = 0; l < p.ll.n_lights; ++l) {
      const LightArgs la = p.ll.lights[l];
      float shadowing = 1.0f;
      for (int base = 0; base < la.n_vpls; base += kVplTile) {
        __syncthreads();
        const int nt = min(kVplTile, la.n_vpls - base);
        const float4* src = reinterpret_cast<const float4*>(la.vpls + base);
        for (int i = threadIdx.x; i < nt * 3; i += kThreads) s_vpl[i] = __ldg(src + i);
        if (p.shadow) {
          const int c0 = base / la.interval, c1 = (base + nt - 1) / la.interval;
          for (int i = threadIdx.x; i <= c1 - c0; i += kThreads)
            s_cone[i] = __ldg(reinterpret_cast<const float4*>(la.cones) + c0 + i);
        }
        __syncthreads();
        const int c0 = base / la.interval;
        for (int j = 0; j < nt; ++j) {
          if (p.shadow && (base + j) % la.interval == 0) {
            float4 c = s_cone[(base + j) / la.interval - c0];
            shadowing = cone_shadow(p, cp, voxel_pos, mkf3(c.x, c.y, c.z), c.w);
          }
          const float4 a = s_vpl[3 * j], b = s_vpl[3 * j + 1], n = s_vpl[3 * j + 2];
          // a = {flux.rgb, area}, b = {position, 0}, n = {normal, 0}
          f3 to = mkf3(b.x, b.y, b.z) - cp;
          float d2 = dot3(to, to);
          to = to * rsqrtf(d2);
          float f = sat(-(n.x * to.x + n.y * to.y + n.z * to.z)) * shadowing;
          float s = f / (d2 + a.w);
          const float L[3] = {a.x * s, a.y * s, a.z * s};
          const float b0 = p.ev[0], b1y = p.ev[1] * to.y, b1z = p.ev[1] * to.z, b1x = p.ev[1] * to.x;
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            acc[0 * 3 + ch] += b0 * L[ch];
            acc[1 * 3 + ch] -= b1y * L[ch];
            acc[2 * 3 + ch] += b1z * L[ch];
            acc[3 * 3 + ch] -= b1x * L[ch];
          }
          if (p.sh2) {
            const float b4 = p.ev[2] * to.x * to.y, b5 = p.ev[2] * to.y * to.z;
            const float b6 = p.ev[3] * (to.z * to.z * 3.0f - 1.0f), b7 = p.ev[2] * to.x * to.z;
            const float b8 = p.ev[4] * (to.x * to.x - to.y * to.y);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
              acc[4 * 3 + ch] -= b4 * L[ch];
              acc[5 * 3 + ch] += b5 * L[ch];
              acc[6 * 3 + ch] += b6 * L[ch];
              acc[7 * 3 + ch] += b7 * L[ch];
              acc[8 * 3 + ch] += b8 * L[ch];
            }
          }
        }
      }
    }
    if (active) {
      float* e = p.entries + (size_t)idx * p.stride_floats;
      const int nk = p.sh2 ? 9 : 4;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        if (k < nk)
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) e[sh_offset(k, ch)] += acc[k * 3 + ch];
    }
  }
}

}  // namespace

cudaError_t launch_light_caches(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                                const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                                const uint32_t* bits, const float* mips, const size_t* mip_offsets, int num_sms) {
  LightParams p;
  p.ll = ll;
  for (int i = 0; i < 3; ++i) p.vol_min[i] = vol.volume_world_min[i];
  p.voxel_size = vol.voxel_size_in_world;
  p.N = cfg.voxel_res;
  int L = 0;
  while ((1 << (L + 1)) <= cfg.voxel_res) ++L;
  p.max_level = L;
  p.bits = bits;
  p.mips = mips;
  for (int i = 0; i < kMaxVoxelLevels; ++i) p.mip_off[i] = mip_offsets[i];
  p.sh2 = cfg.sh_order == 2;
  p.shadow = cfg.indirect_shadow;
  p.max_steps = cfg.max_cone_steps;
  p.counter = counter;
  p.max_caches = cfg.max_caches;
  p.entries = (float*)entries;
  p.stride_floats = (int)(entry_stride / 4);
  const double kPi = 3.14159265358979323846;
  p.ev[0] = (float)(1.0 / (2.0 * std::sqrt(kPi)));
  p.ev[1] = (float)(std::sqrt(3.0) / (2.0 * std::sqrt(kPi)));
  p.ev[2] = (float)std::sqrt(15.0 / (4.0 * kPi));
  p.ev[3] = (float)std::sqrt(5.0 / (16.0 * kPi));
  p.ev[4] = (float)std::sqrt(15.0 / (16.0 * kPi));
  int blocks_per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, light_kernel, kThreads, 0);
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  light_kernel<<<num_sms * blocks_per_sm, kThreads, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace drv
