// k_light.cu — Renderer::LightCachesRSM (renderer.cpp:899-933) /
// cacheLightingRSM.comp:80-374: per cache, gather every VPL of every light
// into RGB spherical harmonics, with the voxel cone-traced indirect shadow of
// cacheLightingRSM.comp:167-232.
//
// Work decomposition (the reference runs one thread per cache and loops over
// all VPLs; a frame has only a few thousand caches, too few to fill 152 SMs):
//  - the shadow blocks of all lights (IndirectShadowComputationSampleInterval
//    consecutive VPLs share one cone) form one index space, cut into
//    `n_chunks` chunks;
//  - a unit of work is (cache, chunk) and belongs to one warp; a persistent
//    grid walks the units up to the device-side cache count (no indirect
//    dispatch: graph-capturable), and warps never wait for each other;
//  - inside a unit, the 32 lanes take blocks round-robin: every lane's cone
//    starts at the same cache, so the first steps of all 32 cones of a warp
//    fetch the same voxel bytes;
//  - the warp reduces its 27 partial SH sums with shuffles; with several
//    chunks, partials go to a scratch slot per unit and the last warp to
//    finish a cache (a ticket counter per cache) adds them in chunk order, so
//    results do not depend on scheduling, then resets the ticket;
//  - the entry's SH is read-modify-written once (`+=`, as the reference's
//    per-light dispatches accumulate).
#include <cmath>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "voxel_sample.cuh"

namespace drv {
namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

struct LightParams {
  LightLaunch ll;
  float casc_min[DRV_MAX_CASCADES][3];  // for BF16 entries: position = cell * size + min (cacheGather.comp:65)
  float casc_cell[DRV_MAX_CASCADES];
  int block_base[DRV_MAX_LIGHTS + 1];  // prefix sum of shadow blocks per light
  int total_blocks;
  int n_chunks;
  int chunk_blocks;
  VoxelView vox;
  float vol_min[3];
  float voxel_size;
  int shadow;
  int max_steps;
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  float* entries;
  int stride_floats;
  float* scratch;     // [max_caches * n_chunks][27] partial sums
  uint32_t* tickets;  // [max_caches], zero between frames
  float ev[5];        // ShEvaFactor0, 1, 2n2_p1_n1, 20, 2p2 (renderer.cpp:302-306)
};

struct VplData {
  float px, py, pz, area, fr, fg, fb, nx, ny, nz;
};

template <bool BF16>
__device__ __forceinline__ VplData load_vpl(const void* base, int i) {
  VplData d;
  if (BF16) {
    const uint4* q = reinterpret_cast<const uint4*>(static_cast<const DrvVPLBF16*>(base) + i);
    const uint4 a = __ldg(q), b = __ldg(q + 1);
    d.px = __uint_as_float(a.x);
    d.py = __uint_as_float(a.y);
    d.pz = __uint_as_float(a.z);
    d.area = __uint_as_float(a.w);
    d.fr = from_bf16((uint16_t)(b.x & 0xFFFFu));
    d.fg = from_bf16((uint16_t)(b.x >> 16));
    d.fb = from_bf16((uint16_t)(b.y & 0xFFFFu));
    d.nx = from_bf16((uint16_t)(b.y >> 16));
    d.ny = from_bf16((uint16_t)(b.z & 0xFFFFu));
    d.nz = from_bf16((uint16_t)(b.z >> 16));
  } else {
    const float4* q = reinterpret_cast<const float4*>(static_cast<const DrvVPL*>(base) + i);
    const float4 a = __ldg(q), b = __ldg(q + 1), n = __ldg(q + 2);  // {flux, area}, {position}, {normal}
    d.fr = a.x;
    d.fg = a.y;
    d.fb = a.z;
    d.area = a.w;
    d.px = b.x;
    d.py = b.y;
    d.pz = b.z;
    d.nx = n.x;
    d.ny = n.y;
    d.nz = n.z;
  }
  return d;
}

// acc (and comp, with KAHAN) point at this thread's column of a
// [NK*3][kThreads] shared array.
template <int NK, bool KAHAN>
__device__ __forceinline__ void accumulate_vpl(const LightParams& p, float* acc, float* comp, const VplData& v,
                                               float cx, float cy, float cz, float shadowing) {
  float tx = v.px - cx, ty = v.py - cy, tz = v.pz - cz;
  const float d2 = tx * tx + ty * ty + tz * tz;
  const float r = rsqrtf(d2);
  tx *= r;
  ty *= r;
  tz *= r;
  const float f = sat(-(v.nx * tx + v.ny * ty + v.nz * tz)) * shadowing;
  const float s = f / (d2 + v.area);
  const float L[3] = {v.fr * s, v.fg * s, v.fb * s};
  const float bs[9] = {p.ev[0], -p.ev[1] * ty, p.ev[1] * tz, -p.ev[1] * tx, -p.ev[2] * tx * ty, p.ev[2] * ty * tz,
                       p.ev[3] * (tz * tz * 3.0f - 1.0f), p.ev[2] * tx * tz, p.ev[4] * (tx * tx - ty * ty)};
#pragma unroll
  for (int k = 0; k < NK; ++k)
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const int o = (3 * k + ch) * kThreads;
      const float x = bs[k] * L[ch];
      if (KAHAN) {
        // Kahan-compensated running sum (FP32 accumulation, BF16 storage).
        const float y = __fsub_rn(x, comp[o]);
        const float t = __fadd_rn(acc[o], y);
        comp[o] = __fsub_rn(__fsub_rn(t, acc[o]), y);
        acc[o] = t;
      } else {
        acc[o] += x;
      }
    }
}

// Adds the finished sum of coefficient `lane` to the entry.
template <int NK, bool BF16>
__device__ __forceinline__ void add_to_entry(float* entry, int lane, float v) {
  if (BF16) {
    uint16_t* sh = reinterpret_cast<uint16_t*>(entry + 1);
    sh[lane] = to_bf16(from_bf16(sh[lane]) + v);
  } else {
    entry[sh_offset(lane / 3, lane % 3)] += v;
  }
}

// One warp = one unit (cache, chunk); warps never wait for each other. The
// SH partial sums live in shared memory (touched once per pair, against
// hundreds of cone instructions), which keeps the cone loop's register
// footprint small enough for 8 CTAs per SM.
template <int NK, bool BF16>
__global__ void __launch_bounds__(kThreads, 8) light_kernel(LightParams p) {
  constexpr bool KAHAN = BF16;
  __shared__ float s_acc[NK * 3 * kThreads * (KAHAN ? 2 : 1)];
  const uint32_t count = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  const uint32_t n_units = count * (uint32_t)p.n_chunks;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * kWarps;
  for (uint32_t u = blockIdx.x * kWarps + (threadIdx.x >> 5); u < n_units; u += warps) {
    const uint32_t cache = u / (uint32_t)p.n_chunks;
    const int chunk = (int)(u % (uint32_t)p.n_chunks);
    float* entry = p.entries + (size_t)cache * p.stride_floats;
    float cx, cy, cz;
    if (BF16) {
      const uint32_t key = __float_as_uint(entry[0]);
      const int c = (int)(key >> 27);
      const float cell = p.casc_cell[c];
      cx = __fadd_rn(__fmul_rn((float)(key & 511u), cell), p.casc_min[c][0]);
      cy = __fadd_rn(__fmul_rn((float)((key >> 9) & 511u), cell), p.casc_min[c][1]);
      cz = __fadd_rn(__fmul_rn((float)((key >> 18) & 511u), cell), p.casc_min[c][2]);
    } else {
      cx = entry[0];
      cy = entry[1];
      cz = entry[2];
    }
    const float scale = 1.0f / (p.voxel_size * p.vox.N);
    const float vx = (cx - p.vol_min[0]) * scale, vy = (cy - p.vol_min[1]) * scale, vz = (cz - p.vol_min[2]) * scale;
    float* acc = s_acc + threadIdx.x;
    float* comp = acc + NK * 3 * kThreads;
#pragma unroll
    for (int k = 0; k < NK * 3; ++k) {
      acc[k * kThreads] = 0.0f;
      if (KAHAN) comp[k * kThreads] = 0.0f;
    }
    const int b0 = chunk * p.chunk_blocks, b1 = min(b0 + p.chunk_blocks, p.total_blocks);
    int l = 0;
    for (int b = b0 + lane; b < b1; b += 32) {
      while (b >= p.block_base[l + 1]) ++l;
      const LightArgs& la = p.ll.lights[l];
      const int lb = b - p.block_base[l];
      float shadowing = 1.0f;
      int v0 = lb, nv = 1;
      if (p.shadow) {
        const float4 c = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
        shadowing = cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, c.x, c.y, c.z, c.w);
        v0 = lb * la.interval;
        nv = la.interval;
      }
      for (int j = 0; j < nv; ++j)
        accumulate_vpl<NK, KAHAN>(p, acc, comp, load_vpl<BF16>(la.vpls, v0 + j), cx, cy, cz, shadowing);
    }
    // Warp reduction: lane k (< NK*3) ends up holding coefficient k.
    float mine = 0.0f;
#pragma unroll
    for (int k = 0; k < NK * 3; ++k) {
      float v = acc[k * kThreads];
      if (KAHAN) v = __fsub_rn(v, comp[k * kThreads]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == k) mine = v;
    }
    if (p.n_chunks == 1) {
      if (lane < NK * 3) add_to_entry<NK, BF16>(entry, lane, mine);
      continue;
    }
    if (lane < NK * 3) p.scratch[(size_t)u * (NK * 3) + lane] = mine;
    __threadfence();
    uint32_t last = 0;
    if (lane == 0) last = atomicAdd(p.tickets + cache, 1u) == (uint32_t)p.n_chunks - 1u;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence();
      if (lane < NK * 3) {
        const volatile float* base = p.scratch + (size_t)cache * p.n_chunks * (NK * 3);
        float v = 0.0f;
        for (int c = 0; c < p.n_chunks; ++c) v += base[c * (NK * 3) + lane];
        add_to_entry<NK, BF16>(entry, lane, v);
      }
      if (lane == 0) p.tickets[cache] = 0u;
    }
  }
}

template <int NK, bool BF16>
void launch_variant(cudaStream_t s, const LightParams& p, int num_sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, light_kernel<NK, BF16>, kThreads, 0);
  light_kernel<NK, BF16><<<num_sms * (per_sm < 1 ? 1 : per_sm), kThreads, 0, s>>>(p);
}

}  // namespace

int light_chunks(int total_blocks) {
  int n = (total_blocks + 255) / 256;
  return n < 1 ? 1 : (n > kMaxLightChunks ? kMaxLightChunks : n);
}

cudaError_t launch_light_caches(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                                const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                                const uint8_t* corners, const void* mips, const size_t* mip_offsets, float* scratch,
                                uint32_t* tickets, int num_sms) {
  LightParams p;
  p.ll = ll;
  p.shadow = cfg.indirect_shadow;
  int base = 0;
  for (int l = 0; l < ll.n_lights; ++l) {
    p.block_base[l] = base;
    base += p.shadow ? ll.lights[l].n_vpls / ll.lights[l].interval : ll.lights[l].n_vpls;
  }
  for (int l = ll.n_lights; l <= DRV_MAX_LIGHTS; ++l) p.block_base[l] = base;
  p.total_blocks = base;
  p.n_chunks = light_chunks(base);
  p.chunk_blocks = (base + p.n_chunks - 1) / p.n_chunks;
  int L = 0;
  while ((1 << (L + 1)) <= cfg.voxel_res) ++L;
  p.vox.corners = corners;
  p.vox.mips = mips;
  for (int i = 0; i < 16; ++i) p.vox.off[i] = (uint32_t)(i < kMaxVoxelLevels ? mip_offsets[i] : 0);
  p.vox.N = cfg.voxel_res;
  p.vox.log2n = L;
  p.vox.max_level = L;
  for (int i = 0; i < 3; ++i) p.vol_min[i] = vol.volume_world_min[i];
  p.voxel_size = vol.voxel_size_in_world;
  p.max_steps = cfg.max_cone_steps;
  p.counter = counter;
  p.max_caches = cfg.max_caches;
  p.entries = (float*)entries;
  p.stride_floats = (int)(entry_stride / 4);
  p.scratch = scratch;
  p.tickets = tickets;
  const double kPi = 3.14159265358979323846;
  p.ev[0] = (float)(1.0 / (2.0 * std::sqrt(kPi)));
  p.ev[1] = (float)(std::sqrt(3.0) / (2.0 * std::sqrt(kPi)));
  p.ev[2] = (float)std::sqrt(15.0 / (4.0 * kPi));
  p.ev[3] = (float)std::sqrt(5.0 / (16.0 * kPi));
  p.ev[4] = (float)std::sqrt(15.0 / (16.0 * kPi));
  const bool bf16 = cfg.precision == DRV_PRECISION_BF16;
  p.vox.half_mips = bf16;
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) {
    p.casc_cell[c] = vol.cascades[c].world_voxel_size;
    for (int i = 0; i < 3; ++i) p.casc_min[c][i] = vol.cascades[c].min[i];
  }
  if (cfg.sh_order == 2) {
    if (bf16)
      launch_variant<9, true>(s, p, num_sms);
    else
      launch_variant<9, false>(s, p, num_sms);
  } else {
    if (bf16)
      launch_variant<4, true>(s, p, num_sms);
    else
      launch_variant<4, false>(s, p, num_sms);
  }
  return cudaGetLastError();
}

}  // namespace drv
