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
#include "light_common.cuh"
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

// Adds the finished sum of coefficient `lane` to the entry.
template <bool BF16>
__device__ __forceinline__ void add_to_entry(float* entry, int lane, float v) {
  if (BF16) {
    uint16_t* sh = reinterpret_cast<uint16_t*>(entry + 1);
    sh[lane] = to_bf16(from_bf16(sh[lane]) + v);
  } else {
    entry[sh_offset(lane / 3, lane % 3)] += v;
  }
}

// Shadow block b (global index) -> light and block within the light.
__device__ __forceinline__ int block_light(const LightParams& p, int b) {
  int l = 0;
  while (b >= p.block_base[l + 1]) ++l;
  return l;
}

// One warp = one unit (cache, chunk); warps never wait for each other.
//  - Lanes first test their shadow blocks: a block none of whose VPLs has
//    positive flux and faces the cache adds exactly zero whatever its
//    shadowing, so its cone is not traced (the reference traces it).
//  - Blocks that can contribute go to a per-warp queue; every 32 queued
//    blocks are traced together, so all lanes march a cone.
// The SH partial sums live in shared memory (touched once per pair, against
// hundreds of cone instructions), which keeps the cone loop's register
// footprint small enough for 8 CTAs per SM.
template <int NK, bool BF16>
__global__ void __launch_bounds__(kThreads, 8) light_kernel(LightParams p) {
  constexpr bool KAHAN = BF16;
  __shared__ float s_acc[NK * 3 * kThreads * (KAHAN ? 2 : 1)];
  __shared__ int s_queue[kWarps][64];
  const uint32_t count = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  const uint32_t n_units = count * (uint32_t)p.n_chunks;
  const int lane = threadIdx.x & 31;
  int* queue = s_queue[threadIdx.x >> 5];
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
    // Traces the cone of block qb and gathers its contributing VPLs.
    auto trace_block = [&](int qb) {
      const int l = block_light(p, qb);
      const LightArgs& la = p.ll.lights[l];
      const int lb = qb - p.block_base[l];
      const float4 c = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
      const float s = cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, c.x, c.y, c.z, c.w);
      for (int j = 0; j < la.interval; ++j) {
        const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
        const Transfer t = transfer(v, cx, cy, cz);
        if (contributes(v, t)) accumulate<NK, KAHAN>(p.ev, acc, comp, kThreads, v, t, s);
      }
    };
    const int b0 = chunk * p.chunk_blocks, b1 = min(b0 + p.chunk_blocks, p.total_blocks);
    int queued = 0;
    for (int base = b0; base < b1; base += 32) {
      const int b = base + lane;
      bool live = false;
      if (b < b1) {
        const int l = block_light(p, b);
        const LightArgs& la = p.ll.lights[l];
        const int lb = b - p.block_base[l];
        if (p.shadow) {
          for (int j = 0; j < la.interval && !live; ++j) {
            const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
            live = contributes(v, transfer(v, cx, cy, cz));
          }
        } else {  // no indirect shadow: blocks are single VPLs, shadowing 1
          const VplData v = load_vpl<BF16>(la.vpls, lb);
          const Transfer t = transfer(v, cx, cy, cz);
          if (contributes(v, t)) accumulate<NK, KAHAN>(p.ev, acc, comp, kThreads, v, t, 1.0f);
        }
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, live);
      if (live) queue[queued + __popc(mask & ((1u << lane) - 1u))] = b;
      queued += __popc(mask);
      __syncwarp();
      if (queued >= 32) {
        trace_block(queue[queued - 32 + lane]);
        queued -= 32;
        __syncwarp();
      }
    }
    if (lane < queued) trace_block(queue[lane]);
    __syncwarp();
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
      if (lane < NK * 3) add_to_entry<BF16>(entry, lane, mine);
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
        const volatile float* sb = p.scratch + (size_t)cache * p.n_chunks * (NK * 3);
        float v = 0.0f;
        for (int c = 0; c < p.n_chunks; ++c) v += sb[c * (NK * 3) + lane];
        add_to_entry<BF16>(entry, lane, v);
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
