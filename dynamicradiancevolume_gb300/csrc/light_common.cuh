// light_common.cuh — per-pair pieces of the cache-lighting stage shared by the
// cone-traced (k_light.cu) and surrogate (k_light_surrogate.cu) kernels:
// VPL loads in both storage precisions, the SH gather of
// cacheLightingRSM.comp:234-279, and the test that a shadow block can
// contribute at all.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "voxel_sample.cuh"

namespace drv {

// Everything a light-stage kernel needs to know about the frame.
struct StageParams {
  LightLaunch ll;
  int block_base[DRV_MAX_LIGHTS + 1];  // prefix sum of shadow blocks per light
  int total_blocks;
  int shadow;     // indirect shadow on
  int max_steps;  // cone steps
  VoxelView vox;
  float vol_min[3];
  float voxel_size;
  float inv_extent;                     // 1 / (voxel_size * N)
  float casc_min[DRV_MAX_CASCADES][3];  // BF16 entries store cells: position = cell * size + min
  float casc_cell[DRV_MAX_CASCADES];
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  float* entries;
  int stride_floats;
  float ev[5];  // ShEvaFactor0, 1, 2n2_p1_n1, 20, 2p2 (renderer.cpp:302-306)
  int spec;     // INDIRECT_SPECULAR: VPLs with a flux sum below 0.001 are skipped
  uint32_t* err;  // device error word for bounded waits (nullptr: none)
};

// Host: the device view of a voxel pyramid of resolution cfg.voxel_res.
inline VoxelView make_voxel_view(const DrvConfig& cfg, const VoxelInputs& in) {
  VoxelView v{};
  int L = 0;
  while ((1 << (L + 1)) <= cfg.voxel_res) ++L;
  v.corners = in.corners;
  v.mips = in.mips;
  for (int i = 0; i < 16; ++i) v.off[i] = (uint32_t)(i < kMaxVoxelLevels && in.mip_offsets ? in.mip_offsets[i] : 0);
  v.N = cfg.voxel_res;
  v.log2n = L;
  v.max_level = L;
  v.half_mips = cfg.precision == DRV_PRECISION_BF16;
  v.records = in.records;
  v.cbias = 0u - tap_index_bias(L);
  v.record_levels = in.records && in.record_offsets ? in.record_levels : 0;
  for (int i = 0; i < 16; ++i)
    v.roff[i] = v.record_levels && i >= 1 && i <= v.record_levels ? in.record_offsets[i] - tap_index_bias(L - i) : 0u;
  return v;
}

// Host: fills StageParams from the stage's arguments (k_light.cu).
StageParams make_stage_params(const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                              const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                              const VoxelInputs& vox);

// Host: the surrogate's pass over the pair list (k_light_surrogate.cu):
// shadowing of the confident pairs, the others marked (cls 0) for the cone.
cudaError_t launch_surrogate_mlp(cudaStream_t s, const StageParams& p, const PairList& L, const SurrogateArgs& sa,
                                 bool bf16, int num_sms);

// Host: resident CTAs per SM of a kernel at this block size and dynamic
// shared memory, queried once per (kernel, block, smem) and device.
int resident_ctas(const void* kernel, int threads, size_t smem);

// Host: persistent launch (SMs x resident CTAs per SM, capped at
// ctas_per_sm when that is positive) of a kernel.
template <typename... KArgs, typename... Args>
cudaError_t launch_persistent(void (*kernel)(KArgs...), int threads, size_t smem, cudaStream_t s, int num_sms,
                              const Args&... args) {
  const int per_sm = resident_ctas(reinterpret_cast<const void*>(kernel), threads, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kernel<<<num_sms * per_sm, threads, smem, s>>>(args...);
  return cudaGetLastError();
}

// Programmatic dependent launch within the split light stage: a grid waits
// here until the previous grid of the stream has completed and its writes
// are visible (a no-op when it was launched without the attribute), then
// lets the next grid of the stream launch, so that the next grid's launch and
// CTA placement overlap this grid's tail.
__device__ __forceinline__ void pdl_wait_and_release() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Host: a launch that may start before the previous kernel of the stream
// has finished (it must call pdl_wait_and_release before reading that
// kernel's output).
template <typename... KArgs, typename... Args>
cudaError_t launch_after(void (*kernel)(KArgs...), int blocks, int threads, size_t smem, cudaStream_t s,
                         const Args&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

__device__ __forceinline__ uint32_t cache_count(const StageParams& p) {
  return min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
}

// Shadow block b (global index) -> light.
__device__ __forceinline__ int block_light(const StageParams& p, int b) {
  int l = 0;
  while (b >= p.block_base[l + 1]) ++l;
  return l;
}

// World position of cache c (BF16 entries hold the packed cell key).
template <bool BF16>
__device__ __forceinline__ void cache_position(const StageParams& p, uint32_t c, float& x, float& y, float& z) {
  const float* entry = p.entries + (size_t)c * p.stride_floats;
  if (BF16) {
    const uint32_t key = __float_as_uint(__ldg(entry));
    const int k = (int)(key >> 27);
    const float cell = p.casc_cell[k];
    x = __fadd_rn(__fmul_rn((float)(key & 511u), cell), p.casc_min[k][0]);
    y = __fadd_rn(__fmul_rn((float)((key >> 9) & 511u), cell), p.casc_min[k][1]);
    z = __fadd_rn(__fmul_rn((float)((key >> 18) & 511u), cell), p.casc_min[k][2]);
  } else {
    x = __ldg(entry);
    y = __ldg(entry + 1);
    z = __ldg(entry + 2);
  }
}

struct VplData {
  float px, py, pz, area, fr, fg, fb, nx, ny, nz;
};

// 16 bytes from global memory through the read-only path, or (SHARED) from
// a copy in shared memory.
template <bool SHARED, typename T>
__device__ __forceinline__ T load16(const T* q) {
  if constexpr (SHARED) return *q;
  else return __ldg(q);
}

// VPL i of an array (DrvVPL, or DrvVPLBF16 with BF16 precision) in global
// memory, or (SHARED) of its copy in shared memory.
template <bool BF16, bool SHARED = false>
__device__ __forceinline__ VplData load_vpl(const void* base, int i) {
  VplData d;
  if (BF16) {
    const uint4* q = reinterpret_cast<const uint4*>(static_cast<const DrvVPLBF16*>(base) + i);
    const uint4 a = load16<SHARED>(q), b = load16<SHARED>(q + 1);
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
    const float4 a = load16<SHARED>(q), b = load16<SHARED>(q + 1), n = load16<SHARED>(q + 2);  // {flux, area}, {position}, {normal}
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

// The light-transfer factor of one VPL at cache c, computed exactly as the
// gather computes it: radianceIn = flux * (g * shadowing).
struct Transfer {
  float tx, ty, tz;  // unit direction cache -> VPL
  float g;           // saturate(dot(n, -dir)) / (d^2 + area)
};

__device__ __forceinline__ Transfer transfer(const VplData& v, float cx, float cy, float cz) {
  Transfer t;
  float tx = v.px - cx, ty = v.py - cy, tz = v.pz - cz;
  const float d2 = tx * tx + ty * ty + tz * tz;
  const float r = rsqrtf(d2);
  t.tx = tx * r;
  t.ty = ty * r;
  t.tz = tz * r;
  t.g = sat(-(v.nx * t.tx + v.ny * t.ty + v.nz * t.tz)) / (d2 + v.area);
  return t;
}

// True when a VPL can add anything to the cache: positive flux and facing it.
// A VPL that fails this adds exactly zero whatever its shadowing is, so its
// shadow cone need not be traced.
__device__ __forceinline__ bool contributes(const VplData& v, const Transfer& t) {
  return t.g > 0.0f && (v.fr > 0.0f || v.fg > 0.0f || v.fb > 0.0f);
}

// Dynamic work distribution of the light stages: work[0] hands out units
// (one atomic per unit, by lane 0), work[1] counts retired CTAs; the last CTA
// to retire zeroes both, so every launch starts from zero without a memset.
__device__ __forceinline__ uint32_t next_unit(uint32_t* work, int lane) {
  uint32_t u = 0;
  if (lane == 0) u = atomicAdd(work, 1u);
  return __shfl_sync(0xffffffffu, u, 0);
}

// Called by every thread of the CTA once it has no more units.
__device__ __forceinline__ void retire_cta(uint32_t* work) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(work + 1, 1u) == gridDim.x - 1u) {
      work[0] = 0u;
      work[1] = 0u;
    }
  }
}

// With INDIRECT_SPECULAR the reference skips a VPL whose flux sum is below
// 0.001 (cacheLightingRSM.comp:240-241), for the SH as well.
__device__ __forceinline__ bool flux_ok(const StageParams& p, const VplData& v) {
  return !p.spec || !(__fadd_rn(__fadd_rn(v.fr, v.fg), v.fb) < 0.001f);
}

// A superset of `contributes` that needs no normalisation or division:
// positive flux and -(n . t) > -1e-6 max|t_i| with t = VPL - cache. The exact
// test's sign of -(n . t / |t|) can differ from the sign of -(n . t) only
// within a few roundings of zero, far inside that margin; a pair that passes
// here but not there is gathered with weight 0.
__device__ __forceinline__ bool may_contribute(const VplData& v, float cx, float cy, float cz) {
  const float tx = v.px - cx, ty = v.py - cy, tz = v.pz - cz;
  const float facing = -(v.nx * tx + v.ny * ty + v.nz * tz);
  const float scale = fmaxf(fmaxf(fabsf(tx), fabsf(ty)), fabsf(tz));
  return facing > -1e-6f * scale && (v.fr > 0.0f || v.fg > 0.0f || v.fb > 0.0f);
}

// True when some VPL of shadow block b may contribute to the cache (a
// superset of the blocks the gather's exact test keeps, see may_contribute).
template <bool BF16>
__device__ __forceinline__ bool block_live(const StageParams& p, int b, float cx, float cy, float cz) {
  const int l = block_light(p, b);
  const LightArgs& la = p.ll.lights[l];
  const int lb = b - p.block_base[l];
  for (int j = 0; j < la.interval; ++j)
    if (may_contribute(load_vpl<BF16>(la.vpls, lb * la.interval + j), cx, cy, cz)) return true;
  return false;
}

// Shadowing of block b seen from the cache (the reference's cone); `reads`
// counts the voxel loads (NoReads: nothing).
template <class R>
__device__ __forceinline__ float block_cone(const StageParams& p, int b, float cx, float cy, float cz, R& reads) {
  const int l = block_light(p, b);
  const float4 c = __ldg(reinterpret_cast<const float4*>(p.ll.lights[l].cones) + (b - p.block_base[l]));
  const float vx = (cx - p.vol_min[0]) * p.inv_extent, vy = (cy - p.vol_min[1]) * p.inv_extent,
              vz = (cz - p.vol_min[2]) * p.inv_extent;
  return cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, c.x, c.y, c.z, c.w, reads);
}
__device__ __forceinline__ float block_cone(const StageParams& p, int b, float cx, float cy, float cz) {
  NoReads r;
  return block_cone(p, b, cx, cy, cz, r);
}

// SH gather of one VPL, cacheLightingRSM.comp:255-278. acc (and comp with
// KAHAN) point at this thread's column of a [NK*3][stride] shared array.
template <int NK, bool KAHAN>
__device__ __forceinline__ void accumulate(const float ev[5], float* acc, float* comp, int stride, const VplData& v,
                                           const Transfer& t, float shadowing) {
  const float s = t.g * shadowing;
  const float L[3] = {v.fr * s, v.fg * s, v.fb * s};
  const float tx = t.tx, ty = t.ty, tz = t.tz;
  const float bs[9] = {ev[0], -ev[1] * ty, ev[1] * tz, -ev[1] * tx, -ev[2] * tx * ty, ev[2] * ty * tz,
                       ev[3] * (tz * tz * 3.0f - 1.0f), ev[2] * tx * tz, ev[4] * (tx * tx - ty * ty)};
  // Red and green as one packed pair, blue alone.
  const float2 Lrg = make_float2(L[0], L[1]);
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int o = 3 * k * stride, ob = (3 * k + 2) * stride;
    const float2 b2 = make_float2(bs[k], bs[k]);
    float2 a2 = make_float2(acc[o], acc[o + stride]);
    if (KAHAN) {
      // Kahan-compensated running sums (FP32 accumulation, BF16 storage).
      const float2 x2 = mul2(b2, Lrg);
      const float2 c2 = make_float2(comp[o], comp[o + stride]);
      const float2 y2 = sub2(x2, c2);
      const float2 t2 = add2(a2, y2);
      const float2 n2 = sub2(sub2(t2, a2), y2);
      comp[o] = n2.x;
      comp[o + stride] = n2.y;
      a2 = t2;
      const float xb = __fmul_rn(bs[k], L[2]);
      const float yb = __fsub_rn(xb, comp[ob]);
      const float tb = __fadd_rn(acc[ob], yb);
      comp[ob] = __fsub_rn(__fsub_rn(tb, acc[ob]), yb);
      acc[ob] = tb;
    } else {
      a2 = fma2(b2, Lrg, a2);
      acc[ob] = __fmaf_rn(bs[k], L[2], acc[ob]);
    }
    acc[o] = a2.x;
    acc[o + stride] = a2.y;
  }
}

}  // namespace drv
