// k_light.cu — Renderer::LightCachesRSM (renderer.cpp:899-933) /
// cacheLightingRSM.comp:80-374: per cache, gather every VPL of every light
// into RGB spherical harmonics, with the voxel cone-traced indirect shadow of
// cacheLightingRSM.comp:167-232.
//
// The reference runs one thread per cache and loops over all VPLs, tracing
// one cone per shadow block (IndirectShadowComputationSampleInterval
// consecutive VPLs). A frame has only a few thousand caches, and per cache
// only a small share of the blocks can contribute at all (a block none of
// whose VPLs has positive flux and faces the cache adds exactly zero whatever
// its shadowing), so the stage is split in three steps (five launches):
//
//  1. cull_records_kernel (K caches per pass against every VPL's plane
//     record, staged in shared memory; cull_kernel, a CTA per cache over the
//     VPL arrays, where the records do not fit) tests every block against
//     the cache and writes the cache's contributing blocks, in block order,
//     to one contiguous run of a global pair list (one atomic per cache
//     claims it), and lists the cache's gather units;
//  2. classify_kernel + scatter_kernel order the pairs by cone class (the
//     number of steps the cone marches and whether it reaches mip samples),
//     and cone_kernel (a thread per pair, persistent grid) traces the cones
//     in that order and stores each pair's shadowing: every warp holds 32
//     pairs, no lane idles on a block that needs no cone, and a warp's lanes
//     march cones of one length along one sampling path; with the learned
//     surrogate, the MLP (k_light_surrogate.cu) fills in the shadowing first
//     and only the pairs it is not confident about are traced;
//  3. gather_kernel (a warp per unit of up to kGatherChunk pairs of one
//     cache; one wave takes every cache at once): each lane gathers a fixed
//     subset of the unit's pairs with their shadowing into SH partial sums
//     in registers, reduced in a fixed order — the result does not depend on
//     scheduling — and read-modify-written into the entry once (`+=`, as the
//     reference's per-light dispatches accumulate).
//
// light_kernel, the single-launch form (warp per (cache, chunk) unit, cones
// traced from a per-warp queue, ticketed chunk reduction), serves the frames
// without indirect shadow and the allocation-free entry point.
#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "light_common.cuh"
#include "voxel_sample.cuh"

namespace drv {

StageParams make_stage_params(const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                              const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                              const VoxelInputs& vox) {
  StageParams p;
  p.ll = ll;
  p.shadow = cfg.indirect_shadow;
  int base = 0;
  for (int l = 0; l < ll.n_lights; ++l) {
    p.block_base[l] = base;
    base += p.shadow ? ll.lights[l].n_vpls / ll.lights[l].interval : ll.lights[l].n_vpls;
  }
  for (int l = ll.n_lights; l <= DRV_MAX_LIGHTS; ++l) p.block_base[l] = base;
  p.total_blocks = base;
  p.max_steps = cfg.max_cone_steps;
  p.vox = make_voxel_view(cfg, vox);
  for (int i = 0; i < 3; ++i) p.vol_min[i] = vol.volume_world_min[i];
  p.voxel_size = vol.voxel_size_in_world;
  p.inv_extent = 1.0f / (p.voxel_size * (float)cfg.voxel_res);
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) {
    p.casc_cell[c] = vol.cascades[c].world_voxel_size;
    for (int i = 0; i < 3; ++i) p.casc_min[c][i] = vol.cascades[c].min[i];
  }
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
  p.spec = cfg.specular_envmap_size > 0;
  p.err = nullptr;
  return p;
}

namespace {

// Adds the finished sum of coefficient k (channel-interleaved, k < 27) to the entry.
template <bool BF16>
__device__ __forceinline__ void add_to_entry(float* entry, int k, float v) {
  if (BF16) {
    uint16_t* sh = reinterpret_cast<uint16_t*>(entry + 1);
    sh[k] = to_bf16(from_bf16(sh[k]) + v);
  } else {
    entry[sh_offset(k / 3, k % 3)] += v;
  }
}

// SH gather of the contributing VPLs of block b with the given shadowing
// into acc/comp (stride 1: register arrays once inlined).
template <int NK, bool BF16, bool KAHAN>
__device__ __forceinline__ void gather_block(const StageParams& p, float* acc, float* comp, int b, float cx, float cy,
                                             float cz, float shadowing) {
  const int l = block_light(p, b);
  const LightArgs& la = p.ll.lights[l];
  const int lb = b - p.block_base[l];
  for (int j = 0; j < la.interval; ++j) {
    const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
    const Transfer t = transfer(v, cx, cy, cz);
    if (contributes(v, t) && flux_ok(p, v)) accumulate<NK, KAHAN>(p.ev, acc, comp, 1, v, t, shadowing);
  }
}

// ------------------------------------------------------------ split stage
// Lists the gather units of cache c's run: one per kGatherChunk listed
// pairs, one for a cache the list could not hold; and zeroes the cache's
// ticket, so that a gather that stopped early (a timed-out copy) leaves no
// count behind for the next stage.
__device__ __forceinline__ void note_gather_units(const PairList& L, uint32_t c, uint32_t total, bool over) {
  L.tickets[c] = 0u;
  const uint32_t n = over ? 1u : (total + kGatherChunk - 1) / kGatherChunk;
  if (!n) return;
  const uint32_t base = atomicAdd(L.counters + kGatherUnitsCounter, n);
  for (uint32_t k = 0; k < n; ++k) L.units[base + k] = make_uint2(c, k);
}

constexpr int kCullThreads = 256;
constexpr int kCullWarps = kCullThreads / 32;

// CTA per cache: contributing blocks -> a contiguous run of the pair list.
template <bool BF16>
__global__ void __launch_bounds__(kCullThreads) cull_kernel(StageParams p, PairList L) {
  pdl_wait_and_release();
  extern __shared__ uint32_t s_dyn[];  // [W] ballot words, [W] exclusive prefix of their popcounts
  __shared__ uint32_t s_warp[kCullWarps];
  __shared__ uint32_t s_base, s_count;
  const int W = (p.total_blocks + 31) >> 5;
  uint32_t* s_mask = s_dyn;
  uint32_t* s_pre = s_dyn + W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per = (W + kCullThreads - 1) / kCullThreads;  // words per thread in the scan
  const uint32_t n_caches = cache_count(p);
  for (uint32_t c = blockIdx.x; c < n_caches; c += gridDim.x) {
    float cx, cy, cz;
    cache_position<BF16>(p, c, cx, cy, cz);
    for (int w = warp; w < W; w += kCullWarps) {
      const int b = (w << 5) + lane;
      const bool live = b < p.total_blocks && block_live<BF16>(p, b, cx, cy, cz);
      const uint32_t m = __ballot_sync(0xffffffffu, live);
      if (lane == 0) s_mask[w] = m;
    }
    __syncthreads();
    // Exclusive scan of the word popcounts (thread t owns words [t*per, t*per + per)).
    const int w0 = threadIdx.x * per;
    uint32_t local = 0;
    for (int k = 0; k < per; ++k)
      if (w0 + k < W) local += __popc(s_mask[w0 + k]);
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t run = incl - local, total = 0;
#pragma unroll
    for (int k = 0; k < kCullWarps; ++k) {
      const uint32_t v = s_warp[k];
      if (k < warp) run += v;
      total += v;
    }
    for (int k = 0; k < per; ++k)
      if (w0 + k < W) {
        s_pre[w0 + k] = run;
        run += __popc(s_mask[w0 + k]);
      }
    if (threadIdx.x == 0) {
      const uint32_t base = total ? atomicAdd(L.counters, total) : 0u;
      const bool over = (uint64_t)base + total > (uint64_t)L.cap;
      L.info[2 * c] = base;
      L.info[2 * c + 1] = over ? kPairOverflow : total;
      note_gather_units(L, c, total, over);
      s_base = base;
      s_count = over ? kPairOverflow : total;
    }
    __syncthreads();
    const uint32_t base = s_base;
    if (s_count != kPairOverflow) {
      for (int w = warp; w < W; w += kCullWarps) {
        const uint32_t m = s_mask[w];
        if ((m >> lane) & 1u) {
          const uint32_t i = base + s_pre[w] + __popc(m & ((1u << lane) - 1u));
          L.cache[i] = c;
          L.block[i] = (uint32_t)((w << 5) + lane);
        }
      }
    } else {
      // The list is full: the gather traces this cache itself; the claimed
      // slots below the capacity stay empty.
      const uint32_t end = (uint32_t)min((uint64_t)base + total, (uint64_t)L.cap);
      for (uint32_t i = base + threadIdx.x; i < end; i += kCullThreads) L.block[i] = kNoPair;
    }
    __syncthreads();
  }
}

// ---- cull over VPL plane records in shared memory
// The test of may_contribute, rewritten as a plane test: a VPL at p with
// normal n faces the cache c when n . c - n . p > 0. Each VPL becomes one
// 16-byte record {n, -n . p + eps (1 + |p|_inf)} (no-flux VPLs: -inf, never
// live), staged once per CTA in shared memory; a cache passes when
// n . c + w > -eps |c|_inf. The margin eps = 1e-5 covers the FP32 rounding of
// both this sum and the gather's normalised test (a few u = 2^-24 relative to
// |p| + |c|), so the cull stays a superset of the pairs the gather's exact
// test keeps; the few extra near-tangent pairs are gathered with weight 0.
// Each CTA tests K caches per pass (the tile: K caches x every record; 4 by
// default, DrvTuning.cull_caches_per_pass): one shared-memory load serves K
// tests of three FMAs each.
constexpr int kCullRecThreads = 512;
constexpr int kCullRecWarps = kCullRecThreads / 32;
constexpr size_t kCullRecMaxSmem = 220 * 1024;

// Shared memory of cull_records_kernel: the records, then per cache of the
// pass the ballot words and their exclusive prefix.
inline size_t cull_records_smem(int total_vpls, int words, int K) {
  return (size_t)total_vpls * 16 + (size_t)2 * K * words * 4;
}

// UNIT: every light's shadow blocks are single VPLs, so block b's record is
// record b. COPY: every light has its records in global memory (written by
// the VPL extraction); one bulk asynchronous copy per light (TMA, completion
// on an mbarrier, bounded wait) stages them, instead of computing them here
// from the VPLs.
// One VPL plane record against K caches, ORed into live[]: n.c + w > lim,
// the three multiply-adds of two caches at a time in packed FP32 pairs (the
// same roundings as fmaf).
template <int K>
__device__ __forceinline__ void plane_tests(const float4 r, const float (&cx)[K], const float (&cy)[K],
                                            const float (&cz)[K], const float (&lim)[K], bool (&live)[K]) {
  const float2 rx = make_float2(r.x, r.x), ry = make_float2(r.y, r.y), rz = make_float2(r.z, r.z),
               rw = make_float2(r.w, r.w);
#pragma unroll
  for (int k = 0; k < K; k += 2) {
    const float2 d = fma2(rx, make_float2(cx[k], cx[k + 1]),
                          fma2(ry, make_float2(cy[k], cy[k + 1]), fma2(rz, make_float2(cz[k], cz[k + 1]), rw)));
    live[k] |= d.x > lim[k];
    live[k + 1] |= d.y > lim[k + 1];
  }
}

template <bool BF16, bool UNIT, bool COPY, int K>
__global__ void __launch_bounds__(kCullRecThreads) cull_records_kernel(StageParams p, PairList L, int total_vpls) {
  pdl_wait_and_release();
  extern __shared__ float4 s_rec[];
  __shared__ uint32_t s_base[K], s_count[K];
  __shared__ __align__(8) uint64_t s_bar;
  const int W = (p.total_blocks + 31) >> 5;
  uint32_t* s_mask = reinterpret_cast<uint32_t*>(s_rec + total_vpls);  // [K][W]
  uint32_t* s_pre = s_mask + K * W;                        // [K][W]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // VPL records, in light order (light l's VPLs from vpl_base(l)).
  if (COPY) {
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_bar);
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(total_vpls * 16)
                   : "memory");
      int base = 0;
      for (int l = 0; l < p.ll.n_lights; ++l) {
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(s_rec + base)),
                     "l"(p.ll.lights[l].records), "r"(p.ll.lights[l].n_vpls * 16), "r"(bar)
                     : "memory");
        base += p.ll.lights[l].n_vpls;
      }
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    bool ok = false;
    const unsigned long long t0 = clock64();
    for (;;) {
      uint32_t done;
      asm volatile(
          "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\nselp.u32 %0, 1, 0, q;\n}\n"
          : "=r"(done)
          : "r"(bar)
          : "memory");
      if (done) {
        ok = true;
        break;
      }
      if ((unsigned long long)(clock64() - t0) > 2000000000ull) break;  // about a second
    }
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0 && p.err) raise_error(p.err, DRV_DEVERR_TIMEOUT);
      // the copies may still be in flight: wait for them once more (bounded)
      // before this CTA's shared memory is released
      const unsigned long long t1 = clock64();
      for (;;) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\nselp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(bar)
            : "memory");
        if (done || (unsigned long long)(clock64() - t1) > 2000000000ull) break;
      }
      return;
    }
  } else {
    for (int g = threadIdx.x; g < total_vpls; g += kCullRecThreads) {
      int l = 0, base = 0;
      while (g >= base + p.ll.lights[l].n_vpls) base += p.ll.lights[l].n_vpls, ++l;
      const VplData v = load_vpl<BF16>(p.ll.lights[l].vpls, g - base);
      s_rec[g] = make_cull_record(v.nx, v.ny, v.nz, v.px, v.py, v.pz, v.fr > 0.0f || v.fg > 0.0f || v.fb > 0.0f);
    }
    __syncthreads();
  }
  const uint32_t n_caches = cache_count(p);
  for (uint32_t c0 = blockIdx.x * K; c0 < n_caches; c0 += gridDim.x * K) {
    float cx[K], cy[K], cz[K], lim[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t c = min(c0 + k, n_caches - 1u);  // past the end: a copy of the last cache, not written
      cache_position<BF16>(p, c, cx[k], cy[k], cz[k]);
      lim[k] = -kCullRecordEps * fmaxf(fmaxf(fabsf(cx[k]), fabsf(cy[k])), fabsf(cz[k]));
    }
    for (int w = warp; w < W; w += kCullRecWarps) {
      const int b = (w << 5) + lane;
      bool live[K];
#pragma unroll
      for (int k = 0; k < K; ++k) live[k] = false;
      if (b < p.total_blocks) {
        if (UNIT) {
          plane_tests<K>(s_rec[b], cx, cy, cz, lim, live);
        } else {
          int l = 0, vbase = 0;
          while (b >= p.block_base[l + 1]) vbase += p.ll.lights[l].n_vpls, ++l;
          const int interval = p.ll.lights[l].interval;
          const int first = vbase + (b - p.block_base[l]) * interval;
          for (int j = 0; j < interval; ++j) plane_tests<K>(s_rec[first + j], cx, cy, cz, lim, live);
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t m = __ballot_sync(0xffffffffu, live[k]);
        if (lane == 0) s_mask[k * W + w] = m;
      }
    }
    __syncthreads();
    // Warp k: exclusive prefix of cache k's word popcounts, then its run of
    // the pair list (one atomic per cache).
    if (warp < K && c0 + warp < n_caches) {
      const int k = warp;
      const uint32_t c = c0 + k;
      const int per = (W + 31) >> 5;
      const int w0 = lane * per;
      uint32_t local = 0;
      for (int q = 0; q < per; ++q)
        if (w0 + q < W) local += __popc(s_mask[k * W + w0 + q]);
      uint32_t incl = local;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
      uint32_t run = incl - local;
      for (int q = 0; q < per; ++q)
        if (w0 + q < W) {
          s_pre[k * W + w0 + q] = run;
          run += __popc(s_mask[k * W + w0 + q]);
        }
      if (lane == 0) {
        const uint32_t base = total ? atomicAdd(L.counters, total) : 0u;
        const bool over = (uint64_t)base + total > (uint64_t)L.cap;
        L.info[2 * c] = base;
        L.info[2 * c + 1] = over ? kPairOverflow : total;
        note_gather_units(L, c, total, over);
        s_base[k] = base;
        s_count[k] = over ? kPairOverflow : total;
      }
    }
    __syncthreads();
    const int nk = (int)min((uint32_t)K, n_caches - c0);
    const uint32_t below = (1u << lane) - 1u;
    for (int k = 0; k < nk; ++k) {
      const uint32_t base = s_base[k], c = c0 + k;
      if (s_count[k] != kPairOverflow) {
        for (int w = warp; w < W; w += kCullRecWarps) {
          const uint32_t m = s_mask[k * W + w];
          if ((m >> lane) & 1u) {
            const uint32_t i = base + s_pre[k * W + w] + __popc(m & below);
            L.cache[i] = c;
            L.block[i] = (uint32_t)((w << 5) + lane);
          }
        }
      } else if (warp == 0) {
        // The list is full: the gather traces this cache itself; the claimed
        // slots below the capacity stay empty.
        uint32_t total = 0;
        for (int q = 0; q < W; ++q) total += __popc(s_mask[k * W + q]);
        const uint32_t end = (uint32_t)min((uint64_t)base + total, (uint64_t)L.cap);
        for (uint32_t i = base + lane; i < end; i += 32) L.block[i] = kNoPair;
      }
    }
    __syncthreads();
  }
}

// Cone class of a pair: about how many steps its cone marches when nothing
// occludes it, in buckets of 4, and at which step, if any, its radius passes
// one voxel (its samples move to mip levels): never, after step 16, after
// step 8, or earlier. cone_shadow steps by max(1, g * dist) with
// g = 2 dsr / (1 - dsr): unit steps up to dist = 1 / g, then the distance
// grows by the factor 1 + g per step, until it reaches the goal. Classes
// only order the cones; results do not depend on them.
__device__ __forceinline__ float cone_steps_to(float dist, float g, float m) {
  // steps until the marched distance reaches `dist`
  return dist <= m ? ceilf(dist) : m + ceilf(__log2f(dist / m) / __log2f(1.0f + g));
}

__device__ __forceinline__ int cone_class(float light_dist, float voxel_size, float dsr, int max_steps) {
  const float goal = fmaxf(light_dist / voxel_size - 2.0f, 1.0f);
  const float g = 2.0f * dsr / (1.0f - dsr);
  const float m = g > 0.0f ? fmaxf(1.0f, floorf(1.0f / g)) : 3.0e38f;  // last unit step
  const float n = fminf(cone_steps_to(goal, g, m), (float)max_steps);
  const float n_mip = dsr > 0.0f ? cone_steps_to(1.0f / dsr, g, m) : 3.0e38f;  // first step with radius > 1
  const int len = min(max((int)n - 1, 0) >> 2, 7);
  const int mip = n_mip > n ? 0 : (n_mip > 16.0f ? 1 : (n_mip > 8.0f ? 2 : 3));
  return mip * 8 + len;
}

constexpr int kClassThreads = 256;

// Thread per listed pair: its cone class; class totals in counters[8 + c].
// MARKED: only the pairs the surrogate left unconfident (cls 0) get a class;
// the others keep 0xFF and are neither ordered nor traced.
template <bool BF16, bool MARKED>
__global__ void __launch_bounds__(kClassThreads) classify_kernel(StageParams p, PairList L) {
  pdl_wait_and_release();
  __shared__ uint32_t s_hist[kConeClasses];
  if (threadIdx.x < kConeClasses) s_hist[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t n = min(L.counters[0], L.cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t b = L.block[i];
    uint8_t c = 0xFF;
    if (b != kNoPair && (!MARKED || L.cls[i] != 0xFF)) {
      float cx, cy, cz;
      cache_position<BF16>(p, L.cache[i], cx, cy, cz);
      const int l = block_light(p, (int)b);
      const float4 cone = __ldg(reinterpret_cast<const float4*>(p.ll.lights[l].cones) + (b - p.block_base[l]));
      const float tx = cone.x - cx, ty = cone.y - cy, tz = cone.z - cz;
      c = (uint8_t)cone_class(sqrtf(tx * tx + ty * ty + tz * tz), p.voxel_size, cone.w, p.max_steps);
      atomicAdd(&s_hist[c], 1u);
    }
    L.cls[i] = c;
  }
  __syncthreads();
  if (threadIdx.x < kConeClasses && s_hist[threadIdx.x]) atomicAdd(L.counters + 8 + threadIdx.x, s_hist[threadIdx.x]);
}

constexpr int kScatterTile = 4 * kClassThreads;

// CTA per tile of kScatterTile pairs (4 per thread): each pair's index goes
// to its class's region of L.order (regions in class order); a CTA reserves
// its share of each region with one atomic per class.
__global__ void __launch_bounds__(kClassThreads) scatter_kernel(PairList L) {
  pdl_wait_and_release();
  __shared__ uint32_t s_region[kConeClasses], s_hist[kConeClasses], s_pos[kConeClasses];
  const uint32_t n = min(L.counters[0], L.cap);
  static_assert(kConeClasses == 32, "one warp scans the class totals");
  if (threadIdx.x < 32) {
    // exclusive scan of the class totals: one load per lane, shuffles
    const uint32_t total = L.counters[8 + threadIdx.x];
    uint32_t incl = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)threadIdx.x >= o) incl += v;
    }
    s_region[threadIdx.x] = incl - total;
  }
  for (uint32_t t0 = blockIdx.x * kScatterTile; t0 < n; t0 += gridDim.x * kScatterTile) {
    if (threadIdx.x < kConeClasses) s_hist[threadIdx.x] = 0u;
    __syncthreads();
    uint8_t c[4];
    uint32_t rank[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t i = t0 + j * kClassThreads + threadIdx.x;
      c[j] = i < n ? L.cls[i] : (uint8_t)0xFF;
      rank[j] = c[j] != 0xFF ? atomicAdd(&s_hist[c[j]], 1u) : 0u;
    }
    __syncthreads();
    if (threadIdx.x < kConeClasses) {
      const uint32_t h = s_hist[threadIdx.x];
      s_pos[threadIdx.x] = s_region[threadIdx.x] + (h ? atomicAdd(L.counters + 8 + kConeClasses + threadIdx.x, h) : 0u);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (c[j] != 0xFF) L.order[s_pos[c[j]] + rank[j]] = t0 + j * kClassThreads + threadIdx.x;
    __syncthreads();
  }
}

// Thread per cone over L.order, the listed pairs in cone-class order (with
// the surrogate, the pairs it left unconfident). COUNT (a separate,
// measuring instance): the voxel loads of all cones are summed into
// counters[1] (level-0 corner bytes), [2] (16-byte mip records) and [7]
// (plain mip texels).
template <bool BF16, bool COUNT = false>
__global__ void __launch_bounds__(128) cone_kernel(StageParams p, PairList L) {
  pdl_wait_and_release();
  uint32_t n = 0;
#pragma unroll
  for (int c = 0; c < kConeClasses; ++c) n += L.counters[8 + c];
  n = min(n, L.cap);
  typename std::conditional<COUNT, VoxelReads, NoReads>::type reads;
  // Warps take 32 cones at a time from counters[6], from the end of the
  // class order (the longest cones) to its start, so the short cones fill
  // the tail of the pass.
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(L.counters + 6, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    if (base + lane >= n) continue;
    const uint32_t i = L.order[n - 1u - (base + lane)];
    const uint32_t b = L.block[i];
    if (b == kNoPair) continue;
    float cx, cy, cz;
    cache_position<BF16>(p, L.cache[i], cx, cy, cz);
    L.shadow[i] = block_cone(p, (int)b, cx, cy, cz, reads);
  }
  if constexpr (COUNT) {
    uint32_t a = reads.level0_bytes, b = reads.records, c = reads.texels;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
      atomicAdd(L.counters + 1, a);
      atomicAdd(L.counters + 2, b);
      atomicAdd(L.counters + 7, c);
    }
  }
}

// Sum over the warp of each lane's v[0..N-1] (N = 16 or 32), returned in
// lane k for value k (lanes >= N get nothing useful): at each step a lane
// keeps the half of its values its own half of the warp will own, sends the
// other half to the partner lane and adds what it receives, so the 32-value
// case takes 16 + 8 + 4 + 2 + 1 = 31 shuffles instead of 32 x 5.
template <int N>
__device__ __forceinline__ float warp_transpose_reduce(float (&v)[32], int lane) {
  // Values N..31 are unused: first fold lane halves when N = 16.
  int n = N;
#pragma unroll
  for (int half = 16; half >= 1; half >>= 1) {
    if (half >= n) {  // fewer values than lanes in this half: plain butterfly on each
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (i < n) v[i] += __shfl_xor_sync(0xffffffffu, v[i], half);
      continue;
    }
    const bool upper = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (i < n / 2) {
        const float send = upper ? v[i] : v[i + n / 2];
        const float keep = upper ? v[i + n / 2] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, half);
      }
    }
    n /= 2;
  }
  return v[0];
}

// The gather's VPLs: as many as fit in kGatherStageBytes of shared memory
// (VPL g of the lights' arrays back to back, in light order) are copied there
// once per CTA; the rest are read from global memory.
constexpr size_t kGatherStageBytes = 220 * 1024;
template <bool BF16>
__host__ __device__ constexpr uint32_t vpl_bytes() {
  return BF16 ? (uint32_t)sizeof(DrvVPLBF16) : (uint32_t)sizeof(DrvVPL);
}
uint32_t gather_staged_vpls(const LightLaunch& ll, bool bf16) {
  uint32_t total = 0;
  for (int l = 0; l < ll.n_lights; ++l) total += (uint32_t)ll.lights[l].n_vpls;
  const uint32_t fit = (uint32_t)(kGatherStageBytes / (bf16 ? vpl_bytes<true>() : vpl_bytes<false>()));
  return total < fit ? total : fit;
}

// SH gather of block b with the given shadowing, its VPLs from the staged
// copy (g < staged) or from global memory.
template <int NK, bool BF16, bool KAHAN>
__device__ __forceinline__ void gather_block_staged(const StageParams& p, const unsigned char* s_vpl,
                                                    const uint32_t* s_vbase, uint32_t staged, float* acc, float* comp,
                                                    int b, float cx, float cy, float cz, float shadowing) {
  const int l = block_light(p, b);
  const LightArgs& la = p.ll.lights[l];
  const int lb = b - p.block_base[l];
  for (int j = 0; j < la.interval; ++j) {
    const int i = lb * la.interval + j;
    const uint32_t g = s_vbase[l] + (uint32_t)i;
    const VplData v = g < staged ? load_vpl<BF16, true>(s_vpl, (int)g) : load_vpl<BF16>(la.vpls, i);
    const Transfer t = transfer(v, cx, cy, cz);
    if (contributes(v, t) && flux_ok(p, v)) accumulate<NK, KAHAN>(p.ev, acc, comp, 1, v, t, shadowing);
  }
}

// Warp per gather unit: kGatherChunk pairs of one cache's run (lane j sums
// the unit's pairs j, j + 32, ... in order), or the whole cache when the list
// could not hold it (the warp tests every block and traces the live ones'
// cones; the k-th live block goes to lane k mod 32, the lane its listed pair
// would have had). The cull lists the units, so one wave of warps takes
// every cache at once and a long run is spread over several warps. A cache
// of one unit adds
// its sums to the entry directly (`+=`, as the reference's per-light
// dispatches accumulate); a longer one writes each unit's sums to its slot
// and the unit that finishes last adds them in unit order: the result does
// not depend on scheduling. One CTA per SM: its VPL copy (a bulk
// asynchronous copy per light, issued before the wait on the previous
// kernel, since the VPLs were written before the light stage began) is
// shared by all its warps. THREADS only sets the warps per CTA.
// hold_copy (test hook): the copies are not issued, so the wait runs out
// after kGatherTestWaitCycles (~10 ms) and the timeout path is taken.
constexpr unsigned long long kGatherWaitCycles = 2000000000ull;  // about a second
constexpr unsigned long long kGatherTestWaitCycles = 20000000ull;
template <int NK, bool BF16, int THREADS>
__global__ void __launch_bounds__(THREADS, 1) gather_kernel(StageParams p, PairList L, uint32_t staged,
                                                            int hold_copy) {
  extern __shared__ __align__(16) unsigned char s_vpl[];
  __shared__ uint32_t s_vbase[DRV_MAX_LIGHTS];
  __shared__ __align__(8) uint64_t s_bar;
  constexpr bool KAHAN = BF16;  // FP32 accumulation of BF16-stored results, compensated
  constexpr int NV = NK * 3;
  const int lane = threadIdx.x & 31;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_bar);
  if (threadIdx.x == 0) {
    uint32_t base = 0;
    for (int l = 0; l < p.ll.n_lights; ++l) {
      s_vbase[l] = base;
      base += (uint32_t)p.ll.lights[l].n_vpls;
    }
    if (staged) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(staged * vpl_bytes<BF16>())
                   : "memory");
      for (int l = 0; l < p.ll.n_lights && !hold_copy; ++l) {
        const uint32_t v0 = s_vbase[l];
        if (v0 >= staged) break;
        const uint32_t n = min((uint32_t)p.ll.lights[l].n_vpls, staged - v0);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(s_vpl + (size_t)v0 * vpl_bytes<BF16>())),
                     "l"(p.ll.lights[l].vpls), "r"(n * vpl_bytes<BF16>()), "r"(bar)
                     : "memory");
      }
    }
  }
  __syncthreads();  // offsets written, barrier initialised before anyone waits on it
  pdl_wait_and_release();
  if (staged) {
    const unsigned long long limit = hold_copy ? kGatherTestWaitCycles : kGatherWaitCycles;
    bool ok = false;
    const unsigned long long t0 = clock64();
    for (;;) {
      uint32_t done;
      asm volatile(
          "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\nselp.u32 %0, 1, 0, q;\n}\n"
          : "=r"(done)
          : "r"(bar)
          : "memory");
      if (done) {
        ok = true;
        break;
      }
      if ((unsigned long long)(clock64() - t0) > limit) break;
    }
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0 && p.err) raise_error(p.err, DRV_DEVERR_TIMEOUT);
      // the copies may still be in flight: wait for them once more (bounded)
      // before this CTA's shared memory is released
      const unsigned long long t1 = clock64();
      for (;;) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\nselp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(bar)
            : "memory");
        if (done || (unsigned long long)(clock64() - t1) > limit) break;
      }
      return;
    }
  }
  const uint32_t n_units = L.counters[kGatherUnitsCounter];
  const uint32_t warps = gridDim.x * (THREADS / 32);
  for (uint32_t u = blockIdx.x * (THREADS / 32) + (threadIdx.x >> 5); u < n_units; u += warps) {
    const uint2 unit = L.units[u];
    const uint32_t c = unit.x, k = unit.y;
    const uint32_t first = L.info[2 * c], count = L.info[2 * c + 1];
    const bool over = count == kPairOverflow;
    const uint32_t units = over ? 1u : (count + kGatherChunk - 1) / kGatherChunk;
    float cx, cy, cz;
    cache_position<BF16>(p, c, cx, cy, cz);
    float acc[NV], comp[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = comp[q] = 0.0f;
    const uint32_t lo = first + k * kGatherChunk;
    if (!over) {
      // the next pair's block and shadowing are loaded while this pair is summed
      const uint32_t hi = first + min(count, (k + 1) * kGatherChunk);
      uint32_t i = lo + lane;
      uint32_t b_next = i < hi ? __ldg(L.block + i) : 0u;
      float s_next = i < hi ? __ldg(L.shadow + i) : 0.0f;
      for (; i < hi; i += 32) {
        const uint32_t b = b_next;
        const float shadowing = s_next;
        if (i + 32 < hi) {
          b_next = __ldg(L.block + i + 32);
          s_next = __ldg(L.shadow + i + 32);
        }
        gather_block_staged<NK, BF16, KAHAN>(p, s_vpl, s_vbase, staged, acc, comp, (int)b, cx, cy, cz, shadowing);
      }
    } else {
      uint32_t before = 0;  // live blocks in earlier rounds
      for (int b0 = 0; b0 < p.total_blocks; b0 += 32) {
        const int b = b0 + lane;
        const bool live = b < p.total_blocks && block_live<BF16>(p, b, cx, cy, cz);
        const uint32_t m = __ballot_sync(0xffffffffu, live);
        const int n = __popc(m);
        const int i = (lane - (int)(before & 31u)) & 31;  // this lane's live block of the round
        const int src = i < n ? (int)__fns(m, 0u, i + 1) : 0;
        const int bb = __shfl_sync(0xffffffffu, b, src);
        if (i < n)
          gather_block_staged<NK, BF16, KAHAN>(p, s_vpl, s_vbase, staged, acc, comp, bb, cx, cy, cz,
                                               block_cone(p, bb, cx, cy, cz));
        before += (uint32_t)n;
      }
    }
    // Warp reduction of the NV sums: lane q ends up with coefficient q.
    float v[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = q < NV ? (KAHAN ? __fsub_rn(acc[q], comp[q]) : acc[q]) : 0.0f;
    const float mine = warp_transpose_reduce<NV <= 16 ? 16 : 32>(v, lane);
    float* entry = p.entries + (size_t)c * p.stride_floats;
    if (units == 1u) {
      if (lane < NV) add_to_entry<BF16>(entry, lane, mine);
      continue;
    }
    auto slot_of = [&](uint32_t j) -> size_t {
      return j + 1 < units ? (first + j * kGatherChunk + kGatherChunk - 1) / kGatherChunk
                           : (size_t)L.partial_tail + c;
    };
    if (lane < NV) L.partials[slot_of(k) * kGatherSlotFloats + lane] = mine;
    __threadfence();
    __syncwarp();
    uint32_t ticket = 0;
    if (lane == 0) ticket = atomicAdd(L.tickets + c, 1u);
    ticket = __shfl_sync(0xffffffffu, ticket, 0);
    if (ticket + 1u != units) continue;
    __threadfence();
    if (lane < NV) {
      float sum = 0.0f;
      for (uint32_t j = 0; j < units; ++j)
        sum += j == k ? mine : __ldcg(L.partials + slot_of(j) * kGatherSlotFloats + lane);
      add_to_entry<BF16>(entry, lane, sum);
    }
  }
}

// ------------------------------------------------------------ single launch
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

struct FusedParams {
  StageParams s;
  int n_chunks;
  int chunk_blocks;
  float* scratch;     // [max_caches * n_chunks][NK*3] partial sums
  uint32_t* tickets;  // [max_caches], zero between launches
  uint32_t* work;     // unit counter + retired CTAs, zero between launches
};

// One warp = one unit (cache, chunk), handed out dynamically; lanes take the
// chunk's blocks round-robin. Blocks that can contribute go to a per-warp
// queue traced 32 at a time; partial SH sums live in shared memory (touched
// once per pair) so the cone loop keeps 8 CTAs per SM.
template <int NK, bool BF16>
__global__ void __launch_bounds__(kThreads, 8) light_kernel(FusedParams fp) {
  const StageParams& p = fp.s;
  constexpr bool KAHAN = BF16;
  __shared__ float s_acc[NK * 3 * kThreads * (KAHAN ? 2 : 1)];
  __shared__ int s_queue[kWarps][64];
  const uint32_t n_units = cache_count(p) * (uint32_t)fp.n_chunks;
  const int lane = threadIdx.x & 31;
  int* queue = s_queue[threadIdx.x >> 5];
  for (uint32_t u = next_unit(fp.work, lane); u < n_units; u = next_unit(fp.work, lane)) {
    const uint32_t cache = u / (uint32_t)fp.n_chunks;
    const int chunk = (int)(u % (uint32_t)fp.n_chunks);
    float* entry = p.entries + (size_t)cache * p.stride_floats;
    float cx, cy, cz;
    cache_position<BF16>(p, cache, cx, cy, cz);
    float* acc = s_acc + threadIdx.x;
    float* comp = acc + NK * 3 * kThreads;
#pragma unroll
    for (int k = 0; k < NK * 3; ++k) {
      acc[k * kThreads] = 0.0f;
      if (KAHAN) comp[k * kThreads] = 0.0f;
    }
    auto trace_block = [&](int qb) {
      const float s = block_cone(p, qb, cx, cy, cz);
      const int l = block_light(p, qb);
      const LightArgs& la = p.ll.lights[l];
      const int lb = qb - p.block_base[l];
      for (int j = 0; j < la.interval; ++j) {
        const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
        const Transfer t = transfer(v, cx, cy, cz);
        if (contributes(v, t) && flux_ok(p, v)) accumulate<NK, KAHAN>(p.ev, acc, comp, kThreads, v, t, s);
      }
    };
    const int b0 = chunk * fp.chunk_blocks, b1 = min(b0 + fp.chunk_blocks, p.total_blocks);
    int queued = 0;
    for (int base = b0; base < b1; base += 32) {
      const int b = base + lane;
      bool live = false;
      if (b < b1) {
        if (p.shadow) {
          live = block_live<BF16>(p, b, cx, cy, cz);
        } else {  // no indirect shadow: blocks are single VPLs, shadowing 1
          const int l = block_light(p, b);
          const VplData v = load_vpl<BF16>(p.ll.lights[l].vpls, b - p.block_base[l]);
          const Transfer t = transfer(v, cx, cy, cz);
          if (contributes(v, t) && flux_ok(p, v)) accumulate<NK, KAHAN>(p.ev, acc, comp, kThreads, v, t, 1.0f);
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
    if (fp.n_chunks == 1) {
      if (lane < NK * 3) add_to_entry<BF16>(entry, lane, mine);
      continue;
    }
    if (lane < NK * 3) fp.scratch[(size_t)u * (NK * 3) + lane] = mine;
    __threadfence();
    uint32_t last = 0;
    if (lane == 0) last = atomicAdd(fp.tickets + cache, 1u) == (uint32_t)fp.n_chunks - 1u;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence();
      if (lane < NK * 3) {
        const volatile float* sb = fp.scratch + (size_t)cache * fp.n_chunks * (NK * 3);
        float v = 0.0f;
        for (int c = 0; c < fp.n_chunks; ++c) v += sb[c * (NK * 3) + lane];
        add_to_entry<BF16>(entry, lane, v);
      }
      if (lane == 0) fp.tickets[cache] = 0u;
    }
  }
  retire_cta(fp.work);
}

// Launch of CTAs_PER_SM x SMs CTAs (at most what fits), or a full persistent grid.
// after: launched with programmatic stream serialisation (launch_after).
template <typename... KArgs, typename... Args>
cudaError_t launch_grid(void (*kernel)(KArgs...), int threads, size_t smem, cudaStream_t s, int num_sms,
                        int ctas_per_sm, bool after, const Args&... args) {
  int per_sm = resident_ctas(reinterpret_cast<const void*>(kernel), threads, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  if (after) return launch_after(kernel, num_sms * per_sm, threads, smem, s, args...);
  kernel<<<num_sms * per_sm, threads, smem, s>>>(args...);
  return cudaGetLastError();
}

// launch_persistent with programmatic stream serialisation.
template <typename... KArgs, typename... Args>
cudaError_t launch_persistent_after(void (*kernel)(KArgs...), int threads, size_t smem, cudaStream_t s, int num_sms,
                                    const Args&... args) {
  const int per_sm = resident_ctas(reinterpret_cast<const void*>(kernel), threads, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  return launch_after(kernel, num_sms * per_sm, threads, smem, s, args...);
}

// The record cull's instance for one-VPL blocks (unit), records copied from
// the extraction (copy) and K caches per pass (2, 4 or 8).
template <bool BF16>
void (*cull_kernel_for(bool unit, bool copy, int K))(StageParams, PairList, int) {
#define DRV_CULL_K(U, CP)                                                   \
  (K == 2 ? cull_records_kernel<BF16, U, CP, 2>                             \
          : (K == 8 ? cull_records_kernel<BF16, U, CP, 8> : cull_records_kernel<BF16, U, CP, 4>))
  if (unit) return copy ? DRV_CULL_K(true, true) : DRV_CULL_K(true, false);
  return copy ? DRV_CULL_K(false, true) : DRV_CULL_K(false, false);
#undef DRV_CULL_K
}

// Raises a kernel's dynamic shared-memory limit, once per (kernel, device).
cudaError_t set_max_smem(const void* kernel, size_t bytes) {
  struct Done {
    const void* kernel;
    int device;
  };
  static std::mutex mu;
  static std::vector<Done> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  for (const Done& d : done)
    if (d.kernel == kernel && d.device == dev) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                 (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess) done.push_back(Done{kernel, dev});
  return e;
}

// events (optional, 2 x DRV_LK_COUNT): slot k's kernel runs between
// events[2k] and events[2k + 1] (both recorded back to back for a slot the
// stage skips), so its time is elapsed(events[2k], events[2k + 1]) whatever
// order the slots run in.
template <int NK, bool BF16>
cudaError_t split_variant(cudaStream_t s, const StageParams& p, const PairList& L, const SurrogateArgs& sur,
                          const SplitKnobs& knobs, int num_sms, cudaEvent_t* ev, cudaEvent_t voxels_ready) {
  const int cone_ctas = knobs.cone_ctas_per_sm;
  const bool count_reads = knobs.count_voxel_reads;
  // Only the cone pass and the surrogate's features read the voxels: with
  // voxels_ready, the cull and the ordering passes overlap the voxel build.
  auto wait_voxels = [&]() { return voxels_ready ? cudaStreamWaitEvent(s, voxels_ready, 0) : cudaSuccess; };
  auto begin = [&](int k) { return ev ? cudaEventRecord(ev[2 * k], s) : cudaSuccess; };
  auto end = [&](int k) { return ev ? cudaEventRecord(ev[2 * k + 1], s) : cudaSuccess; };
  auto skip = [&](int k) {
    cudaError_t r = begin(k);
    return r == cudaSuccess ? end(k) : r;
  };
  cudaError_t e = cudaMemsetAsync(L.counters, 0, kPairCounters * sizeof(uint32_t), s);
  if (e != cudaSuccess || (e = begin(DRV_LK_CULL)) != cudaSuccess) return e;
  int total_vpls = 0;
  for (int l = 0; l < p.ll.n_lights; ++l) total_vpls += p.ll.lights[l].n_vpls;
  const int words = (p.total_blocks + 31) >> 5;
  const int K = knobs.cull_caches_per_pass;
  const size_t rec_smem = cull_records_smem(total_vpls, words, K);
  if (rec_smem <= kCullRecMaxSmem) {
    bool unit = true, copy = true;
    for (int l = 0; l < p.ll.n_lights; ++l) {
      unit = unit && p.ll.lights[l].interval == 1;
      copy = copy && p.ll.lights[l].records != nullptr;
    }
    auto kernel = cull_kernel_for<BF16>(unit, copy, K);
    if ((e = set_max_smem(reinterpret_cast<const void*>(kernel), kCullRecMaxSmem)) != cudaSuccess) return e;
    e = launch_persistent(kernel, kCullRecThreads, rec_smem, s, num_sms, p, L, total_vpls);
  } else {
    const size_t cull_smem = (size_t)words * 2 * sizeof(uint32_t);
    e = launch_persistent(cull_kernel<BF16>, kCullThreads, cull_smem, s, num_sms, p, L);
  }
  if (e != cudaSuccess || (e = end(DRV_LK_CULL)) != cudaSuccess) return e;
  if (sur.weights) {
    // The MLP first: it sets the confident pairs' shadowing and marks the
    // others (cls 0); only those are classified, ordered and traced below.
    if ((e = wait_voxels()) != cudaSuccess || (e = begin(DRV_LK_MLP)) != cudaSuccess) return e;
    if ((e = launch_surrogate_mlp(s, p, L, sur, BF16, num_sms)) != cudaSuccess) return e;
    if ((e = end(DRV_LK_MLP)) != cudaSuccess) return e;
  }
  if ((e = begin(DRV_LK_CLASSIFY)) != cudaSuccess) return e;
  e = sur.weights ? launch_persistent_after(classify_kernel<BF16, true>, kClassThreads, 0, s, num_sms, p, L)
                  : launch_persistent_after(classify_kernel<BF16, false>, kClassThreads, 0, s, num_sms, p, L);
  if (e != cudaSuccess || (e = end(DRV_LK_CLASSIFY)) != cudaSuccess) return e;
  if ((e = begin(DRV_LK_SCATTER)) != cudaSuccess) return e;
  if ((e = launch_persistent_after(scatter_kernel, kClassThreads, 0, s, num_sms, L)) != cudaSuccess) return e;
  if ((e = end(DRV_LK_SCATTER)) != cudaSuccess) return e;
  if (!sur.weights && ((e = skip(DRV_LK_MLP)) != cudaSuccess || (e = wait_voxels()) != cudaSuccess)) return e;
  if ((e = begin(DRV_LK_CONE)) != cudaSuccess) return e;
  e = count_reads ? launch_grid(cone_kernel<BF16, true>, 128, 0, s, num_sms, cone_ctas, true, p, L)
                  : launch_grid(cone_kernel<BF16, false>, 128, 0, s, num_sms, cone_ctas, true, p, L);
  if (e != cudaSuccess || (e = end(DRV_LK_CONE)) != cudaSuccess || (e = begin(DRV_LK_GATHER)) != cudaSuccess) return e;
  {
    const uint32_t staged = gather_staged_vpls(p.ll, BF16);
    const size_t smem = (size_t)staged * vpl_bytes<BF16>();
    auto kernel = knobs.gather_threads == 256 ? gather_kernel<NK, BF16, 256> : gather_kernel<NK, BF16, 512>;
    if ((e = set_max_smem(reinterpret_cast<const void*>(kernel), kGatherStageBytes)) != cudaSuccess) return e;
    e = launch_grid(kernel, knobs.gather_threads == 256 ? 256 : 512, smem, s, num_sms, knobs.gather_ctas_per_sm,
                    true, p, L, staged, knobs.gather_wait_test);
  }
  if (e != cudaSuccess) return e;
  return end(DRV_LK_GATHER);
}

}  // namespace

int resident_ctas(const void* kernel, int threads, size_t smem) {
  struct Entry {
    const void* kernel;
    int threads, device;
    size_t smem;
    int ctas;
  };
  static std::mutex mu;
  static std::vector<Entry> memo;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  for (const Entry& e : memo)
    if (e.kernel == kernel && e.threads == threads && e.smem == smem && e.device == dev) return e.ctas;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) return 0;
  memo.push_back(Entry{kernel, threads, dev, smem, n});
  return n;
}

int light_chunks(int total_blocks, int max_chunks) {
  int n = (total_blocks + kLightChunkMinBlocks - 1) / kLightChunkMinBlocks;
  return n < 1 ? 1 : (n > max_chunks ? max_chunks : n);
}

cudaError_t launch_light_caches(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                                const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                                const VoxelInputs& vox, const LightScratch& scratch, int num_sms) {
  FusedParams fp;
  fp.s = make_stage_params(cfg, vol, ll, counter, entries, entry_stride, vox);
  fp.n_chunks = light_chunks(fp.s.total_blocks, scratch.max_chunks);
  fp.chunk_blocks = (fp.s.total_blocks + fp.n_chunks - 1) / fp.n_chunks;
  fp.scratch = scratch.partials;
  fp.tickets = scratch.tickets;
  fp.work = scratch.work;
  const bool bf16 = cfg.precision == DRV_PRECISION_BF16;
  if (cfg.sh_order == 2)
    return bf16 ? launch_persistent(light_kernel<9, true>, kThreads, 0, s, num_sms, fp)
                : launch_persistent(light_kernel<9, false>, kThreads, 0, s, num_sms, fp);
  return bf16 ? launch_persistent(light_kernel<4, true>, kThreads, 0, s, num_sms, fp)
              : launch_persistent(light_kernel<4, false>, kThreads, 0, s, num_sms, fp);
}

bool light_split_supported(const DrvConfig& cfg, const LightLaunch& ll) {
  if (!cfg.indirect_shadow) return false;
  long blocks = 0;
  for (int l = 0; l < ll.n_lights; ++l) blocks += ll.lights[l].n_vpls / ll.lights[l].interval;
  return blocks >= 1 && blocks <= kMaxSplitBlocks;
}

cudaError_t launch_light_split(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                               const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                               const VoxelInputs& vox, const PairList& pairs, const SurrogateArgs& sur,
                               uint32_t* err, const SplitKnobs& knobs, int num_sms, cudaEvent_t* events,
                               cudaEvent_t voxels_ready) {
  StageParams p = make_stage_params(cfg, vol, ll, counter, entries, entry_stride, vox);
  p.err = err;
  const bool bf16 = cfg.precision == DRV_PRECISION_BF16;
  if (cfg.sh_order == 2)
    return bf16 ? split_variant<9, true>(s, p, pairs, sur, knobs, num_sms, events, voxels_ready)
                : split_variant<9, false>(s, p, pairs, sur, knobs, num_sms, events, voxels_ready);
  return bf16 ? split_variant<4, true>(s, p, pairs, sur, knobs, num_sms, events, voxels_ready)
              : split_variant<4, false>(s, p, pairs, sur, knobs, num_sms, events, voxels_ready);
}

}  // namespace drv
