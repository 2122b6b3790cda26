// k_specular.cu — the indirect-specular path (INDIRECT_SPECULAR) of
// Renderer::LightCachesRSM and Renderer::PrepareSpecularEnvmaps:
//
//  * specular_kernel (a CTA per cache) fills each allocated cache's level-0
//    envmap: every contributing VPL adds its reflected radiance,
//    radianceIn * saturate(h . l), to the texel the cache-local half vector h
//    projects to, and the sum is scaled by the base level's Blinn
//    normalisation (cacheLightingRSM.comp:87-98, 310-335, 376-383). The
//    shadowing is the light stage's: the pair list's cone results after the
//    split stage, otherwise the cones traced here (or 1 without indirect
//    shadow).
//  * envmap_prepare_kernel (a CTA per cache) computes the mip levels
//    (specularenvmap_mipmap.frag) and the optional hole fill
//    (specularenvmap_fillholes.frag) of each allocated cache's envmap, and
//    writes the apply's per-cache FP16 copy of every level (R11/G11/B10
//    values are FP16 values, so the copy is exact and the apply reads its
//    texels without unpacking).
//
// Differences from the reference, each exact to FP32 rounding or documented:
//  - the sum is formed in FP32 and rounded to R11F_G11F_B10F once (the
//    reference's direct write rounds after every added VPL);
//  - the texel coordinate ivec2(proj * size + 0.5) is clamped to size - 1
//    (the reference's can reach size, a texel of the neighbouring cache);
//  - the atlas is not cleared: every allocated cache's region is written
//    whole, and only allocated caches are read.
//
// The sum is deterministic: each warp accumulates into its own shared copy of
// the envmap; within a warp the lanes that hit the same texel are summed in
// lane order by the lowest of them; the copies are added in warp order.
#include <cuda_fp16.h>

#include "drv_internal.h"
#include "light_common.cuh"
#include "specular.cuh"

namespace drv {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Warps (envmap copies) per CTA for envmap side `size`: 8 up to 32, 4 for 64.
inline int spec_warps(int size) { return size <= 32 ? 8 : 4; }

template <bool BF16>
__global__ void __launch_bounds__(256) specular_kernel(StageParams p, PairList L, SpecView sv, int use_list) {
  extern __shared__ float s_env[];  // [warps][size * size][3]
  const int n_warps = (int)(blockDim.x >> 5);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = sv.size, nt = S * S;
  float* mine = s_env + (size_t)warp * nt * 3;
  const uint32_t n_caches = cache_count(p);
  for (uint32_t c = blockIdx.x; c < n_caches; c += gridDim.x) {
    for (int i = threadIdx.x; i < n_warps * nt * 3; i += blockDim.x) s_env[i] = 0.0f;
    __syncthreads();
    float cx, cy, cz;
    cache_position<BF16>(p, c, cx, cy, cz);
    const LocalFrame fr = local_view_space(sv.cam, cx, cy, cz);
    const uint32_t first = use_list ? L.info[2 * c] : 0u;
    const uint32_t count = use_list ? L.info[2 * c + 1] : kPairOverflow;
    const bool listed = count != kPairOverflow;
    const uint32_t n_units = listed ? count : (uint32_t)p.total_blocks;
    // Unit u (a listed pair, or a shadow block) goes to warp (u / 32) % n_warps, lane u % 32.
    for (uint32_t base = 0; base < n_units; base += 32u * (uint32_t)n_warps) {
      const uint32_t u = base + (uint32_t)warp * 32u + (uint32_t)lane;
      bool have = u < n_units;
      int b = 0;
      float shadowing = 1.0f;
      if (have) {
        if (listed) {
          b = (int)L.block[first + u];
          shadowing = L.shadow[first + u];
        } else {
          b = (int)u;
          have = block_live<BF16>(p, b, cx, cy, cz);
          if (have && p.shadow) shadowing = block_cone(p, b, cx, cy, cz);
        }
      }
      if (!__any_sync(kFull, have)) continue;
      const int l = have ? block_light(p, b) : 0;
      const LightArgs& la = p.ll.lights[l];
      const int interval = have ? la.interval : 0;
      const int lb = have ? b - p.block_base[l] : 0;
      const int jmax = (int)__reduce_max_sync(kFull, (unsigned)interval);
      for (int j = 0; j < jmax; ++j) {
        bool valid = false;
        int texel = 0;
        float r = 0.0f, g = 0.0f, bl = 0.0f;
        if (j < interval) {
          const VplData v = load_vpl<BF16>(la.vpls, lb * interval + j);
          const Transfer t = transfer(v, cx, cy, cz);
          if (contributes(v, t) && flux_ok(p, v)) {
            // Cache-local direction to the VPL and half vector with the
            // direction to the camera, (0, 0, 1) in cache-local space.
            const f3 tl = to_local(fr, mkf3(t.tx, t.ty, t.tz));
            f3 h = mkf3(tl.x, tl.y, tl.z + 1.0f);
            const float hl2 = dot3(h, h);
            if (hl2 > 0.0f) {
              h = h * rsqrtf(hl2);
              float pu, pv;
              hemi_projection(h, pu, pv);
              const int tx = min(max((int)(pu * (float)S + 0.5f), 0), S - 1);
              const int ty = min(max((int)(pv * (float)S + 0.5f), 0), S - 1);
              // radianceIn * saturate(h . l); radianceIn = flux * g * shadowing
              const float k = t.g * shadowing * sat(dot3(h, tl));
              r = v.fr * k;
              g = v.fg * k;
              bl = v.fb * k;
              texel = ty * S + tx;
              valid = true;
            }
          }
        }
        if (__any_sync(kFull, valid)) {
          const unsigned peers = __match_any_sync(kFull, valid ? texel : (1 << 20) + lane);
          float sr = 0.0f, sg = 0.0f, sb = 0.0f;
#pragma unroll 4
          for (int k = 0; k < 32; ++k) {
            const float qr = __shfl_sync(kFull, r, k), qg = __shfl_sync(kFull, g, k), qb = __shfl_sync(kFull, bl, k);
            if ((peers >> k) & 1u) {
              sr += qr;
              sg += qg;
              sb += qb;
            }
          }
          if (valid && lane == __ffs(peers) - 1) {
            mine[3 * texel] += sr;
            mine[3 * texel + 1] += sg;
            mine[3 * texel + 2] += sb;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      float r = 0.0f, g = 0.0f, bl = 0.0f;
      for (int w = 0; w < n_warps; ++w) {
        const float* e = s_env + ((size_t)w * nt + t) * 3;
        r += e[0];
        g += e[1];
        bl += e[2];
      }
      sv.levels[env_index(sv, c, 0, t % S, t / S)] = encode_r11g11b10(mkf3(r * sv.norm, g * sv.norm, bl * sv.norm));
    }
    __syncthreads();
  }
}

// Mip levels and hole fill of each allocated cache's envmap, all levels of a
// cache held in shared memory (texel words, level l at loff[l]).
__global__ void __launch_bounds__(256) envmap_prepare_kernel(SpecView sv, const DrvCacheCounter* counter,
                                                             uint32_t max_caches, int fill) {
  extern __shared__ uint32_t s_lv[];
  const int S = sv.size, L = sv.n_levels;
  int loff[8];
  loff[0] = 0;
  for (int l = 1; l < 8; ++l) loff[l] = l < L ? loff[l - 1] + (S >> (l - 1)) * (S >> (l - 1)) : loff[l - 1];
  const uint32_t n_caches = min((uint32_t)max(counter->total_light_cache_count, 0), max_caches);
  for (uint32_t c = blockIdx.x; c < n_caches; c += gridDim.x) {
    for (int t = threadIdx.x; t < S * S; t += blockDim.x) s_lv[t] = sv.levels[env_index(sv, c, 0, t % S, t / S)];
    __syncthreads();
    // specularenvmap_mipmap.frag: level l texel = the mean of its 2x2 texels
    // of level l - 1 (a bilinear fetch at their common corner).
    for (int l = 1; l < L; ++l) {
      const int side = S >> l, below = side * 2;
      const uint32_t* src = s_lv + loff[l - 1];
      for (int t = threadIdx.x; t < side * side; t += blockDim.x) {
        const int x = t % side, y = t / side;
        const f3 a = decode_r11g11b10_fast(src[(2 * y) * below + 2 * x]);
        const f3 b = decode_r11g11b10_fast(src[(2 * y) * below + 2 * x + 1]);
        const f3 cc = decode_r11g11b10_fast(src[(2 * y + 1) * below + 2 * x]);
        const f3 d = decode_r11g11b10_fast(src[(2 * y + 1) * below + 2 * x + 1]);
        s_lv[loff[l] + t] = encode_r11g11b10(mkf3(0.25f * ((a.x + b.x) + (cc.x + d.x)),
                                                  0.25f * ((a.y + b.y) + (cc.y + d.y)),
                                                  0.25f * ((a.z + b.z) + (cc.z + d.z))));
      }
      __syncthreads();
    }
    // specularenvmap_fillholes.frag, from level `fill` down to 1: zero texels
    // of level i - 1 take their parent's colour, and the four are rescaled so
    // that their mean keeps the parent's energy.
    for (int i = fill; i > 0; --i) {
      const int side = S >> i, below = side * 2;
      uint32_t* dst = s_lv + loff[i - 1];
      for (int t = threadIdx.x; t < side * side; t += blockDim.x) {
        const int x = t % side, y = t / side;
        const f3 sc = decode_r11g11b10_fast(s_lv[loff[i] + t]);
        if (sc.x + sc.y + sc.z < 0.0001f) continue;
        const int at[4] = {(2 * y) * below + 2 * x, (2 * y) * below + 2 * x + 1, (2 * y + 1) * below + 2 * x,
                           (2 * y + 1) * below + 2 * x + 1};
        f3 dc[4];
        f3 sum = mkf3(0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          dc[k] = decode_r11g11b10_fast(dst[at[k]]);
          if (dc[k].x + dc[k].y + dc[k].z == 0.0f) dc[k] = sc;
          sum = mkf3(sum.x + dc[k].x, sum.y + dc[k].y, sum.z + dc[k].z);
        }
        sum = mkf3(sum.x + 0.00001f, sum.y + 0.00001f, sum.z + 0.00001f);
        const f3 k4 = mkf3(4.0f * sc.x / sum.x, 4.0f * sc.y / sum.y, 4.0f * sc.z / sum.z);
#pragma unroll
        for (int k = 0; k < 4; ++k) dst[at[k]] = encode_r11g11b10(mkf3(dc[k].x * k4.x, dc[k].y * k4.y, dc[k].z * k4.z));
      }
      __syncthreads();
    }
    for (int l = fill > 0 ? 0 : 1; l < L; ++l) {
      const int side = S >> l;
      for (int t = threadIdx.x; t < side * side; t += blockDim.x)
        sv.levels[env_index(sv, c, l, t % side, t / side)] = s_lv[loff[l] + t];
    }
    // The apply's FP16 copy of all levels (the same values).
    for (uint32_t t = threadIdx.x; t < sv.words; t += blockDim.x) {
      const f3 e = decode_r11g11b10_fast(s_lv[t]);
      const __half2 rg = __floats2half2_rn(e.x, e.y), b0 = __floats2half2_rn(e.z, 0.0f);
      sv.half[(size_t)c * sv.words + t] = make_uint2(*reinterpret_cast<const uint32_t*>(&rg),
                                                     *reinterpret_cast<const uint32_t*>(&b0));
    }
    __syncthreads();
  }
}

template <typename K>
cudaError_t launch_with_smem(K kernel, int threads, size_t smem, cudaStream_t s, int num_sms, const StageParams* p,
                             const PairList* L, const SpecView& sv, int use_list) {
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024 &&
      (e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return e;
  const int per_sm = resident_ctas(reinterpret_cast<const void*>(kernel), threads, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kernel<<<num_sms * per_sm, threads, smem, s>>>(*p, *L, sv, use_list);
  return cudaGetLastError();
}

}  // namespace

SpecView make_spec_view(const DrvConfig& cfg, uint32_t* levels, const uint32_t off[8], int atlas, uint2* half,
                        const DrvPerFrame& f) {
  SpecView v{};
  v.levels = levels;
  v.half = half;
  for (int l = 0; l < 8; ++l) v.off[l] = off[l];
  v.size = cfg.specular_envmap_size;
  int lg = 0;
  while ((1 << (lg + 1)) <= v.size) ++lg;
  v.log2size = lg;
  v.n_levels = lg + 1;
  v.atlas = atlas;
  v.per_row = v.size > 0 ? atlas / v.size : 0;
  // GetBlinnPhongExponentForHemispherePixel (concentric map): size^2 - 1;
  // BlinnNormalization: (e + 8) / (8 pi).
  const double e = (double)v.size * v.size - 1.0;
  v.norm = (float)((e + 8.0) / (8.0 * 3.14159265358979323846));
  for (int i = 0; i < 3; ++i) v.cam[i] = f.camera_position[i];
  uint32_t w = 0;
  for (int l = 0; l < 8; ++l) {
    v.loff[l] = w;
    if (l < v.n_levels) w += (uint32_t)(v.size >> l) * (uint32_t)(v.size >> l);
  }
  v.words = w;
  return v;
}

cudaError_t launch_specular_gather(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol,
                                   const LightLaunch& ll, const DrvCacheCounter* counter, void* entries,
                                   uint32_t entry_stride, const VoxelInputs& vox, const PairList* pairs,
                                   const SpecView& sv, int num_sms) {
  const StageParams p = make_stage_params(cfg, vol, ll, counter, entries, entry_stride, vox);
  const int warps = spec_warps(sv.size);
  const size_t smem = (size_t)warps * sv.size * sv.size * 3 * sizeof(float);
  const PairList none{};
  const PairList& L = pairs ? *pairs : none;
  const int use_list = pairs != nullptr;
  if (cfg.precision == DRV_PRECISION_BF16)
    return launch_with_smem(specular_kernel<true>, warps * 32, smem, s, num_sms, &p, &L, sv, use_list);
  return launch_with_smem(specular_kernel<false>, warps * 32, smem, s, num_sms, &p, &L, sv, use_list);
}

cudaError_t launch_envmap_prepare(cudaStream_t s, const SpecView& sv, const DrvCacheCounter* counter,
                                  uint32_t max_caches, int fill, int num_sms) {
  size_t words = 0;
  for (int l = 0; l < sv.n_levels; ++l) words += (size_t)(sv.size >> l) * (sv.size >> l);
  const size_t smem = words * sizeof(uint32_t);
  const int per_sm = resident_ctas(reinterpret_cast<const void*>(envmap_prepare_kernel), 256, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  envmap_prepare_kernel<<<num_sms * per_sm, 256, smem, s>>>(sv, counter, max_caches, fill);
  return cudaGetLastError();
}

}  // namespace drv
