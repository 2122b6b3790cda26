// k_apply.cu — Renderer::ApplyCaches (renderer.cpp:1047-1079) / cacheApply.frag:
// per pixel, trilinear interpolation of the irradiance of the 8 surrounding
// light caches (SampleCacheIrradiance, lightcache.glsl:137-179) times
// albedo / pi, with the optional cascade-transition blend.
//
// The reference reads the atlas and the entries without bounds checks
// (cacheApply.frag:264-284); here a corner outside the atlas, or whose slot is
// 0 (never allocated) or 0xFFFFFFFF (locked by a capacity overflow),
// contributes zero irradiance and its weight is not redistributed.
//
// With INDIRECT_SPECULAR (cacheApply.frag:76-116, 145-158) each corner cache
// also contributes its specular envmap, fetched trilinearly (the sampler is
// LINEAR/LINEAR/LINEAR, renderer.cpp:1070) at the concentric projection of
// the cache-local normal and the lod of the pixel's Blinn exponent, and the
// material splits into diffuse and specular colours by metallic.
#include <cmath>

#include <cuda_fp16.h>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "specular.cuh"

namespace drv {
namespace {

struct ApplyParams {
  DrvVolumeInfo vol;
  DrvPerFrame frame;
  const float* depth;
  const void* normal;
  int normal_format;
  const void* albedo;
  int albedo_format;
  const float* srgb;
  int w, h;
  int res, n_cascades, transitions, sh2;
  int bf16;  // DrvCacheEntryBF16 entries
  const uint32_t* atlas;
  const float* entries;
  int stride_floats;
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  float cl[5];  // ShCosLobeFactor0, 1, 2n2_p1_n1, 20, 2p2
  float* out;  // RGB F32, or RGBA16F (out_half)
  int out_half, out_add;
  CellRecip rc;
  SpecView spec;             // INDIRECT_SPECULAR only
  const void* rough_metal;   // drv_rough_metal_format
  int rm_f32;
  uint32_t* err;             // DRV_DEVERR_BOUNDS (nullptr: not reported)
};

// Where a pixel reads the corner caches' envmaps. The lookup coordinate and
// the lod are the pixel's, so the bilinear taps of each level — four texel
// offsets within a cache's region and their weights (GL 4.5 section 8.14.2,
// indices clamped to the region: the lookup is clamped half a texel of the
// coarser level inside it, so the clamp only meets zero weights) — are the
// same for all eight corner caches and are formed once.
struct EnvTaps {
  uint32_t at[4];  // (x0,y0), (x1,y0), (x0,y1), (x1,y1) within a cache's FP16 copy
  float w[4];
};

struct EnvLookup {
  EnvTaps t[2];  // level l0, level l1
  int l0, l1;
  float f;       // weight of level l1 (LINEAR mip filtering)
};

__device__ __forceinline__ EnvTaps env_taps(const SpecView& sv, int l, float u, float v) {
  const int side = sv.size >> l;
  const uint32_t stride = (uint32_t)side, base = sv.loff[l];
  const float x = u * (float)side - 0.5f, y = v * (float)side - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float a = x - fx, b = y - fy;
  const uint32_t x0 = (uint32_t)min(max((int)fx, 0), side - 1), x1 = (uint32_t)min(max((int)fx + 1, 0), side - 1);
  const uint32_t y0 = (uint32_t)min(max((int)fy, 0), side - 1), y1 = (uint32_t)min(max((int)fy + 1, 0), side - 1);
  EnvTaps t;
  t.at[0] = base + y0 * stride + x0;
  t.at[1] = base + y0 * stride + x1;
  t.at[2] = base + y1 * stride + x0;
  t.at[3] = base + y1 * stride + x1;
  t.w[0] = (1.0f - a) * (1.0f - b);
  t.w[1] = a * (1.0f - b);
  t.w[2] = (1.0f - a) * b;
  t.w[3] = a * b;
  return t;
}

// Reads the prepared FP16 copy of cache c (the atlas's values exactly).
__device__ __forceinline__ f3 env_bilinear(const uint2* half, const EnvTaps& t) {
  f3 r = mkf3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint2 q = __ldg(half + t.at[k]);
    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    const float b = __low2float(*reinterpret_cast<const __half2*>(&q.y));
    r = mkf3(r.x + t.w[k] * rg.x, r.y + t.w[k] * rg.y, r.z + t.w[k] * b);
  }
  return r;
}

// textureLod with LINEAR mip filtering: the two levels around the lod.
__device__ __forceinline__ f3 env_sample(const SpecView& sv, uint32_t c, const EnvLookup& q) {
  const uint2* half = sv.half + (size_t)c * sv.words;
  f3 r = env_bilinear(half, q.t[0]);
  if (q.f > 0.0f) {
    const f3 r1 = env_bilinear(half, q.t[1]);
    r = mkf3(r.x + (r1.x - r.x) * q.f, r.y + (r1.y - r.y) * q.f, r.z + (r1.z - r.z) * q.f);
  }
  return r;
}

template <bool BF16, bool SH2, bool SPEC>
__device__ __forceinline__ f3 lighting(const ApplyParams& p, const float wp[3], int c, f3 n, uint32_t n_caches,
                                       const EnvLookup& q, f3& spec) {
  const DrvCascade& k = p.vol.cascades[c];
  float wgt[3][2];
  int a0[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float a = div_exact(__fsub_rn(wp[i], k.min[i]), k.world_voxel_size, p.rc.inv_cell[c]);
    a0[i] = __float2int_rz(fminf(fmaxf(a, -1e9f), 1e9f));
    const float t = a - (float)a0[i];
    wgt[i][0] = 1.0f - t;
    wgt[i][1] = t;
  }
  const int aw = p.n_cascades * p.res;
  const int x0 = a0[0] + p.res * c, y0 = a0[1], z0 = a0[2];
  // Corner (ox, oy, oz) is inside the atlas when each axis is.
  const bool vx0 = x0 >= 0 && x0 < aw, vx1 = x0 + 1 >= 0 && x0 + 1 < aw;
  const bool vy0 = y0 >= 0 && y0 < p.res, vy1 = y0 + 1 >= 0 && y0 + 1 < p.res;
  const bool vz0 = z0 >= 0 && z0 < p.res, vz1 = z0 + 1 >= 0 && z0 + 1 < p.res;
  const long long base = ((long long)z0 * p.res + y0) * aw + x0;
  const long long plane = (long long)p.res * aw;
  uint32_t slot[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    // Corner order of cacheApply.frag:219-230: x fastest.
    const int ox = i & 1, oy = (i >> 1) & 1, oz = i >> 2;
    const bool v = (ox ? vx1 : vx0) && (oy ? vy1 : vy0) && (oz ? vz1 : vz0);
    slot[i] = v ? __ldg(p.atlas + (base + ox + oy * aw + oz * plane)) : 0u;
  }
  // Per-normal factors of SampleCacheIrradiance.
  const float f0 = p.cl[0];
  const float f1y = p.cl[1] * n.y, f1z = p.cl[1] * n.z, f1x = p.cl[1] * n.x;
  const float f4 = p.cl[2] * n.x * n.y, f5 = p.cl[2] * n.y * n.z, f6 = p.cl[3] * (n.z * n.z * 3.0f - 1.0f);
  const float f7 = p.cl[2] * n.x * n.z, f8 = p.cl[4] * (n.x * n.x - n.y * n.y);
  f3 irr = mkf3(0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t addr = slot[i];
    // unallocated, outside the atlas, or 0xFFFFFFFF (locked by an overflow);
    // any other index past the count is not read (the reference reads it
    // unchecked, cacheApply.frag:88-100) and is reported
    const bool live = addr != 0u && addr <= n_caches;
    if (addr > n_caches && addr != 0xFFFFFFFFu && p.err) raise_error(p.err, DRV_DEVERR_BOUNDS);
    const int ox = i & 1, oy = (i >> 1) & 1, oz = i >> 2;
    const float w = wgt[0][ox] * wgt[1][oy] * wgt[2][oz];
    float er = 0.0f, eg = 0.0f, eb = 0.0f;
    if (!live) {
    } else if (BF16) {
      // 27 BF16 values from byte 4 of the 64-byte entry, coefficient-major.
      const uint4* e = reinterpret_cast<const uint4*>(p.entries + (size_t)(addr - 1u) * p.stride_floats);
      const uint4 a = __ldg(e), b = __ldg(e + 1), cc = __ldg(e + 2), d = __ldg(e + 3);
      const uint32_t q[16] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, cc.y, cc.z, cc.w, d.x, d.y, d.z, d.w};
      float sh[27];
#pragma unroll
      for (int j = 0; j < 27; ++j) sh[j] = from_bf16((uint16_t)(q[1 + (j >> 1)] >> (16 * (j & 1))));
      er = sh[0] * f0 - sh[3] * f1y + sh[6] * f1z - sh[9] * f1x;
      eg = sh[1] * f0 - sh[4] * f1y + sh[7] * f1z - sh[10] * f1x;
      eb = sh[2] * f0 - sh[5] * f1y + sh[8] * f1z - sh[11] * f1x;
      if (SH2) {
        er += -sh[12] * f4 + sh[15] * f5 + sh[18] * f6 + sh[21] * f7 + sh[24] * f8;
        eg += -sh[13] * f4 + sh[16] * f5 + sh[19] * f6 + sh[22] * f7 + sh[25] * f8;
        eb += -sh[14] * f4 + sh[17] * f5 + sh[20] * f6 + sh[23] * f7 + sh[26] * f8;
      }
    } else {
      const float4* e = reinterpret_cast<const float4*>(p.entries + (size_t)(addr - 1u) * p.stride_floats);
      const float4 q1 = __ldg(e + 1), q2 = __ldg(e + 2), q3 = __ldg(e + 3);
      // q1 = {SH1neg1, SH00_r}, q2 = {SH10, SH00_g}, q3 = {SH1pos1, SH00_b}
      er = q1.w * f0 - q1.x * f1y + q2.x * f1z - q3.x * f1x;
      eg = q2.w * f0 - q1.y * f1y + q2.y * f1z - q3.y * f1x;
      eb = q3.w * f0 - q1.z * f1y + q2.z * f1z - q3.z * f1x;
      if (SH2) {
        const float4 q4 = __ldg(e + 4), q5 = __ldg(e + 5), q6 = __ldg(e + 6), q7 = __ldg(e + 7);
        // q4 = {SH2neg2, SH20_r}, q5 = {SH2neg1, SH20_g}, q6 = {SH2pos1, SH20_b}, q7 = {SH2pos2, pad}
        er += -q4.x * f4 + q5.x * f5 + q4.w * f6 + q6.x * f7 + q7.x * f8;
        eg += -q4.y * f4 + q5.y * f5 + q5.w * f6 + q6.y * f7 + q7.y * f8;
        eb += -q4.z * f4 + q5.z * f5 + q6.w * f6 + q6.z * f7 + q7.z * f8;
      }
    }
    irr.x += fmaxf(er, 0.0f) * w;
    irr.y += fmaxf(eg, 0.0f) * w;
    irr.z += fmaxf(eb, 0.0f) * w;
    if (SPEC && live) {
      const f3 e = env_sample(p.spec, addr - 1u, q);
      spec.x += e.x * w;
      spec.y += e.y * w;
      spec.z += e.z * w;
    }
  }
  return irr;
}

// The pixel's radiance into the target: RGB F32 or RGBA16F, written (alpha
// 1) or added (alpha kept; the sum in FP32, one rounding to FP16).
__device__ __forceinline__ void store_output(const ApplyParams& p, size_t i, f3 c) {
  if (p.out_half) {
    uint2* o = reinterpret_cast<uint2*>(p.out) + i;
    uint2 v = p.out_add ? *o : make_uint2(0u, 0u);
    if (p.out_add) {
      c.x += __half2float(__ushort_as_half((unsigned short)(v.x & 0xFFFFu)));
      c.y += __half2float(__ushort_as_half((unsigned short)(v.x >> 16)));
      c.z += __half2float(__ushort_as_half((unsigned short)(v.y & 0xFFFFu)));
    }
    const uint32_t hx = __half_as_ushort(__float2half_rn(c.x)), hy = __half_as_ushort(__float2half_rn(c.y)),
                   hz = __half_as_ushort(__float2half_rn(c.z));
    const uint32_t alpha = p.out_add ? (v.y >> 16) : 0x3C00u;  // written: alpha 1
    *o = make_uint2(hx | hy << 16, hz | alpha << 16);
    return;
  }
  float* o = p.out + 3 * i;
  if (p.out_add) {
    o[0] += c.x;
    o[1] += c.y;
    o[2] += c.z;
  } else {
    __stcs(o, c.x);
    __stcs(o + 1, c.y);
    __stcs(o + 2, c.z);
  }
}

// Five CTAs per SM (48 registers, a few bytes spilled) hide more of the
// corner loads' latency than four: 0.1215 -> 0.1152 ms (FP32) and 0.1052 ->
// 0.1013 ms (BF16) at 1080p; the specular instances at three (80 registers).
template <bool BF16, bool SH2, bool SPEC>
__global__ void __launch_bounds__(256, SPEC ? 3 : 5) apply_kernel(ApplyParams p) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= p.w || y >= p.h) return;
  const size_t i = (size_t)y * p.w + x;
  // G-buffer texels are read once and the output written once: streaming
  // (evict-first) accesses keep L1/L2 for the atlas and the cache entries.
  const float d = __ldcs(p.depth + i);
  // cacheApply.frag:304-307 (discard). A NaN depth counts as no geometry
  // too (the reference's test passes it and shades NaN).
  if (!(d >= 0.00001f)) {
    if (!p.out_add) store_output(p, i, mkf3(0.0f, 0.0f, 0.0f));
    return;
  }
  f3 n;
  if (p.normal_format == DRV_NORMAL_RG16I) {
    const int q = __ldcs(reinterpret_cast<const int*>(p.normal) + i);  // two int16, x in the low half
    n = unpack_normal16i((int16_t)(q & 0xFFFF), (int16_t)(q >> 16));
  } else {
    const float* q = reinterpret_cast<const float*>(p.normal) + 3 * i;
    n = mkf3(__ldcs(q), __ldcs(q + 1), __ldcs(q + 2));
  }
  const float inv_pi = 1.0f / DRV_SHADER_PI;
  const f3 a = load_albedo(p.albedo, p.albedo_format, p.srgb, i);
  f3 alb = mkf3(a.x * inv_pi, a.y * inv_pi, a.z * inv_pi);
  const uint32_t n_caches = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  float wp[3];
  reconstruct_world(p.frame, x, y, p.w, p.h, d, wp);
  const int c = select_cascade(p.vol, p.n_cascades, wp);
  EnvLookup q{};
  f3 spec_col = mkf3(0.0f, 0.0f, 0.0f);
  if (SPEC) {
    float rough, metal;
    if (p.rm_f32) {
      const float2 rm = __ldcs(reinterpret_cast<const float2*>(p.rough_metal) + i);
      rough = rm.x;
      metal = rm.y;
    } else {
      const unsigned short rm = __ldcs(reinterpret_cast<const unsigned short*>(p.rough_metal) + i);
      rough = (float)(rm & 0xFFu) / 255.0f;
      metal = (float)(rm >> 8) / 255.0f;
    }
    // ComputeMaterialColors (lightingfunctions.glsl:41-49): mix(x, y, a) = x (1 - a) + y a.
    alb = mkf3((a.x * (1.0f - metal) + 0.02f * metal) * inv_pi, (a.y * (1.0f - metal) + 0.02f * metal) * inv_pi,
               (a.z * (1.0f - metal) + 0.02f * metal) * inv_pi);
    spec_col = mkf3(0.04f * (1.0f - metal) + a.x * metal, 0.04f * (1.0f - metal) + a.y * metal,
                    0.04f * (1.0f - metal) + a.z * metal);
    // RoughnessToBlinnExponent, GetHemisphereLodForBlinnPhongExponent and
    // the lookup clamp of cacheApply.frag:150-157.
    const float rsq = rough * rough;
    const float blinn = 2.0f / (rsq * rsq + 0.0005f);
    const float S = (float)p.spec.size;
    const float lod = fmaxf(0.0f, log2f(S * S / (1.0f + blinn)) * 0.5f);
    const float half_px = 0.5f / (exp2f(-ceilf(lod)) * S);
    const LocalFrame fr = local_view_space(p.frame.camera_position, wp[0], wp[1], wp[2]);
    float u, v;
    hemi_projection(to_local(fr, n), u, v);
    u = fminf(fmaxf(u, half_px), 1.0f - half_px);
    v = fminf(fmaxf(v, half_px), 1.0f - half_px);
    const float fl = fminf(floorf(lod), (float)(p.spec.n_levels - 1));
    q.l0 = (int)fl;
    q.l1 = min(q.l0 + 1, p.spec.n_levels - 1);
    q.f = q.l1 > q.l0 ? lod - fl : 0.0f;
    q.t[0] = env_taps(p.spec, q.l0, u, v);
    if (q.f > 0.0f) q.t[1] = env_taps(p.spec, q.l1, u, v);
  }
  f3 spec = mkf3(0.0f, 0.0f, 0.0f);
  f3 irr = lighting<BF16, SH2, SPEC>(p, wp, c, n, n_caches, q, spec);
  f3 col = mkf3(irr.x * alb.x, irr.y * alb.y, irr.z * alb.z);
  if (SPEC) col = mkf3(col.x + spec.x * spec_col.x, col.y + spec.y * spec_col.y, col.z + spec.z * spec_col.z);
  if (p.transitions) {
    const float t = cascade_transition(p.vol, p.rc, c, wp);
    if (t > 0.0f && c < p.n_cascades - 1) {
      f3 spec2 = mkf3(0.0f, 0.0f, 0.0f);
      f3 irr2 = lighting<BF16, SH2, SPEC>(p, wp, c + 1, n, n_caches, q, spec2);
      f3 col2 = mkf3(irr2.x * alb.x, irr2.y * alb.y, irr2.z * alb.z);
      if (SPEC)
        col2 = mkf3(col2.x + spec2.x * spec_col.x, col2.y + spec2.y * spec_col.y, col2.z + spec2.z * spec_col.z);
      col = col * (1.0f - t) + col2 * t;  // mix(), cacheApply.frag:359
    }
  }
  store_output(p, i, col);
}

}  // namespace

cudaError_t launch_apply(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const DrvPerFrame& f,
                         const DrvGBufferView& g, const uint32_t* atlas, const void* entries, uint32_t entry_stride,
                         const DrvCacheCounter* counter, float* out_rgb, const float* srgb, const SpecView* spec,
                         uint32_t* err) {
  ApplyParams p{};
  p.err = err;
  p.rc = make_cell_recip(vol);
  p.vol = vol;
  p.frame = f;
  p.depth = g.depth;
  p.normal = g.normal;
  p.normal_format = g.normal_format;
  p.albedo = g.albedo;
  p.albedo_format = g.albedo_format;
  p.srgb = srgb;
  p.w = g.width;
  p.h = g.height;
  p.res = cfg.cav_res;
  p.n_cascades = cfg.n_cascades;
  p.transitions = cfg.cascade_transition > 0.0f;
  p.sh2 = cfg.sh_order == 2;
  p.bf16 = cfg.precision == DRV_PRECISION_BF16;
  p.atlas = atlas;
  p.entries = (const float*)entries;
  p.stride_floats = (int)(entry_stride / 4);
  p.counter = counter;
  p.max_caches = cfg.max_caches;
  const double kPi = 3.14159265358979323846;
  p.cl[0] = (float)(std::sqrt(kPi) / 2.0);
  p.cl[1] = (float)std::sqrt(kPi / 3.0);
  p.cl[2] = (float)((cfg.sh2_sign == DRV_SH2_SIGN_FIXED ? 1.0 : -1.0) * std::sqrt(15.0 * kPi) / 8.0);
  p.cl[3] = (float)(std::sqrt(5.0 * kPi) / 16.0);
  p.cl[4] = (float)(std::sqrt(15.0 * kPi) / 16.0);
  p.out = out_rgb;
  p.out_half = cfg.output_format == DRV_OUTPUT_RGBA16F;
  p.out_add = cfg.output_blend == DRV_OUTPUT_ADD;
  dim3 block(16, 16), grid((g.width + 15) / 16, (g.height + 15) / 16);
  if (spec) {
    p.spec = *spec;
    p.rough_metal = g.rough_metal;
    p.rm_f32 = g.rough_metal_format == DRV_ROUGH_METAL_F32;
    if (p.bf16)
      p.sh2 ? apply_kernel<true, true, true><<<grid, block, 0, s>>>(p)
            : apply_kernel<true, false, true><<<grid, block, 0, s>>>(p);
    else
      p.sh2 ? apply_kernel<false, true, true><<<grid, block, 0, s>>>(p)
            : apply_kernel<false, false, true><<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
  }
  if (p.bf16)
    p.sh2 ? apply_kernel<true, true, false><<<grid, block, 0, s>>>(p)
          : apply_kernel<true, false, false><<<grid, block, 0, s>>>(p);
  else
    p.sh2 ? apply_kernel<false, true, false><<<grid, block, 0, s>>>(p)
          : apply_kernel<false, false, false><<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace drv
