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
  // Per-normal factors of SampleCacheIrradiance, with the signs of its terms
  // (SH1neg1, SH1pos1 and SH2neg2 enter negated) folded in.
  const float f0 = p.cl[0];
  const float f1y = -(p.cl[1] * n.y), f1z = p.cl[1] * n.z, f1x = -(p.cl[1] * n.x);
  const float f4 = -(p.cl[2] * n.x * n.y), f5 = p.cl[2] * n.y * n.z, f6 = p.cl[3] * (n.z * n.z * 3.0f - 1.0f);
  const float f7 = p.cl[2] * n.x * n.z, f8 = p.cl[4] * (n.x * n.x - n.y * n.y);
  // Red and green are summed as one packed pair, blue alone.
  auto pair = [](float v) { return make_float2(v, v); };
  float2 irr_rg = make_float2(0.f, 0.f);
  float irr_b = 0.0f;
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
    float2 erg = make_float2(0.0f, 0.0f);
    float eb = 0.0f;
    if (!live) {
    } else if (BF16) {
      // 27 BF16 values from byte 4 of the 64-byte entry, coefficient-major.
      const uint4* e = reinterpret_cast<const uint4*>(p.entries + (size_t)(addr - 1u) * p.stride_floats);
      const uint4 a = __ldg(e), b = __ldg(e + 1), cc = __ldg(e + 2), d = __ldg(e + 3);
      const uint32_t q[16] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, cc.y, cc.z, cc.w, d.x, d.y, d.z, d.w};
      float sh[27];
#pragma unroll
      for (int j = 0; j < 27; ++j) sh[j] = from_bf16((uint16_t)(q[1 + (j >> 1)] >> (16 * (j & 1))));
      auto rg = [&](int k) { return make_float2(sh[3 * k], sh[3 * k + 1]); };
      erg = mul2(rg(0), pair(f0));
      erg = fma2(rg(1), pair(f1y), erg);
      erg = fma2(rg(2), pair(f1z), erg);
      erg = fma2(rg(3), pair(f1x), erg);
      eb = __fmaf_rn(sh[11], f1x, __fmaf_rn(sh[8], f1z, __fmaf_rn(sh[5], f1y, __fmul_rn(sh[2], f0))));
      if (SH2) {
        erg = fma2(rg(4), pair(f4), erg);
        erg = fma2(rg(5), pair(f5), erg);
        erg = fma2(rg(6), pair(f6), erg);
        erg = fma2(rg(7), pair(f7), erg);
        erg = fma2(rg(8), pair(f8), erg);
        eb = __fmaf_rn(sh[26], f8, __fmaf_rn(sh[23], f7, __fmaf_rn(sh[20], f6, __fmaf_rn(sh[17], f5,
                       __fmaf_rn(sh[14], f4, eb)))));
      }
    } else {
      const float4* e = reinterpret_cast<const float4*>(p.entries + (size_t)(addr - 1u) * p.stride_floats);
      const float4 q1 = __ldg(e + 1), q2 = __ldg(e + 2), q3 = __ldg(e + 3);
      // q1 = {SH1neg1, SH00_r}, q2 = {SH10, SH00_g}, q3 = {SH1pos1, SH00_b}
      erg = mul2(make_float2(q1.w, q2.w), pair(f0));
      erg = fma2(make_float2(q1.x, q1.y), pair(f1y), erg);
      erg = fma2(make_float2(q2.x, q2.y), pair(f1z), erg);
      erg = fma2(make_float2(q3.x, q3.y), pair(f1x), erg);
      eb = __fmaf_rn(q3.z, f1x, __fmaf_rn(q2.z, f1z, __fmaf_rn(q1.z, f1y, __fmul_rn(q3.w, f0))));
      if (SH2) {
        const float4 q4 = __ldg(e + 4), q5 = __ldg(e + 5), q6 = __ldg(e + 6), q7 = __ldg(e + 7);
        // q4 = {SH2neg2, SH20_r}, q5 = {SH2neg1, SH20_g}, q6 = {SH2pos1, SH20_b}, q7 = {SH2pos2, pad}
        erg = fma2(make_float2(q4.x, q4.y), pair(f4), erg);
        erg = fma2(make_float2(q5.x, q5.y), pair(f5), erg);
        erg = fma2(make_float2(q4.w, q5.w), pair(f6), erg);
        erg = fma2(make_float2(q6.x, q6.y), pair(f7), erg);
        erg = fma2(make_float2(q7.x, q7.y), pair(f8), erg);
        eb = __fmaf_rn(q7.z, f8, __fmaf_rn(q6.z, f7, __fmaf_rn(q6.w, f6, __fmaf_rn(q5.z, f5,
                       __fmaf_rn(q4.z, f4, eb)))));
      }
    }
    irr_rg = fma2(make_float2(fmaxf(erg.x, 0.0f), fmaxf(erg.y, 0.0f)), pair(w), irr_rg);
    irr_b = __fmaf_rn(fmaxf(eb, 0.0f), w, irr_b);
    if (SPEC && live) {
      const f3 e = env_sample(p.spec, addr - 1u, q);
      spec.x += e.x * w;
      spec.y += e.y * w;
      spec.z += e.z * w;
    }
  }
  return mkf3(irr_rg.x, irr_rg.y, irr_b);
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

// ---------------------------------------------------------- tensor-core form
// BF16 entries without specular: the 8 corners' irradiance of a whole warp of
// pixels on the tensor cores. E_ch(pixel, corner) = sum_k F_k(n) SH_k,ch
// (SampleCacheIrradiance, lightcache.glsl:137-179, with the signs of its terms
// folded into F) is a product of a [pixels x 9] matrix of per-pixel factors and
// a [9 x corners] matrix of one cell's SH per channel. The warp (a 16 x 2 pixel
// tile) groups its pixels by cell (cascade and base corner; almost always one
// or two groups); per group, lane (g, t) loads corner g's BF16 entry as the B
// fragment, and mma.sync m16n8k16 (BF16 operands, FP32 accumulation) gives
// every pixel's 8 corner irradiances for each channel. F is split into BF16
// hi + lo parts (two MMAs), so the products keep about 16 bits of F; the SH
// values are the stored BF16 ones exactly. The clamp at zero, the trilinear
// weights and the sum over corners follow on the accumulators (quad shuffles).
// The sum's order differs from the per-pixel form's (FP32 rounding).
constexpr int kTcRow = 24;  // BF16 values per shared-memory row: 16 used + 8 pad (conflict-free ldmatrix)

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <bool SH2>
__global__ void __launch_bounds__(256, 3) apply_tc_kernel(ApplyParams p) {
  constexpr int NK = SH2 ? 9 : 4;
  __shared__ __align__(16) uint16_t s_f[8][2][32 * kTcRow];  // per warp: F hi rows, F lo rows
  const int tid = threadIdx.y * 16 + threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  const bool inside = x < p.w && y < p.h;
  const size_t i = inside ? (size_t)y * p.w + x : 0;
  const float d = inside ? __ldcs(p.depth + i) : 0.0f;
  // cacheApply.frag:304-307 (discard); a NaN depth counts as no geometry.
  const bool geom = inside && d >= 0.00001f;
  f3 n = mkf3(0.0f, 0.0f, 1.0f), alb = mkf3(0.0f, 0.0f, 0.0f);
  float wp[3] = {0.0f, 0.0f, 0.0f};
  int c = 0;
  if (geom) {
    if (p.normal_format == DRV_NORMAL_RG16I) {
      const int q = __ldcs(reinterpret_cast<const int*>(p.normal) + i);
      n = unpack_normal16i((int16_t)(q & 0xFFFF), (int16_t)(q >> 16));
    } else {
      const float* q = reinterpret_cast<const float*>(p.normal) + 3 * i;
      n = mkf3(__ldcs(q), __ldcs(q + 1), __ldcs(q + 2));
    }
    const float inv_pi = 1.0f / DRV_SHADER_PI;
    const f3 a = load_albedo(p.albedo, p.albedo_format, p.srgb, i);
    alb = mkf3(a.x * inv_pi, a.y * inv_pi, a.z * inv_pi);
    reconstruct_world(p.frame, x, y, p.w, p.h, d, wp);
    c = select_cascade(p.vol, p.n_cascades, wp);
  }
  // Per-normal factors of SampleCacheIrradiance, signs folded in (0 without geometry).
  float F[16];
  {
    const float f1y = p.cl[1] * n.y, f1z = p.cl[1] * n.z, f1x = p.cl[1] * n.x;
    F[0] = p.cl[0];
    F[1] = -f1y;
    F[2] = f1z;
    F[3] = -f1x;
    F[4] = -(p.cl[2] * n.x * n.y);
    F[5] = p.cl[2] * n.y * n.z;
    F[6] = p.cl[3] * (n.z * n.z * 3.0f - 1.0f);
    F[7] = p.cl[2] * n.x * n.z;
    F[8] = p.cl[4] * (n.x * n.x - n.y * n.y);
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k >= NK || !geom) F[k] = 0.0f;
  }
  {
    uint32_t hi[8], lo[8];
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
      const uint16_t h0 = to_bf16(F[k]), h1 = to_bf16(F[k + 1]);
      const uint16_t l0 = to_bf16(F[k] - from_bf16(h0)), l1 = to_bf16(F[k + 1] - from_bf16(h1));
      hi[k / 2] = (uint32_t)h0 | (uint32_t)h1 << 16;
      lo[k / 2] = (uint32_t)l0 | (uint32_t)l1 << 16;
    }
    uint4* rh = reinterpret_cast<uint4*>(s_f[warp][0] + lane * kTcRow);
    uint4* rl = reinterpret_cast<uint4*>(s_f[warp][1] + lane * kTcRow);
    rh[0] = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    rh[1] = make_uint4(hi[4], hi[5], hi[6], hi[7]);
    rl[0] = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    rl[1] = make_uint4(lo[4], lo[5], lo[6], lo[7]);
  }
  __syncwarp();
  // A fragments of the two 16-pixel halves of the warp, hi and lo.
  uint32_t ah[2][4], al[2][4];
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const int row = 16 * m + (lane & 7) + ((lane >> 3) & 1) * 8, col = ((lane >> 4) & 1) * 8;
    ldsm_x4(ah[m], (uint32_t)__cvta_generic_to_shared(s_f[warp][0] + row * kTcRow + col));
    ldsm_x4(al[m], (uint32_t)__cvta_generic_to_shared(s_f[warp][1] + row * kTcRow + col));
  }
  const uint32_t n_caches = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  const int g = lane >> 2, t = lane & 3;
  const int aw = p.n_cascades * p.res;
  float tmix = 0.0f;
  bool in_tr = false;
  if (geom && p.transitions) {
    tmix = cascade_transition(p.vol, p.rc, c, wp);
    in_tr = tmix > 0.0f && c < p.n_cascades - 1;
  }
  f3 col = mkf3(0.0f, 0.0f, 0.0f);
  for (int call = 0; call < 2; ++call) {
    const bool part = geom && (call == 0 || in_tr);
    if (call == 1 && !__any_sync(0xffffffffu, part)) break;
    const int cc = c + call;
    // The pixel's cell in cascade cc and its trilinear fractions.
    int a0[3] = {0, 0, 0};
    float fr[3] = {0.0f, 0.0f, 0.0f};
    if (part) {
      const DrvCascade& k = p.vol.cascades[cc];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float a = div_exact(__fsub_rn(wp[j], k.min[j]), k.world_voxel_size, p.rc.inv_cell[cc]);
        a0[j] = __float2int_rz(fminf(fmaxf(a, -1e9f), 1e9f));
        fr[j] = a - (float)a0[j];
      }
    }
    const unsigned long long key =
        part ? ((unsigned long long)(uint32_t)cc << 60) | ((unsigned long long)((uint32_t)a0[0] & 0xFFFFFu) << 40) |
                   ((unsigned long long)((uint32_t)a0[1] & 0xFFFFFu) << 20) | (unsigned long long)((uint32_t)a0[2] & 0xFFFFFu)
             : ~0ull;
    f3 irr = mkf3(0.0f, 0.0f, 0.0f);
    uint32_t remaining = __ballot_sync(0xffffffffu, part);
    while (remaining) {
      const int leader = __ffs(remaining) - 1;
      const unsigned long long gk = __shfl_sync(0xffffffffu, key, leader);
      const bool member = part && key == gk;
      remaining &= ~__ballot_sync(0xffffffffu, member);
      // Corner g of the group's cell (x fastest, cacheApply.frag:219-230).
      const int gc = __shfl_sync(0xffffffffu, cc, leader);
      const int gx = __shfl_sync(0xffffffffu, a0[0], leader) + (g & 1) + p.res * gc;
      const int gy = __shfl_sync(0xffffffffu, a0[1], leader) + ((g >> 1) & 1);
      const int gz = __shfl_sync(0xffffffffu, a0[2], leader) + (g >> 2);
      const bool inside_atlas = gx >= 0 && gx < aw && gy >= 0 && gy < p.res && gz >= 0 && gz < p.res;
      const uint32_t slot = inside_atlas ? __ldg(p.atlas + ((size_t)gz * p.res + gy) * aw + gx) : 0u;
      const bool live = slot != 0u && slot <= n_caches;
      if (slot > n_caches && slot != 0xFFFFFFFFu && p.err && t == 0) raise_error(p.err, DRV_DEVERR_BOUNDS);
      // B fragments: rows k = 2t, 2t + 1 (and 8 for t = 0), column g.
      uint32_t b0[3] = {0u, 0u, 0u}, b1[3] = {0u, 0u, 0u};
      if (live) {
        const uint16_t* sh = reinterpret_cast<const uint16_t*>(p.entries + (size_t)(slot - 1u) * p.stride_floats) + 2;
        const int k0 = 2 * t, k1 = 2 * t + 1;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          const uint32_t v0 = k0 < NK ? __ldg(sh + 3 * k0 + ch) : 0u, v1 = k1 < NK ? __ldg(sh + 3 * k1 + ch) : 0u;
          b0[ch] = v0 | v1 << 16;
          b1[ch] = (SH2 && t == 0) ? (uint32_t)__ldg(sh + 24 + ch) : 0u;
        }
      }
      // Accumulators: lane (g, t) holds pixels 16m + g (+ 8) at corners 2t, 2t + 1.
      float part_sum[2][2][3];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        float dv[3][4];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          dv[ch][0] = dv[ch][1] = dv[ch][2] = dv[ch][3] = 0.0f;
          mma_bf16_16816(dv[ch], ah[m], b0[ch], b1[ch]);
          mma_bf16_16816(dv[ch], al[m], b0[ch], b1[ch]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = 16 * m + g + 8 * h;
          const float fx = __shfl_sync(0xffffffffu, fr[0], r), fy = __shfl_sync(0xffffffffu, fr[1], r),
                      fz = __shfl_sync(0xffffffffu, fr[2], r);
          const float wyz = ((t & 1) ? fy : 1.0f - fy) * ((t >> 1) ? fz : 1.0f - fz);
          const float w0 = (1.0f - fx) * wyz, w1 = fx * wyz;
#pragma unroll
          for (int ch = 0; ch < 3; ++ch)
            part_sum[m][h][ch] = fmaxf(dv[ch][2 * h], 0.0f) * w0 + fmaxf(dv[ch][2 * h + 1], 0.0f) * w1;
        }
      }
      // Sum over the quad's corners, then each pixel takes its own sums.
#pragma unroll
      for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            float v = part_sum[m][h][ch];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            part_sum[m][h][ch] = v;
          }
      const int src = 4 * (lane & 7), mm = lane >> 4, hh = (lane >> 3) & 1;
      float mine[3];
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const float v00 = __shfl_sync(0xffffffffu, part_sum[0][0][ch], src);
        const float v01 = __shfl_sync(0xffffffffu, part_sum[0][1][ch], src);
        const float v10 = __shfl_sync(0xffffffffu, part_sum[1][0][ch], src);
        const float v11 = __shfl_sync(0xffffffffu, part_sum[1][1][ch], src);
        mine[ch] = mm ? (hh ? v11 : v10) : (hh ? v01 : v00);
      }
      if (member) irr = mkf3(mine[0], mine[1], mine[2]);
    }
    const f3 cc_col = mkf3(irr.x * alb.x, irr.y * alb.y, irr.z * alb.z);
    if (call == 0)
      col = cc_col;
    else if (in_tr)
      col = col * (1.0f - tmix) + cc_col * tmix;  // mix(), cacheApply.frag:359
  }
  if (!inside) return;
  if (!geom) {
    if (!p.out_add) store_output(p, i, mkf3(0.0f, 0.0f, 0.0f));
    return;
  }
  store_output(p, i, col);
}

}  // namespace

cudaError_t launch_apply(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const DrvPerFrame& f,
                         const DrvGBufferView& g, const uint32_t* atlas, const void* entries, uint32_t entry_stride,
                         const DrvCacheCounter* counter, float* out_rgb, const float* srgb, const SpecView* spec,
                         uint32_t* err, bool tensor_core) {
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
  if (p.bf16 && tensor_core)
    p.sh2 ? apply_tc_kernel<true><<<grid, block, 0, s>>>(p) : apply_tc_kernel<false><<<grid, block, 0, s>>>(p);
  else if (p.bf16)
    p.sh2 ? apply_kernel<true, true, false><<<grid, block, 0, s>>>(p)
          : apply_kernel<true, false, false><<<grid, block, 0, s>>>(p);
  else
    p.sh2 ? apply_kernel<false, true, false><<<grid, block, 0, s>>>(p)
          : apply_kernel<false, false, false><<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace drv
