// voxel_sample.cuh — quadrilinear opacity lookups of the voxel pyramid on the
// GPU: textureLod(VoxelVolume, s, lod) with the LINEAR/LINEAR/LINEAR CLAMP
// sampler the reference binds for the cone trace (renderer.cpp:916-917),
// written in software (GL 4.5 §8.14: lod <= 0 magnifies level 0; otherwise
// LINEAR_MIPMAP_LINEAR between floor/ceil levels, clamped to the last level;
// texel centres at (i + 0.5) / n; CLAMP_TO_EDGE).
//
// Level 0 is read from the corner-packed byte grid: byte (x, y, z) holds the
// 8 voxels (x + dx, y + dy, z + dz), dx,dy,dz in {0,1}, with +1 clamped to the
// last voxel, x fastest, so one trilinear level-0 sample is one byte load.
// Levels >= 1 are FP32 arrays (x fastest) and, where the context built them,
// corner-packed records of the same values: record (x, y, z) of level l holds
// the 8 texels (x + dx, y + dy, z + dz), +1 clamped, slot dx | dy << 1 |
// dz << 2, as FP16, 16 bytes, x fastest, so one trilinear mip sample is one
// 16-byte load instead of eight. With BF16 precision the texels are FP16 anyway and every level has
// records; with FP32 precision levels 1..3 have them: a level-l texel is
// k / 8^l (a mean of means of binary voxels) and FP16 holds it exactly for
// 8^l <= 512, so the sample is the same FP32 value bit for bit.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "f32x2.cuh"

namespace drv {

// The sampler's taps are integer texel coordinates plus kTapBias (the bit
// pattern of 2^23, see taps()); the linear index x + (y << ln) + (z << 2 ln)
// of a level of 2^ln texels per axis, computed from biased taps in 32-bit
// arithmetic, is the true index plus tap_index_bias(ln) modulo 2^32, which
// the view's offsets subtract in advance.
constexpr uint32_t kTapBias = 0x4B000000u;
__host__ __device__ constexpr uint32_t tap_index_bias(int ln) {
  return kTapBias * (1u + (1u << ln) + (1u << (2 * ln)));
}

struct VoxelView {
  const uint8_t* corners;  // level 0, N^3 bytes, x fastest
  const void* mips;        // levels 1..L concatenated: float, or __half when half_mips
  uint32_t off[16];        // offset (floats) of level l in `mips`
  int N;                   // level-0 resolution (power of two)
  int log2n;
  int max_level;           // L = log2(N)
  int half_mips;
  uint32_t cbias;          // -tap_index_bias(log2n): corner index of biased taps
  const uint4* records;    // corner-packed mip records (nullptr: none)
  uint32_t roff[16];       // record offset of level l minus tap_index_bias(log2n - l)
  int record_levels;       // levels 1..record_levels have records
};

// Voxel loads of the sampler, for the cone pass's memory roofline: every
// sampling function takes a reads object; NoReads (the default) compiles to
// nothing, VoxelReads counts level-0 corner bytes (1 B each), mip records
// (16 B each) and plain mip texels (2 or 4 B each).
struct NoReads {
  __device__ __forceinline__ void on_level0() {}
  __device__ __forceinline__ void on_record() {}
  __device__ __forceinline__ void on_texels(int) {}
};
struct VoxelReads {
  uint32_t level0_bytes = 0, records = 0, texels = 0;
  __device__ __forceinline__ void on_level0() { ++level0_bytes; }
  __device__ __forceinline__ void on_record() { ++records; }
  __device__ __forceinline__ void on_texels(int n) { texels += (uint32_t)n; }
};

// The arithmetic of the sampler and the cone is written with explicit
// rounding intrinsics (no contraction left to the compiler), so every kernel
// that inlines it computes the same bits.
__device__ __forceinline__ float lerp(float a, float b, float t) { return __fmaf_rn(b - a, t, a); }

// Trilinear blend of corners t0..t7 (x fastest): the seven lerps of
// lerp(lerp(lerp(t0, t1, ax), lerp(t2, t3, ax), ay), lerp(lerp(t4, t5, ax),
// lerp(t6, t7, ax), ay), az), the x and y lerps two at a time in packed FP32
// pairs: the same roundings, so the same bits, in fewer instructions.
__device__ __forceinline__ float trilerp(float t0, float t1, float t2, float t3, float t4, float t5, float t6,
                                         float t7, float ax, float ay, float az) {
  const float2 axx = make_float2(ax, ax);
  const float2 lo0 = make_float2(t0, t2), lo1 = make_float2(t4, t6);
  const float2 c0 = fma2(sub2(make_float2(t1, t3), lo0), axx, lo0);  // (c00, c10)
  const float2 c1 = fma2(sub2(make_float2(t5, t7), lo1), axx, lo1);  // (c01, c11)
  const float2 lo = make_float2(c0.x, c1.x);
  const float2 cz = fma2(sub2(make_float2(c0.y, c1.y), lo), make_float2(ay, ay), lo);  // (lerp in y) at z0, z1
  return lerp(cz.x, cz.y, az);
}

__device__ __forceinline__ float mip_texel(const VoxelView& v, uint32_t i) {
  return v.half_mips ? __half2float(__ldg(static_cast<const __half*>(v.mips) + i))
                     : __ldg(static_cast<const float*>(v.mips) + i);
}

// A sample position U in level-0 voxel units (U = s * N for texture
// coordinate s; exact, N is a power of two). Level l reads texel coordinate
// u_l = U * 2^-l - 0.5 = s * n_l - 0.5, one rounding (exact for |U| < 2^22),
// so all levels see the same point and a coarse texel footprint contains the
// finer one.
struct Coord {
  float x, y, z;
};

__device__ __forceinline__ Coord level_coord(const Coord& U, int level) {
  const float sc = __uint_as_float((uint32_t)(127 - level) << 23);  // 2^-level
  const float2 xy = fma2(make_float2(U.x, U.y), make_float2(sc, sc), make_float2(-0.5f, -0.5f));
  return Coord{xy.x, xy.y, __fmaf_rn(U.z, sc, -0.5f)};
}

// Base texel and weight of coordinate u in a level of n texels (nm1 = n - 1):
// below 0 both taps clamp to texel 0, at or above n - 1 both clamp to n - 1;
// clamping u itself to [0, n - 1] gives the same sample, because the
// corner-packed byte / record at n - 1 repeats texel n - 1 for the +1 tap.
//
// The floor is taken without a float-to-int conversion: for 0 <= c < 2^23,
// c + 2^23 rounded toward -infinity is 2^23 + floor(c) exactly (floats in
// [2^23, 2^24) are the integers), so subtracting 2^23 gives floor(c), and
// the bit pattern is floor(c) + kTapBias: the biased tap. The x and y taps
// go in one packed pair.
struct Taps {
  uint32_t x, y, z;  // texel + kTapBias
  float ax, ay, az;
};
__device__ __forceinline__ Taps taps(float ux, float uy, float uz, float nm1) {
  constexpr float kTwo23 = 8388608.0f;
  const float2 c = make_float2(fminf(fmaxf(ux, 0.0f), nm1), fminf(fmaxf(uy, 0.0f), nm1));
  const float cz = fminf(fmaxf(uz, 0.0f), nm1);
  const float2 t = add2_rm(c, make_float2(kTwo23, kTwo23));
  const float tz = __fadd_rd(cz, kTwo23);
  const float2 a = sub2(c, sub2(t, make_float2(kTwo23, kTwo23)));
  return Taps{__float_as_uint(t.x), __float_as_uint(t.y), __float_as_uint(tz), a.x, a.y, cz - (tz - kTwo23)};
}

// Linear index x + (y << ln) + (z << 2 ln) of biased taps, plus `base`
// (an offset that has the taps' bias subtracted).
__device__ __forceinline__ uint32_t tap_index(const Taps& t, int ln, uint32_t base) {
  return base + t.x + (t.y << ln) + (t.z << (2 * ln));
}

// n - 1 as a float for a level of n = 2^ln texels.
__device__ __forceinline__ float last_texel(int ln) { return __uint_as_float((uint32_t)(127 + ln) << 23) - 1.0f; }

template <class R>
__device__ __forceinline__ float level0_taps(const VoxelView& v, const Taps& t, R& reads) {
  reads.on_level0();
  const uint32_t b = __ldg(v.corners + tap_index(t, v.log2n, v.cbias));
  const float ax = t.ax, ay = t.ay, az = t.az;
  // Trilinear weights sum to one, so eight equal corners give that value
  // exactly: empty space (the common case) costs no interpolation.
  if (b == 0u) return 0.0f;
  if (b == 0xFFu) return 1.0f;
  auto bit = [b](int k) { return (b >> k) & 1u ? 1.0f : 0.0f; };
  return trilerp(bit(0), bit(1), bit(2), bit(3), bit(4), bit(5), bit(6), bit(7), ax, ay, az);
}

// Level 0 at position U (texel coordinate U - 0.5, exact).
template <class R>
__device__ __forceinline__ float level0_at(const VoxelView& v, const Coord& U, R& reads) {
  const float2 uxy = add2(make_float2(U.x, U.y), make_float2(-0.5f, -0.5f));
  return level0_taps(v, taps(uxy.x, uxy.y, U.z - 0.5f, last_texel(v.log2n)), reads);
}

template <class R>
__device__ __forceinline__ float level_n_at(const VoxelView& v, int level, const Coord& u, R& reads) {
  reads.on_texels(8);
  const int ln = v.log2n - level, n = 1 << ln;
  const float ax = u.x - floorf(u.x), ay = u.y - floorf(u.y), az = u.z - floorf(u.z);
  const int x0 = (int)floorf(u.x), y0 = (int)floorf(u.y), z0 = (int)floorf(u.z);
  const int xa = min(max(x0, 0), n - 1), xb = min(max(x0 + 1, 0), n - 1);
  const int ya = min(max(y0, 0), n - 1) << ln, yb = min(max(y0 + 1, 0), n - 1) << ln;
  const int za = min(max(z0, 0), n - 1) << (2 * ln), zb = min(max(z0 + 1, 0), n - 1) << (2 * ln);
  const uint32_t m = v.off[level];
  float t0 = mip_texel(v, m + (za | ya | xa)), t1 = mip_texel(v, m + (za | ya | xb));
  float t2 = mip_texel(v, m + (za | yb | xa)), t3 = mip_texel(v, m + (za | yb | xb));
  float t4 = mip_texel(v, m + (zb | ya | xa)), t5 = mip_texel(v, m + (zb | ya | xb));
  float t6 = mip_texel(v, m + (zb | yb | xa)), t7 = mip_texel(v, m + (zb | yb | xb));
  return trilerp(t0, t1, t2, t3, t4, t5, t6, t7, ax, ay, az);
}

__device__ __forceinline__ __half2 u32_as_half2(uint32_t w) {
  __half2 h;
  memcpy(&h, &w, 4);
  return h;
}

// level_n_at from the level's corner-packed record; `zero` reports a record
// whose 8 texels are all 0 (the sample is then 0).
template <class R>
__device__ __forceinline__ float level_record_at(const VoxelView& v, int level, const Coord& u, bool& zero,
                                                 R& reads) {
  reads.on_record();
  const Taps t = taps(u.x, u.y, u.z, last_texel(v.log2n - level));
  const float ax = t.ax, ay = t.ay, az = t.az;
  const uint4 r = __ldg(v.records + tap_index(t, v.log2n - level, v.roff[level]));
  zero = (r.x | r.y | r.z | r.w) == 0u;  // FP16 +0 is the all-zero pattern; texels are >= 0
  if (zero) return 0.0f;
  const float t0 = __low2float(u32_as_half2(r.x)), t1 = __high2float(u32_as_half2(r.x));
  const float t2 = __low2float(u32_as_half2(r.y)), t3 = __high2float(u32_as_half2(r.y));
  const float t4 = __low2float(u32_as_half2(r.z)), t5 = __high2float(u32_as_half2(r.z));
  const float t6 = __low2float(u32_as_half2(r.w)), t7 = __high2float(u32_as_half2(r.w));
  return trilerp(t0, t1, t2, t3, t4, t5, t6, t7, ax, ay, az);
}

// Trilinear sample of mip level >= 1 (from its records where they exist);
// `zero` is set only from a record.
template <class R>
__device__ __forceinline__ float level_any_at(const VoxelView& v, int level, const Coord& u, bool& zero, R& reads) {
  zero = false;
  return level <= v.record_levels ? level_record_at(v, level, u, zero, reads) : level_n_at(v, level, u, reads);
}
__device__ __forceinline__ float level_any_at(const VoxelView& v, int level, const Coord& u, bool& zero) {
  NoReads r;
  return level_any_at(v, level, u, zero, r);
}

// Position U (level-0 voxel units) of texture coordinate s.
__device__ __forceinline__ Coord voxel_pos(const VoxelView& v, float sx, float sy, float sz) {
  const float fn = (float)v.N;
  return Coord{__fmul_rn(sx, fn), __fmul_rn(sy, fn), __fmul_rn(sz, fn)};
}

// Trilinear sample of one mip level at s (no lod blend).
__device__ __forceinline__ float level_any(const VoxelView& v, int level, float sx, float sy, float sz) {
  bool zero;
  return level_any_at(v, level, level_coord(voxel_pos(v, sx, sy, sz), level), zero);
}

// textureLod at position U. For a blended lod the coarser level is read
// first: its footprint contains the finer level's (the finer taps
// floor(u_f), floor(u_f) + 1 lie within the fine texels of coarse taps
// floor(u_c), floor(u_c) + 1, also where both clamp), so an all-zero coarse
// record makes both levels 0.
template <class R>
__device__ __forceinline__ float sample_voxels_at(const VoxelView& v, const Coord& U, float lod, R& reads) {
  if (!(lod > 0.0f)) return level0_at(v, U, reads);
  bool zero;
  if (lod >= (float)v.max_level) return level_any_at(v, v.max_level, level_coord(U, v.max_level), zero, reads);
  const float fl = floorf(lod);
  const int d1 = (int)fl;
  const float fr = lod - fl;
  const float t2 = level_any_at(v, d1 + 1, level_coord(U, d1 + 1), zero, reads);
  if (zero) return 0.0f;
  const float t1 = d1 == 0 ? level0_at(v, U, reads) : level_any_at(v, d1, level_coord(U, d1), zero, reads);
  if (fr == 0.0f) return t1;
  return __fmaf_rn(fr, t2, __fmul_rn(1.0f - fr, t1));
}
__device__ __forceinline__ float sample_voxels_at(const VoxelView& v, const Coord& U, float lod) {
  NoReads r;
  return sample_voxels_at(v, U, lod, r);
}

// textureLod at texture coordinate s.
__device__ __forceinline__ float sample_voxels(const VoxelView& v, float sx, float sy, float sz, float lod) {
  return sample_voxels_at(v, voxel_pos(v, sx, sy, sz), lod);
}

// Indirect-shadow cone, cacheLightingRSM.comp:195-230: march from the cache
// toward the block's average VAL position, growing the sample sphere with the
// distance, front-to-back occlusion, at most max_steps samples. Once the
// occlusion reaches 1 a further step gives occlusion * (1 - s) + s >= 1 for
// any sample s in [0, 1], so the clamped result is 0 (to within one rounding)
// whatever is sampled: the march stops there (the reference marches on).
template <class R>
__device__ __forceinline__ float cone_shadow(const VoxelView& v, float voxel_size, int max_steps, float cx, float cy,
                                             float cz, float px, float py, float pz, float ax, float ay, float az,
                                             float dsr, R& reads) {
  float tx = ax - cx, ty = ay - cy, tz = az - cz;
  const float light_dist = sqrtf(__fmaf_rn(tz, tz, __fmaf_rn(ty, ty, __fmul_rn(tx, tx))));
  const float inv = 1.0f / light_dist;
  // The march in level-0 voxel units: direction D = (t / |t|) = (t / |t| / N) * N
  // and position U = q * N, both exact scalings of the texture-space march
  // q += d * step (rounding commutes with a power-of-two scale).
  const float Dx = __fmul_rn(tx, inv), Dy = __fmul_rn(ty, inv), Dz = __fmul_rn(tz, inv);
  const Coord P = voxel_pos(v, px, py, pz);
  Coord U{__fmaf_rn(Dx, 2.0f, P.x), __fmaf_rn(Dy, 2.0f, P.y), __fmaf_rn(Dz, 2.0f, P.z)};
  float occlusion = 0.0f, step = 1.0f, dist = 0.0f;
  const float goal = light_dist / voxel_size - 2.0f;
  const float k = 2.0f / (1.0f - dsr);
  for (int s = 0; s < max_steps; ++s) {
    const float2 xy = fma2(make_float2(Dx, Dy), make_float2(step, step), make_float2(U.x, U.y));
    U.x = xy.x;
    U.y = xy.y;
    U.z = __fmaf_rn(Dz, step, U.z);
    dist += step;
    const float radius = __fmul_rn(dist, dsr);
    // A sphere of radius <= 1 voxel samples level 0 (its lod log2(radius) is
    // <= 0): the logarithm is taken only on the mip branch.
    const float s_vox = radius > 1.0f ? sample_voxels_at(v, U, __log2f(radius), reads) : level0_at(v, U, reads);
    occlusion = __fmaf_rn(1.0f - occlusion, s_vox, occlusion);
    if (dist >= goal || occlusion >= 1.0f) break;
    step = fmaxf(1.0f, __fmul_rn(radius, k));
  }
  return fminf(fmaxf(1.0f - occlusion, 0.0f), 1.0f);
}
__device__ __forceinline__ float cone_shadow(const VoxelView& v, float voxel_size, int max_steps, float cx, float cy,
                                             float cz, float px, float py, float pz, float ax, float ay, float az,
                                             float dsr) {
  NoReads r;
  return cone_shadow(v, voxel_size, max_steps, cx, cy, cz, px, py, pz, ax, ay, az, dsr, r);
}

}  // namespace drv
