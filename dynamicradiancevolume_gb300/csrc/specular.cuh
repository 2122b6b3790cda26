// specular.cuh — device helpers of the indirect-specular path
// (INDIRECT_SPECULAR): the R11F_G11F_B10F texel format of the envmap atlas,
// the cache-local view space, the concentric hemispherical projection and
// the envmap addressing shared by the light stage, the mip / hole-fill pass
// and the apply.
#pragma once

#include <cstdint>

#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {

constexpr float kPiF = 3.14159265358979323846f;

// Unsigned small float with a 5-bit exponent (bias 15) and mbits of mantissa
// (6 for R and G, 5 for B), the GL packed-float rules (GL 4.5 section
// 2.3.4.3-4): negative values and -inf -> 0, finite values above the largest
// finite value -> that value, +inf -> inf, NaN -> NaN; otherwise rounded to
// nearest, ties to even.
__device__ __forceinline__ uint32_t encode_ufloat(float f, int mbits) {
  const uint32_t mmask = (1u << mbits) - 1u;
  if (f != f) return (31u << mbits) | 1u;
  if (!(f > 0.0f)) return 0u;
  const uint32_t u = __float_as_uint(f);
  if (u >= 0x7F800000u) return 31u << mbits;
  const uint32_t max_finite = (30u << mbits) | mmask;
  const int e = (int)(u >> 23) - 127 + 15;  // biased small-float exponent
  if (e <= 0) {
    // subnormal: m * 2^(-14 - mbits), m = rint(f * 2^(14 + mbits)) (exact scaling)
    return __float2uint_rn(f * __uint_as_float((uint32_t)(127 + 14 + mbits) << 23));
  }
  if (e >= 31) return max_finite;
  const int shift = 23 - mbits;
  const uint32_t mant = u & 0x7FFFFFu;
  const uint32_t r = mant + ((1u << (shift - 1)) - 1u) + ((mant >> shift) & 1u);
  const uint32_t v = ((uint32_t)e << mbits) + (r >> shift);  // a mantissa carry moves into the exponent
  return v > max_finite ? max_finite : v;
}

__device__ __forceinline__ float decode_ufloat(uint32_t v, int mbits) {
  const uint32_t e = v >> mbits, m = v & ((1u << mbits) - 1u);
  if (e == 0u) return (float)m * __uint_as_float((uint32_t)(127 - 14 - mbits) << 23);
  if (e == 31u) return m ? __uint_as_float(0x7FC00000u) : __uint_as_float(0x7F800000u);
  return __uint_as_float(((e - 15u + 127u) << 23) | (m << (23 - mbits)));
}

// The same decode in three instructions for a finite code: its exponent and
// mantissa fields moved into a binary32 give (1 + m 2^-mbits) 2^(e - 127), or
// the denormal m 2^-(mbits + 126) when e = 0, and the product with 2^112 is
// the code's value, exactly (the library is compiled without flushing
// denormals). The all-ones exponent (infinity, NaN) takes the general path.
__device__ __forceinline__ float decode_ufloat_fast(uint32_t v, int mbits) {
  const float x = __fmul_rn(__uint_as_float(v << (23 - mbits)), 0x1p112f);
  return (v >> mbits) == 31u ? decode_ufloat(v, mbits) : x;
}

__device__ __forceinline__ f3 decode_r11g11b10_fast(uint32_t v) {
  return mkf3(decode_ufloat_fast(v & 0x7FFu, 6), decode_ufloat_fast((v >> 11) & 0x7FFu, 6),
              decode_ufloat_fast(v >> 22, 5));
}

__device__ __forceinline__ uint32_t encode_r11g11b10(f3 c) {
  return encode_ufloat(c.x, 6) | encode_ufloat(c.y, 6) << 11 | encode_ufloat(c.z, 5) << 22;
}

__device__ __forceinline__ f3 decode_r11g11b10(uint32_t v) {
  return mkf3(decode_ufloat(v & 0x7FFu, 6), decode_ufloat((v >> 11) & 0x7FFu, 6), decode_ufloat(v >> 22, 5));
}

// ComputeLocalViewSpace (lightcache.glsl:98-106): Z towards the camera,
// X = normalize((Z.z, 0, -Z.x)), Y = Z x X.
struct LocalFrame {
  f3 x, y, z;
};

__device__ __forceinline__ LocalFrame local_view_space(const float cam[3], float px, float py, float pz) {
  LocalFrame f;
  f.z = normalize3(mkf3(cam[0] - px, cam[1] - py, cam[2] - pz));
  f.x = normalize3(mkf3(f.z.z, 0.0f, -f.z.x));
  f.y = cross3(f.z, f.x);
  return f;
}

// v * mat3(X, Y, Z) in GLSL: the components of v along X, Y and Z.
__device__ __forceinline__ f3 to_local(const LocalFrame& f, f3 v) {
  return mkf3(dot3(v, f.x), dot3(v, f.y), dot3(v, f.z));
}

// HemisphericalProjection, the concentric square map (utils.glsl:103-170,
// HEMIPROJECTION_LAMBERT_CONCENTRICQUAD): a direction of the z+ hemisphere
// to [0, 1]^2. 1 - z is clamped at 0 (a rounding above 1 would give NaN).
__device__ __forceinline__ void hemi_projection(f3 d, float& u, float& v) {
  const float r = sqrtf(fmaxf(1.0f - d.z, 0.0f)) * 0.5f;
  float phi = atan2f(d.y, d.x) * (4.0f / kPiF);
  if (phi < -1.0f) phi += 8.0f;
  float px, py;
  if (phi < 3.0f) {
    if (phi < 1.0f) {
      px = r;
      py = phi * r;
    } else {
      px = -(phi - 2.0f) * r;
      py = r;
    }
  } else {
    if (phi < 5.0f) {
      px = -r;
      py = -(phi - 4.0f) * r;
    } else {
      px = (phi - 6.0f) * r;
      py = -r;
    }
  }
  u = px + 0.5f;
  v = py + 0.5f;
}

// Word index of the first texel of cache c's region at level l (the atlas
// geometry is all powers of two: per_row = 2^(log2 atlas - log2 size); the
// whole atlas holds fewer than 2^32 words, which drv_create checks).
__device__ __forceinline__ uint32_t env_region(const SpecView& s, uint32_t c, int l) {
  const int shift = __ffs(s.per_row) - 1;
  const uint32_t side = (uint32_t)(s.size >> l);
  return s.off[l] + ((c >> shift) * (uint32_t)(s.atlas >> l) + (c & (uint32_t)(s.per_row - 1))) * side;
}

// Word index of texel (x, y) of cache c's region at level l.
__device__ __forceinline__ size_t env_index(const SpecView& s, uint32_t c, int l, int x, int y) {
  return env_region(s, c, l) + (size_t)y * (size_t)(s.atlas >> l) + (size_t)x;
}

}  // namespace drv
