// oracle.cpp — CPU FP64 restatement of the DynamicRadianceVolume per-frame
// indirect-lighting path. TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Compiled with -ffp-contract=off: the binary32 "mirror" helpers below must
// round every operation on its own, exactly as the CUDA kernels do with
// __fmul_rn/__fadd_rn/__fdiv_rn.
//
// All reference paths are relative to the DynamicRadianceVolume project.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// utils.glsl:1 defines PI as this literal; the lighting math uses it.
constexpr double kShaderPi = 3.14159265358979;
constexpr double kPi = 3.14159265358979323846;

struct d3 {
  double x, y, z;
};
inline d3 mk(double x, double y, double z) { return {x, y, z}; }
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 cross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double length(d3 a) { return std::sqrt(dot(a, a)); }
inline d3 normalize(d3 a) { return a * (1.0 / length(a)); }
inline double saturate(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }
inline d3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
inline d3 ld3(const double* p) { return {p[0], p[1], p[2]}; }

// ---------------------------------------------------------------------------
// binary32 mirror: M * (x, y, z, 1) with a fixed left-to-right order, each
// product and sum rounded separately (the kernels use the same order).
inline float mrow(const float* r, float x, float y, float z) {
  float a = r[0] * x;
  float b = r[1] * y;
  float s = a + b;
  float c = r[2] * z;
  s = s + c;
  return s + r[3];
}

// World position from a depth-buffer sample (cacheGather.comp:113-119,
// cacheApply.frag:310-311), binary32.
inline void reconstruct_world_f32(const DrvPerFrame* f, int px, int py, int w, int h, float depth, float out[3]) {
  float sx = (float)px + 0.5f;
  float sy = (float)py + 0.5f;
  float nx = sx / (float)w;
  float ny = sy / (float)h;
  nx = nx * 2.0f;
  ny = ny * 2.0f;
  nx = nx - 1.0f;
  ny = ny - 1.0f;
  const float* M = f->inverse_view_projection;
  float X = mrow(M + 0, nx, ny, depth);
  float Y = mrow(M + 4, nx, ny, depth);
  float Z = mrow(M + 8, nx, ny, depth);
  float W = mrow(M + 12, nx, ny, depth);
  out[0] = X / W;
  out[1] = Y / W;
  out[2] = Z / W;
}

// ComputeAddressVolumeCascade, lightcache.glsl:109-122 (binary32 compares).
inline int select_cascade_f32(const DrvVolumeInfo* v, int n_cascades, const float p[3]) {
  int c = 0;
  for (; c < n_cascades - 1; ++c) {
    const DrvCascade& k = v->cascades[c];
    bool inside = p[0] <= k.decision_max[0] && p[1] <= k.decision_max[1] && p[2] <= k.decision_max[2] &&
                  p[0] >= k.decision_min[0] && p[1] >= k.decision_min[1] && p[2] >= k.decision_min[2];
    if (inside) break;
  }
  return c;
}

// ComputeAddressVolumeCascadeTransition, lightcache.glsl:125-134 (binary32).
inline float cascade_transition_f32(const DrvVolumeInfo* v, int c, const float p[3]) {
  const DrvCascade& k = v->cascades[c];
  float dmax0 = k.decision_max[0] - p[0], dmax1 = k.decision_max[1] - p[1], dmax2 = k.decision_max[2] - p[2];
  float dmin0 = p[0] - k.decision_min[0], dmin1 = p[1] - k.decision_min[1], dmin2 = p[2] - k.decision_min[2];
  float m = std::min(std::min(std::min(dmax0, dmax1), dmax2), std::min(std::min(dmin0, dmin1), dmin2));
  float denom = k.world_voxel_size * v->cav_transition_zone_size;
  float q = m / denom;
  float t = 1.0f - q;
  return t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
}

// clamp(ivec3(v), 0, res-1) where ivec3 truncates toward zero.
inline int trunc_clamp(float v, int res) {
  if (!(v > 0.0f)) return 0;
  if (v >= (float)(res - 1)) return res - 1;
  return (int)v;
}

// GetCache1DCoord, cacheGather.comp:20-30 (binary32).
inline int cache_1d_coord_f32(const DrvVolumeInfo* v, int res, int c, const float p[3]) {
  const DrvCascade& k = v->cascades[c];
  int ix = trunc_clamp((p[0] - k.min[0]) / k.world_voxel_size, res);
  int iy = trunc_clamp((p[1] - k.min[1]) / k.world_voxel_size, res);
  int iz = trunc_clamp((p[2] - k.min[2]) / k.world_voxel_size, res);
  return ix + iy * res + iz * res * res + c * res * res * res;
}

// Matrices -----------------------------------------------------------------
struct m4 {
  double m[16];
};
m4 mul(const m4& a, const m4& b) {
  m4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += a.m[i * 4 + k] * b.m[k * 4 + j];
      r.m[i * 4 + j] = s;
    }
  return r;
}
bool invert(const m4& a, m4& out) {
  // Gauss-Jordan with partial pivoting in FP64.
  double t[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 8; ++j) t[i][j] = j < 4 ? a.m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int p = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(t[r][c]) > std::fabs(t[p][c])) p = r;
    if (t[p][c] == 0.0) return false;
    if (p != c)
      for (int j = 0; j < 8; ++j) std::swap(t[p][j], t[c][j]);
    double inv = 1.0 / t[c][c];
    for (int j = 0; j < 8; ++j) t[c][j] *= inv;
    for (int r = 0; r < 4; ++r)
      if (r != c) {
        double f = t[r][c];
        if (f != 0.0)
          for (int j = 0; j < 8; ++j) t[r][j] -= f * t[c][j];
      }
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out.m[i * 4 + j] = t[i][j + 4];
  return true;
}
// Look-at basis: +z forward (DX-style, left-handed), up fallback when the
// direction is (anti)parallel to the requested up.
void basis(d3 dir, d3 up, d3& right, d3& up_out, d3& fwd) {
  fwd = normalize(dir);
  if (std::fabs(dot(normalize(up), fwd)) > 0.999) up = std::fabs(fwd.z) < 0.9 ? mk(0, 0, 1) : mk(1, 0, 0);
  right = normalize(cross(up, fwd));
  up_out = cross(fwd, right);
}
m4 view_matrix(d3 pos, d3 dir, d3 up) {
  d3 r, u, f;
  basis(dir, up, r, u, f);
  m4 v = {{r.x, r.y, r.z, -dot(r, pos), u.x, u.y, u.z, -dot(u, pos), f.x, f.y, f.z, -dot(f, pos), 0, 0, 0, 1}};
  return v;
}
// ei::perspectiveDX(fov, aspect, far, near) with near/far swapped: reversed-Z,
// depth 1 at the near plane, 0 at the far plane (camera.hpp:27-28).
m4 proj_reversed(double fovy, double aspect, double n, double f) {
  double sy = 1.0 / std::tan(fovy * 0.5), sx = sy / aspect;
  double A = n / (n - f), B = n * f / (f - n);
  m4 p = {{sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, A, B, 0, 0, 1, 0}};
  return p;
}
void store(const m4& a, float* out) {
  for (int i = 0; i < 16; ++i) out[i] = (float)a.m[i];
}

// Ray vs. axis-aligned boxes; returns box index or -1, hit distance, axis.
int trace(const DrvBox* boxes, int n, d3 o, d3 d, double& t_hit, int& axis_hit) {
  int best = -1;
  t_hit = 1e300;
  double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  for (int b = 0; b < n; ++b) {
    double tn = -1e300, tf = 1e300;
    int an = 0, af = 0;
    bool miss = false;
    for (int a = 0; a < 3; ++a) {
      if (dd[a] == 0.0) {
        if (oo[a] < boxes[b].min[a] || oo[a] > boxes[b].max[a]) miss = true;
        continue;
      }
      double t0 = (boxes[b].min[a] - oo[a]) / dd[a];
      double t1 = (boxes[b].max[a] - oo[a]) / dd[a];
      if (t0 > t1) std::swap(t0, t1);
      if (t0 > tn) { tn = t0; an = a; }
      if (t1 < tf) { tf = t1; af = a; }
    }
    if (miss || tn > tf) continue;
    double t;
    int ax;
    if (boxes[b].inward) {
      t = tf;
      ax = af;
    } else {
      t = tn;
      ax = an;
    }
    if (t > 1e-6 && t < t_hit) {
      t_hit = t;
      best = b;
      axis_hit = ax;
    }
  }
  return best;
}

// Texture-space helpers -----------------------------------------------------
inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

inline double voxel_l0(int N, const uint32_t* bits, int x, int y, int z) {
  size_t i = ((size_t)z * N + y) * N + x;
  return (bits[i >> 5] >> (i & 31)) & 1u ? 1.0 : 0.0;
}

size_t mip_offset(int N, int level) {  // offset of `level` (>= 1) in the concatenated mips
  size_t off = 0;
  for (int l = 1; l < level; ++l) {
    size_t n = (size_t)(N >> l);
    off += n * n * n;
  }
  return off;
}

inline double texel(int N, const uint32_t* bits, const double* mips, int level, int x, int y, int z) {
  if (level == 0) return voxel_l0(N, bits, x, y, z);
  int n = N >> level;
  return mips[mip_offset(N, level) + ((size_t)z * n + y) * n + x];
}

// LINEAR filter within one level with CLAMP_TO_EDGE (GL 4.5 §8.14.2).
double trilinear(int N, const uint32_t* bits, const double* mips, int level, const double s[3]) {
  int n = N >> level;
  int i0[3];
  double a[3];
  for (int k = 0; k < 3; ++k) {
    double u = s[k] * n - 0.5;
    double f = std::floor(u);
    i0[k] = (int)f;
    a[k] = u - f;
  }
  double r = 0.0;
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        double w = (dx ? a[0] : 1 - a[0]) * (dy ? a[1] : 1 - a[1]) * (dz ? a[2] : 1 - a[2]);
        int x = clampi(i0[0] + dx, 0, n - 1), y = clampi(i0[1] + dy, 0, n - 1), z = clampi(i0[2] + dz, 0, n - 1);
        r += w * texel(N, bits, mips, level, x, y, z);
      }
  return r;
}

int ilog2(int v) {
  int l = 0;
  while ((1 << (l + 1)) <= v) ++l;
  return l;
}

// Bilinear sample of a 2-channel RSM level (sampler2D LINEAR, CLAMP).
void bilinear2(int n, const float* img, double u, double v, double out[2]) {
  double x = u * n - 0.5, y = v * n - 0.5;
  double fx = std::floor(x), fy = std::floor(y);
  int x0 = (int)fx, y0 = (int)fy;
  double ax = x - fx, ay = y - fy;
  out[0] = out[1] = 0;
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      double w = (dx ? ax : 1 - ax) * (dy ? ay : 1 - ay);
      int xx = clampi(x0 + dx, 0, n - 1), yy = clampi(y0 + dy, 0, n - 1);
      out[0] += w * img[((size_t)yy * n + xx) * 2 + 0];
      out[1] += w * img[((size_t)yy * n + xx) * 2 + 1];
    }
}

d3 unproject_dir(const float* inv_vp, double u, double v, d3 from) {
  // vec4(uv*2-1, 0, 1) * InverseLightViewProjection (cacheLightingRSM.comp:154-155)
  double x = u * 2.0 - 1.0, y = v * 2.0 - 1.0;
  double c[4];
  for (int r = 0; r < 4; ++r) c[r] = inv_vp[r * 4 + 0] * x + inv_vp[r * 4 + 1] * y + inv_vp[r * 4 + 3];
  d3 p = mk(c[0] / c[3], c[1] / c[3], c[2] / c[3]);
  return normalize(p - from);
}

void set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // namespace

extern "C" {

// cacheLightingRSM.comp:46-62
void orc_morton_decode(uint32_t morton, uint32_t* x, uint32_t* y) {
  uint32_t c[2] = {morton, morton >> 1};
  for (int i = 0; i < 2; ++i) {
    uint32_t v = c[i] & 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0f0f0f0fu;
    v = (v | (v >> 4)) & 0x00ff00ffu;
    v = (v | (v >> 8)) & 0x0000ffffu;
    c[i] = v;
  }
  *x = c[0];
  *y = c[1];
}

// PackNormal / PackNormal16I, utils.glsl:61-89. The conversion to a 16-bit
// integer target saturates to [-32768, 32767] (the reference writes +32768
// for n.z = 1 into an RG16I target, which GL leaves undefined).
void orc_pack_normal16i(const double n[3], int16_t out[2]) {
  double px = n[0] == 0.0 ? ((n[1] > 0) - (n[1] < 0)) * kShaderPi / 2 : std::atan2(n[1], n[0]);
  double py = n[2];
  // (x / PI) * 32768, the same product as the reference's x * (32768 / PI),
  // ordered so that axis-aligned normals pack exactly on every side.
  double vx = std::trunc((px / kShaderPi) * 32768.0);
  double vy = std::trunc(py * 32768.0);
  if (!(vx == vx)) vx = 0;
  if (!(vy == vy)) vy = 0;
  out[0] = (int16_t)std::max(-32768.0, std::min(32767.0, vx));
  out[1] = (int16_t)std::max(-32768.0, std::min(32767.0, vy));
}

// UnpackNormal16I / UnpackNormal, utils.glsl:44-58.
void orc_unpack_normal16i(const int16_t packed[2], double out[3]) {
  double px = packed[0] * (kShaderPi / 32768.0);
  double py = packed[1] * (1.0 / 32768.0);
  double sin_phi = std::sqrt(1.0 - py * py);
  d3 v = normalize(mk(std::cos(px) * sin_phi, std::sin(px) * sin_phi, py));
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
}

// Renderer::UpdateConstantUBO, renderer.cpp:296-306.
void orc_sh_constants(int sh2_sign, double cl[5], double ev[5]) {
  cl[0] = std::sqrt(kPi) / 2.0;
  cl[1] = std::sqrt(kPi / 3.0);
  cl[2] = (sh2_sign == DRV_SH2_SIGN_FIXED ? 1.0 : -1.0) * std::sqrt(15.0 * kPi) / 8.0;
  cl[3] = std::sqrt(5.0 * kPi) / 16.0;
  cl[4] = std::sqrt(15.0 * kPi) / 16.0;
  ev[0] = 1.0 / (2.0 * std::sqrt(kPi));
  ev[1] = std::sqrt(3.0) / (2.0 * std::sqrt(kPi));
  ev[2] = std::sqrt(15.0 / (4.0 * kPi));
  ev[3] = std::sqrt(5.0 / (16.0 * kPi));
  ev[4] = std::sqrt(15.0 / (16.0 * kPi));
}

// SampleCacheIrradiance, lightcache.glsl:137-179.
void orc_sh_irradiance(int sh_order, int sh2_sign, const double* sh, const double nn[3], double out[3]) {
  double cl[5], ev[5];
  orc_sh_constants(sh2_sign, cl, ev);
  double nx = nn[0], ny = nn[1], nz = nn[2];
  for (int ch = 0; ch < 3; ++ch) {
    double e = sh[0 * 3 + ch] * cl[0];
    e -= sh[1 * 3 + ch] * (cl[1] * ny);
    e += sh[2 * 3 + ch] * (cl[1] * nz);
    e -= sh[3 * 3 + ch] * (cl[1] * nx);
    if (sh_order == 2) {
      e -= sh[4 * 3 + ch] * (cl[2] * nx * ny);
      e += sh[5 * 3 + ch] * (cl[2] * ny * nz);
      e += sh[6 * 3 + ch] * (cl[3] * (nz * nz * 3.0 - 1.0));
      e += sh[7 * 3 + ch] * (cl[2] * nx * nz);
      e += sh[8 * 3 + ch] * (cl[4] * (nx * nx - ny * ny));
    }
    out[ch] = std::max(e, 0.0);
  }
}

// textureLod(VoxelVolume, s, lod) with the LINEAR/LINEAR/LINEAR CLAMP sampler
// bound at renderer.cpp:916-917 (GL 4.5 §8.14: lambda <= 0 magnifies on the
// base level; otherwise LINEAR_MIPMAP_LINEAR between floor/ceil levels,
// clamped to the last level).
double orc_sample_voxels(int N, const uint32_t* bits, const double* mips, const double s[3], double lod) {
  int q = ilog2(N);
  if (!(lod > 0.0)) return trilinear(N, bits, mips, 0, s);
  if (lod >= q) return trilinear(N, bits, mips, q, s);
  double fl = std::floor(lod);
  int d1 = (int)fl;
  double fr = lod - fl;
  double t1 = trilinear(N, bits, mips, d1, s);
  if (fr == 0.0) return t1;
  double t2 = trilinear(N, bits, mips, d1 + 1, s);
  return (1.0 - fr) * t1 + fr * t2;
}

// cacheLightingRSM.comp:103-104, 195-230.
double orc_cone_shadow(const DrvVolumeInfo* vol, int N, const uint32_t* bits, const double* mips, const double cp[3],
                       const double av[3], double dsr, int max_steps) {
  d3 world = ld3(cp);
  d3 vmin = ld3(vol->volume_world_min);
  double vs = vol->voxel_size_in_world;
  d3 voxel_pos = (world - vmin) * (1.0 / (vs * N));
  d3 to = ld3(av) - world;
  double light_dist = length(to);
  to = to * (1.0 / light_dist);
  d3 dir_in_voxel = to * (1.0 / N);
  d3 cur = voxel_pos + dir_in_voxel * 2.0;
  double occlusion = 0.0, step = 1.0, dist = 0.0;
  double goal = light_dist / vs - 2.0;
  double k = 2.0 / (1.0 - dsr);
  for (int s = 0; s < max_steps; ++s) {
    cur = cur + dir_in_voxel * step;
    dist += step;
    double radius = dist * dsr;
    double p[3] = {cur.x, cur.y, cur.z};
    double occ = orc_sample_voxels(N, bits, mips, p, std::log2(radius));
    occlusion += (1.0 - occlusion) * occ;
    if (dist >= goal) break;
    step = std::max(1.0, radius * k);
  }
  return saturate(1.0 - occlusion);
}

// Renderer::PrepareLights, renderer.cpp:664-725 (float host math as there;
// matrices computed in FP64 and rounded, a convention shared with the product).
void orc_prepare_light(const DrvLightDesc* L, DrvSpotLight* o) {
  std::memset(o, 0, sizeof(*o));
  for (int i = 0; i < 3; ++i) {
    o->intensity[i] = L->intensity[i];
    o->position[i] = L->position[i];
  }
  d3 dir = normalize(ld3(L->direction));
  o->direction[0] = (float)dir.x;
  o->direction[1] = (float)dir.y;
  o->direction[2] = (float)dir.z;
  o->shadow_normal_offset = 0.01f;
  o->shadow_bias = 0.0001f;
  o->cos_half_angle = cosf(L->half_angle);
  m4 v = view_matrix(ld3(L->position), dir, mk(0, 1, 0));
  m4 p = proj_reversed(2.0 * L->half_angle, 1.0, L->near_plane, L->far_plane);
  m4 vp = mul(p, v), inv;
  invert(vp, inv);
  store(vp, o->view_projection);
  store(inv, o->inverse_view_projection);
  int r = 1;
  while ((uint32_t)r < L->rsm_resolution) r <<= 1;
  o->rsm_render_resolution = r;
  int read = r >> L->rsm_read_lod;
  o->rsm_read_resolution = read;
  float clip_w = sinf(L->half_angle) * L->near_plane * 2.0f;
  float vaf = clip_w * clip_w / (L->near_plane * L->near_plane * (float)read * (float)read);
  o->val_area_factor = vaf;
  o->indirect_shadow_lod = (float)L->indirect_shadow_lod;
  float bs = (float)(1 << L->indirect_shadow_lod);
  o->indirect_shadow_block_size = bs;
  o->indirect_shadow_sample_interval = (int)(bs * bs);
  o->indirect_shadow_super_val_width = sqrtf(vaf) * bs;
  o->indirect_shadow_sampling_offset = 0.5f + sqrtf(2.0f) * bs / 2.0f;
}

// Renderer::UpdatePerFrameUBO, renderer.cpp:324-344, camera.hpp:27-30.
void orc_prepare_camera(const DrvCamera* c, DrvPerFrame* o) {
  std::memset(o, 0, sizeof(*o));
  d3 dir = normalize(ld3(c->direction));
  m4 v = view_matrix(ld3(c->position), dir, ld3(c->up));
  m4 p = proj_reversed(c->fov_y_deg * (kPi / 180.0), c->aspect, c->near_plane, c->far_plane);
  m4 vp = mul(p, v), inv;
  invert(vp, inv);
  store(vp, o->view_projection);
  store(inv, o->inverse_view_projection);
  for (int i = 0; i < 3; ++i) o->camera_position[i] = c->position[i];
  o->camera_direction[0] = (float)dir.x;
  o->camera_direction[1] = (float)dir.y;
  o->camera_direction[2] = (float)dir.z;
}

// Renderer::UpdateVolumeUBO, renderer.cpp:346-431 ("simple version"), float.
void orc_compute_volume_info(const DrvConfig* cfg, const float amin[3], const float amax[3], const float cam[3],
                             DrvVolumeInfo* o) {
  std::memset(o, 0, sizeof(*o));
  float mn[3], mx[3], ext[3];
  for (int i = 0; i < 3; ++i) {
    mn[i] = amin[i] - 0.001f;
    mx[i] = amax[i] + 0.001f;
    ext[i] = mx[i] - mn[i];
  }
  float largest = std::max(std::max(ext[0], ext[1]), ext[2]);
  for (int i = 0; i < 3; ++i) {
    float grow = largest - ext[i];
    mx[i] = mx[i] + grow;
    o->volume_world_min[i] = mn[i];
    o->volume_world_max[i] = mx[i];
  }
  o->voxel_size_in_world = (mx[0] - mn[0]) / (float)cfg->voxel_res;
  o->cav_transition_zone_size = cfg->cascade_transition;
  for (int c = 0; c < cfg->n_cascades; ++c) {
    float size = cfg->cascade_world_size[c];
    float cell = size / (float)cfg->cav_res;
    DrvCascade& k = o->cascades[c];
    k.world_voxel_size = cell;
    for (int i = 0; i < 3; ++i) {
      float snapped = roundf(cam[i] / cell) * cell;
      float half = size * 0.5f;
      k.min[i] = snapped - half;
      k.max[i] = snapped + half;
      float off = cell * 1.5f;
      k.decision_min[i] = (cam[i] - half) + off;
      k.decision_max[i] = (cam[i] + half) - off;
    }
  }
}

// fillgbuffer.frag:21-43 as a ray cast (no normal maps: the shading normal is
// the face normal; base colour is the box albedo).
void orc_raycast_gbuffer(const DrvBox* boxes, int n, const DrvPerFrame* f, const DrvCamera* cam, int W, int H,
                         float* depth, int16_t* n16, float* n32, float* alb) {
  d3 r, u, fw;
  basis(ld3(cam->direction), ld3(cam->up), r, u, fw);
  double ty = std::tan(cam->fov_y_deg * (kPi / 180.0) * 0.5), tx = ty * cam->aspect;
  d3 o = ld3(cam->position);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      double nx = ((x + 0.5) / W) * 2.0 - 1.0, ny = ((y + 0.5) / H) * 2.0 - 1.0;
      d3 d = normalize(fw + r * (nx * tx) + u * (ny * ty));
      double t;
      int ax = 0;
      int b = trace(boxes, n, o, d, t, ax);
      if (b < 0) {
        depth[i] = 0.0f;
        if (n16) n16[2 * i] = n16[2 * i + 1] = 0;
        if (n32) n32[3 * i] = n32[3 * i + 1] = n32[3 * i + 2] = 0.0f;
        for (int c = 0; c < 3; ++c) alb[3 * i + c] = 0.0f;
        continue;
      }
      d3 p = o + d * t;
      double cz = 0, cw = 0;
      const float* M = f->view_projection;
      cz = M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11];
      cw = M[12] * p.x + M[13] * p.y + M[14] * p.z + M[15];
      depth[i] = (float)(cz / cw);
      double nrm[3] = {0, 0, 0};
      double dd[3] = {d.x, d.y, d.z};
      nrm[ax] = dd[ax] > 0 ? -1.0 : 1.0;
      if (n16) orc_pack_normal16i(nrm, n16 + 2 * i);
      if (n32)
        for (int c = 0; c < 3; ++c) n32[3 * i + c] = (float)nrm[c];
      for (int c = 0; c < 3; ++c) alb[3 * i + c] = boxes[b].albedo[c];
    }
}

// fillrsm.frag:24-62 (+ lightingfunctions.glsl:3-15) as a ray cast from the
// spot light through each RSM texel centre; the ray direction is the one the
// VPL reconstruction uses (unprojection at depth 0, cacheLightingRSM.comp:154-155).
void orc_raycast_rsm(const DrvBox* boxes, int n, const DrvSpotLight* L, float* flux, int16_t* n16, float* dls) {
  int R = L->rsm_render_resolution;
  d3 o = ld3(L->position);
  d3 ldir = ld3(L->direction);
  double cos_half = L->cos_half_angle;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < R; ++y)
    for (int x = 0; x < R; ++x) {
      size_t i = (size_t)y * R + x;
      d3 d = unproject_dir(L->inverse_view_projection, (x + 0.5) / R, (y + 0.5) / R, o);
      double th;
      int ax = 0;
      int b = trace(boxes, n, o, d, th, ax);
      if (b < 0) {
        flux[3 * i] = flux[3 * i + 1] = flux[3 * i + 2] = 0.0f;
        n16[2 * i] = n16[2 * i + 1] = 0;
        dls[2 * i] = dls[2 * i + 1] = 0.0f;
        continue;
      }
      d3 p = o + d * th;
      d3 to_light = o - p;
      double dist = length(to_light);
      to_light = to_light * (1.0 / dist);
      double cos_to_light = saturate(dot(to_light * -1.0, ldir));
      double total_sr = 2.0 * kShaderPi * (1.0 - cos_half);
      double pixel_sr = total_sr * cos_to_light / R / R;
      double falloff = saturate(cos_to_light - cos_half) / (1.0 - cos_half);
      for (int c = 0; c < 3; ++c)
        flux[3 * i + c] = (float)(boxes[b].albedo[c] * L->intensity[c] * (falloff * pixel_sr / kShaderPi));
      dls[2 * i] = (float)dist;
      dls[2 * i + 1] = (float)(dist * dist);
      double nrm[3] = {0, 0, 0};
      double dd[3] = {d.x, d.y, d.z};
      nrm[ax] = dd[ax] > 0 ? -1.0 : 1.0;
      orc_pack_normal16i(nrm, n16 + 2 * i);
    }
}

// The same producers for a triangle mesh (positions xyz per vertex, optional
// vertex normals, optional RGB albedo per triangle, optional indices): the
// nearest triangle along each ray (either face, inside the depth range),
// normal = face normal or the barycentric blend of the vertex normals, turned
// towards the ray.
namespace {
struct MeshIn {
  const float* pos;
  const float* nrm;
  const float* alb;
  const uint32_t* idx;
  int nt;
};

d3 mesh_vertex(const MeshIn& m, uint32_t i) { return {m.pos[3 * i], m.pos[3 * i + 1], m.pos[3 * i + 2]}; }

void mesh_tri(const MeshIn& m, int k, uint32_t v[3]) {
  for (int j = 0; j < 3; ++j) v[j] = m.idx ? m.idx[3 * k + j] : 3u * k + j;
}

// Clip-space depth z/w of p under the row-major view-projection M, and
// whether it lies in the rasteriser's depth range [0, 1] (near and far
// planes; reversed-Z, so nearer is larger).
bool in_depth_range(const float* M, d3 p) {
  const double cz = M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11];
  const double cw = M[12] * p.x + M[13] * p.y + M[14] * p.z + M[15];
  if (!(cw > 0.0)) return false;
  const double z = cz / cw;
  return z >= 0.0 && z <= 1.0;
}

// Nearest hit (Moller-Trumbore, both faces, t > 1e-6) inside the target's
// depth range, as a rasteriser clips against the near and far planes:
// triangle or -1.
int mesh_trace(const MeshIn& m, const float* M, d3 o, d3 d, double& t_hit, double& l1, double& l2) {
  int best = -1;
  t_hit = 1e300;
  for (int k = 0; k < m.nt; ++k) {
    uint32_t v[3];
    mesh_tri(m, k, v);
    const d3 v0 = mesh_vertex(m, v[0]), e1 = mesh_vertex(m, v[1]) - v0, e2 = mesh_vertex(m, v[2]) - v0;
    const d3 pv = cross(d, e2);
    const double det = dot(e1, pv);
    if (std::fabs(det) < 1e-300) continue;
    const double inv = 1.0 / det;
    const d3 tv = o - v0;
    const double a = dot(tv, pv) * inv;
    if (a < 0.0 || a > 1.0) continue;
    const d3 qv = cross(tv, e1);
    const double b = dot(d, qv) * inv;
    if (b < 0.0 || a + b > 1.0) continue;
    const double t = dot(e2, qv) * inv;
    if (t > 1e-6 && t < t_hit && in_depth_range(M, o + d * t)) {
      t_hit = t;
      best = k;
      l1 = a;
      l2 = b;
    }
  }
  return best;
}

d3 mesh_normal(const MeshIn& m, int k, double l1, double l2, d3 d) {
  uint32_t v[3];
  mesh_tri(m, k, v);
  d3 n;
  if (m.nrm) {
    auto vn = [&](uint32_t i) { return d3{m.nrm[3 * i], m.nrm[3 * i + 1], m.nrm[3 * i + 2]}; };
    n = vn(v[0]) * (1.0 - l1 - l2) + vn(v[1]) * l1 + vn(v[2]) * l2;
  } else {
    const d3 v0 = mesh_vertex(m, v[0]);
    n = cross(mesh_vertex(m, v[1]) - v0, mesh_vertex(m, v[2]) - v0);
  }
  // Normalised through the largest component first, so that an axis-aligned
  // normal comes out exactly (+-1 on its axis, as the box casters give it).
  const double big = std::max(std::max(std::fabs(n.x), std::fabs(n.y)), std::fabs(n.z));
  n = big > 0.0 ? normalize(d3{n.x / big, n.y / big, n.z / big}) : d3{0.0, 0.0, 1.0};
  if (dot(n, d) > 0.0) n = n * -1.0;
  return d3{n.x + 0.0, n.y + 0.0, n.z + 0.0};  // no negative zeros (they pack to the other end of the atan2 range)
}
}  // namespace

void orc_raycast_gbuffer_mesh(const float* pos, const float* nrm, const float* alb, const uint32_t* idx, int n_tris,
                              const DrvPerFrame* f, const DrvCamera* cam, int W, int H, float* depth, int16_t* n16,
                              float* n32, float* albedo) {
  const MeshIn m{pos, nrm, alb, idx, n_tris};
  d3 r, u, fw;
  basis(ld3(cam->direction), ld3(cam->up), r, u, fw);
  double ty = std::tan(cam->fov_y_deg * (kPi / 180.0) * 0.5), tx = ty * cam->aspect;
  d3 o = ld3(cam->position);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      double nx = ((x + 0.5) / W) * 2.0 - 1.0, ny = ((y + 0.5) / H) * 2.0 - 1.0;
      d3 d = normalize(fw + r * (nx * tx) + u * (ny * ty));
      double t, l1 = 0, l2 = 0;
      const int k = mesh_trace(m, f->view_projection, o, d, t, l1, l2);
      if (k < 0) {
        depth[i] = 0.0f;
        if (n16) n16[2 * i] = n16[2 * i + 1] = 0;
        if (n32) n32[3 * i] = n32[3 * i + 1] = n32[3 * i + 2] = 0.0f;
        for (int c = 0; c < 3; ++c) albedo[3 * i + c] = 0.0f;
        continue;
      }
      d3 p = o + d * t;
      const float* M = f->view_projection;
      double cz = M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11];
      double cw = M[12] * p.x + M[13] * p.y + M[14] * p.z + M[15];
      depth[i] = (float)(cz / cw);
      const d3 n = mesh_normal(m, k, l1, l2, d);
      double nn[3] = {n.x, n.y, n.z};
      if (n16) orc_pack_normal16i(nn, n16 + 2 * i);
      if (n32)
        for (int c = 0; c < 3; ++c) n32[3 * i + c] = (float)nn[c];
      for (int c = 0; c < 3; ++c) albedo[3 * i + c] = alb ? alb[3 * k + c] : 1.0f;
    }
}

void orc_raycast_rsm_mesh(const float* pos, const float* nrm, const float* alb, const uint32_t* idx, int n_tris,
                          const DrvSpotLight* L, float* flux, int16_t* n16, float* dls) {
  const MeshIn m{pos, nrm, alb, idx, n_tris};
  int R = L->rsm_render_resolution;
  d3 o = ld3(L->position);
  d3 ldir = ld3(L->direction);
  double cos_half = L->cos_half_angle;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < R; ++y)
    for (int x = 0; x < R; ++x) {
      size_t i = (size_t)y * R + x;
      d3 d = unproject_dir(L->inverse_view_projection, (x + 0.5) / R, (y + 0.5) / R, o);
      double th, l1 = 0, l2 = 0;
      const int k = mesh_trace(m, L->view_projection, o, d, th, l1, l2);
      if (k < 0) {
        flux[3 * i] = flux[3 * i + 1] = flux[3 * i + 2] = 0.0f;
        n16[2 * i] = n16[2 * i + 1] = 0;
        dls[2 * i] = dls[2 * i + 1] = 0.0f;
        continue;
      }
      d3 p = o + d * th;
      d3 to_light = o - p;
      double dist = length(to_light);
      to_light = to_light * (1.0 / dist);
      double cos_to_light = saturate(dot(to_light * -1.0, ldir));
      double total_sr = 2.0 * kShaderPi * (1.0 - cos_half);
      double pixel_sr = total_sr * cos_to_light / R / R;
      double falloff = saturate(cos_to_light - cos_half) / (1.0 - cos_half);
      for (int c = 0; c < 3; ++c)
        flux[3 * i + c] = (float)((alb ? alb[3 * k + c] : 1.0f) * L->intensity[c] * (falloff * pixel_sr / kShaderPi));
      dls[2 * i] = (float)dist;
      dls[2 * i + 1] = (float)(dist * dist);
      const d3 n = mesh_normal(m, k, l1, l2, d);
      double nn[3] = {n.x, n.y, n.z};
      orc_pack_normal16i(nn, n16 + 2 * i);
    }
}

// downsamplersm.frag:15-33: flux = sum of the 2x2 children (textureGather),
// normal = PackNormal16I(normalize(sum of unpacked)), (d, d^2) = bilinear at
// the shared corner = mean of the 4 children.
void orc_downsample_rsm(int res, const float* flux, const int16_t* nrm, const float* dls, float* fo, int16_t* no,
                        float* dlo) {
  int h = res / 2;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < h; ++x) {
      double fs[3] = {0, 0, 0}, ns[3] = {0, 0, 0}, ds[2] = {0, 0};
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          size_t j = (size_t)(2 * y + dy) * res + (2 * x + dx);
          for (int c = 0; c < 3; ++c) fs[c] += flux[3 * j + c];
          double un[3];
          orc_unpack_normal16i(nrm + 2 * j, un);
          for (int c = 0; c < 3; ++c) ns[c] += un[c];
          ds[0] += dls[2 * j];
          ds[1] += dls[2 * j + 1];
        }
      size_t i = (size_t)y * h + x;
      for (int c = 0; c < 3; ++c) fo[3 * i + c] = (float)fs[c];
      double len = std::sqrt(ns[0] * ns[0] + ns[1] * ns[1] + ns[2] * ns[2]);
      if (len > 0.0) {
        double nn[3] = {ns[0] / len, ns[1] / len, ns[2] / len};
        orc_pack_normal16i(nn, no + 2 * i);
      } else {
        no[2 * i] = no[2 * i + 1] = 0;
      }
      dlo[2 * i] = (float)(ds[0] * 0.25);
      dlo[2 * i + 1] = (float)(ds[1] * 0.25);
    }
}

// cacheLightingRSM.comp:141-158 (VPL) and 168-192 (shadow cone source).
void orc_extract_vpls(const DrvSpotLight* L, int R, const float* flux, const int16_t* nrm, const float* dls,
                      const float* dls_shadow, double* vo, double* co) {
  d3 lp = ld3(L->position);
  int n = R * R;
  for (int i = 0; i < n; ++i) {
    uint32_t x, y;
    orc_morton_decode((uint32_t)i, &x, &y);
    size_t t = (size_t)y * R + x;
    double u = (x + 0.5) / R, v = (y + 0.5) / R;
    double d = dls[2 * t];
    for (int c = 0; c < 3; ++c) vo[10 * i + c] = flux[3 * t + c];
    vo[10 * i + 3] = d * d * L->val_area_factor;
    d3 p = lp + unproject_dir(L->inverse_view_projection, u, v, lp) * d;
    vo[10 * i + 4] = p.x;
    vo[10 * i + 5] = p.y;
    vo[10 * i + 6] = p.z;
    double un[3];
    orc_unpack_normal16i(nrm + 2 * t, un);
    vo[10 * i + 7] = un[0];
    vo[10 * i + 8] = un[1];
    vo[10 * i + 9] = un[2];
  }
  int interval = L->indirect_shadow_sample_interval;
  int lod = (int)L->indirect_shadow_lod;
  int rs = R >> lod;
  for (int b = 0; b * interval < n; ++b) {
    uint32_t x, y;
    orc_morton_decode((uint32_t)(b * interval), &x, &y);
    double u = (x + (double)L->indirect_shadow_sampling_offset) / R;
    double v = (y + (double)L->indirect_shadow_sampling_offset) / R;
    double dd[2];
    bilinear2(rs, dls_shadow, u, v, dd);
    d3 avg = lp + unproject_dir(L->inverse_view_projection, u, v, lp) * dd[0];
    // depthVariance can round below zero; clamped (sqrt of a negative is
    // undefined in GLSL).
    double var = std::max(0.0, dd[1] - dd[0] * dd[0]);
    double dsr = std::max((double)L->indirect_shadow_super_val_width, std::sqrt(var) * 2.0 / dd[0]);
    co[4 * b + 0] = avg.x;
    co[4 * b + 1] = avg.y;
    co[4 * b + 2] = avg.z;
    co[4 * b + 3] = dsr;
  }
}

// voxelize.{vert,geom,frag}: conservative surface voxelization. For an
// axis-aligned face the dominant axis is its normal axis, the depth gradient
// is zero (no +-1 depth voxels, voxelize.frag:295-313) and the dilated
// triangles with their half-voxel raster AABB (voxelize.geom:201-225,
// voxelize.frag:280-283) cover every voxel whose square touches the face
// rectangle (closed intervals). Binary32 mirror with the kernel.
void orc_voxelize(const DrvBox* boxes, int n, const DrvVolumeInfo* vol, int N, uint32_t* bits) {
  size_t words = ((size_t)N * N * N + 31) / 32;
  std::memset(bits, 0, words * 4);
  const float* vm = vol->volume_world_min;
  float vs = vol->voxel_size_in_world;
  for (int b = 0; b < n; ++b)
    for (int axis = 0; axis < 3; ++axis)
      for (int side = 0; side < 2; ++side) {
        int ua = (axis + 1) % 3, va = (axis + 2) % 3;
        float plane = side ? boxes[b].max[axis] : boxes[b].min[axis];
        float kc = (plane - vm[axis]) / vs;
        if (!(kc >= 0.0f) || !(kc < (float)N)) continue;
        int k = (int)kc;
        float lo_u = (boxes[b].min[ua] - vm[ua]) / vs, hi_u = (boxes[b].max[ua] - vm[ua]) / vs;
        float lo_v = (boxes[b].min[va] - vm[va]) / vs, hi_v = (boxes[b].max[va] - vm[va]) / vs;
        int u0 = std::max(0, (int)std::ceil(lo_u) - 1), u1 = std::min(N - 1, (int)std::floor(hi_u));
        int v0 = std::max(0, (int)std::ceil(lo_v) - 1), v1 = std::min(N - 1, (int)std::floor(hi_v));
        for (int vv = v0; vv <= v1; ++vv)
          for (int uu = u0; uu <= u1; ++uu) {
            int c[3];
            c[axis] = k;
            c[ua] = uu;
            c[va] = vv;
            size_t i = ((size_t)c[2] * N + c[1]) * N + c[0];
            bits[i >> 5] |= 1u << (i & 31);
          }
      }
}

// voxelize.{vert,geom,frag} for a triangle mesh (binary32, no contraction):
// positions in voxel units w = (p - VolumeWorldMin) / VoxelSizeInWorld
// (window coordinates of the reference's VoxelResolution^2 viewport); the
// dominant axis of the normal picks the projection (voxelize.geom:24-51,
// ties as there); each edge line is moved outward by half a voxel in the L1
// sense (voxelize.geom:70-86) and the pixel centres inside all three moved
// lines (inclusive) and inside the triangle's AABB grown by half a voxel
// (voxelize.geom:59-62, voxelize.frag:22-26; inclusive) are covered; the
// depth is the plane through the moved vertices with the original vertices'
// depths (voxelize.geom:89-107), voxel z = int(depth), plus z - 1 / z + 1 where
// int(depth -+ 1.414 |grad depth|) differs (voxelize.frag:39-55); fragments
// with depth outside [0, N] are clipped, stores outside the grid ignored.
namespace {
struct TriSetup {
  int side;
  float r[3][3];       // swizzled vertices (raster x, raster y, depth)
  float plane[3][3];   // moved edge lines a x + b y + c (inside: <= 0)
  float aabb[4];       // x0, y0, x1, y1
  float zA, zB, zC;    // depth plane z = zA x + zB y + zC
  float max_change;
  bool ok;
};

TriSetup tri_setup(const float* p0, const float* p1, const float* p2, const float* vm, float vs) {
  TriSetup t{};
  float w[3][3];
  const float* P[3] = {p0, p1, p2};
  for (int i = 0; i < 3; ++i)
    for (int a = 0; a < 3; ++a) w[i][a] = (P[i][a] - vm[a]) / vs;
  const float e0[3] = {w[1][0] - w[0][0], w[1][1] - w[0][1], w[1][2] - w[0][2]};
  const float e1[3] = {w[2][0] - w[0][0], w[2][1] - w[0][1], w[2][2] - w[0][2]};
  const float n[3] = {std::fabs(e0[1] * e1[2] - e0[2] * e1[1]), std::fabs(e0[2] * e1[0] - e0[0] * e1[2]),
                      std::fabs(e0[0] * e1[1] - e0[1] * e1[0])};
  int side = n[0] > n[1] ? 0 : 1;
  side = n[side] > n[2] ? side : 2;
  t.side = side;
  for (int i = 0; i < 3; ++i) {
    const float x = w[i][0], y = w[i][1], z = w[i][2];
    if (side == 0) { t.r[i][0] = z; t.r[i][1] = y; t.r[i][2] = x; }
    else if (side == 1) { t.r[i][0] = x; t.r[i][1] = z; t.r[i][2] = y; }
    else { t.r[i][0] = x; t.r[i][1] = y; t.r[i][2] = z; }
  }
  t.aabb[0] = std::min(std::min(t.r[0][0], t.r[1][0]), t.r[2][0]) - 0.5f;
  t.aabb[1] = std::min(std::min(t.r[0][1], t.r[1][1]), t.r[2][1]) - 0.5f;
  t.aabb[2] = std::max(std::max(t.r[0][0], t.r[1][0]), t.r[2][0]) + 0.5f;
  t.aabb[3] = std::max(std::max(t.r[0][1], t.r[1][1]), t.r[2][1]) + 0.5f;
  // Edge i runs from vertex from[i] to vertex to[i] (voxelize.geom:66-71).
  const int from[3] = {2, 0, 1}, to[3] = {0, 1, 2};
  const float ax = t.r[0][0] - t.r[2][0], ay = t.r[0][1] - t.r[2][1];
  const float bx = t.r[1][0] - t.r[0][0], by = t.r[1][1] - t.r[0][1];
  const float area = ax * by - bx * ay;
  if (!(area != 0.0f)) return t;  // degenerate in its own projection: nothing rasterised
  const float wind = area > 0.0f ? 1.0f : -1.0f;
  for (int i = 0; i < 3; ++i) {
    const float dx = t.r[to[i]][0] - t.r[from[i]][0], dy = t.r[to[i]][1] - t.r[from[i]][1];
    const float px = t.r[from[i]][0], py = t.r[from[i]][1];
    const float a = dy * wind, b = -dx * wind, c = (dx * py - dy * px) * wind;
    t.plane[i][0] = a;
    t.plane[i][1] = b;
    t.plane[i][2] = c - 0.5f * (std::fabs(a) + std::fabs(b));
  }
  // Moved vertices: vertex i = moved line i intersected with moved line i+1
  // (voxelize.geom:95-107), with vertex i's depth.
  float V[3][2];
  for (int i = 0; i < 3; ++i) {
    const float* L0 = t.plane[i];
    const float* L1 = t.plane[(i + 1) % 3];
    const float hx = L0[1] * L1[2] - L0[2] * L1[1], hy = L0[2] * L1[0] - L0[0] * L1[2],
                hw = L0[0] * L1[1] - L0[1] * L1[0];
    if (!(hw != 0.0f)) return t;
    V[i][0] = hx / hw;
    V[i][1] = hy / hw;
  }
  const float x10 = V[1][0] - V[0][0], y10 = V[1][1] - V[0][1], x20 = V[2][0] - V[0][0], y20 = V[2][1] - V[0][1];
  const float z10 = t.r[1][2] - t.r[0][2], z20 = t.r[2][2] - t.r[0][2];
  const float det = x10 * y20 - x20 * y10;
  if (!(det != 0.0f)) return t;
  t.zA = (z10 * y20 - z20 * y10) / det;
  t.zB = (x10 * z20 - x20 * z10) / det;
  t.zC = t.r[0][2] - t.zA * V[0][0] - t.zB * V[0][1];
  t.max_change = std::sqrt(t.zA * t.zA + t.zB * t.zB) * 1.414f;
  t.ok = true;
  return t;
}

inline void set_voxel_swz(uint32_t* bits, int N, int side, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= N || y >= N || z >= N) return;
  int c[3];
  if (side == 0) { c[0] = z; c[1] = y; c[2] = x; }
  else if (side == 1) { c[0] = x; c[1] = z; c[2] = y; }
  else { c[0] = x; c[1] = y; c[2] = z; }
  const size_t i = ((size_t)c[2] * N + c[1]) * N + c[0];
  bits[i >> 5] |= 1u << (i & 31);
}
}  // namespace

void orc_voxelize_triangles(const float* positions, const uint32_t* indices, int n_tris, const DrvVolumeInfo* vol,
                            int N, uint32_t* bits) {
  std::memset(bits, 0, (((size_t)N * N * N + 31) / 32) * 4);
  for (int k = 0; k < n_tris; ++k) {
    const uint32_t i0 = indices ? indices[3 * k] : 3u * k, i1 = indices ? indices[3 * k + 1] : 3u * k + 1,
                   i2 = indices ? indices[3 * k + 2] : 3u * k + 2;
    const TriSetup t = tri_setup(positions + 3 * i0, positions + 3 * i1, positions + 3 * i2,
                                 vol->volume_world_min, vol->voxel_size_in_world);
    if (!t.ok) continue;
    const int x0 = std::max(0, (int)std::floor(t.aabb[0])), y0 = std::max(0, (int)std::floor(t.aabb[1]));
    const int x1 = std::min(N - 1, (int)std::floor(t.aabb[2])), y1 = std::min(N - 1, (int)std::floor(t.aabb[3]));
    for (int py = y0; py <= y1; ++py)
      for (int px = x0; px <= x1; ++px) {
        const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
        if (cx < t.aabb[0] || cy < t.aabb[1] || cx > t.aabb[2] || cy > t.aabb[3]) continue;
        bool in = true;
        for (int e = 0; e < 3; ++e) in = in && (t.plane[e][0] * cx + t.plane[e][1] * cy + t.plane[e][2] <= 0.0f);
        if (!in) continue;
        const float z = t.zA * cx + t.zB * cy + t.zC;
        if (!(z >= 0.0f && z <= (float)N)) continue;
        const int zi = (int)z;
        set_voxel_swz(bits, N, t.side, px, py, zi);
        if ((int)(z - t.max_change) != zi) set_voxel_swz(bits, N, t.side, px, py, zi - 1);
        if ((int)(z + t.max_change) != zi) set_voxel_swz(bits, N, t.side, px, py, zi + 1);
      }
  }
}

// voxelmipmap.comp:8-13: a linear sample at the corner shared by 8 children
// is their mean (stored as R8 in the reference; kept exact here).
void orc_build_mips(int N, const uint32_t* bits, double* mips) {
  int L = ilog2(N);
  for (int l = 1; l <= L; ++l) {
    int n = N >> l;
    double* dst = mips + mip_offset(N, l);
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          double s = 0;
          for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
              for (int dx = 0; dx < 2; ++dx) s += texel(N, bits, mips, l - 1, 2 * x + dx, 2 * y + dy, 2 * z + dz);
          dst[((size_t)z * n + y) * n + x] = s / 8.0;
        }
  }
}

// cacheGather.comp:32-164 executed workgroup by workgroup (16x16 tiles).
int orc_allocate_caches(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* f, int W, int H,
                        const float* depth, uint32_t* atlas, float* pos, uint32_t* count_out) {
  const int res = cfg->cav_res, nC = cfg->n_cascades;
  const int res2 = res * res, res3 = res2 * res;
  const int AW = nC * res;  // atlas width
  std::memset(atlas, 0, (size_t)AW * res * res * 4);
  const bool transitions = cfg->cascade_transition > 0.0f;
  uint32_t count = 0;
  int status = DRV_OK;
  // AllocateCaches, cacheGather.comp:32-91. Out-of-atlas corners are skipped.
  auto allocate = [&](int coord, int cascade) {
    static const int off[8][3] = {{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}, {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}};
    int base = coord - res3 * cascade;
    int bz = base / res2, by = (base - bz * res2) / res, bx = base % res;
    for (int i = 0; i < 8; ++i) {
      int lx = bx + off[i][0], ly = by + off[i][1], lz = bz + off[i][2];
      int ax = lx + cascade * res;
      if (ax >= AW || ly >= res || lz >= res) continue;
      size_t a = ((size_t)lz * res + ly) * AW + ax;
      if (atlas[a] != 0u) continue;
      atlas[a] = 0xFFFFFFFFu;
      uint32_t idx = count++;
      if (idx >= cfg->max_caches) {
        status = DRV_ERR_CAPACITY;
        continue;  // stays locked; apply treats it as empty
      }
      const DrvCascade& k = vol->cascades[cascade];
      float fx = (float)lx * k.world_voxel_size;
      float fy = (float)ly * k.world_voxel_size;
      float fz = (float)lz * k.world_voxel_size;
      pos[3 * idx + 0] = fx + k.min[0];
      pos[3 * idx + 1] = fy + k.min[1];
      pos[3 * idx + 2] = fz + k.min[2];
      atlas[a] = idx + 1;
    }
  };
  const int TS = 16;
  int tiles_x = (W + TS - 1) / TS, tiles_y = (H + TS - 1) / TS;
  int list1[TS][TS], list2[TS][TS], own1[TS][TS], own2[TS][TS], casc[TS][TS];
  for (int ty = 0; ty < tiles_y; ++ty)
    for (int tx = 0; tx < tiles_x; ++tx) {
      for (int ly = 0; ly < TS; ++ly)
        for (int lx = 0; lx < TS; ++lx) {
          list1[lx][ly] = list2[lx][ly] = -1;
          own1[lx][ly] = own2[lx][ly] = -1;
          casc[lx][ly] = -1;
          int px = tx * TS + lx, py = ty * TS + ly;
          if (px >= W || py >= H) continue;
          float d = depth[(size_t)py * W + px];
          if (!(d > 0.0001f)) continue;
          float p[3];
          reconstruct_world_f32(f, px, py, W, H, d, p);
          int c = select_cascade_f32(vol, nC, p);
          casc[lx][ly] = c;
          own1[lx][ly] = list1[lx][ly] = cache_1d_coord_f32(vol, res, c, p);
          if (transitions) {
            float t = cascade_transition_f32(vol, c, p);
            if (t > 0.0f && c < nC - 1) own2[lx][ly] = list2[lx][ly] = cache_1d_coord_f32(vol, res, c + 1, p);
          }
        }
      // Threads run in x-fastest order within the tile (the allocation index
      // order is not part of the contract; only the set is).
      for (int ly = 0; ly < TS; ++ly)
        for (int lx = 0; lx < TS; ++lx) {
          int own = own1[lx][ly];
          int ux = std::max(0, lx - 1), uy = std::max(0, ly - 1);
          bool self = (ux == lx && uy == ly);
          if (((list1[lx][uy] != own && list1[ux][ly] != own && list1[ux][uy] != own) || self) && own != -1)
            allocate(own, casc[lx][ly]);
          if (transitions) {
            int own_b = own2[lx][ly];
            int dx = std::min(TS - 1, lx + 1), dy = std::min(TS - 1, ly + 1);
            bool corner = (dx == TS - 1 && dy == TS - 1);
            if (((list2[lx][dy] != own_b && list2[dx][ly] != own_b && list2[dx][dy] != own_b) || corner) &&
                own_b != -1)
              allocate(own_b, casc[lx][ly] + 1);
          }
        }
    }
  *count_out = count;
  return status;
}

// cacheLightingRSM.comp:80-374, all lights accumulated (the reference
// dispatches once per light and adds into the entries).
void orc_light_caches(const DrvConfig* cfg, const DrvVolumeInfo* vol, int n_caches, const float* positions,
                      int n_lights, const DrvSpotLight* lights, const double* const* vpls,
                      const double* const* cones, const int* n_vpls, const uint32_t* bits, const double* mips,
                      double* sh_out, int n_threads) {
  orc_light_caches_specular(cfg, vol, n_caches, positions, nullptr, n_lights, lights, vpls, cones, n_vpls, bits, mips,
                            sh_out, nullptr, n_threads);
}

namespace {
// ComputeLocalViewSpace (lightcache.glsl:98-106).
void local_view_space(d3 cam, d3 p, d3& x, d3& y, d3& z) {
  z = normalize(cam - p);
  x = normalize(mk(z.z, 0.0, -z.x));
  y = cross(z, x);
}

// HemisphericalProjection, concentric square map (utils.glsl:103-170).
void hemi_projection(d3 d, double& u, double& v) {
  const double r = std::sqrt(std::max(1.0 - d.z, 0.0)) * 0.5;
  double phi = std::atan2(d.y, d.x) * (4.0 / kShaderPi);
  if (phi < -1.0) phi += 8.0;
  double px, py;
  if (phi < 3.0) {
    if (phi < 1.0) {
      px = r;
      py = phi * r;
    } else {
      px = -(phi - 2.0) * r;
      py = r;
    }
  } else if (phi < 5.0) {
    px = -r;
    py = -(phi - 4.0) * r;
  } else {
    px = (phi - 6.0) * r;
    py = -r;
  }
  u = px + 0.5;
  v = py + 0.5;
}

// GL unsigned 11/10-bit float (5-bit exponent, bias 15, mbits of mantissa)
// from a double: negative -> 0, NaN -> NaN, +inf -> inf, above the largest
// finite value -> that value, else the nearest value (ties to even).
uint32_t encode_ufloat(double x, int mbits) {
  const uint32_t mmask = (1u << mbits) - 1u;
  if (std::isnan(x)) return (31u << mbits) | 1u;
  if (!(x > 0.0)) return 0u;
  if (std::isinf(x)) return 31u << mbits;
  int e;
  std::frexp(x, &e);  // x = m 2^e, m in [0.5, 1)
  int E = e + 14;     // biased exponent of a normal result
  if (E < 1) return (uint32_t)std::nearbyint(std::ldexp(x, 14 + mbits));  // subnormal (2^mbits: smallest normal)
  double q = std::nearbyint(std::ldexp(x, mbits - (e - 1)));               // in [2^mbits, 2^(mbits+1)]
  if (q >= (double)(2u << mbits)) {
    q = (double)(1u << mbits);
    ++E;
  }
  if (E > 30) return (30u << mbits) | mmask;
  return ((uint32_t)E << mbits) | ((uint32_t)q - (1u << mbits));
}

double decode_ufloat(uint32_t v, int mbits) {
  const uint32_t e = v >> mbits, m = v & ((1u << mbits) - 1u);
  if (e == 0) return std::ldexp((double)m, -14 - mbits);
  if (e == 31) return m ? std::nan("") : INFINITY;
  return std::ldexp(1.0 + (double)m / (double)(1u << mbits), (int)e - 15);
}
}  // namespace

void orc_hemi_projection(const double d[3], double uv[2]) { hemi_projection(d3{d[0], d[1], d[2]}, uv[0], uv[1]); }

uint32_t orc_encode_r11g11b10(const double rgb[3]) {
  return encode_ufloat(rgb[0], 6) | encode_ufloat(rgb[1], 6) << 11 | encode_ufloat(rgb[2], 5) << 22;
}

void orc_encode_r11g11b10_n(const double* rgb, int64_t n, uint32_t* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = orc_encode_r11g11b10(rgb + 3 * i);
}

void orc_decode_r11g11b10(uint32_t v, double rgb[3]) {
  rgb[0] = decode_ufloat(v & 0x7FFu, 6);
  rgb[1] = decode_ufloat((v >> 11) & 0x7FFu, 6);
  rgb[2] = decode_ufloat(v >> 22, 5);
}

void orc_light_caches_specular(const DrvConfig* cfg, const DrvVolumeInfo* vol, int n_caches, const float* positions,
                               const float* cam, int n_lights, const DrvSpotLight* lights,
                               const double* const* vpls, const double* const* cones, const int* n_vpls,
                               const uint32_t* bits, const double* mips, double* sh_out, double* env_out,
                               int n_threads) {
  set_threads(n_threads);
  double cl[5], ev[5];
  orc_sh_constants(DRV_SH2_SIGN_REFERENCE, cl, ev);
  const bool sh2 = cfg->sh_order == 2;
  const int S = cfg->specular_envmap_size;
  const bool spec = S > 0;
  const bool env = spec && env_out && cam;
  // BlinnNormalization(GetBlinnPhongExponentForHemispherePixel(S)) (utils.glsl:180-190,
  // lightingfunctions.glsl:37-40).
  const double norm = ((double)S * S - 1.0 + 8.0) / (8.0 * kShaderPi);
#pragma omp parallel for schedule(dynamic, 16)
  for (int c = 0; c < n_caches; ++c) {
    double acc[27];
    for (int k = 0; k < 27; ++k) acc[k] = 0.0;
    d3 wp = ld3(positions + 3 * c);
    double cp[3] = {wp.x, wp.y, wp.z};
    double* E = env ? env_out + (size_t)c * S * S * 3 : nullptr;
    if (E)
      for (int k = 0; k < S * S * 3; ++k) E[k] = 0.0;
    d3 fx{}, fy{}, fz{};
    if (env) local_view_space(ld3(cam), wp, fx, fy, fz);
    for (int l = 0; l < n_lights; ++l) {
      const double* V = vpls[l];
      const double* C = cones[l];
      int interval = lights[l].indirect_shadow_sample_interval;
      double shadowing = 1.0;
      for (int j = 0; j < n_vpls[l]; ++j) {
        if (cfg->indirect_shadow && j % interval == 0) {
          const double* cone = C + 4 * (j / interval);
          shadowing = orc_cone_shadow(vol, cfg->voxel_res, bits, mips, cp, cone, cone[3], cfg->max_cone_steps);
        }
        const double* v = V + 10 * j;
        // INDIRECT_SPECULAR skips VPLs of little flux (cacheLightingRSM.comp:240-241)
        if (spec && v[0] + v[1] + v[2] < 0.001) continue;
        d3 to = mk(v[4], v[5], v[6]) - wp;
        double d2 = dot(to, to);
        to = to * (1.0 / std::sqrt(d2));
        double f = saturate(-dot(mk(v[7], v[8], v[9]), to)) * shadowing;
        double s = f / (d2 + v[3]);
        if (E && s > 0.0) {
          // cacheLightingRSM.comp:310-335: the reflected radiance into the
          // texel of the cache-local half vector (texel clamped to S - 1).
          const d3 tl = mk(dot(to, fx), dot(to, fy), dot(to, fz));
          d3 h = mk(tl.x, tl.y, tl.z + 1.0);
          const double hl = length(h);
          if (hl > 0.0) {
            h = h * (1.0 / hl);
            double pu, pv;
            hemi_projection(h, pu, pv);
            const int tx = std::min(std::max((int)(pu * S + 0.5), 0), S - 1);
            const int ty = std::min(std::max((int)(pv * S + 0.5), 0), S - 1);
            const double k = s * saturate(dot(h, tl));
            for (int ch = 0; ch < 3; ++ch) E[3 * (ty * S + tx) + ch] += v[ch] * k;
          }
        }
        for (int ch = 0; ch < 3; ++ch) {
          double L = v[ch] * s;
          acc[0 * 3 + ch] += ev[0] * L;
          acc[1 * 3 + ch] -= (ev[1] * to.y) * L;
          acc[2 * 3 + ch] += (ev[1] * to.z) * L;
          acc[3 * 3 + ch] -= (ev[1] * to.x) * L;
          if (sh2) {
            acc[4 * 3 + ch] -= (ev[2] * to.x * to.y) * L;
            acc[5 * 3 + ch] += (ev[2] * to.y * to.z) * L;
            acc[6 * 3 + ch] += (ev[3] * (to.z * to.z * 3.0 - 1.0)) * L;
            acc[7 * 3 + ch] += (ev[2] * to.x * to.z) * L;
            acc[8 * 3 + ch] += (ev[4] * (to.x * to.x - to.y * to.y)) * L;
          }
        }
      }
    }
    for (int k = 0; k < 27; ++k) sh_out[(size_t)c * 27 + k] = acc[k];
    if (E)
      for (int k = 0; k < S * S * 3; ++k) E[k] *= norm;
  }
}

// Renderer::PrepareSpecularEnvmaps (renderer.cpp:994-1043) on per-cache
// envmaps (cache c's levels at c * words, level l at the sum of the sizes of
// the levels above it, (S >> l)^2 texels row-major): mips
// (specularenvmap_mipmap.frag, the mean of the 2x2 texels below), then the
// hole fill from `fill` down to 1 (specularenvmap_fillholes.frag); every
// texel stored rounded to R11F_G11F_B10F.
void orc_specular_prepare(int S, int fill, int n_caches, uint32_t* env, int n_threads) {
  set_threads(n_threads);
  int L = 0;
  while ((1 << L) <= S) ++L;  // log2(S) + 1 levels
  std::vector<int> off(L + 1, 0);
  for (int l = 1; l <= L; ++l) off[l] = off[l - 1] + (S >> (l - 1)) * (S >> (l - 1));
  const int words = off[L];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < n_caches; ++c) {
    uint32_t* e = env + (size_t)c * words;
    for (int l = 1; l < L; ++l) {
      const int side = S >> l, below = 2 * side;
      for (int y = 0; y < side; ++y)
        for (int x = 0; x < side; ++x) {
          double a[3], b[3], cc[3], d[3], m[3];
          orc_decode_r11g11b10(e[off[l - 1] + (2 * y) * below + 2 * x], a);
          orc_decode_r11g11b10(e[off[l - 1] + (2 * y) * below + 2 * x + 1], b);
          orc_decode_r11g11b10(e[off[l - 1] + (2 * y + 1) * below + 2 * x], cc);
          orc_decode_r11g11b10(e[off[l - 1] + (2 * y + 1) * below + 2 * x + 1], d);
          for (int ch = 0; ch < 3; ++ch) m[ch] = 0.25 * ((a[ch] + b[ch]) + (cc[ch] + d[ch]));
          e[off[l] + y * side + x] = orc_encode_r11g11b10(m);
        }
    }
    for (int i = fill; i > 0; --i) {
      const int side = S >> i, below = 2 * side;
      for (int y = 0; y < side; ++y)
        for (int x = 0; x < side; ++x) {
          double sc[3];
          orc_decode_r11g11b10(e[off[i] + y * side + x], sc);
          if (sc[0] + sc[1] + sc[2] < 0.0001) continue;
          const int at[4] = {(2 * y) * below + 2 * x, (2 * y) * below + 2 * x + 1, (2 * y + 1) * below + 2 * x,
                             (2 * y + 1) * below + 2 * x + 1};
          double dc[4][3], sum[3] = {0, 0, 0};
          for (int k = 0; k < 4; ++k) {
            orc_decode_r11g11b10(e[off[i - 1] + at[k]], dc[k]);
            if (dc[k][0] + dc[k][1] + dc[k][2] == 0.0)
              for (int ch = 0; ch < 3; ++ch) dc[k][ch] = sc[ch];
            for (int ch = 0; ch < 3; ++ch) sum[ch] += dc[k][ch];
          }
          for (int k = 0; k < 4; ++k) {
            double o[3];
            for (int ch = 0; ch < 3; ++ch) o[ch] = dc[k][ch] * (4.0 * sc[ch] / (sum[ch] + 0.00001));
            e[off[i - 1] + at[k]] = orc_encode_r11g11b10(o);
          }
        }
    }
  }
}

// The SH gather of cacheLightingRSM.comp:234-279 with the shadowing of every
// (cache, shadow block) pair given (shadow[c * total_blocks + b], blocks of all
// lights in light order) instead of cone-traced: checks a learned visibility.
void orc_light_caches_shadowed(const DrvConfig* cfg, int n_caches, const float* positions, int n_lights,
                               const DrvSpotLight* lights, const double* const* vpls, const int* n_vpls,
                               const double* shadow, int total_blocks, double* sh_out, int n_threads) {
  set_threads(n_threads);
  double cl[5], ev[5];
  orc_sh_constants(DRV_SH2_SIGN_REFERENCE, cl, ev);
  const bool sh2 = cfg->sh_order == 2;
#pragma omp parallel for schedule(dynamic, 16)
  for (int c = 0; c < n_caches; ++c) {
    double acc[27];
    for (int k = 0; k < 27; ++k) acc[k] = 0.0;
    d3 wp = ld3(positions + 3 * c);
    int block_base = 0;
    for (int l = 0; l < n_lights; ++l) {
      const double* V = vpls[l];
      const int interval = cfg->indirect_shadow ? lights[l].indirect_shadow_sample_interval : 1;
      for (int j = 0; j < n_vpls[l]; ++j) {
        const double shadowing = shadow[(size_t)c * total_blocks + block_base + j / interval];
        const double* v = V + 10 * j;
        d3 to = mk(v[4], v[5], v[6]) - wp;
        double d2 = dot(to, to);
        to = to * (1.0 / std::sqrt(d2));
        double f = saturate(-dot(mk(v[7], v[8], v[9]), to)) * shadowing;
        double s = f / (d2 + v[3]);
        for (int ch = 0; ch < 3; ++ch) {
          double L = v[ch] * s;
          acc[0 * 3 + ch] += ev[0] * L;
          acc[1 * 3 + ch] -= (ev[1] * to.y) * L;
          acc[2 * 3 + ch] += (ev[1] * to.z) * L;
          acc[3 * 3 + ch] -= (ev[1] * to.x) * L;
          if (sh2) {
            acc[4 * 3 + ch] -= (ev[2] * to.x * to.y) * L;
            acc[5 * 3 + ch] += (ev[2] * to.y * to.z) * L;
            acc[6 * 3 + ch] += (ev[3] * (to.z * to.z * 3.0 - 1.0)) * L;
            acc[7 * 3 + ch] += (ev[2] * to.x * to.z) * L;
            acc[8 * 3 + ch] += (ev[4] * (to.x * to.x - to.y * to.y)) * L;
          }
        }
      }
      block_base += n_vpls[l] / interval;
    }
    for (int k = 0; k < 27; ++k) sh_out[(size_t)c * 27 + k] = acc[k];
  }
}

// cacheApply.frag:204-294 (ComputeLightingFromCaches) and :296-362 (main).
// Corners outside the atlas, or whose atlas slot holds 0 (never allocated) or
// 0xFFFFFFFF (locked, capacity overflow), contribute zero irradiance; their
// weight is not redistributed (GL robust access returns zeros there).
void orc_apply(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* f, int W, int H, const float* depth,
               const void* normal, int normal_format, const float* albedo, const uint32_t* atlas, int n_caches,
               const double* sh, double* out, int n_threads) {
  orc_apply_specular(cfg, vol, f, W, H, depth, normal, normal_format, albedo, nullptr, atlas, n_caches, sh, nullptr,
                     out, n_threads);
}

namespace {
// Bilinear fetch of one level of a per-cache envmap (GL 4.5 section 8.14.2),
// texel indices clamped to the level.
void env_bilinear(const uint32_t* lv, int side, double u, double v, double out[3]) {
  const double x = u * side - 0.5, y = v * side - 0.5;
  const double fx = std::floor(x), fy = std::floor(y), a = x - fx, b = y - fy;
  auto cl = [&](double q) { return std::min(std::max((int)q, 0), side - 1); };
  const int x0 = cl(fx), x1 = cl(fx + 1), y0 = cl(fy), y1 = cl(fy + 1);
  double t00[3], t10[3], t01[3], t11[3];
  orc_decode_r11g11b10(lv[y0 * side + x0], t00);
  orc_decode_r11g11b10(lv[y0 * side + x1], t10);
  orc_decode_r11g11b10(lv[y1 * side + x0], t01);
  orc_decode_r11g11b10(lv[y1 * side + x1], t11);
  for (int ch = 0; ch < 3; ++ch)
    out[ch] = (1 - a) * (1 - b) * t00[ch] + a * (1 - b) * t10[ch] + (1 - a) * b * t01[ch] + a * b * t11[ch];
}
}  // namespace

// cacheApply.frag with INDIRECT_SPECULAR (:76-116, 145-158) when
// cfg->specular_envmap_size > 0: rough_metal (RG F32 per pixel) and env (the
// per-cache envmaps as orc_specular_prepare lays them out) give each corner
// cache's trilinear envmap sample, and the material splits by metallic.
void orc_apply_specular(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* f, int W, int H,
                        const float* depth, const void* normal, int normal_format, const float* albedo,
                        const float* rough_metal, const uint32_t* atlas, int n_caches, const double* sh,
                        const uint32_t* env, double* out, int n_threads) {
  set_threads(n_threads);
  const int res = cfg->cav_res, nC = cfg->n_cascades, AW = nC * res;
  const bool transitions = cfg->cascade_transition > 0.0f;
  const int S = cfg->specular_envmap_size;
  const bool spec = S > 0 && rough_metal && env;
  int L = 0;
  while (spec && (1 << L) <= S) ++L;
  std::vector<int> eoff(L + 1, 0);
  for (int l = 1; l <= L; ++l) eoff[l] = eoff[l - 1] + (S >> (l - 1)) * (S >> (l - 1));
  const int ewords = spec ? eoff[L] : 0;
  struct Lookup {
    double u, v, f;
    int l0, l1;
  };
  auto env_sample = [&](uint32_t cache, const Lookup& q, double o[3]) {
    const uint32_t* e = env + (size_t)cache * ewords;
    env_bilinear(e + eoff[q.l0], S >> q.l0, q.u, q.v, o);
    if (q.f > 0.0) {
      double o1[3];
      env_bilinear(e + eoff[q.l1], S >> q.l1, q.u, q.v, o1);
      for (int ch = 0; ch < 3; ++ch) o[ch] = o[ch] * (1.0 - q.f) + o1[ch] * q.f;
    }
  };
  auto lighting = [&](const float p[3], int c, const double n[3], const double alb[3], const Lookup* q,
                      const double* spec_col, double col[3]) {
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    const DrvCascade& k = vol->cascades[c];
    float a[3];
    int a0[3];
    double t[3];
    for (int i = 0; i < 3; ++i) {
      a[i] = (p[i] - k.min[i]) / k.world_voxel_size;
      a0[i] = (int)std::trunc(std::max(-1e9f, std::min(1e9f, a[i])));
      t[i] = (double)a[i] - (double)a0[i];
    }
    double irr[3] = {0, 0, 0}, sp[3] = {0, 0, 0};
    for (int i = 0; i < 8; ++i) {
      double w = (off[i][0] ? t[0] : 1 - t[0]) * (off[i][1] ? t[1] : 1 - t[1]) * (off[i][2] ? t[2] : 1 - t[2]);
      int x = a0[0] + off[i][0], y = a0[1] + off[i][1], z = a0[2] + off[i][2];
      x += res * c;
      if (x < 0 || y < 0 || z < 0 || x >= AW || y >= res || z >= res) continue;
      uint32_t addr = atlas[((size_t)z * res + y) * AW + x];
      if (addr == 0u || addr == 0xFFFFFFFFu || addr > (uint32_t)n_caches) continue;
      double e[3];
      orc_sh_irradiance(cfg->sh_order, cfg->sh2_sign, sh + (size_t)(addr - 1) * 27, n, e);
      for (int ch = 0; ch < 3; ++ch) irr[ch] += e[ch] * w;
      if (q) {
        double es[3];
        env_sample(addr - 1, *q, es);
        for (int ch = 0; ch < 3; ++ch) sp[ch] += es[ch] * w;
      }
    }
    for (int ch = 0; ch < 3; ++ch) col[ch] = irr[ch] * alb[ch] / kShaderPi + (q ? sp[ch] * spec_col[ch] : 0.0);
  };
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t i = (size_t)y * W + x;
      double* o = out + 3 * i;
      o[0] = o[1] = o[2] = 0.0;
      float d = depth[i];
      if (d < 0.00001f) continue;
      float p[3];
      reconstruct_world_f32(f, x, y, W, H, d, p);
      int c = select_cascade_f32(vol, nC, p);
      double n[3];
      if (normal_format == DRV_NORMAL_RG16I) {
        orc_unpack_normal16i((const int16_t*)normal + 2 * i, n);
      } else {
        const float* nf = (const float*)normal + 3 * i;
        n[0] = nf[0];
        n[1] = nf[1];
        n[2] = nf[2];
      }
      double alb[3] = {albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2]};
      Lookup q{};
      double spec_col[3] = {0, 0, 0};
      if (spec) {
        // ComputeMaterialColors, RoughnessToBlinnExponent,
        // GetHemisphereLodForBlinnPhongExponent and the lookup clamp
        // (lightingfunctions.glsl:27-49, utils.glsl:193-200, cacheApply.frag:150-157).
        const double rough = rough_metal[2 * i], metal = rough_metal[2 * i + 1];
        for (int ch = 0; ch < 3; ++ch) {
          spec_col[ch] = 0.04 * (1.0 - metal) + alb[ch] * metal;
          alb[ch] = alb[ch] * (1.0 - metal) + 0.02 * metal;
        }
        const double rsq = rough * rough, blinn = 2.0 / (rsq * rsq + 0.0005);
        const double lod = std::max(0.0, std::log2((double)S * S / (1.0 + blinn)) * 0.5);
        const double half_px = 0.5 / (std::exp2(-std::ceil(lod)) * S);
        d3 fx, fy, fz;
        local_view_space(ld3(f->camera_position), mk(p[0], p[1], p[2]), fx, fy, fz);
        const d3 nv = mk(n[0], n[1], n[2]);
        hemi_projection(mk(dot(nv, fx), dot(nv, fy), dot(nv, fz)), q.u, q.v);
        q.u = std::min(std::max(q.u, half_px), 1.0 - half_px);
        q.v = std::min(std::max(q.v, half_px), 1.0 - half_px);
        const double fl = std::min(std::floor(lod), (double)(L - 1));
        q.l0 = (int)fl;
        q.l1 = std::min(q.l0 + 1, L - 1);
        q.f = q.l1 > q.l0 ? lod - fl : 0.0;
      }
      double col[3];
      lighting(p, c, n, alb, spec ? &q : nullptr, spec_col, col);
      if (transitions) {
        float t = cascade_transition_f32(vol, c, p);
        if (t > 0.0f && c < nC - 1) {
          double col2[3];
          lighting(p, c + 1, n, alb, spec ? &q : nullptr, spec_col, col2);
          for (int ch = 0; ch < 3; ++ch) col[ch] = col[ch] * (1.0 - t) + col2[ch] * t;
        }
      }
      o[0] = col[0];
      o[1] = col[1];
      o[2] = col[2];
    }
}

// bruteforcersm.frag:15-82 (see oracle.h).
void orc_bruteforce_rsm(const DrvPerFrame* f, int W, int H, const float* depth, const int16_t* normal16,
                        const float* albedo, const float* rough_metal, int n_lights, const double* const* vpls,
                        const int* n_vpls, double* out, int n_threads) {
  set_threads(n_threads);
  const d3 cam = mk(f->camera_position[0], f->camera_position[1], f->camera_position[2]);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = (size_t)y * W + x;
      double* o = out + 3 * i;
      o[0] = o[1] = o[2] = 0.0;
      const float d = depth[i];
      if (d < 0.00001f) continue;
      float pf[3];
      reconstruct_world_f32(f, x, y, W, H, d, pf);
      const d3 p = mk(pf[0], pf[1], pf[2]);
      double nn[3];
      orc_unpack_normal16i(normal16 + 2 * i, nn);
      const d3 n = mk(nn[0], nn[1], nn[2]);
      const d3 base = mk(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2]);
      // BRDF parameters, lightingfunctions.glsl:27-50.
      d3 diffuse = base, specular = mk(0, 0, 0);
      double blinn_exp = 0.0, blinn_norm = 0.0;
      d3 to_cam = mk(0, 0, 0);
      if (rough_metal) {
        const double r = rough_metal[2 * i], m = rough_metal[2 * i + 1];
        const double rsq = r * r;
        blinn_exp = 2.0 / (rsq * rsq + 0.0005);
        blinn_norm = (blinn_exp + 8.0) / (8.0 * kShaderPi);
        diffuse = base * (1.0 - m) + mk(0.02, 0.02, 0.02) * m;
        specular = mk(0.04, 0.04, 0.04) * (1.0 - m) + base * m;
        d3 tc = cam - p;
        to_cam = tc * (1.0 / std::sqrt(dot(tc, tc)));
      }
      double acc[3] = {0, 0, 0};
      for (int l = 0; l < n_lights; ++l) {
        const double* V = vpls[l];
        for (int j = 0; j < n_vpls[l]; ++j) {
          const double* v = V + 10 * j;
          d3 to = mk(v[4], v[5], v[6]) - p;
          const double d2 = dot(to, to);
          to = to * (1.0 / std::sqrt(d2));
          const double cos_theta = saturate(dot(to, n));
          const double flux_to_intensity = saturate(dot(mk(v[7], v[8], v[9]), to * -1.0));
          const double g = flux_to_intensity * cos_theta / (d2 + v[3]);
          double brdf[3];
          if (rough_metal) {
            d3 h = to_cam + to;
            h = h * (1.0 / std::sqrt(dot(h, h)));
            const double bp = blinn_norm * std::pow(saturate(dot(n, h)), blinn_exp);
            brdf[0] = diffuse.x / kShaderPi + bp * specular.x;
            brdf[1] = diffuse.y / kShaderPi + bp * specular.y;
            brdf[2] = diffuse.z / kShaderPi + bp * specular.z;
          } else {
            brdf[0] = diffuse.x / kShaderPi;
            brdf[1] = diffuse.y / kShaderPi;
            brdf[2] = diffuse.z / kShaderPi;
          }
          for (int ch = 0; ch < 3; ++ch) acc[ch] += brdf[ch] * v[ch] * g;
        }
      }
      o[0] = acc[0];
      o[1] = acc[1];
      o[2] = acc[2];
    }
}

// ---------------------------------------------------------------- scenes
// The seeded box rooms of the benchmark workloads: splitmix64 draws, an
// inward unit-cube room (box 0) and n_boxes boxes inside it; camera and spot
// light rejection-sampled clear of the boxes. Same draws in the same order as
// the product's generator, so both give the same floats.
namespace {
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double u(double a, double b) { return a + (b - a) * u01(); }
};

// Signed distance from p to the nearest non-room box (negative inside).
double box_clearance(const DrvScene* scene, const double p[3]) {
  double best = 1e30;
  for (int b = 0; b < scene->n_boxes; ++b) {
    const DrvBox& x = scene->boxes[b];
    if (x.inward) continue;
    double outside2 = 0.0, depth = 1e30;
    bool inside = true;
    for (int i = 0; i < 3; ++i) {
      const double e = std::max((double)x.min[i] - p[i], p[i] - (double)x.max[i]);
      if (e > 0) {
        outside2 += e * e;
        inside = false;
      } else {
        depth = std::min(depth, -e);
      }
    }
    best = std::min(best, inside ? -depth : std::sqrt(outside2));
  }
  return best;
}

void clear_sample(SplitMix& r, const DrvScene* scene, const double lo[3], const double hi[3], double margin,
                  double p[3]) {
  for (int tries = 0; tries < 4096; ++tries) {
    for (int i = 0; i < 3; ++i) p[i] = r.u(lo[i], hi[i]);
    if (!scene || box_clearance(scene, p) >= margin) return;
  }
}

void unit_towards(const double from[3], const double to[3], float out[3]) {
  const double d[3] = {to[0] - from[0], to[1] - from[1], to[2] - from[2]};
  const double inv = 1.0 / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (int i = 0; i < 3; ++i) out[i] = (float)(d[i] * inv);
}
}  // namespace

void orc_generate_scene(uint64_t seed, int n_boxes, float size_min, float size_max, float albedo_min,
                        float albedo_max, DrvBox* boxes, DrvScene* scene) {
  SplitMix r{seed * 0x2545F4914F6CDD1Dull + 1};
  std::memset(boxes, 0, sizeof(DrvBox) * (size_t)(n_boxes + 1));
  for (int i = 0; i < 3; ++i) {
    boxes[0].max[i] = 1.0f;
    boxes[0].albedo[i] = (float)r.u(albedo_min, albedo_max);
  }
  boxes[0].inward = 1;
  for (int b = 1; b <= n_boxes; ++b) {
    for (int i = 0; i < 3; ++i) {
      const float size = (float)r.u(size_min, size_max);
      const float lo = (float)r.u(0.0, 1.0 - size);
      boxes[b].min[i] = lo;
      boxes[b].max[i] = lo + size;
    }
    for (int i = 0; i < 3; ++i) boxes[b].albedo[i] = (float)r.u(albedo_min, albedo_max);
  }
  scene->n_boxes = n_boxes + 1;
  scene->boxes = boxes;
  for (int i = 0; i < 3; ++i) {
    scene->aabb_min[i] = 0.0f;
    scene->aabb_max[i] = 1.0f;
  }
}

void orc_generate_camera(uint64_t seed, const DrvScene* scene, float aspect, DrvCamera* c) {
  SplitMix r{seed * 0x9E3779B97F4A7C15ull + 7};
  std::memset(c, 0, sizeof(*c));
  const double lo[3] = {0.15, 0.35, 0.05}, hi[3] = {0.85, 0.8, 0.25};
  double p[3];
  clear_sample(r, scene, lo, hi, 0.08, p);
  const double t[3] = {r.u(0.3, 0.7), r.u(0.15, 0.45), r.u(0.7, 0.95)};
  for (int i = 0; i < 3; ++i) c->position[i] = (float)p[i];
  unit_towards(p, t, c->direction);
  c->up[1] = 1.0f;
  c->fov_y_deg = 60.0f;
  c->aspect = aspect;
  c->near_plane = 0.01f;
  c->far_plane = 1000.0f;
}

void orc_generate_light(uint64_t seed, const DrvScene* scene, uint32_t rsm_resolution, uint32_t rsm_read_lod,
                        uint32_t indirect_shadow_lod, DrvLightDesc* L) {
  SplitMix r{seed * 0xD1B54A32D192ED03ull + 13};
  std::memset(L, 0, sizeof(*L));
  const double lo[3] = {0.2, 0.75, 0.2}, hi[3] = {0.8, 0.95, 0.8};
  double p[3];
  clear_sample(r, scene, lo, hi, 0.05, p);
  const double t[3] = {r.u(0.25, 0.75), r.u(0.0, 0.2), r.u(0.25, 0.75)};
  for (int i = 0; i < 3; ++i) {
    L->intensity[i] = 10.0f;
    L->position[i] = (float)p[i];
  }
  unit_towards(p, t, L->direction);
  L->half_angle = (float)(30.0 * kPi / 180.0);
  L->rsm_resolution = rsm_resolution;
  L->rsm_read_lod = rsm_read_lod;
  L->indirect_shadow_lod = indirect_shadow_lod;
  L->near_plane = 0.1f;
  L->far_plane = 10000.0f;
}

}  // extern "C"
