// host_params.cpp — host-side parameter setup of the path: the reference's
// UBO fills (Renderer::UpdateConstantUBO/UpdatePerFrameUBO/UpdateVolumeUBO/
// PrepareLights, rendering/renderer.cpp:290-431, 664-725) and the seeded
// procedural scene that replaces its mesh scenes.
//
// Compiled with -ffp-contract=off so its float results do not depend on the
// host architecture's fused multiply-add.
#include <cmath>
#include <cstring>

#include "drv_internal.h"

namespace drv {
namespace {

constexpr double kPi = 3.14159265358979323846;

struct v3 {
  double x, y, z;
};
v3 sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
v3 cross(v3 a, v3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
v3 scale(v3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
v3 norm(v3 a) { return scale(a, 1.0 / std::sqrt(dot(a, a))); }
v3 ld(const float* p) { return {p[0], p[1], p[2]}; }

struct m4 {
  double m[16];
};
m4 mul(const m4& a, const m4& b) {
  m4 r{};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += a.m[i * 4 + k] * b.m[k * 4 + j];
      r.m[i * 4 + j] = s;
    }
  return r;
}
// Gauss-Jordan inverse with partial pivoting (ei::invert is not available).
bool inverse(const m4& a, m4& out) {
  double t[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 8; ++j) t[i][j] = j < 4 ? a.m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int p = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(t[r][c]) > std::fabs(t[p][c])) p = r;
    if (t[p][c] == 0.0) return false;
    if (p != c)
      for (int j = 0; j < 8; ++j) {
        double tmp = t[p][j];
        t[p][j] = t[c][j];
        t[c][j] = tmp;
      }
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

// Left-handed look-at frame (+z forward, +y up), the convention of the
// DX-style projection used by the reference (camera.hpp:27-30).
void frame(v3 dir, v3 up, v3& right, v3& up_out, v3& fwd) {
  fwd = norm(dir);
  if (std::fabs(dot(norm(up), fwd)) > 0.999) up = std::fabs(fwd.z) < 0.9 ? v3{0, 0, 1} : v3{1, 0, 0};
  right = norm(cross(up, fwd));
  up_out = cross(fwd, right);
}
m4 look(v3 pos, v3 dir, v3 up) {
  v3 r, u, f;
  frame(dir, up, r, u, f);
  return m4{{r.x, r.y, r.z, -dot(r, pos), u.x, u.y, u.z, -dot(u, pos), f.x, f.y, f.z, -dot(f, pos), 0, 0, 0, 1}};
}
// perspectiveDX(fov, aspect, far, near): near/far swapped -> reversed Z.
m4 perspective_reversed(double fovy, double aspect, double n, double f) {
  double sy = 1.0 / std::tan(fovy * 0.5), sx = sy / aspect;
  return m4{{sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, n / (n - f), n * f / (f - n), 0, 0, 1, 0}};
}
void put(const m4& a, float* o) {
  for (int i = 0; i < 16; ++i) o[i] = (float)a.m[i];
}

// splitmix64: a small seeded generator with identical output on every host.
struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

}  // namespace

RayFrame make_ray_frame(const float pos[3], const float dir[3], const float up[3], double tan_x, double tan_y) {
  v3 r, u, f;
  frame(ld(dir), ld(up), r, u, f);
  RayFrame rf;
  for (int i = 0; i < 3; ++i) rf.origin[i] = pos[i];
  rf.fwd[0] = (float)f.x;
  rf.fwd[1] = (float)f.y;
  rf.fwd[2] = (float)f.z;
  rf.right[0] = (float)(r.x * tan_x);
  rf.right[1] = (float)(r.y * tan_x);
  rf.right[2] = (float)(r.z * tan_x);
  rf.up[0] = (float)(u.x * tan_y);
  rf.up[1] = (float)(u.y * tan_y);
  rf.up[2] = (float)(u.z * tan_y);
  return rf;
}

}  // namespace drv

using namespace drv;

extern "C" {

int drv_abi_version(void) { return DRV_ABI_VERSION; }

// Defaults of the reference Renderer (renderer.cpp:37-50, 86-90, light.hpp:12-14)
// where they exist; FP32 storage and cone visibility.
void drv_default_config(DrvConfig* c) {
  std::memset(c, 0, sizeof(*c));
  c->width = 1920;
  c->height = 1080;
  c->sh_order = 1;
  c->indirect_shadow = 1;
  c->max_cone_steps = 32;
  c->cascade_transition = 2.0f;
  c->n_cascades = 3;
  c->cav_res = 32;
  c->cascade_world_size[0] = 4.0f;
  c->cascade_world_size[1] = 8.0f;
  c->cascade_world_size[2] = 16.0f;
  c->cascade_world_size[3] = 32.0f;
  c->voxel_res = 128;
  c->max_caches = 16384;
  c->precision = DRV_PRECISION_FP32;
  c->visibility = DRV_VISIBILITY_CONE;
  c->surrogate_conf_threshold = 0.5f;
  c->sh2_sign = DRV_SH2_SIGN_REFERENCE;
  c->max_lights = 1;
  c->max_rsm_resolution = 1024;
}

// Renderer::UpdateVolumeUBO, renderer.cpp:346-431 ("simple version": cascades
// centred on the camera, snapped to their cell size; decision boxes shrunk by
// 1.5 cells and not snapped).
drv_status drv_compute_volume_info(const DrvConfig* cfg, const float amin[3], const float amax[3], const float cam[3],
                                   DrvVolumeInfo* o) {
  if (!cfg || !amin || !amax || !cam || !o) return DRV_ERR_INVALID_ARG;
  if (cfg->n_cascades < 1 || cfg->n_cascades > DRV_MAX_CASCADES || cfg->cav_res < 2 || cfg->voxel_res < 2)
    return DRV_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  float mn[3], mx[3], ext[3];
  for (int i = 0; i < 3; ++i) {
    mn[i] = amin[i] - 0.001f;
    mx[i] = amax[i] + 0.001f;
    ext[i] = mx[i] - mn[i];
  }
  float largest = ext[0] > ext[1] ? ext[0] : ext[1];
  largest = largest > ext[2] ? largest : ext[2];
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
    if (!(size > 0.0f)) return DRV_ERR_INVALID_ARG;
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
  return DRV_OK;
}

// Renderer::PrepareLights, renderer.cpp:664-725.
drv_status drv_prepare_light(const DrvLightDesc* L, DrvSpotLight* o) {
  if (!L || !o) return DRV_ERR_INVALID_ARG;
  if (L->rsm_resolution == 0 || L->half_angle <= 0.0f || L->near_plane <= 0.0f || L->far_plane <= L->near_plane)
    return DRV_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  for (int i = 0; i < 3; ++i) {
    o->intensity[i] = L->intensity[i];
    o->position[i] = L->position[i];
  }
  v3 dir = norm(ld(L->direction));
  o->direction[0] = (float)dir.x;
  o->direction[1] = (float)dir.y;
  o->direction[2] = (float)dir.z;
  o->shadow_normal_offset = 0.01f;  // Light::normalOffsetShadowBias default
  o->shadow_bias = 0.0001f;         // Light::shadowBias default
  o->cos_half_angle = cosf(L->half_angle);
  m4 vp = mul(perspective_reversed(2.0 * L->half_angle, 1.0, L->near_plane, L->far_plane),
              look(ld(L->position), dir, v3{0, 1, 0}));
  m4 inv;
  if (!inverse(vp, inv)) return DRV_ERR_INVALID_ARG;
  put(vp, o->view_projection);
  put(inv, o->inverse_view_projection);
  int r = 1;
  while ((uint32_t)r < L->rsm_resolution) r <<= 1;  // next power of two (renderer.cpp:694-696)
  o->rsm_render_resolution = r;
  int read = r >> L->rsm_read_lod;
  if (read < 1) return DRV_ERR_INVALID_ARG;
  o->rsm_read_resolution = read;
  float clip_w = sinf(L->half_angle) * L->near_plane * 2.0f;
  float vaf = clip_w * clip_w / (L->near_plane * L->near_plane * (float)read * (float)read);
  o->val_area_factor = vaf;
  o->indirect_shadow_lod = (float)L->indirect_shadow_lod;
  float bs = (float)(1 << L->indirect_shadow_lod);
  if (bs > (float)read) return DRV_ERR_INVALID_ARG;  // renderer.cpp:712
  o->indirect_shadow_block_size = bs;
  o->indirect_shadow_sample_interval = (int)(bs * bs);
  o->indirect_shadow_super_val_width = sqrtf(vaf) * bs;
  o->indirect_shadow_sampling_offset = 0.5f + sqrtf(2.0f) * bs / 2.0f;
  return DRV_OK;
}

// Renderer::UpdatePerFrameUBO, renderer.cpp:324-344.
drv_status drv_prepare_camera(const DrvCamera* c, DrvPerFrame* o) {
  if (!c || !o || c->aspect <= 0.0f || c->near_plane <= 0.0f || c->far_plane <= c->near_plane)
    return DRV_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  v3 dir = norm(ld(c->direction));
  m4 vp = mul(perspective_reversed(c->fov_y_deg * (kPi / 180.0), c->aspect, c->near_plane, c->far_plane),
              look(ld(c->position), dir, ld(c->up)));
  m4 inv;
  if (!inverse(vp, inv)) return DRV_ERR_INVALID_ARG;
  put(vp, o->view_projection);
  put(inv, o->inverse_view_projection);
  for (int i = 0; i < 3; ++i) o->camera_position[i] = c->position[i];
  o->camera_direction[0] = (float)dir.x;
  o->camera_direction[1] = (float)dir.y;
  o->camera_direction[2] = (float)dir.z;
  return DRV_OK;
}

// Inward unit-cube room [0,1]^3 (box 0) plus n_boxes boxes fully inside it.
drv_status drv_generate_scene(uint64_t seed, int32_t n_boxes, float size_min, float size_max, float albedo_min,
                              float albedo_max, DrvBox* boxes, DrvScene* scene) {
  if (!boxes || !scene || n_boxes < 0 || !(size_min > 0.0f) || size_max < size_min || size_max >= 1.0f)
    return DRV_ERR_INVALID_ARG;
  Rng rng{seed * 0x2545F4914F6CDD1Dull + 1};
  DrvBox& room = boxes[0];
  for (int i = 0; i < 3; ++i) {
    room.min[i] = 0.0f;
    room.max[i] = 1.0f;
    room.albedo[i] = (float)rng.uniform(albedo_min, albedo_max);
  }
  room.inward = 1;
  for (int b = 1; b <= n_boxes; ++b) {
    DrvBox& x = boxes[b];
    for (int i = 0; i < 3; ++i) {
      float size = (float)rng.uniform(size_min, size_max);
      float lo = (float)rng.uniform(0.0, 1.0 - size);
      x.min[i] = lo;
      x.max[i] = lo + size;
    }
    for (int i = 0; i < 3; ++i) x.albedo[i] = (float)rng.uniform(albedo_min, albedo_max);
    x.inward = 0;
  }
  scene->n_boxes = n_boxes + 1;
  scene->boxes = boxes;
  for (int i = 0; i < 3; ++i) {
    scene->aabb_min[i] = 0.0f;
    scene->aabb_max[i] = 1.0f;
  }
  return DRV_OK;
}

namespace {
// Distance from p to the nearest non-room box (negative inside a box).
double clearance(const DrvScene* scene, v3 p) {
  double best = 1e30;
  for (int b = 0; b < scene->n_boxes; ++b) {
    const DrvBox& x = scene->boxes[b];
    if (x.inward) continue;
    double q[3] = {p.x, p.y, p.z}, d2 = 0.0, inside = 1e30;
    bool in = true;
    for (int i = 0; i < 3; ++i) {
      double lo = x.min[i] - q[i], hi = q[i] - x.max[i];
      double e = lo > hi ? lo : hi;
      if (e > 0) {
        d2 += e * e;
        in = false;
      } else {
        inside = inside < -e ? inside : -e;
      }
    }
    double d = in ? -inside : std::sqrt(d2);
    if (d < best) best = d;
  }
  return best;
}
// Rejection-samples a point inside [lo, hi] at least `margin` away from every box.
v3 clear_point(Rng& rng, const DrvScene* scene, v3 lo, v3 hi, double margin) {
  v3 p{};
  for (int tries = 0; tries < 4096; ++tries) {
    p = v3{rng.uniform(lo.x, hi.x), rng.uniform(lo.y, hi.y), rng.uniform(lo.z, hi.z)};
    if (!scene || clearance(scene, p) >= margin) return p;
  }
  return p;
}
}  // namespace

// Camera inside the room, clear of the boxes, looking across it (fov 60 as
// application.cpp:51-52; near 0.01 / far 1000 for the unit room).
drv_status drv_generate_camera(uint64_t seed, const DrvScene* scene, float aspect, DrvCamera* c) {
  if (!c || !(aspect > 0.0f)) return DRV_ERR_INVALID_ARG;
  Rng rng{seed * 0x9E3779B97F4A7C15ull + 7};
  std::memset(c, 0, sizeof(*c));
  v3 p = clear_point(rng, scene, v3{0.15, 0.35, 0.05}, v3{0.85, 0.8, 0.25}, 0.08);
  v3 t{rng.uniform(0.3, 0.7), rng.uniform(0.15, 0.45), rng.uniform(0.7, 0.95)};
  v3 d = norm(sub(t, p));
  c->position[0] = (float)p.x;
  c->position[1] = (float)p.y;
  c->position[2] = (float)p.z;
  c->direction[0] = (float)d.x;
  c->direction[1] = (float)d.y;
  c->direction[2] = (float)d.z;
  c->up[1] = 1.0f;
  c->fov_y_deg = 60.0f;
  c->aspect = aspect;
  c->near_plane = 0.01f;
  c->far_plane = 1000.0f;
  return DRV_OK;
}

// Spot light in the upper part of the room, clear of the boxes, aimed down
// into it (half angle 30 degrees as application.cpp:91; near/far 0.1/10000 as
// scene.cpp:6-7).
drv_status drv_generate_light(uint64_t seed, const DrvScene* scene, uint32_t rsm_resolution, uint32_t rsm_read_lod,
                              uint32_t indirect_shadow_lod, DrvLightDesc* L) {
  if (!L || rsm_resolution == 0) return DRV_ERR_INVALID_ARG;
  Rng rng{seed * 0xD1B54A32D192ED03ull + 13};
  std::memset(L, 0, sizeof(*L));
  v3 p = clear_point(rng, scene, v3{0.2, 0.75, 0.2}, v3{0.8, 0.95, 0.8}, 0.05);
  v3 t{rng.uniform(0.25, 0.75), rng.uniform(0.0, 0.2), rng.uniform(0.25, 0.75)};
  v3 d = norm(sub(t, p));
  for (int i = 0; i < 3; ++i) L->intensity[i] = 10.0f;
  L->position[0] = (float)p.x;
  L->position[1] = (float)p.y;
  L->position[2] = (float)p.z;
  L->direction[0] = (float)d.x;
  L->direction[1] = (float)d.y;
  L->direction[2] = (float)d.z;
  L->half_angle = (float)(30.0 * kPi / 180.0);
  L->rsm_resolution = rsm_resolution;
  L->rsm_read_lod = rsm_read_lod;
  L->indirect_shadow_lod = indirect_shadow_lod;
  L->near_plane = 0.1f;
  L->far_plane = 10000.0f;
  return DRV_OK;
}

}  // extern "C"
