// k_bruteforce.cu — Renderer::ApplyRSMsBruteForce (renderer.cpp:851-871) /
// bruteforcersm.frag:15-82: per pixel, the unshadowed sum over every VAL of
// every light, without caches — the ground truth the cache volume
// interpolates. The VALs are the context's extracted VPLs (the same
// position / normal / flux / disc-area formulas, bruteforcersm.frag:51-73),
// read at each light's RSM read resolution (the reference's texelFetch reads
// RSM level 0 with read-resolution coordinates, which is the same at read
// lod 0).
//
// A CTA is a 16x16 pixel tile; the VPLs stream through shared memory in
// tiles of 256 (one per thread), so every VPL is read from L2 once per CTA
// and the inner loop is FP32 arithmetic only.
#include "drv_device.cuh"
#include "drv_internal.h"
#include "light_common.cuh"

namespace drv {
namespace {

constexpr int kTile = 16;
constexpr int kThreads = kTile * kTile;

struct BruteParams {
  DrvPerFrame frame;
  const float* depth;
  const void* normal;
  int normal_format;
  const void* albedo;
  int albedo_format;
  const float* srgb;
  const float* rough_metal;  // RG per pixel, or null: diffuse BRDF
  int w, h;
  LightLaunch ll;
  float* out;
};

template <bool BF16, bool SPECULAR>
__global__ void __launch_bounds__(kThreads) brute_kernel(BruteParams p) {
  __shared__ float s_v[10][kThreads];  // px py pz area fr fg fb nx ny nz
  const int x = blockIdx.x * kTile + threadIdx.x, y = blockIdx.y * kTile + threadIdx.y;
  const int tid = threadIdx.y * kTile + threadIdx.x;
  const bool inside = x < p.w && y < p.h;
  const size_t i = inside ? (size_t)y * p.w + x : 0;
  const float d = inside ? p.depth[i] : 0.0f;
  const bool valid = inside && d >= 0.00001f;
  float px = 0.f, py = 0.f, pz = 0.f;
  f3 n = mkf3(0.f, 0.f, 1.f);
  f3 base = mkf3(0.f, 0.f, 0.f), diffuse = base, specular = base, to_cam = base;
  float blinn_exp = 0.f, blinn_norm = 0.f;
  if (valid) {
    float wp[3];
    reconstruct_world(p.frame, x, y, p.w, p.h, d, wp);
    px = wp[0];
    py = wp[1];
    pz = wp[2];
    if (p.normal_format == DRV_NORMAL_RG16I) {
      const int16_t* q = reinterpret_cast<const int16_t*>(p.normal) + 2 * i;
      n = unpack_normal16i(q[0], q[1]);
    } else {
      const float* q = reinterpret_cast<const float*>(p.normal) + 3 * i;
      n = mkf3(q[0], q[1], q[2]);
    }
    base = load_albedo(p.albedo, p.albedo_format, p.srgb, i);
    diffuse = base;
    if (SPECULAR) {
      // lightingfunctions.glsl:27-50
      const float r = p.rough_metal[2 * i], m = p.rough_metal[2 * i + 1];
      const float rsq = r * r;
      blinn_exp = 2.0f / (rsq * rsq + 0.0005f);
      blinn_norm = (blinn_exp + 8.0f) / (8.0f * DRV_SHADER_PI);
      diffuse = base * (1.0f - m) + mkf3(0.02f, 0.02f, 0.02f) * m;
      specular = mkf3(0.04f, 0.04f, 0.04f) * (1.0f - m) + base * m;
      to_cam = normalize3(mkf3(p.frame.camera_position[0] - px, p.frame.camera_position[1] - py,
                               p.frame.camera_position[2] - pz));
    }
  }
  float ar = 0.f, ag = 0.f, ab = 0.f;  // irradiance (diffuse), or BRDF-weighted radiance (specular)
  for (int l = 0; l < p.ll.n_lights; ++l) {
    const int nv = p.ll.lights[l].n_vpls;
    const void* vpls = p.ll.lights[l].vpls;
    for (int b0 = 0; b0 < nv; b0 += kThreads) {
      __syncthreads();
      if (b0 + tid < nv) {
        const VplData v = load_vpl<BF16>(vpls, b0 + tid);
        s_v[0][tid] = v.px;
        s_v[1][tid] = v.py;
        s_v[2][tid] = v.pz;
        s_v[3][tid] = v.area;
        s_v[4][tid] = v.fr;
        s_v[5][tid] = v.fg;
        s_v[6][tid] = v.fb;
        s_v[7][tid] = v.nx;
        s_v[8][tid] = v.ny;
        s_v[9][tid] = v.nz;
      }
      __syncthreads();
      if (!valid) continue;
      const int cnt = min(kThreads, nv - b0);
      for (int j = 0; j < cnt; ++j) {
        const float tx = s_v[0][j] - px, ty = s_v[1][j] - py, tz = s_v[2][j] - pz;
        const float d2 = tx * tx + ty * ty + tz * tz;
        const float r = rsqrtf(d2);
        const float wx = tx * r, wy = ty * r, wz = tz * r;
        const float cos_theta = sat(wx * n.x + wy * n.y + wz * n.z);
        const float to_intensity = sat(-(s_v[7][j] * wx + s_v[8][j] * wy + s_v[9][j] * wz));
        const float g = __fdividef(to_intensity * cos_theta, d2 + s_v[3][j]);
        if (SPECULAR) {
          const f3 hv = normalize3(mkf3(to_cam.x + wx, to_cam.y + wy, to_cam.z + wz));
          const float bp = blinn_norm * powf(sat(n.x * hv.x + n.y * hv.y + n.z * hv.z), blinn_exp);
          ar += (diffuse.x * (1.0f / DRV_SHADER_PI) + bp * specular.x) * s_v[4][j] * g;
          ag += (diffuse.y * (1.0f / DRV_SHADER_PI) + bp * specular.y) * s_v[5][j] * g;
          ab += (diffuse.z * (1.0f / DRV_SHADER_PI) + bp * specular.z) * s_v[6][j] * g;
        } else {
          ar += s_v[4][j] * g;
          ag += s_v[5][j] * g;
          ab += s_v[6][j] * g;
        }
      }
    }
  }
  if (!inside) return;
  float* o = p.out + 3 * i;
  if (SPECULAR) {
    o[0] = ar;
    o[1] = ag;
    o[2] = ab;
  } else {
    o[0] = diffuse.x * (1.0f / DRV_SHADER_PI) * ar;
    o[1] = diffuse.y * (1.0f / DRV_SHADER_PI) * ag;
    o[2] = diffuse.z * (1.0f / DRV_SHADER_PI) * ab;
  }
}

}  // namespace

cudaError_t launch_bruteforce_rsm(cudaStream_t s, const DrvPerFrame& f, const DrvGBufferView& g,
                                  const float* rough_metal, const LightLaunch& ll, int bf16, float* out_rgb,
                                  const float* srgb) {
  BruteParams p;
  p.frame = f;
  p.depth = g.depth;
  p.normal = g.normal;
  p.normal_format = g.normal_format;
  p.albedo = g.albedo;
  p.albedo_format = g.albedo_format;
  p.srgb = srgb;
  p.rough_metal = rough_metal;
  p.w = g.width;
  p.h = g.height;
  p.ll = ll;
  p.out = out_rgb;
  dim3 block(kTile, kTile), grid((g.width + kTile - 1) / kTile, (g.height + kTile - 1) / kTile);
  if (bf16) {
    if (rough_metal)
      brute_kernel<true, true><<<grid, block, 0, s>>>(p);
    else
      brute_kernel<true, false><<<grid, block, 0, s>>>(p);
  } else {
    if (rough_metal)
      brute_kernel<false, true><<<grid, block, 0, s>>>(p);
    else
      brute_kernel<false, false><<<grid, block, 0, s>>>(p);
  }
  return cudaGetLastError();
}

}  // namespace drv
