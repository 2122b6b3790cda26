// k_raycast.cu — input producers: the G-buffer fill (fillgbuffer.frag:21-43)
// and the RSM fill (fillrsm.frag:24-62) as ray casts against the procedural
// box scene. They replace the reference's rasterisation passes; their output
// layouts are the reference's G-buffer/RSM texture layouts.
#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

constexpr int kMaxSmemBoxes = 512;

struct Hit {
  int box;
  int axis;
  float t;
};

__device__ __forceinline__ Hit trace(const DrvBox* boxes, int n, f3 o, f3 d) {
  Hit h{-1, 0, 3.0e38f};
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  for (int b = 0; b < n; ++b) {
    float tn = -3.0e38f, tf = 3.0e38f;
    int an = 0, af = 0;
    bool miss = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (dd[a] == 0.0f) {
        if (oo[a] < boxes[b].min[a] || oo[a] > boxes[b].max[a]) miss = true;
        continue;
      }
      float t0 = __fdiv_rn(boxes[b].min[a] - oo[a], dd[a]);
      float t1 = __fdiv_rn(boxes[b].max[a] - oo[a], dd[a]);
      if (t0 > t1) {
        float tmp = t0;
        t0 = t1;
        t1 = tmp;
      }
      if (t0 > tn) {
        tn = t0;
        an = a;
      }
      if (t1 < tf) {
        tf = t1;
        af = a;
      }
    }
    if (miss || tn > tf) continue;
    float t = boxes[b].inward ? tf : tn;
    int ax = boxes[b].inward ? af : an;
    if (t > 1e-6f && t < h.t) {
      h.t = t;
      h.box = b;
      h.axis = ax;
    }
  }
  return h;
}

__device__ __forceinline__ f3 face_normal(int axis, f3 d) {
  float dd = axis == 0 ? d.x : (axis == 1 ? d.y : d.z);
  float s = dd > 0.0f ? -1.0f : 1.0f;
  return mkf3(axis == 0 ? s : 0.0f, axis == 1 ? s : 0.0f, axis == 2 ? s : 0.0f);
}

__global__ void __launch_bounds__(256) gbuffer_kernel(const DrvBox* __restrict__ boxes, int n_boxes, RayFrame rf,
                                                      DrvPerFrame vp, int w, int h, DrvGBufferOut out) {
  __shared__ DrvBox sb[kMaxSmemBoxes];
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < n_boxes; i += blockDim.x * blockDim.y) sb[i] = boxes[i];
  __syncthreads();
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  size_t i = (size_t)y * w + x;
  float nx = ((x + 0.5f) / w) * 2.0f - 1.0f, ny = ((y + 0.5f) / h) * 2.0f - 1.0f;
  f3 d = normalize3(ldf3(rf.fwd) + ldf3(rf.right) * nx + ldf3(rf.up) * ny);
  f3 o = ldf3(rf.origin);
  Hit hit = trace(sb, n_boxes, o, d);
  if (hit.box < 0) {
    out.depth[i] = 0.0f;
    if (out.normal_rg16i) {
      out.normal_rg16i[2 * i] = 0;
      out.normal_rg16i[2 * i + 1] = 0;
    }
    if (out.normal_f32) out.normal_f32[3 * i] = out.normal_f32[3 * i + 1] = out.normal_f32[3 * i + 2] = 0.0f;
    out.albedo[3 * i] = out.albedo[3 * i + 1] = out.albedo[3 * i + 2] = 0.0f;
    return;
  }
  f3 p = o + d * hit.t;
  const float* M = vp.view_projection;
  float cz = M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11];
  float cw = M[12] * p.x + M[13] * p.y + M[14] * p.z + M[15];
  out.depth[i] = cz / cw;
  f3 n = face_normal(hit.axis, d);
  if (out.normal_rg16i) {
    int16_t pk[2];
    pack_normal16i(n, pk);
    out.normal_rg16i[2 * i] = pk[0];
    out.normal_rg16i[2 * i + 1] = pk[1];
  }
  if (out.normal_f32) {
    out.normal_f32[3 * i] = n.x;
    out.normal_f32[3 * i + 1] = n.y;
    out.normal_f32[3 * i + 2] = n.z;
  }
  out.albedo[3 * i] = sb[hit.box].albedo[0];
  out.albedo[3 * i + 1] = sb[hit.box].albedo[1];
  out.albedo[3 * i + 2] = sb[hit.box].albedo[2];
}

// Direction from the light through RSM texel centre (u, v): the unprojection
// at depth 0 that the VPL reconstruction uses (cacheLightingRSM.comp:154-155).
__device__ __forceinline__ f3 light_ray(const DrvSpotLight& L, float u, float v) {
  float x = u * 2.0f - 1.0f, y = v * 2.0f - 1.0f;
  const float* M = L.inverse_view_projection;
  float c0 = M[0] * x + M[1] * y + M[3];
  float c1 = M[4] * x + M[5] * y + M[7];
  float c2 = M[8] * x + M[9] * y + M[11];
  float c3 = M[12] * x + M[13] * y + M[15];
  f3 p = mkf3(c0 / c3, c1 / c3, c2 / c3);
  return normalize3(p - ldf3(L.position));
}

__global__ void __launch_bounds__(256) rsm_kernel(const DrvBox* __restrict__ boxes, int n_boxes, DrvSpotLight L,
                                                  DrvRSMOut out) {
  __shared__ DrvBox sb[kMaxSmemBoxes];
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < n_boxes; i += blockDim.x * blockDim.y) sb[i] = boxes[i];
  __syncthreads();
  const int R = L.rsm_render_resolution;
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= R || y >= R) return;
  size_t i = (size_t)y * R + x;
  f3 o = ldf3(L.position);
  f3 d = light_ray(L, (x + 0.5f) / R, (y + 0.5f) / R);
  Hit hit = trace(sb, n_boxes, o, d);
  if (hit.box < 0) {
    out.flux[3 * i] = out.flux[3 * i + 1] = out.flux[3 * i + 2] = 0.0f;
    out.normal[2 * i] = out.normal[2 * i + 1] = 0;
    out.depth_lin_sq[2 * i] = out.depth_lin_sq[2 * i + 1] = 0.0f;
    return;
  }
  f3 p = o + d * hit.t;
  f3 to_light = o - p;
  float dist = sqrtf(dot3(to_light, to_light));
  to_light = to_light * (1.0f / dist);
  float cos_to_light = sat(-dot3(to_light, ldf3(L.direction)));
  float total_sr = 2.0f * DRV_SHADER_PI * (1.0f - L.cos_half_angle);
  float pixel_sr = total_sr * cos_to_light / R / R;
  float falloff = sat(cos_to_light - L.cos_half_angle) / (1.0f - L.cos_half_angle);
  float k = falloff * pixel_sr / DRV_SHADER_PI;
  for (int c = 0; c < 3; ++c) out.flux[3 * i + c] = sb[hit.box].albedo[c] * L.intensity[c] * k;
  out.depth_lin_sq[2 * i] = dist;
  out.depth_lin_sq[2 * i + 1] = dist * dist;
  int16_t pk[2];
  pack_normal16i(face_normal(hit.axis, d), pk);
  out.normal[2 * i] = pk[0];
  out.normal[2 * i + 1] = pk[1];
}

}  // namespace

cudaError_t launch_raycast_gbuffer(cudaStream_t s, const DrvBox* boxes, int n_boxes, RayFrame rf,
                                   const float* view_proj, int w, int h, DrvGBufferOut out) {
  if (n_boxes > kMaxSmemBoxes) return cudaErrorInvalidValue;
  DrvPerFrame vp{};
  for (int i = 0; i < 16; ++i) vp.view_projection[i] = view_proj[i];
  dim3 block(16, 16), grid((w + 15) / 16, (h + 15) / 16);
  gbuffer_kernel<<<grid, block, 0, s>>>(boxes, n_boxes, rf, vp, w, h, out);
  return cudaGetLastError();
}

cudaError_t launch_raycast_rsm(cudaStream_t s, const DrvBox* boxes, int n_boxes, const DrvSpotLight& L,
                               DrvRSMOut out) {
  if (n_boxes > kMaxSmemBoxes) return cudaErrorInvalidValue;
  int R = L.rsm_render_resolution;
  dim3 block(16, 16), grid((R + 15) / 16, (R + 15) / 16);
  rsm_kernel<<<grid, block, 0, s>>>(boxes, n_boxes, L, out);
  return cudaGetLastError();
}

}  // namespace drv
