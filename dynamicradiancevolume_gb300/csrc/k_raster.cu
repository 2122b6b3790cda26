// k_raster.cu — the input producers for triangle meshes: the G-buffer fill
// (fillgbuffer.frag) and the RSM fill (fillrsm.frag:24-62) of an arbitrary
// mesh, untextured (linear RGB albedo per triangle, optional vertex normals).
//
// Two passes per target. Visibility: a warp per triangle projects it with the
// target's view-projection (row-major M v), clips it against the near plane
// (reversed-Z: z/w <= 1, i.e. w - z >= 0; a polygon of up to 4 vertices,
// drawn as a fan), and for every pixel centre inside with depth in [0, 1]
// takes the 64-bit maximum of (depth bits, triangle + 1) — reversed-Z, the
// nearest surface has the largest depth; equal depths go to the higher
// triangle index. Coverage is watertight: each edge function is evaluated with
// its endpoints in a canonical order and without contraction, so the two
// triangles that share an edge get exactly opposite values at every pixel
// centre, and ties count as inside for both. Resolve: a thread per pixel intersects its
// centre ray (the same ray as the box ray caster) with the winning triangle's
// plane and shades as the box producer does: depth from the hit point,
// normal (the face normal, or the barycentric blend of the vertex normals)
// turned towards the ray, albedo of the triangle; for the RSM the flux of
// fillrsm.frag at the hit point.
#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

struct MeshView {
  const float* pos;
  const float* nrm;
  const float* alb;
  const uint32_t* idx;
  int nv, nt;
};

__device__ __forceinline__ bool tri_indices(const MeshView& m, int k, uint32_t v[3]) {
  for (int j = 0; j < 3; ++j) v[j] = m.idx ? __ldg(m.idx + 3 * k + j) : 3u * k + j;
  return v[0] < (uint32_t)m.nv && v[1] < (uint32_t)m.nv && v[2] < (uint32_t)m.nv;
}

__device__ __forceinline__ f3 vertex(const MeshView& m, uint32_t i) {
  return mkf3(__ldg(m.pos + 3 * (size_t)i), __ldg(m.pos + 3 * (size_t)i + 1), __ldg(m.pos + 3 * (size_t)i + 2));
}

struct Mat4 {
  float m[16];
};

// M p with explicit rounding: a vertex projects to the same bits in every
// triangle that uses it, wherever the call is inlined.
__device__ __forceinline__ float mrow(const float* r, f3 p) {
  return __fmaf_rn(r[2], p.z, __fmaf_rn(r[1], p.y, __fmaf_rn(r[0], p.x, r[3])));
}

__device__ __forceinline__ float4 to_clip(const Mat4& M, f3 p) {
  return make_float4(mrow(M.m, p), mrow(M.m + 4, p), mrow(M.m + 8, p), mrow(M.m + 12, p));
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}

// Signed distance to the near plane in clip space (reversed-Z: inside when
// z/w <= 1 with w > 0; w - z is proportional to the view depth past the near
// plane, so it is >= 0 exactly in front of it).
__device__ __forceinline__ float near_distance(float4 c) { return c.w - c.z; }

// Edge function of p against the directed edge a -> b (positive on the left
// for y up), computed with the endpoints in lexicographic order and explicit
// rounding, then negated if they were swapped: the triangles on either side
// of an edge get bitwise opposite values.
__device__ __forceinline__ float edge_fn(float ax, float ay, float bx, float by, float px, float py) {
  const bool swap = ax > bx || (ax == bx && ay > by);
  const float x0 = swap ? bx : ax, y0 = swap ? by : ay, x1 = swap ? ax : bx, y1 = swap ? ay : by;
  const float e = __fsub_rn(__fmul_rn(__fsub_rn(x1, x0), __fsub_rn(py, y0)),
                            __fmul_rn(__fsub_rn(y1, y0), __fsub_rn(px, x0)));
  return swap ? -e : e;
}

// Visibility pass: a warp per triangle (grid-stride).
__global__ void __launch_bounds__(256) raster_kernel(MeshView m, Mat4 M, int W, int H,
                                                     unsigned long long* __restrict__ keys) {
  const int lane = threadIdx.x & 31;
  const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); k < m.nt; k += n_warps) {
    uint32_t vi[3];
    if (!tri_indices(m, k, vi)) continue;
    const float4 c[3] = {to_clip(M, vertex(m, vi[0])), to_clip(M, vertex(m, vi[1])), to_clip(M, vertex(m, vi[2]))};
    // Clip against the near plane (Sutherland-Hodgman, one plane). The cut
    // point is interpolated from the inside end, so the two triangles sharing
    // a cut edge compute the same vertex.
    float4 poly[4];
    int n = 0;
    for (int e = 0; e < 3; ++e) {
      const float4 a = c[e], b = c[(e + 1) % 3];
      const float da = near_distance(a), db = near_distance(b);
      const bool ia = da >= 0.0f, ib = db >= 0.0f;
      if (ia) poly[n++] = a;
      if (ia != ib) poly[n++] = ia ? lerp4(a, b, da / (da - db)) : lerp4(b, a, db / (db - da));
    }
    if (n < 3) continue;
    float sx[4], sy[4], sz[4];
    for (int i = 0; i < n; ++i) {
      const float iw = __fdiv_rn(1.0f, poly[i].w);
      sx[i] = __fmul_rn(__fmaf_rn(__fmul_rn(poly[i].x, iw), 0.5f, 0.5f), (float)W);
      sy[i] = __fmul_rn(__fmaf_rn(__fmul_rn(poly[i].y, iw), 0.5f, 0.5f), (float)H);
      sz[i] = __fmul_rn(poly[i].z, iw);
    }
    for (int f = 1; f + 1 < n; ++f) {  // fan (0, f, f + 1)
      const float x0 = sx[0], y0 = sy[0], x1 = sx[f], y1 = sy[f], x2 = sx[f + 1], y2 = sy[f + 1];
      const float area = edge_fn(x0, y0, x1, y1, x2, y2);
      if (!(area != 0.0f)) continue;
      const float orient = area > 0.0f ? 1.0f : -1.0f;
      const int bx0 = max(0, (int)floorf(fminf(fminf(x0, x1), x2))), by0 = max(0, (int)floorf(fminf(fminf(y0, y1), y2)));
      const int bx1 = min(W - 1, (int)floorf(fmaxf(fmaxf(x0, x1), x2))), by1 = min(H - 1, (int)floorf(fmaxf(fmaxf(y0, y1), y2)));
      if (bx1 < bx0 || by1 < by0) continue;
      const int bw = bx1 - bx0 + 1;
      const int total = bw * (by1 - by0 + 1);
      for (int q = lane; q < total; q += 32) {
        const int px = bx0 + q % bw, py = by0 + q / bw;
        const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
        // edge functions opposite vertices 0, f, f+1, made positive inside
        const float e0 = orient * edge_fn(x1, y1, x2, y2, cx, cy);
        const float e1 = orient * edge_fn(x2, y2, x0, y0, cx, cy);
        const float e2 = orient * edge_fn(x0, y0, x1, y1, cx, cy);
        if (e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) continue;
        const float sum = e0 + e1 + e2;
        if (!(sum > 0.0f)) continue;
        const float z = (e0 * sz[0] + e1 * sz[f] + e2 * sz[f + 1]) / sum;
        if (!(z >= 0.0f && z <= 1.0f)) continue;
        const unsigned long long key = (unsigned long long)__float_as_uint(z) << 32 | (unsigned long long)(k + 1);
        atomicMax(keys + (size_t)py * W + px, key);
      }
    }
  }
}

// Hit point of ray (o, d) on the plane of triangle tri, the normal turned
// towards the ray, and the triangle's albedo. False when the plane is parallel
// to the ray or behind it.
__device__ __forceinline__ bool resolve_hit(const MeshView& m, int tri, f3 o, f3 d, f3& p, f3& n, f3& alb) {
  uint32_t vi[3];
  if (!tri_indices(m, tri, vi)) return false;
  const f3 v0 = vertex(m, vi[0]), v1 = vertex(m, vi[1]), v2 = vertex(m, vi[2]);
  const f3 e1 = v1 - v0, e2 = v2 - v0;
  const f3 fn = cross3(e1, e2);
  const float denom = dot3(fn, d);
  if (!(denom != 0.0f)) return false;
  const float t = dot3(fn, v0 - o) / denom;
  if (!(t > 0.0f)) return false;
  p = o + d * t;
  if (m.nrm) {
    const float nn = dot3(fn, fn);
    const f3 q = p - v0;
    const float l1 = dot3(cross3(q, e2), fn) / nn, l2 = dot3(cross3(e1, q), fn) / nn, l0 = 1.0f - l1 - l2;
    auto vn = [&](uint32_t i) {
      return mkf3(__ldg(m.nrm + 3 * (size_t)i), __ldg(m.nrm + 3 * (size_t)i + 1), __ldg(m.nrm + 3 * (size_t)i + 2));
    };
    n = vn(vi[0]) * l0 + vn(vi[1]) * l1 + vn(vi[2]) * l2;
  } else {
    n = fn;
  }
  // Normalised through the largest component first, so that an axis-aligned
  // normal comes out exactly (+-1 on its axis, as the box producers write it).
  const float big = fmaxf(fmaxf(fabsf(n.x), fabsf(n.y)), fabsf(n.z));
  if (big > 0.0f) {
    n = mkf3(n.x / big, n.y / big, n.z / big);
    const float len = sqrtf(dot3(n, n));
    n = mkf3(n.x / len, n.y / len, n.z / len);
  } else {
    n = mkf3(0.0f, 0.0f, 1.0f);
  }
  if (dot3(n, d) > 0.0f) n = n * -1.0f;
  n = mkf3(n.x + 0.0f, n.y + 0.0f, n.z + 0.0f);  // no negative zeros (they pack to the other end of the atan2 range)
  alb = m.alb ? mkf3(__ldg(m.alb + 3 * tri), __ldg(m.alb + 3 * tri + 1), __ldg(m.alb + 3 * tri + 2))
              : mkf3(1.0f, 1.0f, 1.0f);
  return true;
}

__global__ void __launch_bounds__(256) gbuffer_resolve_kernel(MeshView m, RayFrame rf, Mat4 M, int w, int h,
                                                              const unsigned long long* __restrict__ keys,
                                                              DrvGBufferOut out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const size_t i = (size_t)y * w + x;
  const unsigned long long key = keys[i];
  f3 p, n, alb;
  bool hit = false;
  if (key) {
    const float nx = ((x + 0.5f) / w) * 2.0f - 1.0f, ny = ((y + 0.5f) / h) * 2.0f - 1.0f;
    const f3 d = normalize3(ldf3(rf.fwd) + ldf3(rf.right) * nx + ldf3(rf.up) * ny);
    hit = resolve_hit(m, (int)(key & 0xFFFFFFFFull) - 1, ldf3(rf.origin), d, p, n, alb);
  }
  if (!hit) {
    out.depth[i] = 0.0f;
    if (out.normal_rg16i) out.normal_rg16i[2 * i] = out.normal_rg16i[2 * i + 1] = 0;
    if (out.normal_f32) out.normal_f32[3 * i] = out.normal_f32[3 * i + 1] = out.normal_f32[3 * i + 2] = 0.0f;
    out.albedo[3 * i] = out.albedo[3 * i + 1] = out.albedo[3 * i + 2] = 0.0f;
    return;
  }
  const float4 c = to_clip(M, p);
  out.depth[i] = c.z / c.w;
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
  out.albedo[3 * i] = alb.x;
  out.albedo[3 * i + 1] = alb.y;
  out.albedo[3 * i + 2] = alb.z;
}

// Direction from the light through RSM texel centre (u, v) (as the box RSM
// producer and the VPL reconstruction, cacheLightingRSM.comp:154-155).
__device__ __forceinline__ f3 light_ray_dir(const DrvSpotLight& L, float u, float v) {
  const float x = u * 2.0f - 1.0f, y = v * 2.0f - 1.0f;
  const float* M = L.inverse_view_projection;
  const float c0 = M[0] * x + M[1] * y + M[3], c1 = M[4] * x + M[5] * y + M[7];
  const float c2 = M[8] * x + M[9] * y + M[11], c3 = M[12] * x + M[13] * y + M[15];
  return normalize3(mkf3(c0 / c3, c1 / c3, c2 / c3) - ldf3(L.position));
}

__global__ void __launch_bounds__(256) rsm_resolve_kernel(MeshView m, DrvSpotLight L,
                                                          const unsigned long long* __restrict__ keys, DrvRSMOut out) {
  const int R = L.rsm_render_resolution;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= R || y >= R) return;
  const size_t i = (size_t)y * R + x;
  const unsigned long long key = keys[i];
  const f3 o = ldf3(L.position);
  f3 p, n, alb;
  bool hit = false;
  if (key) hit = resolve_hit(m, (int)(key & 0xFFFFFFFFull) - 1, o, light_ray_dir(L, (x + 0.5f) / R, (y + 0.5f) / R), p, n, alb);
  if (!hit) {
    out.flux[3 * i] = out.flux[3 * i + 1] = out.flux[3 * i + 2] = 0.0f;
    out.normal[2 * i] = out.normal[2 * i + 1] = 0;
    out.depth_lin_sq[2 * i] = out.depth_lin_sq[2 * i + 1] = 0.0f;
    return;
  }
  // fillrsm.frag:32-50
  f3 to_light = o - p;
  const float dist = sqrtf(dot3(to_light, to_light));
  to_light = to_light * (1.0f / dist);
  const float cos_to_light = sat(-dot3(to_light, ldf3(L.direction)));
  const float total_sr = 2.0f * DRV_SHADER_PI * (1.0f - L.cos_half_angle);
  const float pixel_sr = total_sr * cos_to_light / R / R;
  const float falloff = sat(cos_to_light - L.cos_half_angle) / (1.0f - L.cos_half_angle);
  const float kf = falloff * pixel_sr / DRV_SHADER_PI;
  out.flux[3 * i] = alb.x * L.intensity[0] * kf;
  out.flux[3 * i + 1] = alb.y * L.intensity[1] * kf;
  out.flux[3 * i + 2] = alb.z * L.intensity[2] * kf;
  out.depth_lin_sq[2 * i] = dist;
  out.depth_lin_sq[2 * i + 1] = dist * dist;
  int16_t pk[2];
  pack_normal16i(n, pk);
  out.normal[2 * i] = pk[0];
  out.normal[2 * i + 1] = pk[1];
}

MeshView mesh_view(const DrvMesh& mesh) {
  return MeshView{mesh.positions, mesh.normals, mesh.albedo, mesh.indices, mesh.n_vertices, mesh.n_triangles};
}

cudaError_t raster(cudaStream_t s, const MeshView& m, const float* view_proj, int W, int H, unsigned long long* keys,
                   int num_sms) {
  cudaError_t e = cudaMemsetAsync(keys, 0, (size_t)W * H * sizeof(unsigned long long), s);
  if (e != cudaSuccess || m.nt <= 0) return e;
  Mat4 M;
  for (int i = 0; i < 16; ++i) M.m[i] = view_proj[i];
  const int warps = m.nt < num_sms * 64 ? m.nt : num_sms * 64;
  raster_kernel<<<(warps + 7) / 8, 256, 0, s>>>(m, M, W, H, keys);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_raster_gbuffer(cudaStream_t s, const DrvMesh& mesh, RayFrame rf, const float* view_proj, int w,
                                  int h, unsigned long long* keys, DrvGBufferOut out, int num_sms) {
  const MeshView m = mesh_view(mesh);
  cudaError_t e = raster(s, m, view_proj, w, h, keys, num_sms);
  if (e != cudaSuccess) return e;
  Mat4 M;
  for (int i = 0; i < 16; ++i) M.m[i] = view_proj[i];
  dim3 block(16, 16), grid((w + 15) / 16, (h + 15) / 16);
  gbuffer_resolve_kernel<<<grid, block, 0, s>>>(m, rf, M, w, h, keys, out);
  return cudaGetLastError();
}

cudaError_t launch_raster_rsm(cudaStream_t s, const DrvMesh& mesh, const DrvSpotLight& L, unsigned long long* keys,
                              DrvRSMOut out, int num_sms) {
  const MeshView m = mesh_view(mesh);
  const int R = L.rsm_render_resolution;
  cudaError_t e = raster(s, m, L.view_projection, R, R, keys, num_sms);
  if (e != cudaSuccess) return e;
  dim3 block(16, 16), grid((R + 15) / 16, (R + 15) / 16);
  rsm_resolve_kernel<<<grid, block, 0, s>>>(m, L, keys, out);
  return cudaGetLastError();
}

}  // namespace drv
