// k_rsm.cu — RSM mip chain (downsamplersm.frag:15-33, renderer.cpp:1300-1339)
// and VPL extraction at RSMReadResolution (cacheLightingRSM.comp:141-158)
// plus the per-block indirect-shadow cone sources (cacheLightingRSM.comp:168-192).
//
// The reference re-extracts every VPL tile inside every lighting workgroup
// (redundant by caches/64); here extraction runs once per light into a packed
// 48-byte VPL array that the light stage streams through shared memory.
#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

// Element i of an F32 or F16 RSM array.
__device__ __forceinline__ float rsm_at(const void* a, int half, size_t i) {
  return half ? __half2float(static_cast<const __half*>(a)[i]) : static_cast<const float*>(a)[i];
}

// One downsample pass res -> res/2: flux = sum of the 2x2 children
// (textureGather), normal = PackNormal16I(normalize(sum of unpacked normals)),
// (d, d^2) = mean (linear sample at the shared corner).
__global__ void __launch_bounds__(256) downsample_kernel(int res, const void* __restrict__ flux,
                                                         const int16_t* __restrict__ nrm, const void* __restrict__ dls,
                                                         int src_half, float* __restrict__ fo,
                                                         int16_t* __restrict__ no, float* __restrict__ dlo) {
  int h = res >> 1;
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= h || y >= h) return;
  float fs[3] = {0, 0, 0}, d0 = 0, d1 = 0;
  f3 ns = mkf3(0, 0, 0);
#pragma unroll
  for (int dy = 0; dy < 2; ++dy)
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
      size_t j = (size_t)(2 * y + dy) * res + (2 * x + dx);
      fs[0] += rsm_at(flux, src_half, 3 * j);
      fs[1] += rsm_at(flux, src_half, 3 * j + 1);
      fs[2] += rsm_at(flux, src_half, 3 * j + 2);
      ns = ns + unpack_normal16i(nrm[2 * j], nrm[2 * j + 1]);
      d0 += rsm_at(dls, src_half, 2 * j);
      d1 += rsm_at(dls, src_half, 2 * j + 1);
    }
  size_t i = (size_t)y * h + x;
  fo[3 * i] = fs[0];
  fo[3 * i + 1] = fs[1];
  fo[3 * i + 2] = fs[2];
  float len2 = dot3(ns, ns);
  int16_t pk[2] = {0, 0};
  if (len2 > 0.0f) pack_normal16i(ns * rsqrtf(len2), pk);
  no[2 * i] = pk[0];
  no[2 * i + 1] = pk[1];
  dlo[2 * i] = d0 * 0.25f;
  dlo[2 * i + 1] = d1 * 0.25f;
}

__device__ __forceinline__ f3 unproject_dir(const DrvSpotLight& L, float u, float v) {
  float x = u * 2.0f - 1.0f, y = v * 2.0f - 1.0f;
  const float* M = L.inverse_view_projection;
  float c0 = M[0] * x + M[1] * y + M[3];
  float c1 = M[4] * x + M[5] * y + M[7];
  float c2 = M[8] * x + M[9] * y + M[11];
  float c3 = M[12] * x + M[13] * y + M[15];
  return normalize3(mkf3(c0 / c3, c1 / c3, c2 / c3) - ldf3(L.position));
}

template <bool BF16>
__global__ void __launch_bounds__(256) extract_kernel(DrvSpotLight L, int R, const void* __restrict__ flux,
                                                      const int16_t* __restrict__ nrm, const void* __restrict__ dls,
                                                      int read_half, const void* __restrict__ dls_shadow,
                                                      int shadow_half, void* __restrict__ vpls_out,
                                                      DrvShadowCone* __restrict__ cones,
                                                      float4* __restrict__ records) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = R * R;
  if (i >= n) return;
  const f3 lp = ldf3(L.position);
  {
    uint32_t x, y;
    morton_decode((uint32_t)i, x, y);
    size_t t = (size_t)y * R + x;
    float u = (x + 0.5f) / R, v = (y + 0.5f) / R;
    float d = rsm_at(dls, read_half, 2 * t);
    const f3 p = lp + unproject_dir(L, u, v) * d;
    const f3 nn = unpack_normal16i(nrm[2 * t], nrm[2 * t + 1]);
    const float area = d * d * L.val_area_factor;
    if (BF16) {
      DrvVPLBF16 o;
      o.position[0] = p.x;
      o.position[1] = p.y;
      o.position[2] = p.z;
      o.disc_area = area;
      for (int c = 0; c < 3; ++c) o.flux_bf16[c] = to_bf16(rsm_at(flux, read_half, 3 * t + c));
      o.normal_bf16[0] = to_bf16(nn.x);
      o.normal_bf16[1] = to_bf16(nn.y);
      o.normal_bf16[2] = to_bf16(nn.z);
      o._pad = 0u;
      reinterpret_cast<DrvVPLBF16*>(vpls_out)[i] = o;
      // the cull's record of the stored (BF16) normal and flux
      if (records)
        records[i] = make_cull_record(from_bf16(o.normal_bf16[0]), from_bf16(o.normal_bf16[1]),
                                      from_bf16(o.normal_bf16[2]), p.x, p.y, p.z,
                                      from_bf16(o.flux_bf16[0]) > 0.0f || from_bf16(o.flux_bf16[1]) > 0.0f ||
                                          from_bf16(o.flux_bf16[2]) > 0.0f);
    } else {
      DrvVPL o;
      o.flux[0] = rsm_at(flux, read_half, 3 * t);
      o.flux[1] = rsm_at(flux, read_half, 3 * t + 1);
      o.flux[2] = rsm_at(flux, read_half, 3 * t + 2);
      o.disc_area = area;
      o.position[0] = p.x;
      o.position[1] = p.y;
      o.position[2] = p.z;
      o._pad0 = 0.0f;
      o.normal[0] = nn.x;
      o.normal[1] = nn.y;
      o.normal[2] = nn.z;
      o._pad1 = 0.0f;
      reinterpret_cast<DrvVPL*>(vpls_out)[i] = o;
      if (records)
        records[i] = make_cull_record(nn.x, nn.y, nn.z, p.x, p.y, p.z,
                                      o.flux[0] > 0.0f || o.flux[1] > 0.0f || o.flux[2] > 0.0f);
    }
  }
  const int interval = L.indirect_shadow_sample_interval;
  if (i * interval < n) {
    // Shadow cone source of block i (VPLs i*interval ... (i+1)*interval-1).
    uint32_t x, y;
    morton_decode((uint32_t)(i * interval), x, y);
    const float off = L.indirect_shadow_sampling_offset;
    float u = (x + off) / R, v = (y + off) / R;
    const int rs = R >> (int)L.indirect_shadow_lod;
    // Bilinear (d, d^2) at the shadow LOD, CLAMP_TO_EDGE.
    float fx = u * rs - 0.5f, fy = v * rs - 0.5f;
    float flx = floorf(fx), fly = floorf(fy);
    int x0 = (int)flx, y0 = (int)fly;
    float ax = fx - flx, ay = fy - fly;
    float dd0 = 0.0f, dd1 = 0.0f;
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay);
        int xx = min(max(x0 + dx, 0), rs - 1), yy = min(max(y0 + dy, 0), rs - 1);
        dd0 += w * rsm_at(dls_shadow, shadow_half, ((size_t)yy * rs + xx) * 2);
        dd1 += w * rsm_at(dls_shadow, shadow_half, ((size_t)yy * rs + xx) * 2 + 1);
      }
    f3 avg = lp + unproject_dir(L, u, v) * dd0;
    float var = fmaxf(0.0f, dd1 - dd0 * dd0);  // clamped: rounding can push it below 0
    float dsr = fmaxf(L.indirect_shadow_super_val_width, sqrtf(var) * 2.0f / dd0);
    cones[i] = DrvShadowCone{{avg.x, avg.y, avg.z}, dsr};
  }
}

}  // namespace

cudaError_t launch_downsample_rsm(cudaStream_t s, int res, const void* flux, const int16_t* nrm, const void* dls,
                                  int src_half, float* fo, int16_t* no, float* dlo) {
  int h = res / 2;
  dim3 block(16, 16), grid((h + 15) / 16, (h + 15) / 16);
  downsample_kernel<<<grid, block, 0, s>>>(res, flux, nrm, dls, src_half, fo, no, dlo);
  return cudaGetLastError();
}

cudaError_t launch_extract_vpls(cudaStream_t s, const DrvSpotLight& L, int res, const void* flux, const int16_t* nrm,
                                const void* dls, int read_half, const void* dls_shadow, int shadow_half, void* vpls,
                                DrvShadowCone* cones, int precision, float4* records) {
  int n = res * res;
  if (precision == DRV_PRECISION_BF16)
    extract_kernel<true><<<(n + 255) / 256, 256, 0, s>>>(L, res, flux, nrm, dls, read_half, dls_shadow, shadow_half,
                                                         vpls, cones, records);
  else
    extract_kernel<false><<<(n + 255) / 256, 256, 0, s>>>(L, res, flux, nrm, dls, read_half, dls_shadow, shadow_half,
                                                          vpls, cones, records);
  return cudaGetLastError();
}

}  // namespace drv
