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

// The RSM mip chain, downsamplersm.frag:15-33 per pass res -> res/2: flux =
// sum of the 2x2 children (textureGather), normal = PackNormal16I(normalize(
// sum of unpacked normals)), (d, d^2) = mean (linear sample at the shared
// corner). Up to three passes run in one launch: a CTA takes a 32 x 32
// region of the source level and produces its 16 x 16, 8 x 8 and 4 x 4
// texels of the next levels (a thread per level-1 texel, then the first 64
// and 16 threads), keeping each level in shared memory for the next in the
// form it has in global memory (F32 flux and (d, d^2), packed RG16I
// normals), so each texel is the one a pass from global memory would give.
// Every level is written out. P: passes (1..3).
struct RsmChainArgs {
  int res;  // source resolution
  const void* flux;
  const int16_t* nrm;
  const void* dls;
  int src_half;
  float* fo[3];
  int16_t* no[3];
  float* dlo[3];
};

template <int P>
__global__ void __launch_bounds__(256) rsm_chain_kernel(RsmChainArgs a) {
  __shared__ float s_flux[2][3][256];
  __shared__ float s_dls[2][2][256];
  __shared__ int16_t s_nrm[2][2][256];
  const int t = threadIdx.x;
#pragma unroll
  for (int k = 1; k <= P; ++k) {
    const int side = 32 >> k;          // this level's texels per CTA row
    const int res_k = a.res >> k;      // this level's resolution
    const int src_res = a.res >> (k - 1);
    if (t < side * side) {
      const int lx = t & (side - 1), ly = t / side;
      const int gx = blockIdx.x * side + lx, gy = blockIdx.y * side + ly;
      float fs[3] = {0, 0, 0}, d0 = 0, d1 = 0;
      f3 ns = mkf3(0, 0, 0);
      if (gx < res_k && gy < res_k) {
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
          for (int dx = 0; dx < 2; ++dx) {
            if (k == 1) {
              const size_t j = (size_t)(2 * gy + dy) * src_res + (2 * gx + dx);
              fs[0] += rsm_at(a.flux, a.src_half, 3 * j);
              fs[1] += rsm_at(a.flux, a.src_half, 3 * j + 1);
              fs[2] += rsm_at(a.flux, a.src_half, 3 * j + 2);
              ns = ns + unpack_normal16i(a.nrm[2 * j], a.nrm[2 * j + 1]);
              d0 += rsm_at(a.dls, a.src_half, 2 * j);
              d1 += rsm_at(a.dls, a.src_half, 2 * j + 1);
            } else {
              const int b = (k - 2) & 1, ps = 2 * side;  // the previous level's buffer and row
              const int j = (2 * ly + dy) * ps + (2 * lx + dx);
              fs[0] += s_flux[b][0][j];
              fs[1] += s_flux[b][1][j];
              fs[2] += s_flux[b][2][j];
              ns = ns + unpack_normal16i(s_nrm[b][0][j], s_nrm[b][1][j]);
              d0 += s_dls[b][0][j];
              d1 += s_dls[b][1][j];
            }
          }
        const float len2 = dot3(ns, ns);
        int16_t pk[2] = {0, 0};
        if (len2 > 0.0f) pack_normal16i(ns * rsqrtf(len2), pk);
        d0 *= 0.25f;
        d1 *= 0.25f;
        const size_t i = (size_t)gy * res_k + gx;
        a.fo[k - 1][3 * i] = fs[0];
        a.fo[k - 1][3 * i + 1] = fs[1];
        a.fo[k - 1][3 * i + 2] = fs[2];
        a.no[k - 1][2 * i] = pk[0];
        a.no[k - 1][2 * i + 1] = pk[1];
        a.dlo[k - 1][2 * i] = d0;
        a.dlo[k - 1][2 * i + 1] = d1;
        if (k < P) {
          const int b = (k - 1) & 1;
          s_flux[b][0][t] = fs[0];
          s_flux[b][1][t] = fs[1];
          s_flux[b][2][t] = fs[2];
          s_nrm[b][0][t] = pk[0];
          s_nrm[b][1][t] = pk[1];
          s_dls[b][0][t] = d0;
          s_dls[b][1][t] = d1;
        }
      } else if (k < P) {  // outside the level (a ragged edge): never read by an in-range texel
        const int b = (k - 1) & 1;
        s_flux[b][0][t] = s_flux[b][1][t] = s_flux[b][2][t] = 0.0f;
        s_nrm[b][0][t] = s_nrm[b][1][t] = 0;
        s_dls[b][0][t] = s_dls[b][1][t] = 0.0f;
      }
    }
    if (k < P) __syncthreads();
  }
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

cudaError_t launch_rsm_chain(cudaStream_t s, int res, int passes, const void* flux, const int16_t* nrm,
                             const void* dls, int src_half, float* const* fo, int16_t* const* no, float* const* dlo) {
  if (passes < 1 || passes > 3) return cudaErrorInvalidValue;
  RsmChainArgs a{};
  a.res = res;
  a.flux = flux;
  a.nrm = nrm;
  a.dls = dls;
  a.src_half = src_half;
  for (int k = 0; k < passes; ++k) {
    a.fo[k] = fo[k];
    a.no[k] = no[k];
    a.dlo[k] = dlo[k];
  }
  const dim3 grid((res + 31) / 32, (res + 31) / 32);
  if (passes == 1) rsm_chain_kernel<1><<<grid, 256, 0, s>>>(a);
  else if (passes == 2) rsm_chain_kernel<2><<<grid, 256, 0, s>>>(a);
  else rsm_chain_kernel<3><<<grid, 256, 0, s>>>(a);
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
