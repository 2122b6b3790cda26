// light_common.cuh — per-pair pieces of the cache-lighting stage shared by the
// cone-traced (k_light.cu) and surrogate (k_light_surrogate.cu) kernels:
// VPL loads in both storage precisions, the SH gather of
// cacheLightingRSM.comp:234-279, and the test that a shadow block can
// contribute at all.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "drv_device.cuh"

namespace drv {

struct VplData {
  float px, py, pz, area, fr, fg, fb, nx, ny, nz;
};

template <bool BF16>
__device__ __forceinline__ VplData load_vpl(const void* base, int i) {
  VplData d;
  if (BF16) {
    const uint4* q = reinterpret_cast<const uint4*>(static_cast<const DrvVPLBF16*>(base) + i);
    const uint4 a = __ldg(q), b = __ldg(q + 1);
    d.px = __uint_as_float(a.x);
    d.py = __uint_as_float(a.y);
    d.pz = __uint_as_float(a.z);
    d.area = __uint_as_float(a.w);
    d.fr = from_bf16((uint16_t)(b.x & 0xFFFFu));
    d.fg = from_bf16((uint16_t)(b.x >> 16));
    d.fb = from_bf16((uint16_t)(b.y & 0xFFFFu));
    d.nx = from_bf16((uint16_t)(b.y >> 16));
    d.ny = from_bf16((uint16_t)(b.z & 0xFFFFu));
    d.nz = from_bf16((uint16_t)(b.z >> 16));
  } else {
    const float4* q = reinterpret_cast<const float4*>(static_cast<const DrvVPL*>(base) + i);
    const float4 a = __ldg(q), b = __ldg(q + 1), n = __ldg(q + 2);  // {flux, area}, {position}, {normal}
    d.fr = a.x;
    d.fg = a.y;
    d.fb = a.z;
    d.area = a.w;
    d.px = b.x;
    d.py = b.y;
    d.pz = b.z;
    d.nx = n.x;
    d.ny = n.y;
    d.nz = n.z;
  }
  return d;
}

// The light-transfer factor of one VPL at cache c, computed exactly as the
// gather computes it: radianceIn = flux * (g * shadowing).
struct Transfer {
  float tx, ty, tz;  // unit direction cache -> VPL
  float g;           // saturate(dot(n, -dir)) / (d^2 + area)
};

__device__ __forceinline__ Transfer transfer(const VplData& v, float cx, float cy, float cz) {
  Transfer t;
  float tx = v.px - cx, ty = v.py - cy, tz = v.pz - cz;
  const float d2 = tx * tx + ty * ty + tz * tz;
  const float r = rsqrtf(d2);
  t.tx = tx * r;
  t.ty = ty * r;
  t.tz = tz * r;
  t.g = sat(-(v.nx * t.tx + v.ny * t.ty + v.nz * t.tz)) / (d2 + v.area);
  return t;
}

// True when a VPL can add anything to the cache: positive flux and facing it.
// A VPL that fails this adds exactly zero whatever its shadowing is, so its
// shadow cone need not be traced.
__device__ __forceinline__ bool contributes(const VplData& v, const Transfer& t) {
  return t.g > 0.0f && (v.fr > 0.0f || v.fg > 0.0f || v.fb > 0.0f);
}

// SH gather of one VPL, cacheLightingRSM.comp:255-278. acc (and comp with
// KAHAN) point at this thread's column of a [NK*3][stride] shared array.
template <int NK, bool KAHAN>
__device__ __forceinline__ void accumulate(const float ev[5], float* acc, float* comp, int stride, const VplData& v,
                                           const Transfer& t, float shadowing) {
  const float s = t.g * shadowing;
  const float L[3] = {v.fr * s, v.fg * s, v.fb * s};
  const float tx = t.tx, ty = t.ty, tz = t.tz;
  const float bs[9] = {ev[0], -ev[1] * ty, ev[1] * tz, -ev[1] * tx, -ev[2] * tx * ty, ev[2] * ty * tz,
                       ev[3] * (tz * tz * 3.0f - 1.0f), ev[2] * tx * tz, ev[4] * (tx * tx - ty * ty)};
#pragma unroll
  for (int k = 0; k < NK; ++k)
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const int o = (3 * k + ch) * stride;
      const float x = bs[k] * L[ch];
      if (KAHAN) {
        // Kahan-compensated running sum (FP32 accumulation, BF16 storage).
        const float y = __fsub_rn(x, comp[o]);
        const float tt = __fadd_rn(acc[o], y);
        comp[o] = __fsub_rn(__fsub_rn(tt, acc[o]), y);
        acc[o] = tt;
      } else {
        acc[o] += x;
      }
    }
}

}  // namespace drv
