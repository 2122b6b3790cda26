// k_light_surrogate.cu — the learned visibility surrogate in place of the
// indirect-shadow cone (cacheLightingRSM.comp:167-232), as the middle pass of
// the split light stage (k_light.cu): after the cull has listed the
// (cache, shadow block) pairs that can contribute, mlp_kernel takes them 32
// per warp:
//  1. each lane computes its pair's 32 input features (surrogate.cuh) and
//     stores them as BF16 in the warp's shared-memory tile;
//  2. the MLP runs on tensor cores with mma.sync m16n8k16 (BF16 in, FP32
//     accumulate): the accumulator fragment of one layer is, after bias and
//     GELU, exactly the A fragment of the next, so activations never leave
//     registers; weights are read from shared memory (rows padded so the
//     fragment loads are bank-conflict free);
//  3. each lane gets its (visibility, confidence) back by shuffles; confident
//     pairs store sigmoid(visibility) as their shadowing, the others are
//     appended to the re-trace list (narrow cones at its front, wide ones at
//     its back) that cone_kernel then traces.
#include <cmath>
#include <mutex>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "light_common.cuh"
#include "surrogate.cuh"
#include "voxel_sample.cuh"

namespace drv {
namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kLd1 = kMlpIn + 8;      // padded row (bf16) of W1 and of the feature tile
constexpr int kLdH = kMlpHidden + 8;  // padded row (bf16) of W2, W3, W4

// Inference weights as stored by drv_set_surrogate_params: BF16 matrices with
// padded rows, FP32 biases.
struct __align__(16) MlpWeights {
  uint16_t w1[kMlpHidden * kLd1];
  uint16_t w2[kMlpHidden * kLdH];
  uint16_t w3[kMlpHidden * kLdH];
  uint16_t w4[kMlpOutPad * kLdH];
  float b1[kMlpHidden], b2[kMlpHidden], b3[kMlpHidden], b4[kMlpOutPad];
};



__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* smem_row) {
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(smem_row);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// One hidden layer for one 16-row m-tile: in = A fragments [KSTEPS][4], out
// = A fragments of the next layer [4][4] after bias + GELU. The accumulators
// start at the bias (D = A B + C with C = bias).
template <int KSTEPS, int LD>
__device__ __forceinline__ void hidden_layer(const uint32_t (&in)[KSTEPS][4], const uint16_t* w, const float* bias,
                                             uint32_t (&out)[4][4], int g, int tig) {
#pragma unroll
  for (int j = 0; j < kMlpHidden / 8; ++j) {
    const float bl = bias[8 * j + 2 * tig], bh = bias[8 * j + 2 * tig + 1];
    float acc[4] = {bl, bh, bl, bh};
    const uint16_t* wr = w + (8 * j + g) * LD + 2 * tig;
#pragma unroll
    for (int kk = 0; kk < KSTEPS; ++kk) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk + 8);
      mma_bf16(acc, in[kk], b0, b1);
    }
    // n-tile j feeds k-step j/2 of the next layer: even tiles are its low k
    // half (regs 0,1), odd tiles its high half (regs 2,3).
    out[j >> 1][(j & 1) * 2 + 0] = gelu_bf16x2(pack_bf16x2(acc[0], acc[1]));
    out[j >> 1][(j & 1) * 2 + 1] = gelu_bf16x2(pack_bf16x2(acc[2], acc[3]));
  }
}

// Dynamic shared memory of one CTA (about 36 KB).
struct __align__(16) MlpSmem {
  MlpWeights w;
  uint16_t x[kWarps][32 * kLd1];  // per-warp BF16 feature tile, 80-byte rows
};

// Warp per 32 listed pairs: features -> MLP -> shadowing or re-trace.
// counters[5] receives the number of pairs evaluated.
template <bool BF16>
__global__ void __launch_bounds__(kThreads) mlp_kernel(StageParams p, PairList L, const MlpWeights* weights,
                                                       float conf_threshold) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem_raw);
  const MlpWeights& s_w = S.w;
  {
    const uint4* src = reinterpret_cast<const uint4*>(weights);
    uint4* dst = reinterpret_cast<uint4*>(&S.w);
    for (int i = threadIdx.x; i < (int)(sizeof(MlpWeights) / 16); i += kThreads) dst[i] = src[i];
  }
  __syncthreads();
  const uint32_t n = min(L.counters[0], L.cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  uint16_t* xt = S.x[warp];
  uint32_t evaluated = 0;
  for (uint32_t base = (blockIdx.x * kWarps + warp) * 32u; base < n; base += gridDim.x * kWarps * 32u) {
    const uint32_t i = base + lane;
    const uint32_t b = i < n ? L.block[i] : kNoPair;
    const bool valid = b != kNoPair;
    float f[kMlpIn];
    bool wide = false;
    if (valid) {
      float cx, cy, cz;
      cache_position<BF16>(p, L.cache[i], cx, cy, cz);
      const int l = block_light(p, (int)b);
      const LightArgs& la = p.ll.lights[l];
      const int lb = (int)b - p.block_base[l];
      const float4 cone = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
      const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval);
      surrogate_features(p.vox, p.inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x, cone.y,
                         cone.z, v.nx, v.ny, v.nz, cone.w, f);
      wide = wide_cone(cone.w, p.max_steps);
    } else {
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) f[k] = 0.0f;
    }
    uint32_t* row = reinterpret_cast<uint32_t*>(xt + lane * kLd1);
#pragma unroll
    for (int k = 0; k < kMlpIn / 2; ++k) row[k] = pack_bf16x2(f[2 * k], f[2 * k + 1]);
    __syncwarp();
    // The two 16-row m-tiles one after the other: one tile's fragments are
    // live at a time, which keeps the kernel near 64 registers.
    float o[2][4];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      uint32_t a1[2][4];
#pragma unroll
      for (int kk = 0; kk < 2; ++kk)
        ldmatrix_x4(a1[kk], xt + (16 * m + (lane & 7) + ((lane >> 3) & 1) * 8) * kLd1 + 16 * kk +
                                ((lane >> 4) & 1) * 8);
      uint32_t h1[4][4], h2[4][4];
      hidden_layer<2, kLd1>(a1, s_w.w1, s_w.b1, h1, g, tig);
      // Layers 2 and 3 have one shape: one copy of their code (instruction cache).
#pragma unroll 1
      for (int layer = 0; layer < 2; ++layer) {
        hidden_layer<4, kLdH>(h1, layer ? s_w.w3 : s_w.w2, layer ? s_w.b3 : s_w.b2, h2, g, tig);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int r = 0; r < 4; ++r) h1[kk][r] = h2[kk][r];
      }
      o[m][0] = o[m][1] = o[m][2] = o[m][3] = 0.0f;
      const uint16_t* wr = s_w.w4 + g * kLdH + 2 * tig;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t bb0 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk);
        const uint32_t bb1 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk + 8);
        mma_bf16(o[m], h1[kk], bb0, bb1);
      }
    }
    __syncwarp();
    // (visibility, confidence) of row `lane`: held by lane 4*(row&7),
    // registers 0,1 (rows 0-7 of an m-tile) or 2,3 (rows 8-15).
    const int src = 4 * (lane & 7);
    const float r00 = __shfl_sync(0xffffffffu, o[0][0], src), r01 = __shfl_sync(0xffffffffu, o[0][1], src);
    const float r02 = __shfl_sync(0xffffffffu, o[0][2], src), r03 = __shfl_sync(0xffffffffu, o[0][3], src);
    const float r10 = __shfl_sync(0xffffffffu, o[1][0], src), r11 = __shfl_sync(0xffffffffu, o[1][1], src);
    const float r12 = __shfl_sync(0xffffffffu, o[1][2], src), r13 = __shfl_sync(0xffffffffu, o[1][3], src);
    const bool hi_rows = (lane & 8) != 0;
    const float ov = lane < 16 ? (hi_rows ? r02 : r00) : (hi_rows ? r12 : r10);
    const float oc = lane < 16 ? (hi_rows ? r03 : r01) : (hi_rows ? r13 : r11);
    const float vis = sigmoidf(ov + s_w.b4[0]);
    const float conf = sigmoidf(oc + s_w.b4[1]);
    const bool retrace = valid && !(conf >= conf_threshold);
    if (valid && !retrace) L.shadow[i] = vis;
    // Re-traced pairs: narrow cones to the front of L.retrace, wide ones to its back.
    const uint32_t mn = __ballot_sync(0xffffffffu, retrace && !wide), mw = __ballot_sync(0xffffffffu, retrace && wide);
    if (mn | mw) {
      uint32_t fn = 0, fw = 0;
      if (lane == 0) {
        if (mn) fn = atomicAdd(L.counters + 3, (uint32_t)__popc(mn));
        if (mw) fw = atomicAdd(L.counters + 4, (uint32_t)__popc(mw));
      }
      fn = __shfl_sync(0xffffffffu, fn, 0);
      fw = __shfl_sync(0xffffffffu, fw, 0);
      const uint32_t below = (1u << lane) - 1u;
      if (retrace && !wide) L.retrace[fn + __popc(mn & below)] = i;
      if (retrace && wide) L.retrace[L.cap - 1u - (fw + __popc(mw & below))] = i;
    }
    evaluated += (uint32_t)__popc(__ballot_sync(0xffffffffu, valid));
    __syncwarp();
  }
  if (lane == 0 && evaluated) atomicAdd(L.counters + 5, evaluated);
}

// FP32 master parameters -> padded BF16 inference layout.
__global__ void pack_weights_kernel(const float* __restrict__ params, MlpWeights* __restrict__ w) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < kMlpHidden * kLd1) {
    const int r = t / kLd1, c = t % kLd1;
    w->w1[t] = to_bf16(c < kMlpIn ? params[kOffW1 + r * kMlpIn + c] : 0.0f);
  }
  if (t < kMlpHidden * kLdH) {
    const int r = t / kLdH, c = t % kLdH;
    w->w2[t] = to_bf16(c < kMlpHidden ? params[kOffW2 + r * kMlpHidden + c] : 0.0f);
    w->w3[t] = to_bf16(c < kMlpHidden ? params[kOffW3 + r * kMlpHidden + c] : 0.0f);
  }
  if (t < kMlpOutPad * kLdH) {
    const int r = t / kLdH, c = t % kLdH;
    w->w4[t] = to_bf16(r < kMlpOut && c < kMlpHidden ? params[kOffW4 + r * kMlpHidden + c] : 0.0f);
  }
  if (t < kMlpHidden) {
    w->b1[t] = params[kOffB1 + t];
    w->b2[t] = params[kOffB2 + t];
    w->b3[t] = params[kOffB3 + t];
  }
  if (t < kMlpOutPad) w->b4[t] = t < kMlpOut ? params[kOffB4 + t] : 0.0f;
}

// Evaluates the inference MLP for validation: BF16 weights and inputs, FP32
// sums one row per thread, and the tensor-core path's bias + bf16x2 GELU.
__global__ void eval_kernel(const MlpWeights* __restrict__ w, const float* __restrict__ X, int n,
                            float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x[kMlpIn], h[kMlpHidden], h2[kMlpHidden];
  for (int k = 0; k < kMlpIn; ++k) x[k] = from_bf16(to_bf16(X[(size_t)i * kMlpIn + k]));
  // bias + GELU of a layer's 64 outputs in pairs, as the tensor-core path forms them
  auto act = [](float* v) {
    for (int j = 0; j < kMlpHidden; j += 2) {
      const uint32_t a = gelu_bf16x2(pack_bf16x2(v[j], v[j + 1]));
      v[j] = __uint_as_float(a << 16);
      v[j + 1] = __uint_as_float(a & 0xFFFF0000u);
    }
  };
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = w->b1[j];
    for (int k = 0; k < kMlpIn; ++k) s += from_bf16(w->w1[j * kLd1 + k]) * x[k];
    h[j] = s;
  }
  act(h);
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = w->b2[j];
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w2[j * kLdH + k]) * h[k];
    h2[j] = s;
  }
  act(h2);
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = w->b3[j];
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w3[j * kLdH + k]) * h2[k];
    h[j] = s;
  }
  act(h);
  for (int j = 0; j < kMlpOut; ++j) {
    float s = 0.0f;
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w4[j * kLdH + k]) * h[k];
    out[(size_t)i * 2 + j] = sigmoidf(s + w->b4[j]);
  }
}

}  // namespace

size_t surrogate_weights_bytes() { return sizeof(MlpWeights); }

cudaError_t launch_pack_surrogate_weights(cudaStream_t s, const float* params, void* weights) {
  pack_weights_kernel<<<(kMlpHidden * kLdH + 255) / 256, 256, 0, s>>>(params, (MlpWeights*)weights);
  return cudaGetLastError();
}

cudaError_t launch_surrogate_eval(cudaStream_t s, const void* weights, const float* X, int n, float* out) {
  eval_kernel<<<(n + 127) / 128, 128, 0, s>>>((const MlpWeights*)weights, X, n, out);
  return cudaGetLastError();
}

cudaError_t launch_surrogate_mlp(cudaStream_t s, const StageParams& p, const PairList& L, const void* weights,
                                 float conf_threshold, bool bf16, int num_sms) {
  const size_t smem = sizeof(MlpSmem);
  auto kernel = bf16 ? mlp_kernel<true> : mlp_kernel<false>;
  // The attribute belongs to the function (on the current device); setting it
  // again costs a driver call per launch, so it is set once per device.
  static std::mutex mu;
  static uint64_t done[2] = {0, 0};  // bit d: set on device d
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 64 || !((done[bf16] >> dev) & 1u)) {
      e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      if (dev < 64) done[bf16] |= 1ull << dev;
    }
  }
  return launch_persistent(kernel, kThreads, smem, s, num_sms, p, L, (const MlpWeights*)weights, conf_threshold);
}

}  // namespace drv
