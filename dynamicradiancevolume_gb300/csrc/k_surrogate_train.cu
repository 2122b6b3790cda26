// k_surrogate_train.cu — training data and training for the visibility
// surrogate (surrogate.cuh): the pair generator runs the plain cone tracer on
// random (cache, shadow block) pairs of the context's current frame; the
// trainer is a fused FP32 forward + backward pass per 64-sample CTA (weights
// and per-sample activations in shared memory, gradients reduced per CTA into
// a slot) followed by an Adam step that sums the slots in a fixed order.
//
// Losses: visibility = binary cross-entropy of sigmoid(out0) against the cone
// visibility; confidence = binary cross-entropy of sigmoid(out1) against
// "|sigmoid(out0) - visibility| < tau".
#include <cmath>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "light_common.cuh"
#include "surrogate.cuh"
#include "voxel_sample.cuh"

namespace drv {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct PairParams {
  LightLaunch ll;
  int block_base[DRV_MAX_LIGHTS + 1];
  int total_blocks;
  VoxelView vox;
  float vol_min[3];
  float voxel_size;
  int max_steps;
  int bf16;
  float casc_min[DRV_MAX_CASCADES][3];
  float casc_cell[DRV_MAX_CASCADES];
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  const float* entries;
  int stride_floats;
  uint64_t seed;
  int n_pairs;
  float* features;
  float* targets;
  int feature_set;
};

__device__ __forceinline__ void vpl_normal(const void* vpls, int bf16, int i, float& nx, float& ny, float& nz) {
  if (bf16) {
    const DrvVPLBF16& v = static_cast<const DrvVPLBF16*>(vpls)[i];
    nx = from_bf16(v.normal_bf16[0]);
    ny = from_bf16(v.normal_bf16[1]);
    nz = from_bf16(v.normal_bf16[2]);
  } else {
    const DrvVPL& v = static_cast<const DrvVPL*>(vpls)[i];
    nx = v.normal[0];
    ny = v.normal[1];
    nz = v.normal[2];
  }
}

__global__ void __launch_bounds__(128) pairs_kernel(PairParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_pairs) return;
  const uint32_t count = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  float* f = p.features + (size_t)i * kMlpIn;
  if (count == 0 || p.total_blocks == 0) {
    for (int k = 0; k < kMlpIn; ++k) f[k] = k == kOneInput ? 1.0f : 0.0f;
    p.targets[i] = 1.0f;
    return;
  }
  uint32_t cache;
  int b;
  if (p.seed == DRV_SURROGATE_ENUMERATE) {  // pair i = (cache i / blocks, block i % blocks)
    cache = (uint32_t)(i / p.total_blocks);
    b = i % p.total_blocks;
    if (cache >= count) {
      for (int k = 0; k < kMlpIn; ++k) f[k] = k == kOneInput ? 1.0f : 0.0f;
      p.targets[i] = 1.0f;
      return;
    }
  } else {
    // Random pairs that can contribute (positive flux, facing the cache): the
    // light stage never asks for the visibility of the others.
    for (int attempt = 0; attempt < 64; ++attempt) {
      const uint64_t h = mix64(p.seed * 0x9E3779B97F4A7C15ull + (uint64_t)i * 64u + (uint64_t)attempt);
      cache = (uint32_t)(h % count);
      b = (int)((h >> 32) % (uint64_t)p.total_blocks);
      int l = 0;
      while (b >= p.block_base[l + 1]) ++l;
      const LightArgs& la = p.ll.lights[l];
      const int lb = b - p.block_base[l];
      const float* e = p.entries + (size_t)cache * p.stride_floats;
      float ex, ey, ez;
      if (p.bf16) {
        const uint32_t key = __float_as_uint(e[0]);
        const int c = (int)(key >> 27);
        ex = __fadd_rn(__fmul_rn((float)(key & 511u), p.casc_cell[c]), p.casc_min[c][0]);
        ey = __fadd_rn(__fmul_rn((float)((key >> 9) & 511u), p.casc_cell[c]), p.casc_min[c][1]);
        ez = __fadd_rn(__fmul_rn((float)((key >> 18) & 511u), p.casc_cell[c]), p.casc_min[c][2]);
      } else {
        ex = e[0];
        ey = e[1];
        ez = e[2];
      }
      bool live = false;
      for (int j = 0; j < la.interval && !live; ++j) {
        const VplData v = p.bf16 ? load_vpl<true>(la.vpls, lb * la.interval + j)
                                 : load_vpl<false>(la.vpls, lb * la.interval + j);
        live = contributes(v, transfer(v, ex, ey, ez));
      }
      if (live) break;
    }
  }
  int l = 0;
  while (b >= p.block_base[l + 1]) ++l;
  const LightArgs& la = p.ll.lights[l];
  const int lb = b - p.block_base[l];
  const float* entry = p.entries + (size_t)cache * p.stride_floats;
  float cx, cy, cz;
  if (p.bf16) {
    const uint32_t key = __float_as_uint(entry[0]);
    const int c = (int)(key >> 27);
    cx = __fadd_rn(__fmul_rn((float)(key & 511u), p.casc_cell[c]), p.casc_min[c][0]);
    cy = __fadd_rn(__fmul_rn((float)((key >> 9) & 511u), p.casc_cell[c]), p.casc_min[c][1]);
    cz = __fadd_rn(__fmul_rn((float)((key >> 18) & 511u), p.casc_cell[c]), p.casc_min[c][2]);
  } else {
    cx = entry[0];
    cy = entry[1];
    cz = entry[2];
  }
  const float4 cone = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
  float nx, ny, nz;
  vpl_normal(la.vpls, p.bf16, lb * la.interval, nx, ny, nz);
  const float inv_extent = 1.0f / (p.voxel_size * p.vox.N);
  if (p.feature_set == kFeatureCone8)
    pair_features<kFeatureCone8>(p.vox, inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x, cone.y,
                                 cone.z, nx, ny, nz, cone.w, f);
  else if (p.feature_set == kFeatureCone4)
    pair_features<kFeatureCone4>(p.vox, inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x, cone.y,
                                 cone.z, nx, ny, nz, cone.w, f);
  else
    pair_features<kFeatureSegment8>(p.vox, inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x,
                                    cone.y, cone.z, nx, ny, nz, cone.w, f);
  const float vx = (cx - p.vol_min[0]) * inv_extent, vy = (cy - p.vol_min[1]) * inv_extent,
              vz = (cz - p.vol_min[2]) * inv_extent;
  p.targets[i] = cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, cone.x, cone.y, cone.z, cone.w);
}

// ---------------------------------------------------------------- training
constexpr int kTB = 64;      // samples per CTA
constexpr int kLd = 65;      // padded per-sample row stride (conflict-free column access)

struct TrainSmem {
  float w[kMlpParams];
  float x[kTB * (kMlpIn + 1)];
  float z1[kTB * kLd], z2[kTB * kLd], z3[kTB * kLd];  // pre-activations
  float a1[kTB * kLd], a2[kTB * kLd], a3[kTB * kLd];  // GELU(z)
  float d1[kTB * kLd], d2[kTB * kLd], d3[kTB * kLd];  // dLoss/dz
  float g4[kTB * 2];
  float loss[kTB * 2];
};

// One 64-sample chunk per CTA: forward, backward, per-CTA gradient slot.
__global__ void __launch_bounds__(kTB) train_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                                    const float* __restrict__ Y, int n, float conf_tau,
                                                    float* __restrict__ grad_slots, float* __restrict__ loss_slots) {
  extern __shared__ float smem_raw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
  const int t = threadIdx.x;
  for (int i = t; i < kMlpParams; i += kTB) S.w[i] = params[i];
  const int sample = blockIdx.x * kTB + t;
  const bool valid = sample < n;
  float* xr = S.x + t * (kMlpIn + 1);
  for (int i = 0; i < kMlpIn; ++i) xr[i] = valid ? X[(size_t)sample * kMlpIn + i] : 0.0f;
  __syncthreads();
  // forward
  const float* W1 = S.w + kOffW1;
  const float* W2 = S.w + kOffW2;
  const float* W3 = S.w + kOffW3;
  const float* W4 = S.w + kOffW4;
  float* z1 = S.z1 + t * kLd;
  float* z2 = S.z2 + t * kLd;
  float* z3 = S.z3 + t * kLd;
  float* a1 = S.a1 + t * kLd;
  float* a2 = S.a2 + t * kLd;
  float* a3 = S.a3 + t * kLd;
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = S.w[kOffB1 + j];
    for (int i = 0; i < kMlpIn; ++i) s += W1[j * kMlpIn + i] * xr[i];
    z1[j] = s;
    a1[j] = gelu(s);
  }
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = S.w[kOffB2 + j];
    for (int i = 0; i < kMlpHidden; ++i) s += W2[j * kMlpHidden + i] * a1[i];
    z2[j] = s;
    a2[j] = gelu(s);
  }
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = S.w[kOffB3 + j];
    for (int i = 0; i < kMlpHidden; ++i) s += W3[j * kMlpHidden + i] * a2[i];
    z3[j] = s;
    a3[j] = gelu(s);
  }
  float o[2];
  for (int j = 0; j < 2; ++j) {
    float s = S.w[kOffB4 + j];
    for (int i = 0; i < kMlpHidden; ++i) s += W4[j * kMlpHidden + i] * a3[i];
    o[j] = s;
  }
  // losses and output gradients (mean over the whole batch is applied in Adam)
  const float y = valid ? Y[sample] : 0.0f;
  const float v = sigmoidf(o[0]), c = sigmoidf(o[1]);
  const float c_target = fabsf(v - y) < conf_tau ? 1.0f : 0.0f;
  float g0 = valid ? v - y : 0.0f, g1 = valid ? c - c_target : 0.0f;
  S.g4[t * 2] = g0;
  S.g4[t * 2 + 1] = g1;
  const float eps = 1e-7f;
  S.loss[t * 2] = valid ? -(y * __logf(v + eps) + (1.0f - y) * __logf(1.0f - v + eps)) : 0.0f;
  S.loss[t * 2 + 1] = valid ? -(c_target * __logf(c + eps) + (1.0f - c_target) * __logf(1.0f - c + eps)) : 0.0f;
  // backward
  float* d3 = S.d3 + t * kLd;
  float* d2 = S.d2 + t * kLd;
  float* d1 = S.d1 + t * kLd;
  for (int i = 0; i < kMlpHidden; ++i)
    d3[i] = (W4[i] * g0 + W4[kMlpHidden + i] * g1) * gelu_grad(z3[i]);
  for (int i = 0; i < kMlpHidden; ++i) {
    float s = 0.0f;
    for (int j = 0; j < kMlpHidden; ++j) s += W3[j * kMlpHidden + i] * d3[j];
    d2[i] = s * gelu_grad(z2[i]);
  }
  for (int i = 0; i < kMlpHidden; ++i) {
    float s = 0.0f;
    for (int j = 0; j < kMlpHidden; ++j) s += W2[j * kMlpHidden + i] * d2[j];
    d1[i] = s * gelu_grad(z1[i]);
  }
  __syncthreads();
  // per-CTA gradients: each thread owns a strided set of parameters and sums
  // over the 64 samples in order.
  float* slot = grad_slots + (size_t)blockIdx.x * kMlpParams;
  for (int p = t; p < kMlpParams; p += kTB) {
    float s = 0.0f;
    if (p < kOffB1) {
      const int j = p / kMlpIn, i = p % kMlpIn;
      for (int q = 0; q < kTB; ++q) s += S.d1[q * kLd + j] * S.x[q * (kMlpIn + 1) + i];
    } else if (p < kOffW2) {
      const int j = p - kOffB1;
      for (int q = 0; q < kTB; ++q) s += S.d1[q * kLd + j];
    } else if (p < kOffB2) {
      const int j = (p - kOffW2) / kMlpHidden, i = (p - kOffW2) % kMlpHidden;
      for (int q = 0; q < kTB; ++q) s += S.d2[q * kLd + j] * S.a1[q * kLd + i];
    } else if (p < kOffW3) {
      const int j = p - kOffB2;
      for (int q = 0; q < kTB; ++q) s += S.d2[q * kLd + j];
    } else if (p < kOffB3) {
      const int j = (p - kOffW3) / kMlpHidden, i = (p - kOffW3) % kMlpHidden;
      for (int q = 0; q < kTB; ++q) s += S.d3[q * kLd + j] * S.a2[q * kLd + i];
    } else if (p < kOffW4) {
      const int j = p - kOffB3;
      for (int q = 0; q < kTB; ++q) s += S.d3[q * kLd + j];
    } else if (p < kOffB4) {
      const int j = (p - kOffW4) / kMlpHidden, i = (p - kOffW4) % kMlpHidden;
      for (int q = 0; q < kTB; ++q) s += S.g4[q * 2 + j] * S.a3[q * kLd + i];
    } else {
      const int j = p - kOffB4;
      for (int q = 0; q < kTB; ++q) s += S.g4[q * 2 + j];
    }
    slot[p] = s;
  }
  if (t < 2) {
    float s = 0.0f;
    for (int q = 0; q < kTB; ++q) s += S.loss[q * 2 + t];
    loss_slots[blockIdx.x * 2 + t] = s;
  }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters; the gradient is the
// fixed-order sum of the CTA slots divided by the batch size.
__global__ void __launch_bounds__(256) adam_kernel(float* __restrict__ params, float* __restrict__ m,
                                                   float* __restrict__ v, const float* __restrict__ grad_slots,
                                                   int n_slots, float inv_batch, float lr, float beta1, float beta2,
                                                   float eps, float bc1, float bc2, float weight_decay) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  float g = 0.0f;
  for (int s = 0; s < n_slots; ++s) g += grad_slots[(size_t)s * kMlpParams + p];
  g *= inv_batch;
  const float mm = beta1 * m[p] + (1.0f - beta1) * g;
  const float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
  m[p] = mm;
  v[p] = vv;
  const float update = (mm / bc1) / (sqrtf(vv / bc2) + eps);
  params[p] -= lr * (update + weight_decay * params[p]);
}

__global__ void __launch_bounds__(256) loss_sum_kernel(const float* __restrict__ loss_slots, int n_slots,
                                                       float* __restrict__ out) {
  __shared__ float s0[256], s1[256];
  float a = 0.0f, b = 0.0f;
  for (int i = threadIdx.x; i < n_slots; i += 256) {
    a += loss_slots[2 * i];
    b += loss_slots[2 * i + 1];
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s0[threadIdx.x] += s0[threadIdx.x + o];
      s1[threadIdx.x] += s1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s0[0];
    out[1] = s1[0];
  }
}

}  // namespace

cudaError_t launch_surrogate_pairs(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol,
                                   const LightLaunch& ll, const DrvCacheCounter* counter, const void* entries,
                                   uint32_t entry_stride, const VoxelInputs& vox, uint64_t seed, int n_pairs,
                                   float* features, float* targets, int feature_set) {
  PairParams p;
  p.ll = ll;
  int base = 0;
  for (int l = 0; l < ll.n_lights; ++l) {
    p.block_base[l] = base;
    base += ll.lights[l].n_vpls / ll.lights[l].interval;
  }
  for (int l = ll.n_lights; l <= DRV_MAX_LIGHTS; ++l) p.block_base[l] = base;
  p.total_blocks = base;
  p.vox = make_voxel_view(cfg, vox);
  for (int i = 0; i < 3; ++i) p.vol_min[i] = vol.volume_world_min[i];
  p.voxel_size = vol.voxel_size_in_world;
  p.max_steps = cfg.max_cone_steps;
  p.bf16 = cfg.precision == DRV_PRECISION_BF16;
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) {
    p.casc_cell[c] = vol.cascades[c].world_voxel_size;
    for (int i = 0; i < 3; ++i) p.casc_min[c][i] = vol.cascades[c].min[i];
  }
  p.counter = counter;
  p.max_caches = cfg.max_caches;
  p.entries = (const float*)entries;
  p.stride_floats = (int)(entry_stride / 4);
  p.seed = seed;
  p.n_pairs = n_pairs;
  p.features = features;
  p.targets = targets;
  p.feature_set = feature_set;
  pairs_kernel<<<(n_pairs + 127) / 128, 128, 0, s>>>(p);
  return cudaGetLastError();
}

size_t surrogate_train_scratch_floats(int n) {
  const size_t slots = (size_t)(n + kTB - 1) / kTB;
  return slots * kMlpParams + slots * 2 + 2;
}

cudaError_t launch_surrogate_train_step(cudaStream_t s, const float* X, const float* Y, int n, float* params,
                                        float* m, float* v, float* scratch, int step, float lr, float conf_tau,
                                        float weight_decay, float* loss_out) {
  const int slots = (n + kTB - 1) / kTB;
  float* grads = scratch;
  float* losses = scratch + (size_t)slots * kMlpParams;
  const size_t smem = sizeof(TrainSmem);
  cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  train_kernel<<<slots, kTB, smem, s>>>(params, X, Y, n, conf_tau, grads, losses);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(params, m, v, grads, slots, 1.0f / (float)n, lr, b1, b2,
                                                      1e-8f, bc1, bc2, weight_decay);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (loss_out) {
    loss_sum_kernel<<<1, 256, 0, s>>>(losses, slots, loss_out);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace drv
