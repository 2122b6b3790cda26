// k_light_surrogate.cu — the cache-lighting stage with the learned visibility
// surrogate in place of the indirect-shadow cone (cacheLightingRSM.comp:167-232).
//
// Same work decomposition as k_light.cu (a warp owns a (cache, chunk) unit,
// lanes take shadow blocks round-robin, ticketed chunk reduction). Per warp
// iteration the 32 lanes' pairs form a 32-row batch:
//  1. each lane computes its pair's 32 input features (surrogate.cuh) and
//     stores them as BF16 in the warp's shared-memory tile;
//  2. the MLP runs on tensor cores with mma.sync m16n8k16 (BF16 in, FP32
//     accumulate): the accumulator fragment of one layer is, after bias and
//     GELU, exactly the A fragment of the next, so activations never leave
//     registers; weights are read from shared memory (rows padded so the
//     fragment loads are bank-conflict free);
//  3. each lane gets its (visibility, confidence) back by shuffles; confident
//     pairs use sigmoid(visibility), the others are appended to a per-warp
//     queue that is cone-traced 32 pairs at a time, so a single uncertain pair
//     never holds a whole warp in the cone loop;
//  4. the SH gather is the plain stage's (accumulate_vpl).
#include <cmath>

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

struct SurrogateParams {
  LightLaunch ll;
  int block_base[DRV_MAX_LIGHTS + 1];
  int total_blocks;
  int n_chunks;
  int chunk_blocks;
  VoxelView vox;
  float vol_min[3];
  float voxel_size;
  int max_steps;
  float casc_min[DRV_MAX_CASCADES][3];
  float casc_cell[DRV_MAX_CASCADES];
  const DrvCacheCounter* counter;
  uint32_t max_caches;
  float* entries;
  int stride_floats;
  float* scratch;
  uint32_t* tickets;
  const MlpWeights* weights;
  float conf_threshold;
  uint32_t* fallback_count;  // optional: [0] re-traced pairs, [1] pairs the MLP evaluated
  float ev[5];
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
  const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
  return a | (b << 16);
}

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

// One hidden layer for both 16-row m-tiles: in = A fragments [2][KSTEPS][4],
// out = A fragments of the next layer [2][4][4] after bias + GELU.
template <int KSTEPS, int LD>
__device__ __forceinline__ void hidden_layer(const uint32_t (&in)[2][KSTEPS][4], const uint16_t* w, const float* bias,
                                             uint32_t (&out)[2][4][4], int g, int tig) {
#pragma unroll
  for (int j = 0; j < kMlpHidden / 8; ++j) {
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    const uint16_t* wr = w + (8 * j + g) * LD + 2 * tig;
#pragma unroll
    for (int kk = 0; kk < KSTEPS; ++kk) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk + 8);
      mma_bf16(acc[0], in[0][kk], b0, b1);
      mma_bf16(acc[1], in[1][kk], b0, b1);
    }
    const float bl = bias[8 * j + 2 * tig], bh = bias[8 * j + 2 * tig + 1];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const uint32_t lo = pack_bf16x2(gelu_fast(acc[m][0] + bl), gelu_fast(acc[m][1] + bh));
      const uint32_t hi = pack_bf16x2(gelu_fast(acc[m][2] + bl), gelu_fast(acc[m][3] + bh));
      // n-tile j feeds k-step j/2 of the next layer: even tiles are its low
      // k half (regs 0,1), odd tiles its high half (regs 2,3).
      out[m][j >> 1][(j & 1) * 2 + 0] = lo;
      out[m][j >> 1][(j & 1) * 2 + 1] = hi;
    }
  }
}

// Shadow block b (global index) -> light index.
__device__ __forceinline__ int block_light(const SurrogateParams& p, int b) {
  int l = 0;
  while (b >= p.block_base[l + 1]) ++l;
  return l;
}

// SH gather of the contributing VPLs of shadow block b with the given
// shadowing; acc is this thread's column of a [NK*3][kThreads] shared array.
template <int NK, bool BF16>
__device__ __forceinline__ void gather_block(const SurrogateParams& p, float* acc, int b, float cx, float cy,
                                             float cz, float shadowing) {
  const int l = block_light(p, b);
  const LightArgs& la = p.ll.lights[l];
  const int lb = b - p.block_base[l];
  for (int j = 0; j < la.interval; ++j) {
    const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
    const Transfer t = transfer(v, cx, cy, cz);
    if (contributes(v, t)) accumulate<NK, false>(p.ev, acc, nullptr, kThreads, v, t, shadowing);
  }
}

// Dynamic shared memory of one CTA (about 51 KB with SH2).
template <int NK>
struct __align__(16) SurrogateSmem {
  MlpWeights w;
  uint16_t x[kWarps][32 * kLd1];  // per-warp BF16 feature tile, 80-byte rows
  int queue[kWarps][64];          // per-warp re-trace queue
  int live[kWarps][64];           // per-warp queue of blocks that can contribute
  float acc[NK * 3 * kThreads];   // per-thread SH partial sums, column per thread
};

template <int NK, bool BF16>
__global__ void __launch_bounds__(kThreads) light_surrogate_kernel(SurrogateParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SurrogateSmem<NK>& S = *reinterpret_cast<SurrogateSmem<NK>*>(smem_raw);
  MlpWeights& s_w = S.w;
  auto& s_x = S.x;
  auto& s_queue = S.queue;
  float* s_acc = S.acc;
  {
    const uint4* src = reinterpret_cast<const uint4*>(p.weights);
    uint4* dst = reinterpret_cast<uint4*>(&s_w);
    for (int i = threadIdx.x; i < (int)(sizeof(MlpWeights) / 16); i += kThreads) dst[i] = src[i];
  }
  __syncthreads();
  const uint32_t count = min((uint32_t)max(p.counter->total_light_cache_count, 0), p.max_caches);
  const uint32_t n_units = count * (uint32_t)p.n_chunks;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  const uint32_t warps = gridDim.x * kWarps;
  uint16_t* xt = s_x[warp];
  int* queue = s_queue[warp];
  const float inv_extent = 1.0f / (p.voxel_size * p.vox.N);
  uint32_t retraced = 0, evaluated = 0;
  for (uint32_t u = blockIdx.x * kWarps + warp; u < n_units; u += warps) {
    const uint32_t cache = u / (uint32_t)p.n_chunks;
    const int chunk = (int)(u % (uint32_t)p.n_chunks);
    float* entry = p.entries + (size_t)cache * p.stride_floats;
    float cx, cy, cz;
    if (BF16) {
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
    const float vx = (cx - p.vol_min[0]) * inv_extent, vy = (cy - p.vol_min[1]) * inv_extent,
                vz = (cz - p.vol_min[2]) * inv_extent;
    float* acc = s_acc + threadIdx.x;
#pragma unroll
    for (int k = 0; k < NK * 3; ++k) acc[k * kThreads] = 0.0f;
    int* live = S.live[warp];
    int queued = 0, n_live = 0;
    // Runs the MLP on the n (<= 32) live blocks at live[first ...]: confident
    // pairs are gathered with the predicted visibility, the others queued for
    // the cone, which runs once 32 are waiting.
    auto mlp_batch = [&](int first, int n) {
      const bool valid = lane < n;
      evaluated += n;
      const int b = valid ? live[first + lane] : 0;
      __syncwarp();
      float f[kMlpIn];
      if (valid) {
        const int l = block_light(p, b);
        const LightArgs& la = p.ll.lights[l];
        const int lb = b - p.block_base[l];
        const float4 cone = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
        const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval);
        surrogate_features(p.vox, inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x, cone.y,
                           cone.z, v.nx, v.ny, v.nz, cone.w, f);
      } else {
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) f[i] = 0.0f;
      }
      uint32_t* row = reinterpret_cast<uint32_t*>(xt + lane * kLd1);
#pragma unroll
      for (int i = 0; i < kMlpIn / 2; ++i) row[i] = pack_bf16x2(f[2 * i], f[2 * i + 1]);
      __syncwarp();
      uint32_t a1[2][2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int kk = 0; kk < 2; ++kk)
          ldmatrix_x4(a1[m][kk], xt + (16 * m + (lane & 7) + ((lane >> 3) & 1) * 8) * kLd1 + 16 * kk +
                                     ((lane >> 4) & 1) * 8);
      __syncwarp();
      uint32_t h1[2][4][4], h2[2][4][4];
      hidden_layer<2, kLd1>(a1, s_w.w1, s_w.b1, h1, g, tig);
      hidden_layer<4, kLdH>(h1, s_w.w2, s_w.b2, h2, g, tig);
      hidden_layer<4, kLdH>(h2, s_w.w3, s_w.b3, h1, g, tig);
      float o[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      {
        const uint16_t* wr = s_w.w4 + g * kLdH + 2 * tig;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint32_t bb0 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk);
          const uint32_t bb1 = *reinterpret_cast<const uint32_t*>(wr + 16 * kk + 8);
          mma_bf16(o[0], h1[0][kk], bb0, bb1);
          mma_bf16(o[1], h1[1][kk], bb0, bb1);
        }
      }
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
      const bool retrace = valid && !(conf >= p.conf_threshold);
      if (valid && !retrace) gather_block<NK, BF16>(p, acc, b, cx, cy, cz, vis);
      const uint32_t mask = __ballot_sync(0xffffffffu, retrace);
      if (retrace) queue[queued + __popc(mask & ((1u << lane) - 1u))] = b;
      queued += __popc(mask);
      __syncwarp();
      if (queued >= 32) {
        const int qb = queue[queued - 32 + lane];
        const int l = block_light(p, qb);
        const float4 c = __ldg(reinterpret_cast<const float4*>(p.ll.lights[l].cones) + (qb - p.block_base[l]));
        const float sh = cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, c.x, c.y, c.z, c.w);
        gather_block<NK, BF16>(p, acc, qb, cx, cy, cz, sh);
        queued -= 32;
        retraced += 32;
        __syncwarp();
      }
    };
    const int b0 = chunk * p.chunk_blocks, b1 = min(b0 + p.chunk_blocks, p.total_blocks);
    for (int base = b0; base < b1; base += 32) {
      const int b = base + lane;
      bool is_live = false;
      if (b < b1) {
        const int l = block_light(p, b);
        const LightArgs& la = p.ll.lights[l];
        const int lb = b - p.block_base[l];
        for (int j = 0; j < la.interval && !is_live; ++j) {
          const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval + j);
          is_live = contributes(v, transfer(v, cx, cy, cz));
        }
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, is_live);
      if (is_live) live[n_live + __popc(mask & ((1u << lane) - 1u))] = b;
      n_live += __popc(mask);
      __syncwarp();
      if (n_live >= 32) {
        mlp_batch(n_live - 32, 32);
        n_live -= 32;
      }
    }
    if (n_live > 0) mlp_batch(0, n_live);
    if (queued > 0) {
      if (lane < queued) {
        const int qb = queue[lane];
        const int l = block_light(p, qb);
        const float4 c = __ldg(reinterpret_cast<const float4*>(p.ll.lights[l].cones) + (qb - p.block_base[l]));
        const float sh = cone_shadow(p.vox, p.voxel_size, p.max_steps, cx, cy, cz, vx, vy, vz, c.x, c.y, c.z, c.w);
        gather_block<NK, BF16>(p, acc, qb, cx, cy, cz, sh);
      }
      retraced += queued;
      __syncwarp();
    }
    // warp reduction + chunk combination (as k_light.cu)
    float mine = 0.0f;
#pragma unroll
    for (int k = 0; k < NK * 3; ++k) {
      float v = acc[k * kThreads];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == k) mine = v;
    }
    auto add = [&](float v) {
      if (BF16) {
        uint16_t* sh = reinterpret_cast<uint16_t*>(entry + 1);
        sh[lane] = to_bf16(from_bf16(sh[lane]) + v);
      } else {
        entry[sh_offset(lane / 3, lane % 3)] += v;
      }
    };
    if (p.n_chunks == 1) {
      if (lane < NK * 3) add(mine);
      continue;
    }
    if (lane < NK * 3) p.scratch[(size_t)u * (NK * 3) + lane] = mine;
    __threadfence();
    uint32_t last = 0;
    if (lane == 0) last = atomicAdd(p.tickets + cache, 1u) == (uint32_t)p.n_chunks - 1u;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence();
      if (lane < NK * 3) {
        const volatile float* sb = p.scratch + (size_t)cache * p.n_chunks * (NK * 3);
        float v = 0.0f;
        for (int c = 0; c < p.n_chunks; ++c) v += sb[c * (NK * 3) + lane];
        add(v);
      }
      if (lane == 0) p.tickets[cache] = 0u;
    }
  }
  if (p.fallback_count && lane == 0) {
    if (retraced) atomicAdd(p.fallback_count, retraced);
    if (evaluated) atomicAdd(p.fallback_count + 1, evaluated);
  }
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

// Evaluates the inference MLP (BF16 weights, same arithmetic as the light
// kernel's tensor-core path but one row per thread in FP32) for validation.
__global__ void eval_kernel(const MlpWeights* __restrict__ w, const float* __restrict__ X, int n,
                            float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x[kMlpIn], h[kMlpHidden], h2[kMlpHidden];
  for (int k = 0; k < kMlpIn; ++k) x[k] = from_bf16(to_bf16(X[(size_t)i * kMlpIn + k]));
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = 0.0f;
    for (int k = 0; k < kMlpIn; ++k) s += from_bf16(w->w1[j * kLd1 + k]) * x[k];
    h[j] = from_bf16(to_bf16(gelu_fast(s + w->b1[j])));
  }
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = 0.0f;
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w2[j * kLdH + k]) * h[k];
    h2[j] = from_bf16(to_bf16(gelu_fast(s + w->b2[j])));
  }
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = 0.0f;
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w3[j * kLdH + k]) * h2[k];
    h[j] = from_bf16(to_bf16(gelu_fast(s + w->b3[j])));
  }
  for (int j = 0; j < kMlpOut; ++j) {
    float s = 0.0f;
    for (int k = 0; k < kMlpHidden; ++k) s += from_bf16(w->w4[j * kLdH + k]) * h[k];
    out[(size_t)i * 2 + j] = sigmoidf(s + w->b4[j]);
  }
}

template <int NK, bool BF16>
cudaError_t launch_sur(cudaStream_t s, const SurrogateParams& p, int num_sms) {
  const int smem = (int)sizeof(SurrogateSmem<NK>);
  cudaError_t e = cudaFuncSetAttribute(light_surrogate_kernel<NK, BF16>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, light_surrogate_kernel<NK, BF16>, kThreads, smem);
  light_surrogate_kernel<NK, BF16><<<num_sms * (per_sm < 1 ? 1 : per_sm), kThreads, smem, s>>>(p);
  return cudaGetLastError();
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

cudaError_t launch_light_surrogate(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol,
                                   const LightLaunch& ll, const DrvCacheCounter* counter, void* entries,
                                   uint32_t entry_stride, const uint8_t* corners, const void* mips,
                                   const size_t* mip_offsets, float* scratch, uint32_t* tickets, const void* weights,
                                   uint32_t* fallback_count, int num_sms) {
  SurrogateParams p;
  p.ll = ll;
  int base = 0;
  for (int l = 0; l < ll.n_lights; ++l) {
    p.block_base[l] = base;
    base += ll.lights[l].n_vpls / ll.lights[l].interval;
  }
  for (int l = ll.n_lights; l <= DRV_MAX_LIGHTS; ++l) p.block_base[l] = base;
  p.total_blocks = base;
  p.n_chunks = light_chunks(base);
  p.chunk_blocks = (base + p.n_chunks - 1) / p.n_chunks;
  int L = 0;
  while ((1 << (L + 1)) <= cfg.voxel_res) ++L;
  p.vox.corners = corners;
  p.vox.mips = mips;
  for (int i = 0; i < 16; ++i) p.vox.off[i] = (uint32_t)(i < kMaxVoxelLevels ? mip_offsets[i] : 0);
  p.vox.N = cfg.voxel_res;
  p.vox.log2n = L;
  p.vox.max_level = L;
  const bool bf16 = cfg.precision == DRV_PRECISION_BF16;
  p.vox.half_mips = bf16;
  for (int i = 0; i < 3; ++i) p.vol_min[i] = vol.volume_world_min[i];
  p.voxel_size = vol.voxel_size_in_world;
  p.max_steps = cfg.max_cone_steps;
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) {
    p.casc_cell[c] = vol.cascades[c].world_voxel_size;
    for (int i = 0; i < 3; ++i) p.casc_min[c][i] = vol.cascades[c].min[i];
  }
  p.counter = counter;
  p.max_caches = cfg.max_caches;
  p.entries = (float*)entries;
  p.stride_floats = (int)(entry_stride / 4);
  p.scratch = scratch;
  p.tickets = tickets;
  p.weights = (const MlpWeights*)weights;
  p.conf_threshold = cfg.surrogate_conf_threshold;
  p.fallback_count = fallback_count;
  const double kPi = 3.14159265358979323846;
  p.ev[0] = (float)(1.0 / (2.0 * std::sqrt(kPi)));
  p.ev[1] = (float)(std::sqrt(3.0) / (2.0 * std::sqrt(kPi)));
  p.ev[2] = (float)std::sqrt(15.0 / (4.0 * kPi));
  p.ev[3] = (float)std::sqrt(5.0 / (16.0 * kPi));
  p.ev[4] = (float)std::sqrt(15.0 / (16.0 * kPi));
  if (cfg.sh_order == 2) return bf16 ? launch_sur<9, true>(s, p, num_sms) : launch_sur<9, false>(s, p, num_sms);
  return bf16 ? launch_sur<4, true>(s, p, num_sms) : launch_sur<4, false>(s, p, num_sms);
}

}  // namespace drv
