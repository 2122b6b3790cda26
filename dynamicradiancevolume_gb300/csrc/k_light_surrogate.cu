// k_light_surrogate.cu — the learned visibility surrogate in place of the
// indirect-shadow cone (cacheLightingRSM.comp:167-232), as the middle pass of
// the split light stage (k_light.cu), on the fifth-generation tensor cores.
//
// After the cull has listed the (cache, shadow block) pairs that can
// contribute, mlp_tc_kernel takes them 128 at a time (one tile per CTA
// iteration, persistent grid, four CTAs per SM):
//  1. each thread computes its pair's 32 input features (surrogate.cuh) and
//     stores them as BF16 in its row of the CTA's A tile in shared memory;
//  2. one thread issues the layer's tcgen05.mma (M = 128 pairs, N = 64
//     hidden units, K = 16 per instruction, BF16 in, FP32 accumulators in
//     tensor memory) and commits it to an mbarrier;
//  3. every thread reads its row of the accumulators back with tcgen05.ld,
//     applies GELU on bf16x2 pairs and writes the activations over its row
//     of the A tile: the next layer's A operand. Four layers; the fourth has
//     N = 16 (the two outputs and zero rows);
//  4. confident pairs store sigmoid(visibility) as their shadowing; the
//     others are marked (cls 0) for the classify pass, which orders them by
//     cone class like every pair of the plain stage, and cone_kernel traces
//     them.
// The weights (27 KB of BF16 B operands) are staged once per CTA by one bulk
// asynchronous copy (cp.async.bulk, completion on an mbarrier).
//
// Arithmetic folded into the packed weights: the biases ride on a constant-1
// input column (input 31 of layer 1; column 64 of layers 2-4, whose K is 80),
// and GELU x sigmoid(1.702 x) = (1/1.702) y (1 + tanh(y)) with y = 0.851 x, so
// each layer's weights carry the 0.851 of its own activation and the 1/1.702
// of the previous one: an activation is then y + y tanh(y), two bf16x2
// operations (tanh.approx, fma) per pair of values.
//
// Every wait (the weights' copy, each layer's commit) is bounded by a cycle
// count; a wait that runs out latches DRV_DEVERR_TIMEOUT, the CTA waits once
// more (bounded) for what it issued, frees its tensor memory and returns.
#include <cmath>
#include <mutex>

#include "drv_device.cuh"
#include "drv_internal.h"
#include "light_common.cuh"
#include "surrogate.cuh"
#include "voxel_sample.cuh"

namespace drv {
namespace {

constexpr int kThreads = 128;             // one thread per row of the M = 128 tile
constexpr int kK1 = kMlpIn;               // layer-1 K: 31 features + the constant 1
constexpr int kKH = kMlpHidden + 16;      // layers 2-4 K: 64 activations, the constant 1, 15 zeros
constexpr int kN4 = 16;                   // layer-4 N: 2 outputs, padded to the smallest N of an M = 128 MMA
constexpr int kTmemCols = 64;             // FP32 accumulator columns (N of layers 1-3)
constexpr float kGeluHalfK = 0.851f;      // 1.702 / 2
constexpr unsigned long long kWaitCycles = 2000000000ull;  // about one second at 2 GHz
constexpr unsigned long long kTestWaitCycles = 20000000ull;

// Shared-memory image of a [R][K] BF16 operand, K-major, no swizzle (the
// canonical layout of a tcgen05 shared-memory descriptor): 8 rows x 16 bytes
// "core matrices" stored as 128 contiguous bytes; core matrices adjacent in
// K are 128 B apart (the leading-dimension byte offset) and 8-row groups
// (K / 8) * 128 B apart (the stride-dimension byte offset).
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

constexpr uint32_t kW1Off = 0;
constexpr uint32_t kW2Off = kW1Off + kMlpHidden * kK1 * 2;  // 4096
constexpr uint32_t kW3Off = kW2Off + kMlpHidden * kKH * 2;  // 14336
constexpr uint32_t kW4Off = kW3Off + kMlpHidden * kKH * 2;  // 24576
constexpr uint32_t kWBytes = kW4Off + kN4 * kKH * 2;        // 27136
constexpr uint32_t kABytes = kThreads * kKH * 2;            // 20480

struct __align__(128) TcSmem {
  uint8_t w[kWBytes];
  uint8_t a[kABytes];
  uint64_t bar_w;    // the weights' bulk copy
  uint64_t bar_mma;  // each layer's commit
  uint32_t tmem;     // tensor-memory base address (written by tcgen05.alloc)
};

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits until the barrier's phase of this parity has completed, at most
// `cycles` SM clocks; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned long long cycles) {
  const unsigned long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if ((unsigned long long)(clock64() - t0) > cycles) return false;
  return true;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 64-bit shared-memory matrix descriptor: start address, leading- and
// stride-dimension byte offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulators (bits 4-5 = 1), A and
// B BF16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28 (M = 128).
__host__ __device__ constexpr uint32_t instr_desc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Row (TMEM lane) of this thread, 64 consecutive FP32 columns.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
      "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
      "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float& a, float& b) {
  uint32_t r0, r1;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  a = __uint_as_float(r0);
  b = __uint_as_float(r1);
}

// y + y tanh(y) on a bf16x2 pair made of two FP32 accumulators (lo, hi).
__device__ __forceinline__ uint32_t act_bf16x2(float lo, float hi) {
  uint32_t h, y;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(hi), "f"(lo));
  asm("{\n.reg .b32 t;\n"
      "tanh.approx.bf16x2 t, %1;\n"
      "fma.rn.bf16x2 %0, %1, t, %1;\n}\n"
      : "=r"(y)
      : "r"(h));
  return y;
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  uint32_t h;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(hi), "f"(lo));
  return h;
}

// ------------------------------------------------------------ row sources
// The pairs of the split light stage: features of listed pair `row`,
// shadowing or re-trace after the MLP.
template <bool BF16, int FS>
struct PairRows {
  StageParams p;
  PairList L;
  float threshold;

  __device__ uint32_t rows() const { return min(L.counters[0], L.cap); }

  // Writes the row's 32 inputs; false for an empty list slot (inputs 0).
  __device__ bool features(uint32_t i, float* f) const {
    const uint32_t b = L.block[i];
    if (b == kNoPair) return false;
    float cx, cy, cz;
    cache_position<BF16>(p, L.cache[i], cx, cy, cz);
    const int l = block_light(p, (int)b);
    const LightArgs& la = p.ll.lights[l];
    const int lb = (int)b - p.block_base[l];
    const float4 cone = __ldg(reinterpret_cast<const float4*>(la.cones) + lb);
    const VplData v = load_vpl<BF16>(la.vpls, lb * la.interval);
    pair_features<FS>(p.vox, p.inv_extent, p.vol_min, p.voxel_size, p.max_steps, cx, cy, cz, cone.x, cone.y, cone.z,
                      v.nx, v.ny, v.nz, cone.w, f);
    return true;
  }

  // Called by every thread of a warp (rows past the end are not valid);
  // `evaluated` counts this thread's warp's valid rows (lane 0's copy).
  __device__ void finish(uint32_t i, bool valid, float o_vis, float o_conf, uint32_t& evaluated) const {
    const int lane = threadIdx.x & 31;
    const float vis = sigmoidf(o_vis), conf = sigmoidf(o_conf);
    const bool retrace = valid && !(conf >= threshold);
    if (valid && !retrace) L.shadow[i] = vis;
    // cls 0: classified, ordered and traced after this pass; 0xFF: done
    if (valid) L.cls[i] = retrace ? (uint8_t)0 : (uint8_t)0xFF;
    const uint32_t m = __ballot_sync(0xffffffffu, retrace);
    if (lane == 0 && m) atomicAdd(L.counters + 3, (uint32_t)__popc(m));
    evaluated += (uint32_t)__popc(__ballot_sync(0xffffffffu, valid));
  }

  __device__ void done(uint32_t evaluated) const {
    if ((threadIdx.x & 31) == 0 && evaluated) atomicAdd(L.counters + 5, evaluated);
  }
};

// Given feature rows (validation): out[row] = (sigmoid(visibility),
// sigmoid(confidence)). Input 31 is taken as the constant 1.
struct GivenRows {
  const float* X;
  uint32_t n;
  float* out;

  __device__ uint32_t rows() const { return n; }
  __device__ bool features(uint32_t i, float* f) const {
    const float4* x = reinterpret_cast<const float4*>(X + (size_t)i * kMlpIn);
#pragma unroll
    for (int k = 0; k < kMlpIn / 4; ++k) {
      const float4 q = __ldg(x + k);
      f[4 * k] = q.x;
      f[4 * k + 1] = q.y;
      f[4 * k + 2] = q.z;
      f[4 * k + 3] = q.w;
    }
    f[kOneInput] = 1.0f;
    return true;
  }
  __device__ void finish(uint32_t i, bool valid, float o_vis, float o_conf, uint32_t&) const {
    if (valid) {
      out[2 * (size_t)i] = sigmoidf(o_vis);
      out[2 * (size_t)i + 1] = sigmoidf(o_conf);
    }
  }
  __device__ void done(uint32_t) const {}
};

// ------------------------------------------------------------ the MLP kernel
// hold_commit: the first layer-1 commit is withheld (its MMAs are not issued
// either), so that the bounded wait runs out: tests the timeout path.
template <class Rows>
__global__ void __launch_bounds__(kThreads, 4) mlp_tc_kernel(Rows src, const uint8_t* __restrict__ wimg,
                                                             uint32_t* err, int hold_commit) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned long long wait_cycles = hold_commit ? kTestWaitCycles : kWaitCycles;
  if (tid == 0) {
    mbar_init(&S.bar_w, 1);
    mbar_init(&S.bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // This row's constant columns of layers 2-4: 1 (BF16 0x3F80), then zeros.
  *reinterpret_cast<uint4*>(S.a + kmajor_offset(tid, kMlpHidden, kKH)) = make_uint4(0x3F80u, 0u, 0u, 0u);
  *reinterpret_cast<uint4*>(S.a + kmajor_offset(tid, kMlpHidden + 8, kKH)) = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  if (tid == 0) bulk_copy_g2s(S.w, wimg, kWBytes, &S.bar_w);
  bool abort = __syncthreads_or(!mbar_wait_bounded(&S.bar_w, 0, wait_cycles));

  const uint32_t a_addr = smem_u32(S.a), w_addr = smem_u32(S.w);
  const uint32_t sbo_a = (kKH / 8) * 128;  // 1280
  const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 TMEM lanes
  const uint32_t n_rows = src.rows();
  const uint32_t n_tiles = (n_rows + kThreads - 1) / kThreads;
  uint32_t phase = 0, evaluated = 0;
  bool held = false;

  // One layer: MMAs over k_steps (K = 16 each) of A x W^T into TMEM columns
  // [0, n), committed; every thread waits for them. False: the wait ran out.
  auto layer = [&](uint32_t w_off, uint32_t sbo_w, int k_steps, uint32_t idesc) -> bool {
    fence_proxy_async();  // this thread's A-tile stores -> the tensor cores' reads
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      if (hold_commit && !held) {
        held = true;  // nothing issued, nothing committed: the wait below runs out
      } else {
        for (int ks = 0; ks < k_steps; ++ks)
          mma_bf16(tmem, smem_desc(a_addr + ks * 256, 128, sbo_a), smem_desc(w_addr + w_off + ks * 256, 128, sbo_w),
                   idesc, ks > 0 ? 1u : 0u);
        mma_commit(&S.bar_mma);
      }
    }
    const bool ok = mbar_wait_bounded(&S.bar_mma, phase, wait_cycles);
    phase ^= 1u;
    tc_fence_after();
    return !__syncthreads_or(!ok);
  };
  // Accumulators -> activations -> this thread's row of the A tile.
  auto activate = [&]() {
    float v[64];
    tmem_ld64(t_row, v);
#pragma unroll
    for (int c = 0; c < kMlpHidden / 8; ++c) {
      uint4 q;
      q.x = act_bf16x2(v[8 * c + 0], v[8 * c + 1]);
      q.y = act_bf16x2(v[8 * c + 2], v[8 * c + 3]);
      q.z = act_bf16x2(v[8 * c + 4], v[8 * c + 5]);
      q.w = act_bf16x2(v[8 * c + 6], v[8 * c + 7]);
      *reinterpret_cast<uint4*>(S.a + kmajor_offset(tid, 8 * c, kKH)) = q;
    }
  };

  for (uint32_t tile = blockIdx.x; tile < n_tiles && !abort; tile += gridDim.x) {
    const uint32_t row = tile * kThreads + tid;
    bool valid = false;
    {
      float f[kMlpIn];
      if (row < n_rows) valid = src.features(row, f);
      if (!valid) {
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) f[k] = 0.0f;
      }
#pragma unroll
      for (int c = 0; c < kMlpIn / 8; ++c) {
        uint4 q;
        q.x = pack2(f[8 * c + 0], f[8 * c + 1]);
        q.y = pack2(f[8 * c + 2], f[8 * c + 3]);
        q.z = pack2(f[8 * c + 4], f[8 * c + 5]);
        q.w = pack2(f[8 * c + 6], f[8 * c + 7]);
        *reinterpret_cast<uint4*>(S.a + kmajor_offset(tid, 8 * c, kKH)) = q;
      }
    }
    if (!(abort = !layer(kW1Off, (kK1 / 8) * 128, kK1 / 16, instr_desc(kMlpHidden)))) activate();
    if (!abort && !(abort = !layer(kW2Off, sbo_a, kKH / 16, instr_desc(kMlpHidden)))) activate();
    if (!abort && !(abort = !layer(kW3Off, sbo_a, kKH / 16, instr_desc(kMlpHidden)))) activate();
    if (!abort && !(abort = !layer(kW4Off, sbo_a, kKH / 16, instr_desc(kN4)))) {
      float o_vis, o_conf;
      tmem_ld2(t_row, o_vis, o_conf);
      src.finish(row, valid && row < n_rows, o_vis, o_conf, evaluated);
    }
  }
  if (abort) {
    if (tid == 0) raise_error(err, DRV_DEVERR_TIMEOUT);
    // What this CTA issued may still be in flight: wait for it once more
    // (bounded) before the tensor memory and shared memory are released.
    mbar_wait_bounded(&S.bar_w, 0, wait_cycles);
    if (phase) mbar_wait_bounded(&S.bar_mma, phase ^ 1u, wait_cycles);
  } else {
    src.done(evaluated);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// FP32 master parameters -> the packed BF16 B-operand image (folded biases
// and GELU constants, see the file header). One thread per image element.
__global__ void pack_weights_kernel(const float* __restrict__ params, uint16_t* __restrict__ img) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int n1 = kMlpHidden * kK1, nh = kMlpHidden * kKH, n4 = kN4 * kKH;
  float w = 0.0f;
  uint32_t off;
  if (t < n1) {
    const int r = t / kK1, k = t % kK1;
    const float x = k == kOneInput ? __fadd_rn(params[kOffW1 + r * kMlpIn + k], params[kOffB1 + r])
                                   : params[kOffW1 + r * kMlpIn + k];
    w = __fmul_rn(kGeluHalfK, x);
    off = kW1Off + kmajor_offset(r, k, kK1);
  } else if (t < n1 + 2 * nh) {
    const int u = t - n1, layer = u / nh, r = (u % nh) / kKH, k = (u % nh) % kKH;
    const int wo = layer ? kOffW3 : kOffW2, bo = layer ? kOffB3 : kOffB2;
    w = k < kMlpHidden ? __fmul_rn(0.5f, params[wo + r * kMlpHidden + k])
                       : (k == kMlpHidden ? __fmul_rn(kGeluHalfK, params[bo + r]) : 0.0f);
    off = (layer ? kW3Off : kW2Off) + kmajor_offset(r, k, kKH);
  } else if (t < n1 + 2 * nh + n4) {
    const int u = t - n1 - 2 * nh, r = u / kKH, k = u % kKH;
    if (r < kMlpOut)
      w = k < kMlpHidden ? __fdiv_rn(params[kOffW4 + r * kMlpHidden + k], 1.702f)
                         : (k == kMlpHidden ? params[kOffB4 + r] : 0.0f);
    off = kW4Off + kmajor_offset(r, k, kKH);
  } else {
    return;
  }
  img[off / 2] = to_bf16(w);
}

constexpr int kPackElems = kMlpHidden * kK1 + 2 * kMlpHidden * kKH + kN4 * kKH;

// Dynamic shared memory: set once per (kernel, device).
template <class Rows>
cudaError_t launch_tc(cudaStream_t s, const Rows& rows, uint32_t n_rows, const void* weights, uint32_t* err,
                      int hold_commit, int num_sms) {
  auto kernel = mlp_tc_kernel<Rows>;
  const size_t smem = sizeof(TcSmem);
  static std::mutex mu;
  static uint64_t done = 0;  // bit d: attribute set on device d
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 64 || !((done >> dev) & 1u)) {
      e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      // Four CTAs of ~47 KB per SM need the largest shared-memory carveout.
      e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
      if (dev < 64) done |= 1ull << dev;
    }
  }
  // Four CTAs per SM (__launch_bounds__; 4 x 64 of the SM's 512 tensor-memory
  // columns): the CTAs of one SM overlap each other's MMA round trips.
  const int per_sm = 4;
  const uint32_t tiles = (n_rows + kThreads - 1) / kThreads;
  const uint32_t grid = tiles == 0 ? 1u : (tiles < (uint32_t)(num_sms * per_sm) ? tiles : (uint32_t)(num_sms * per_sm));
  kernel<<<grid, kThreads, smem, s>>>(rows, static_cast<const uint8_t*>(weights), err, hold_commit);
  return cudaGetLastError();
}

}  // namespace

size_t surrogate_weights_bytes() { return kWBytes; }

cudaError_t launch_pack_surrogate_weights(cudaStream_t s, const float* params, void* weights) {
  pack_weights_kernel<<<(kPackElems + 255) / 256, 256, 0, s>>>(params, static_cast<uint16_t*>(weights));
  return cudaGetLastError();
}

cudaError_t launch_surrogate_eval(cudaStream_t s, const void* weights, const float* X, int n, float* out,
                                  uint32_t* err, int num_sms) {
  GivenRows rows{X, (uint32_t)n, out};
  return launch_tc(s, rows, (uint32_t)n, weights, err, 0, num_sms);
}

cudaError_t launch_surrogate_mlp(cudaStream_t s, const StageParams& p, const PairList& L, const SurrogateArgs& sa,
                                 bool bf16, int num_sms) {
  // The row count is on the device (pairs the cull listed): the grid covers
  // the list's capacity and idle CTAs return after the first tile check.
  const uint32_t cap_rows = L.cap;
  if (sa.feature_set == kFeatureCone8) {
    if (bf16) return launch_tc(s, PairRows<true, kFeatureCone8>{p, L, sa.threshold}, cap_rows, sa.weights, sa.err,
                               sa.hold_commit, num_sms);
    return launch_tc(s, PairRows<false, kFeatureCone8>{p, L, sa.threshold}, cap_rows, sa.weights, sa.err,
                     sa.hold_commit, num_sms);
  }
  if (sa.feature_set == kFeatureCone4) {
    if (bf16) return launch_tc(s, PairRows<true, kFeatureCone4>{p, L, sa.threshold}, cap_rows, sa.weights, sa.err,
                               sa.hold_commit, num_sms);
    return launch_tc(s, PairRows<false, kFeatureCone4>{p, L, sa.threshold}, cap_rows, sa.weights, sa.err,
                     sa.hold_commit, num_sms);
  }
  if (bf16) return launch_tc(s, PairRows<true, kFeatureSegment8>{p, L, sa.threshold}, cap_rows, sa.weights,
                             sa.err, sa.hold_commit, num_sms);
  return launch_tc(s, PairRows<false, kFeatureSegment8>{p, L, sa.threshold}, cap_rows, sa.weights, sa.err,
                   sa.hold_commit, num_sms);
}

}  // namespace drv
