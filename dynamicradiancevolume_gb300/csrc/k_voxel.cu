// k_voxel.cu — VoxelizeScene (voxelization.cpp:90-142, voxelize.{vert,geom,frag})
// for the procedural box scene, and the opacity mip chain (voxelmipmap.comp:8-13,
// voxelization.cpp:155-172).
//
// Level 0 is a binary surface-voxel grid stored as a bitmask (bit x&31 of
// word ((z*N + y)*N + x) / 32). Levels 1..L are FP32 means of their 8
// children; every level is an exact dyadic rational (count / 8^l with
// 8^l <= 2^24 for N <= 256), so FP32 holds them exactly.
#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

constexpr int kMaxBoxes = 512;

struct Face {
  int16_t axis, k, u0, u1, v0, v1;
};

// Face rectangle -> covered voxel ranges (binary32 mirror). For an
// axis-aligned face the dominant axis is its normal axis and the
// conservative raster (voxelize.geom:201-225 + voxelize.frag:280-283) covers
// every voxel square that touches the closed rectangle; the depth gradient is
// zero, so the +-1 depth voxels of voxelize.frag:295-313 never trigger.
__device__ __forceinline__ bool make_face(const DrvBox& b, int axis, int side, const float* vm, float vs, int N,
                                          Face& f) {
  int ua = (axis + 1) % 3, va = (axis + 2) % 3;
  float plane = side ? b.max[axis] : b.min[axis];
  float kc = __fdiv_rn(__fsub_rn(plane, vm[axis]), vs);
  if (!(kc >= 0.0f) || !(kc < (float)N)) return false;
  float lu = __fdiv_rn(__fsub_rn(b.min[ua], vm[ua]), vs), hu = __fdiv_rn(__fsub_rn(b.max[ua], vm[ua]), vs);
  float lv = __fdiv_rn(__fsub_rn(b.min[va], vm[va]), vs), hv = __fdiv_rn(__fsub_rn(b.max[va], vm[va]), vs);
  int u0 = max(0, (int)ceilf(lu) - 1), u1 = min(N - 1, (int)floorf(hu));
  int v0 = max(0, (int)ceilf(lv) - 1), v1 = min(N - 1, (int)floorf(hv));
  if (u0 > u1 || v0 > v1) return false;
  f.axis = (int16_t)axis;
  f.k = (int16_t)(int)kc;
  f.u0 = (int16_t)u0;
  f.u1 = (int16_t)u1;
  f.v0 = (int16_t)v0;
  f.v1 = (int16_t)v1;
  return true;
}

__device__ __forceinline__ uint32_t range_mask(int lo, int hi, int base) {
  // bits [lo, hi] of the 32-voxel run starting at x = base
  int a = max(lo, base), b = min(hi, base + 31);
  if (a > b) return 0u;
  int n = b - a + 1;
  uint32_t m = n == 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  return m << (a - base);
}

// Box faces x kVoxelSplit CTAs (grid n_boxes*6 by kVoxelSplit): the face's
// covered voxel rectangle is ORed into the zeroed bitmask, one atomicOr per
// touched 32-voxel word (per voxel for faces on the x axis, whose rows cross
// words), the face's items dealt out over its CTAs. OR is order-independent,
// so the mask does not depend on scheduling.
constexpr int kVoxelSplit = 16;

__global__ void __launch_bounds__(256) voxelize_kernel(const DrvBox* __restrict__ boxes, DrvVolumeInfo vol, int N,
                                                       uint32_t* __restrict__ bits) {
  Face fc;
  if (!make_face(boxes[blockIdx.x / 6], (blockIdx.x % 6) >> 1, blockIdx.x & 1, vol.volume_world_min,
                 vol.voxel_size_in_world, N, fc))
    return;
  const int wpr = N / 32;  // words per row
  const int u0 = fc.u0, u1 = fc.u1, v0 = fc.v0, v1 = fc.v1, k = fc.k;
  if (fc.axis == 0) {  // plane x = k: y in [u0,u1], z in [v0,v1]
    const int ny = u1 - u0 + 1, nz = v1 - v0 + 1;
    const uint32_t bit = 1u << (k & 31);
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < ny * nz; i += gridDim.y * blockDim.x) {
      const int y = u0 + i % ny, z = v0 + i / ny;
      atomicOr(bits + ((size_t)z * N + y) * wpr + (k >> 5), bit);
    }
  } else {
    // axis 2, plane z = k: x in [u0,u1] for rows y in [v0,v1];
    // axis 1, plane y = k: x in [v0,v1] for slices z in [u0,u1].
    const int xl = fc.axis == 2 ? u0 : v0, xh = fc.axis == 2 ? u1 : v1;
    const int rl = fc.axis == 2 ? v0 : u0, rh = fc.axis == 2 ? v1 : u1;
    const int w0 = xl >> 5, nw = (xh >> 5) - w0 + 1, nr = rh - rl + 1;
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < nw * nr; i += gridDim.y * blockDim.x) {
      const int w = w0 + i % nw, r = rl + i / nw;
      const size_t row = fc.axis == 2 ? (size_t)k * N + r : (size_t)r * N + k;
      atomicOr(bits + row * wpr + w, range_mask(xl, xh, w * 32));
    }
  }
}

// ---- triangle meshes ----------------------------------------------------
// voxelize.{vert,geom,frag} for a triangle mesh, in binary32 with every
// operation rounded as written (the oracle restates the same sequence):
// positions in voxel units w = (p - VolumeWorldMin) / VoxelSizeInWorld (the
// window coordinates of the reference's VoxelResolution^2 viewport); the
// dominant axis of the normal picks the projection (voxelize.geom:24-51, ties
// as there); each edge line moves outward by half a voxel in the L1 sense
// (voxelize.geom:70-86); a pixel centre inside the three moved lines and
// inside the triangle's AABB grown by half a voxel (voxelize.geom:59-62,
// voxelize.frag:22-26), both inclusive, is a fragment; its depth is the
// plane through the moved vertices carrying the original vertices' depths
// (voxelize.geom:89-107); voxel z = int(depth), plus z - 1 / z + 1 where
// int(depth -+ 1.414 |grad depth|) differs (voxelize.frag:39-55); depth
// outside [0, N] is clipped and stores outside the grid are dropped.
struct TriSetup {
  int side;
  float r[3][3];      // swizzled vertices: raster x, raster y, depth
  float plane[3][3];  // moved edge lines a x + b y + c, inside <= 0
  float aabb[4];      // x0, y0, x1, y1
  float zA, zB, zC;   // depth plane
  float max_change;
  bool ok;
};

__device__ __forceinline__ float dmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dadd(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ TriSetup tri_setup(const float* P0, const float* P1, const float* P2, const float* vm,
                                              float vs) {
  TriSetup t;
  t.ok = false;
  float w[3][3];
  const float* P[3] = {P0, P1, P2};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) w[i][a] = __fdiv_rn(dsub(P[i][a], vm[a]), vs);
  const float e0[3] = {dsub(w[1][0], w[0][0]), dsub(w[1][1], w[0][1]), dsub(w[1][2], w[0][2])};
  const float e1[3] = {dsub(w[2][0], w[0][0]), dsub(w[2][1], w[0][1]), dsub(w[2][2], w[0][2])};
  const float n[3] = {fabsf(dsub(dmul(e0[1], e1[2]), dmul(e0[2], e1[1]))),
                      fabsf(dsub(dmul(e0[2], e1[0]), dmul(e0[0], e1[2]))),
                      fabsf(dsub(dmul(e0[0], e1[1]), dmul(e0[1], e1[0])))};
  int side = n[0] > n[1] ? 0 : 1;
  side = (side == 0 ? n[0] : n[1]) > n[2] ? side : 2;
  t.side = side;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float x = w[i][0], y = w[i][1], z = w[i][2];
    t.r[i][0] = side == 0 ? z : x;
    t.r[i][1] = side == 1 ? z : y;
    t.r[i][2] = side == 0 ? x : (side == 1 ? y : z);
  }
  t.aabb[0] = dsub(fminf(fminf(t.r[0][0], t.r[1][0]), t.r[2][0]), 0.5f);
  t.aabb[1] = dsub(fminf(fminf(t.r[0][1], t.r[1][1]), t.r[2][1]), 0.5f);
  t.aabb[2] = dadd(fmaxf(fmaxf(t.r[0][0], t.r[1][0]), t.r[2][0]), 0.5f);
  t.aabb[3] = dadd(fmaxf(fmaxf(t.r[0][1], t.r[1][1]), t.r[2][1]), 0.5f);
  const float ax = dsub(t.r[0][0], t.r[2][0]), ay = dsub(t.r[0][1], t.r[2][1]);
  const float bx = dsub(t.r[1][0], t.r[0][0]), by = dsub(t.r[1][1], t.r[0][1]);
  const float area = dsub(dmul(ax, by), dmul(bx, ay));
  if (!(area != 0.0f)) return t;
  const float wind = area > 0.0f ? 1.0f : -1.0f;
  // Edge i runs from vertex (i + 2) % 3 to vertex i (voxelize.geom:66-71).
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int f = (i + 2) % 3;
    const float dx = dsub(t.r[i][0], t.r[f][0]), dy = dsub(t.r[i][1], t.r[f][1]);
    const float px = t.r[f][0], py = t.r[f][1];
    const float a = dmul(dy, wind), b = dmul(-dx, wind), c = dmul(dsub(dmul(dx, py), dmul(dy, px)), wind);
    t.plane[i][0] = a;
    t.plane[i][1] = b;
    t.plane[i][2] = dsub(c, dmul(0.5f, dadd(fabsf(a), fabsf(b))));
  }
  // Moved vertex i: moved line i meets moved line i + 1.
  float V[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float* L0 = t.plane[i];
    const float* L1 = t.plane[(i + 1) % 3];
    const float hx = dsub(dmul(L0[1], L1[2]), dmul(L0[2], L1[1]));
    const float hy = dsub(dmul(L0[2], L1[0]), dmul(L0[0], L1[2]));
    const float hw = dsub(dmul(L0[0], L1[1]), dmul(L0[1], L1[0]));
    if (!(hw != 0.0f)) return t;
    V[i][0] = __fdiv_rn(hx, hw);
    V[i][1] = __fdiv_rn(hy, hw);
  }
  const float x10 = dsub(V[1][0], V[0][0]), y10 = dsub(V[1][1], V[0][1]);
  const float x20 = dsub(V[2][0], V[0][0]), y20 = dsub(V[2][1], V[0][1]);
  const float z10 = dsub(t.r[1][2], t.r[0][2]), z20 = dsub(t.r[2][2], t.r[0][2]);
  const float det = dsub(dmul(x10, y20), dmul(x20, y10));
  if (!(det != 0.0f)) return t;
  t.zA = __fdiv_rn(dsub(dmul(z10, y20), dmul(z20, y10)), det);
  t.zB = __fdiv_rn(dsub(dmul(x10, z20), dmul(x20, z10)), det);
  t.zC = dsub(dsub(t.r[0][2], dmul(t.zA, V[0][0])), dmul(t.zB, V[0][1]));
  t.max_change = dmul(__fsqrt_rn(dadd(dmul(t.zA, t.zA), dmul(t.zB, t.zB))), 1.414f);
  t.ok = true;
  return t;
}

__device__ __forceinline__ void set_voxel_swizzled(uint32_t* bits, int N, int side, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= N || y >= N || z >= N) return;
  const int cx = side == 0 ? z : x, cy = side == 1 ? z : y, cz = side == 0 ? x : (side == 1 ? y : z);
  const size_t i = ((size_t)cz * N + cy) * N + cx;
  atomicOr(bits + (i >> 5), 1u << (i & 31));
}

struct TriVolume {
  float vm[3];
  float vs;
};

// A warp per triangle (grid-stride): every lane forms the same setup, the
// lanes share the pixels of the grown AABB.
__global__ void __launch_bounds__(256) triangles_kernel(const float* __restrict__ pos, int n_vertices,
                                                        const uint32_t* __restrict__ idx, int n_tris, TriVolume tv,
                                                        int N, uint32_t* __restrict__ bits) {
  const int lane = threadIdx.x & 31;
  const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); k < n_tris; k += n_warps) {
    const uint32_t i0 = idx ? __ldg(idx + 3 * k) : 3u * k, i1 = idx ? __ldg(idx + 3 * k + 1) : 3u * k + 1,
                   i2 = idx ? __ldg(idx + 3 * k + 2) : 3u * k + 2;
    if (i0 >= (uint32_t)n_vertices || i1 >= (uint32_t)n_vertices || i2 >= (uint32_t)n_vertices) continue;
    float P[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      P[0][a] = __ldg(pos + 3 * (size_t)i0 + a);
      P[1][a] = __ldg(pos + 3 * (size_t)i1 + a);
      P[2][a] = __ldg(pos + 3 * (size_t)i2 + a);
    }
    const TriSetup t = tri_setup(P[0], P[1], P[2], tv.vm, tv.vs);
    if (!t.ok) continue;
    const int x0 = max(0, (int)floorf(t.aabb[0])), y0 = max(0, (int)floorf(t.aabb[1]));
    const int x1 = min(N - 1, (int)floorf(t.aabb[2])), y1 = min(N - 1, (int)floorf(t.aabb[3]));
    if (x1 < x0 || y1 < y0) continue;
    const int W = x1 - x0 + 1, total = W * (y1 - y0 + 1);
    for (int q = lane; q < total; q += 32) {
      const int px = x0 + q % W, py = y0 + q / W;
      const float cx = dadd((float)px, 0.5f), cy = dadd((float)py, 0.5f);
      if (cx < t.aabb[0] || cy < t.aabb[1] || cx > t.aabb[2] || cy > t.aabb[3]) continue;
      bool in = true;
#pragma unroll
      for (int e = 0; e < 3; ++e)
        in = in && dadd(dadd(dmul(t.plane[e][0], cx), dmul(t.plane[e][1], cy)), t.plane[e][2]) <= 0.0f;
      if (!in) continue;
      const float z = dadd(dadd(dmul(t.zA, cx), dmul(t.zB, cy)), t.zC);
      if (!(z >= 0.0f && z <= (float)N)) continue;
      const int zi = (int)z;
      set_voxel_swizzled(bits, N, t.side, px, py, zi);
      if ((int)dsub(z, t.max_change) != zi) set_voxel_swizzled(bits, N, t.side, px, py, zi - 1);
      if ((int)dadd(z, t.max_change) != zi) set_voxel_swizzled(bits, N, t.side, px, py, zi + 1);
    }
  }
}

struct MipOffsets {
  size_t off[kMaxVoxelLevels];
};

// a[i] for a runtime i by an unrolled select over constant indices: a
// runtime index into a by-value kernel argument makes the compiler copy the
// whole array to the local-memory stack of every thread.
template <typename T, int K>
__device__ __forceinline__ T pick(const T (&a)[K], int i) {
  T r = a[0];
#pragma unroll
  for (int k = 1; k < K; ++k)
    if (k == i) r = a[k];
  return r;
}

// Fused mips over one B^3 level-0 block (B = min(32, N)): levels 1..log2(B)
// computed in shared memory from one read of the block's bits.
template <typename T>
__device__ __forceinline__ void store_mip(T* p, float v);
template <>
__device__ __forceinline__ void store_mip<float>(float* p, float v) { *p = v; }
template <>
__device__ __forceinline__ void store_mip<__half>(__half* p, float v) { *p = __float2half_rn(v); }
__device__ __forceinline__ float load_mip(const float* p) { return *p; }
__device__ __forceinline__ float load_mip(const __half* p) { return __half2float(*p); }
// The same through L2 (another CTA's writes of this launch).
__device__ __forceinline__ float load_mip_l2(const float* p) { return __ldcg(p); }
__device__ __forceinline__ float load_mip_l2(const __half* p) {
  return __half2float(__ushort_as_half(__ldcg(reinterpret_cast<const unsigned short*>(p))));
}

template <typename T>
__global__ void __launch_bounds__(256) mips_kernel(int N, int B, const uint32_t* __restrict__ bits,
                                                   T* __restrict__ mips, MipOffsets mo, uint32_t* ticket,
                                                   int tail_first, int tail_last) {
  __shared__ uint32_t sbits[32 * 32];  // B rows x B slices of (B <= 32)-voxel runs
  __shared__ float lv[2][16 * 16 * 16];
  // N and B are powers of two: indices split by shifts and masks (a
  // division by a runtime divisor costs tens of instructions).
  const int lB = 31 - __clz(B), lnb = 31 - __clz(N) - lB, nbx = 1 << lnb;
  const int bx = blockIdx.x & (nbx - 1), by = (blockIdx.x >> lnb) & (nbx - 1), bz = blockIdx.x >> (2 * lnb);
  for (int i = threadIdx.x; i < B * B; i += blockDim.x) {
    int y = i & (B - 1), z = i >> lB;
    int gx = bx * B, gy = by * B + y, gz = bz * B + z;
    size_t bit = ((size_t)gz * N + gy) * N + gx;
    uint32_t word = bits[bit >> 5];
    sbits[i] = B == 32 ? word : ((word >> (bit & 31)) & ((1u << B) - 1u));
  }
  __syncthreads();
  // Level 1 from bits.
  int n = B / 2, ln = lB - 1;
  for (int i = threadIdx.x; i < n * n * n; i += blockDim.x) {
    int x = i & (n - 1), y = (i >> ln) & (n - 1), z = i >> (2 * ln);
    int c = 0;
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        uint32_t w = sbits[(2 * z + dz) * B + (2 * y + dy)];
        c += __popc((w >> (2 * x)) & 3u);
      }
    float v = (float)c * 0.125f;
    lv[0][i] = v;
    int gn = N / 2;
    size_t g = ((size_t)(bz * n + z) * gn + (by * n + y)) * gn + (bx * n + x);
    store_mip(mips + mo.off[1] + g, v);
  }
  __syncthreads();
  // Levels 2 .. log2(B).
  int cur = 0, level = 1;
  for (int m = n / 2, lm = ln - 1; m >= 1; m /= 2, --lm) {
    ++level;
    for (int i = threadIdx.x; i < m * m * m; i += blockDim.x) {
      int x = i & (m - 1), y = (i >> lm) & (m - 1), z = i >> (2 * lm);
      int p = 2 * m;
      float s = 0.0f;
#pragma unroll
      for (int dz = 0; dz < 2; ++dz)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
          for (int dx = 0; dx < 2; ++dx) s += lv[cur][((2 * z + dz) * p + (2 * y + dy)) * p + (2 * x + dx)];
      float v = s * 0.125f;
      lv[cur ^ 1][i] = v;
      int gn = N >> level;
      size_t g = ((size_t)(bz * m + z) * gn + (by * m + y)) * gn + (bx * m + x);
      store_mip(mips + pick(mo.off, level) + g, v);
    }
    __syncthreads();
    cur ^= 1;
  }
  // Levels tail_first..tail_last, above one block: built by the CTA that
  // finishes last (a ticket per build, reset by that CTA for the next), from
  // the level below as every CTA wrote it (each CTA fences its writes before
  // taking its ticket; the last one reads through L2). Like the levels
  // above, each comes from the level below as stored (FP32, or the FP16
  // values: the chain an FP16 texture would hold).
  if (tail_first > tail_last) return;
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int log2n = lB + lnb;
  for (int lv = tail_first; lv <= tail_last; ++lv) {
    const int lm = log2n - lv, m = 1 << lm, p = m * 2;
    const T* src = mips + pick(mo.off, lv - 1);
    T* dst = mips + pick(mo.off, lv);
    for (int i = threadIdx.x; i < m * m * m; i += blockDim.x) {
      const int x = i & (m - 1), y = (i >> lm) & (m - 1), z = i >> (2 * lm);
      float s = 0.0f;
      for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx)
            s += load_mip_l2(src + ((size_t)(2 * z + dz) * p + (2 * y + dy)) * p + (2 * x + dx));
      store_mip(dst + i, s * 0.125f);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// Corner-packed level 0 (see voxel_sample.cuh): byte (x, y, z) = the 8 voxels
// (x + dx, y + dy, z + dz) with +1 clamped to N - 1, bit dx | dy << 1 | dz << 2,
// x fastest. One thread per 16 bytes of a row: it reads bits x0..x0+16 of
// the four voxel rows (y, z), (y+1, z), (y, z+1), (y+1, z+1) and writes one
// 16-byte store (consecutive threads take consecutive 16-byte pieces, so a
// warp writes 512 contiguous bytes).
__device__ __forceinline__ uint32_t corner_row_bits(const uint32_t* __restrict__ bits, int N, int y, int z, int x0) {
  // bits x0..x0+15 of row (y, z) and, in bit 16, voxel x0 + 16 (clamped to N - 1)
  const uint32_t* row = bits + ((size_t)z * N + y) * (N >> 5);
  const int w = x0 >> 5, sh = x0 & 31;  // sh is 0 or 16
  const uint32_t a = __ldg(row + w);
  const uint32_t r = (a >> sh) & 0xFFFFu;
  uint32_t next;
  if (x0 + 16 >= N) next = (r >> 15) & 1u;
  else next = sh ? (__ldg(row + w + 1) & 1u) : ((a >> 16) & 1u);
  return r | next << 16;
}

// 8 x 8 bit-matrix transpose (bit j of byte i to bit i of byte j) by three
// rounds of masked swaps (the classic delta-swap transpose).
__device__ __forceinline__ uint64_t transpose_bits8x8(uint64_t x) {
  uint64_t t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
  x ^= t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
  x ^= t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
  x ^= t ^ (t << 28);
  return x;
}

__global__ void __launch_bounds__(256) corners_kernel(int N, int log2n, const uint32_t* __restrict__ bits,
                                                      uint8_t* __restrict__ out) {
  const int lq = log2n - 4;  // 16-byte pieces per row = N / 16
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ((uint32_t)N * N << lq)) return;
  const int x0 = (int)(t & ((1u << lq) - 1u)) << 4;
  const int y = (int)((t >> lq) & (uint32_t)(N - 1)), z = (int)(t >> (lq + log2n));
  const int y1 = min(y + 1, N - 1), z1 = min(z + 1, N - 1);
  // rows[dy | dz << 1]
  const uint32_t rows[4] = {corner_row_bits(bits, N, y, z, x0), corner_row_bits(bits, N, y1, z, x0),
                            corner_row_bits(bits, N, y, z1, x0), corner_row_bits(bits, N, y1, z1, x0)};
  // Bit k of byte lx is voxel lx + (k & 1) of row k >> 1: with vector k =
  // bits lx (0..7, or 8..15) of row k >> 1 shifted right by k & 1, the 8
  // bytes of an 8-byte half are the 8 x 8 bit transpose of the 8 vectors.
  // Byte permutes gather the vectors (byte k = vector k), three rounds of
  // masked swaps transpose them.
  uint32_t p[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) p[q] = __byte_perm(rows[q], rows[q] >> 1, 0x5140);  // lx 0..7 and 8..15, dx 0, 1
  const uint64_t lo = transpose_bits8x8((uint64_t)__byte_perm(p[0], p[1], 0x5410) |
                                        (uint64_t)__byte_perm(p[2], p[3], 0x5410) << 32);
  const uint64_t hi = transpose_bits8x8((uint64_t)__byte_perm(p[0], p[1], 0x7632) |
                                        (uint64_t)__byte_perm(p[2], p[3], 0x7632) << 32);
  *reinterpret_cast<uint4*>(out + ((size_t)z * N + y) * N + x0) =
      make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// Corner-packed mip records (voxel_sample.cuh), x fastest: one thread per
// 2x2x2 block of records, over the blocks of all levels back to back. It
// reads the 3x3x3 texels its 8 records cover (+1 clamped) once and writes
// the 8 records (consecutive threads take consecutive blocks along x, so
// the record pairs (x0, x0 + 1) of a warp fill contiguous rows). Records
// hold FP16 texels: a copy with BF16 precision; with FP32 precision the
// records cover levels 1..3, whose texels k / 8^l (8^l <= 512) FP16 holds
// exactly.
struct RecordLevels {
  uint32_t blocks;  // 2x2x2 record blocks of levels 1..K
  int levels;       // K
  int log2n;
};

__device__ __forceinline__ uint32_t half_bits(float v) { return (uint32_t)__half_as_ushort(__float2half_rn(v)); }
__device__ __forceinline__ uint32_t half_bits(__half v) { return (uint32_t)__half_as_ushort(v); }

template <typename T>
__global__ void __launch_bounds__(256) records_kernel(const T* __restrict__ mips, MipOffsets mo, RecordLevels rl,
                                                      uint4* __restrict__ out) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= rl.blocks) return;
  // Level of block g: level l has max(n / 2, 1)^3 blocks and n^3 records
  // (n = N >> l), levels back to back from level 1 (found without indexing
  // the parameter arrays, which would copy them to local memory).
  int level = 1, ln = rl.log2n - 1;
  uint32_t bstart = 0, rstart = 0;
  for (;;) {
    const uint32_t nblocks = 1u << (3 * max(ln - 1, 0));
    if (level == rl.levels || g < bstart + nblocks) break;
    bstart += nblocks;
    rstart += 1u << (3 * ln);
    ++level;
    --ln;
  }
  const int n = 1 << ln, lb = ln > 0 ? ln - 1 : 0, nb = 1 << lb;
  const uint32_t block = g - bstart;
  const int x0 = (int)(block & (nb - 1)) << 1, y0 = (int)((block >> lb) & (nb - 1)) << 1,
            z0 = (int)(block >> (2 * lb)) << 1;
  const T* src = mips + pick(mo.off, level);
  uint32_t h[3][3][3];
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      const T* row = src + ((size_t)min(z0 + dz, n - 1) * n + min(y0 + dy, n - 1)) * n;
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) h[dz][dy][dx] = half_bits(row[min(x0 + dx, n - 1)]);
    }
  uint4* dst = out + rstart;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int rx = r & 1, ry = (r >> 1) & 1, rz = r >> 2;
    if (x0 + rx >= n || y0 + ry >= n || z0 + rz >= n) continue;  // a 1-texel level has one record
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j0 = 2 * q, j1 = 2 * q + 1;  // slot j = dx | dy << 1 | dz << 2
      w[q] = h[rz + (j0 >> 2)][ry + ((j0 >> 1) & 1)][rx + (j0 & 1)] |
             h[rz + (j1 >> 2)][ry + ((j1 >> 1) & 1)][rx + (j1 & 1)] << 16;
    }
    dst[((size_t)(z0 + rz) * n + (y0 + ry)) * n + x0 + rx] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

}  // namespace

cudaError_t launch_build_records(cudaStream_t s, int n, const void* mips, const size_t* mip_offsets, int precision,
                                 uint4* records, const uint32_t* record_offsets, int record_levels) {
  if (record_levels <= 0) return cudaSuccess;
  MipOffsets mo{};
  RecordLevels rl{};
  for (int i = 0; i < kMaxVoxelLevels; ++i) mo.off[i] = mip_offsets[i];
  rl.levels = record_levels;
  while ((1 << (rl.log2n + 1)) <= n) ++rl.log2n;
  // the records of level l at record_offsets[l] = sum of (n >> j)^3 over j < l
  for (int l = 1, ln = rl.log2n - 1; l <= record_levels; ++l, --ln) {
    if (record_offsets[l] != (l == 1 ? 0u : record_offsets[l - 1] + (1u << (3 * (ln + 1)))))
      return cudaErrorInvalidValue;
    rl.blocks += 1u << (3 * (ln > 0 ? ln - 1 : 0));
  }
  const dim3 grid((rl.blocks + 255) / 256);
  if (precision == DRV_PRECISION_BF16)
    records_kernel<__half><<<grid, 256, 0, s>>>((const __half*)mips, mo, rl, records);
  else
    records_kernel<float><<<grid, 256, 0, s>>>((const float*)mips, mo, rl, records);
  return cudaGetLastError();
}

cudaError_t launch_build_corners(cudaStream_t s, int n, const uint32_t* bits, uint8_t* corners) {
  int l = 0;
  while ((1 << (l + 1)) <= n) ++l;
  const uint32_t pieces = (uint32_t)n * n * (n / 16);  // 16-byte pieces of the grid
  corners_kernel<<<(pieces + 255) / 256, 256, 0, s>>>(n, l, bits, corners);
  return cudaGetLastError();
}

cudaError_t launch_voxelize(cudaStream_t s, const DrvBox* boxes, int n_boxes, const DrvVolumeInfo& vol, int n,
                            uint32_t* bits) {
  if (n_boxes > kMaxBoxes || n < 32 || (n & 31)) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(bits, 0, (size_t)n * n * (n / 32) * sizeof(uint32_t), s);
  if (e != cudaSuccess || n_boxes == 0) return e;
  voxelize_kernel<<<dim3(n_boxes * 6, kVoxelSplit), 256, 0, s>>>(boxes, vol, n, bits);
  return cudaGetLastError();
}

cudaError_t launch_voxelize_triangles(cudaStream_t s, const float* positions, int n_vertices, const uint32_t* indices,
                                      int n_triangles, const DrvVolumeInfo& vol, int n, uint32_t* bits, int num_sms) {
  if (n < 32 || (n & 31)) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(bits, 0, (size_t)n * n * (n / 32) * sizeof(uint32_t), s);
  if (e != cudaSuccess || n_triangles <= 0) return e;
  TriVolume tv{{vol.volume_world_min[0], vol.volume_world_min[1], vol.volume_world_min[2]}, vol.voxel_size_in_world};
  const int warps = (n_triangles + 0) < num_sms * 64 ? n_triangles : num_sms * 64;  // <= 64 warps per SM in flight
  triangles_kernel<<<(warps + 7) / 8, 256, 0, s>>>(positions, n_vertices, indices, n_triangles, tv, n, bits);
  return cudaGetLastError();
}

cudaError_t launch_build_mips(cudaStream_t s, int n, const uint32_t* bits, void* mips, const size_t* offsets,
                              int n_levels, int precision, uint32_t* ticket) {
  MipOffsets mo{};
  for (int i = 0; i < n_levels && i < kMaxVoxelLevels; ++i) mo.off[i] = offsets[i];
  int B = n < 32 ? n : 32;
  int lb = 0;
  while ((1 << (lb + 1)) <= B) ++lb;
  int blocks = (n / B) * (n / B) * (n / B);
  const bool half = precision == DRV_PRECISION_BF16;
  const int L = n_levels - 1;  // levels lb + 1 .. L by the last CTA
  if (half)
    mips_kernel<__half><<<blocks, 256, 0, s>>>(n, B, bits, (__half*)mips, mo, ticket, lb + 1, L);
  else
    mips_kernel<float><<<blocks, 256, 0, s>>>(n, B, bits, (float*)mips, mo, ticket, lb + 1, L);
  return cudaGetLastError();
}

}  // namespace drv
