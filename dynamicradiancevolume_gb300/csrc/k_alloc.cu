// k_alloc.cu — Renderer::AllocateCaches (renderer.cpp:951-992):
// cacheGather.comp (16x16 workgroups, shared-memory neighbour dedupe, corner
// lock by compare-and-swap, compaction by an atomic counter) and
// cachePrepareLighting.comp (indirect-dispatch arguments, a one-thread
// launch after it).
#include "drv_device.cuh"
#include "drv_internal.h"

namespace drv {
namespace {

constexpr int kTile = 16;  // LOCAL_SIZE, cacheGather.comp:11

struct AllocParams {
  DrvVolumeInfo vol;
  DrvPerFrame frame;
  const float* depth;
  int w, h;
  int res, n_cascades;
  int transitions;
  uint32_t max_caches;
  uint32_t* atlas;
  float4* entries;
  int entry_vec4;  // entry stride in float4 units
  int bf16;        // DrvCacheEntryBF16 entries (cell key + BF16 SH) instead of LightCacheEntry
  DrvCacheCounter* counter;
  uint32_t* err;
  CellRecip rc;
  const float* ndc_x;  // NDC x of every pixel column, y of every row (or nullptr: computed)
  const float* ndc_y;
};

// AllocateCaches, cacheGather.comp:32-91. Corners outside the atlas are
// skipped (the reference performs an image atomic there, which GL defines to
// do nothing and return 0, and then allocates an entry nobody can address).
// The 8 compare-and-swaps are independent, so all are issued before any
// result is used, and the won corners take consecutive entries from one
// atomicAdd (entry order is atomic order in the reference as well).
__device__ void allocate_cell(const AllocParams& p, int coord, int cascade) {
  const int res = p.res, res2 = res * res, res3 = res2 * res;
  const int aw = p.n_cascades * res;
  const int base = coord - res3 * cascade;
  const int bz = base / res2, by = (base - bz * res2) / res, bx = base % res;
  const DrvCascade& k = p.vol.cascades[cascade];
  uint32_t won = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    // Corner order of cacheGather.comp:34-44: (0,0,0) (0,1,0) (0,0,1) (0,1,1) (1,...)
    const int lx = bx + (i >> 2), ly = by + (i & 1), lz = bz + ((i >> 1) & 1);
    const int ax = lx + cascade * res;
    if (ax < aw && ly < res && lz < res &&
        atomicCAS(p.atlas + ((size_t)lz * res + ly) * aw + ax, 0u, 0xFFFFFFFFu) == 0u)
      won |= 1u << i;
  }
  if (!won) return;
  const uint32_t first = (uint32_t)atomicAdd(&p.counter->total_light_cache_count, __popc(won));
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (!((won >> i) & 1u)) continue;
    const int lx = bx + (i >> 2), ly = by + (i & 1), lz = bz + ((i >> 1) & 1);
    uint32_t* slot = p.atlas + ((size_t)lz * res + ly) * aw + (lx + cascade * res);
    const uint32_t idx = first + __popc(won & ((1u << i) - 1u));
    if (idx >= p.max_caches) {
      raise_error(p.err, DRV_DEVERR_CAPACITY);  // slot stays locked = empty for apply
      continue;
    }
    float4* e = p.entries + (size_t)idx * p.entry_vec4;
    if (p.bf16) {
      e[0] = make_float4(__uint_as_float(pack_cell(lx, ly, lz, cascade)), 0.f, 0.f, 0.f);
    } else {
      e[0] = make_float4(__fadd_rn(__fmul_rn((float)lx, k.world_voxel_size), k.min[0]),
                         __fadd_rn(__fmul_rn((float)ly, k.world_voxel_size), k.min[1]),
                         __fadd_rn(__fmul_rn((float)lz, k.world_voxel_size), k.min[2]), 0.0f);
    }
    for (int v = 1; v < p.entry_vec4; ++v) e[v] = make_float4(0.f, 0.f, 0.f, 0.f);
    *slot = idx + 1u;  // +1: zero means "cleared" (cacheGather.comp:88)
  }
}

// Eight CTAs per SM (32 registers, no spill): 0.054 -> 0.048 ms at 1080p,
// the compare-and-swap chains' latency hidden by more resident tiles.
__global__ void __launch_bounds__(kTile* kTile, 8) allocate_kernel(AllocParams p) {
  __shared__ int list1[kTile][kTile];
  __shared__ int list2[kTile][kTile];
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int px = blockIdx.x * kTile + lx, py = blockIdx.y * kTile + ly;
  list1[lx][ly] = -1;
  list2[lx][ly] = -1;
  __syncthreads();
  int own = -1, own2 = -1, cascade = -1;
  if (px < p.w && py < p.h) {
    float d = __ldcs(p.depth + (size_t)py * p.w + px);  // read once: streaming
    if (d > 0.0001f) {
      float wp[3];
      if (p.ndc_x)
        reconstruct_world_ndc(p.frame, __ldg(p.ndc_x + px), __ldg(p.ndc_y + py), d, wp);
      else
        reconstruct_world(p.frame, px, py, p.w, p.h, d, wp);
      cascade = select_cascade(p.vol, p.n_cascades, wp);
      own = cache_1d_coord(p.vol, p.rc, p.res, cascade, wp);
      list1[lx][ly] = own;
      if (p.transitions) {
        float t = cascade_transition(p.vol, p.rc, cascade, wp);
        if (t > 0.0f && cascade < p.n_cascades - 1) {
          own2 = cache_1d_coord(p.vol, p.rc, p.res, cascade + 1, wp);
          list2[lx][ly] = own2;
        }
      }
    }
  }
  __syncthreads();
  // cacheGather.comp:141-150: allocate unless the up, left or up-left
  // neighbour registered the same cell; the vector equality of :146 holds
  // only for thread (0,0), so the other threads of row 0 / column 0 compare
  // against themselves and never allocate (kept as in the reference).
  {
    const int ux = max(0, lx - 1), uy = max(0, ly - 1);
    const bool self = (ux == lx && uy == ly);
    if (((list1[lx][uy] != own && list1[ux][ly] != own && list1[ux][uy] != own) || self) && own != -1)
      allocate_cell(p, own, cascade);
  }
  // cacheGather.comp:153-162: transition cells, looking down/right.
  if (p.transitions) {
    const int dx = min(kTile - 1, lx + 1), dy = min(kTile - 1, ly + 1);
    const bool corner = (dx == kTile - 1 && dy == kTile - 1);
    if (((list2[lx][dy] != own2 && list2[dx][ly] != own2 && list2[dx][dy] != own2) || corner) && own2 != -1)
      allocate_cell(p, own2, cascade + 1);
  }
}

// cachePrepareLighting.comp: dispatch size of the lighting pass.
__global__ void prepare_lighting_kernel(DrvCacheCounter* counter, uint32_t max_caches) {
  const uint32_t lit = min((uint32_t)max(counter->total_light_cache_count, 0), max_caches);
  counter->groups_x = (lit + DRV_LIGHTING_THREADS_PER_GROUP - 1) / DRV_LIGHTING_THREADS_PER_GROUP;
  counter->groups_y = 1;
  counter->groups_z = 1;
}

}  // namespace

cudaError_t launch_allocate(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const DrvPerFrame& f,
                            const float* depth, int w, int h, uint32_t* atlas, void* entries, uint32_t entry_stride,
                            DrvCacheCounter* counter, uint32_t* /*ticket: unused*/, uint32_t* err, const float* ndc) {
  AllocParams p;
  p.rc = make_cell_recip(vol);
  p.ndc_x = ndc;
  p.ndc_y = ndc ? ndc + w : nullptr;
  p.vol = vol;
  p.frame = f;
  p.depth = depth;
  p.w = w;
  p.h = h;
  p.res = cfg.cav_res;
  p.n_cascades = cfg.n_cascades;
  p.transitions = cfg.cascade_transition > 0.0f;
  p.max_caches = cfg.max_caches;
  p.atlas = atlas;
  p.entries = (float4*)entries;
  p.entry_vec4 = (int)(entry_stride / 16);
  p.bf16 = cfg.precision == DRV_PRECISION_BF16;
  p.counter = counter;
  p.err = err;
  dim3 block(kTile, kTile), grid((w + kTile - 1) / kTile, (h + kTile - 1) / kTile);
  allocate_kernel<<<grid, block, 0, s>>>(p);
  prepare_lighting_kernel<<<1, 1, 0, s>>>(counter, cfg.max_caches);
  return cudaGetLastError();
}

}  // namespace drv
