// drv_internal.h — context layout and kernel launchers shared by the
// translation units of libdrv_gb300.so. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/drv.h"

namespace drv {

constexpr int kMaxVoxelLevels = 16;
constexpr int kMaxRsmLevels = 16;
constexpr int kMaxLightChunks = 32;       // VPL-block chunks per cache in the light stage
constexpr int kLightChunkMinBlocks = 128;  // shadow blocks per chunk, at least

struct RsmChain {
  int res0 = 0;      // render resolution
  int n_levels = 0;  // levels res0, res0/2, ..., 1
  void* flux[kMaxRsmLevels] = {};  // level 0 (the caller's): F32 or F16 per half0; below: F32
  int16_t* normal[kMaxRsmLevels] = {};
  void* dls[kMaxRsmLevels] = {};
  int half0 = 0;  // level 0's flux and (d, d^2) are F16 (DRV_RSM_F16)
  bool half(int level) const { return level == 0 && half0; }
};

// The per-cache specular envmap atlas (INDIRECT_SPECULAR) and the scalars of
// its path.
struct SpecView {
  uint32_t* levels;  // all levels, level l at levels + off[l] (R11F_G11F_B10F words)
  uint32_t off[8];
  int size;          // SPECULARENVMAP_PERCACHESIZE (power of two)
  int log2size;
  int n_levels;      // log2size + 1
  int atlas;         // atlas side at level 0 (power of two)
  int per_row;       // caches per atlas row: atlas / size
  float norm;        // BlinnNormalization(GetBlinnPhongExponentForHemispherePixel(size))
  float cam[3];      // CameraPosition
  // The apply's copy of every level, per cache and in FP16 (RGB + 0, 8 bytes
  // a texel; exact: R11/G11/B10 values are FP16 values): cache c's level l
  // texel (x, y) at half[c * words + loff[l] + y * (size >> l) + x].
  uint2* half;
  uint32_t words;
  uint32_t loff[8];
};

// Per-light arguments of the light stage.
struct LightArgs {
  const void* vpls;  // DrvVPL (FP32 precision) or DrvVPLBF16
  const DrvShadowCone* cones;
  int n_vpls;
  int interval;  // IndirectShadowComputationSampleInterval
  const float4* records = nullptr;  // the cull's VPL plane records (make_cull_record), or none
};

struct LightLaunch {
  LightArgs lights[DRV_MAX_LIGHTS];
  int n_lights;
};

// The voxel pyramid as the cone tracer reads it.
struct VoxelInputs {
  const uint8_t* corners = nullptr;     // level 0, corner-packed bytes, x fastest
  const void* mips = nullptr;           // levels 1..L concatenated (float, or half with BF16 precision)
  const size_t* mip_offsets = nullptr;  // texel offset of each level in mips
  const uint4* records = nullptr;       // corner-packed mip records of levels 1..record_levels (optional)
  const uint32_t* record_offsets = nullptr;  // record offset of each level (index 1..record_levels + 1)
  int record_levels = 0;
};

// Levels that get corner-packed FP16 mip records: every level with BF16
// precision (FP16 texels); levels 1..3 with FP32 precision, whose texels
// k / 8^l (8^l <= 512) are exact in FP16.
inline int record_levels_for(int precision, int n_levels) {
  const int L = n_levels - 1;
  return precision == DRV_PRECISION_BF16 ? L : (L < 3 ? L : 3);
}

// Bytes between consecutive cache entries: DrvCacheEntryBF16 (64 B) with BF16
// precision, else LightCacheEntry std430 (lightcache.glsl:33-76): 64 B for
// SH1, 128 B for SH2. Every path that addresses entries takes it from here.
inline uint32_t entry_stride_for(const DrvConfig& cfg) {
  return cfg.precision == DRV_PRECISION_BF16 ? 64u : (cfg.sh_order == 2 ? 128u : 64u);
}

// Device scratch of the light stage. partials: [max_caches * max_chunks][27]
// chunk sums; tickets: one per cache; work: {next unit, retired CTAs}. Tickets
// and work are zero between launches (each launch leaves them zero).
struct LightScratch {
  float* partials;
  uint32_t* tickets;
  uint32_t* work;
  int max_chunks;
};

// Compacted (cache, shadow block) pairs that can contribute, in the split
// light stage. Pair i: cache[i], block[i] (kNoPair: unused slot), shadow[i].
// info[c] = {first pair of cache c, pair count} (count kPairOverflow: the
// list was full, the gather traces that cache's cones itself).
// order lists the pairs to trace by cone class (kConeClasses classes of
// expected step count and width, cls[i]; 0xFF: not traced), so that a
// warp's lanes march cones of one length that take one sampling path; with
// the surrogate only the pairs it is not confident about are classified.
// counters (zeroed before each light stage): [0] pairs claimed, [1] level-0
// corner bytes, [2] mip records and [7] plain mip texels the cone pass read
// (its counting instance only), [3] pairs the surrogate left to the cone
// ([4] zero), [5] pairs the surrogate evaluated, [6] the cone pass's work cursor,
// [8 + c] pairs of class c, [8 + kConeClasses + c] class c's scatter cursor,
// [kGatherUnitsCounter] the gather units listed in units.
// The gather takes a cache's run in units of kGatherChunk pairs (units[u] =
// {cache, unit index}, listed by the cull), a warp per unit; a cache of
// several units sums their partials (partials: a slot per
// unit, full units at the index of the multiple of kGatherChunk they cover,
// each cache's last unit at partial_tail + cache) in unit order, done by the
// unit that finishes last (tickets: per cache, zeroed by the cull).
constexpr uint32_t kNoPair = 0xFFFFFFFFu;
constexpr uint32_t kPairOverflow = 0xFFFFFFFFu;
constexpr int kMaxSplitBlocks = 65536;  // shadow blocks per frame the split stage handles
constexpr int kConeClasses = 32;
constexpr int kGatherUnitsCounter = 8 + 2 * kConeClasses;
constexpr int kPairCounters = kGatherUnitsCounter + 8;
constexpr uint32_t kGatherChunk = 512;  // pairs per gather unit (a multiple of 32)
constexpr int kGatherSlotFloats = 27;   // partial sums per unit slot (NK * 3 <= 27)
struct PairList {
  uint32_t* cache;
  uint32_t* block;
  float* shadow;
  uint32_t* order;
  uint8_t* cls;
  uint32_t* info;
  uint32_t* counters;
  uint32_t* tickets;    // [max_caches]
  float* partials;      // [partial_tail + max_caches][kGatherSlotFloats]
  uint2* units;         // [partial_tail + max_caches]
  uint32_t partial_tail;
  uint32_t cap;
};
// Slots of the gather's partial sums (and bound on its units) a pair list of
// `cap` pairs needs.
inline size_t gather_partial_slots(uint64_t cap, uint32_t max_caches) {
  return (size_t)(cap / kGatherChunk + 1) + max_caches;
}

// Ray frame of a pinhole camera: direction = normalize(fwd + nx*right + ny*up).
struct RayFrame {
  float origin[3];
  float fwd[3];
  float right[3];  // already scaled by tan(fov_x / 2)
  float up[3];     // already scaled by tan(fov_y / 2)
};

struct Context {
  DrvConfig cfg{};
  cudaStream_t stream = nullptr;       // owned
  cudaStream_t user_stream = nullptr;  // set by drv_set_stream, borrowed (may be the legacy stream 0)
  bool has_user_stream = false;
  // drv_frame runs the RSM/VPL stage and the voxel stage on two side streams,
  // concurrently with the cache allocation on the context's stream (fork and
  // join by events, so the frame stays one capturable DAG); while a stage is
  // issued there, `cur` redirects s() to its side stream.
  // Side stream 2 builds the corner grid while the mips are built.
  cudaStream_t side[3] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[3] = {}, vox_fork_ev = nullptr;
  cudaStream_t cur = nullptr;
  cudaStream_t s() const { return cur ? cur : (has_user_stream ? user_stream : stream); }
  int device = 0;
  int num_sms = 0;
  std::string last_error;

  // Caches (LightCacheBuffer, CAV atlas, counter).
  void* entries = nullptr;
  uint32_t entry_stride = 0;
  uint32_t* atlas = nullptr;
  size_t atlas_words = 0;
  DrvCacheCounter* counter = nullptr;
  uint32_t* scratch_words = nullptr;  // [0] alloc ticket, [1] device error bits, [4] input-check bits, [5] mips ticket
  uint32_t* mips_ticket() const { return scratch_words + 5; }
  uint32_t* input_err() const { return scratch_words + 4; }
  // Voxels.
  uint32_t* voxel_bits = nullptr;
  size_t voxel_words = 0;
  float* ndc = nullptr;  // NDC x of each pixel column (width), then y of each row (height): allocation
  float* srgb = nullptr;  // the GL sRGB decode of the 256 byte values (DRV_ALBEDO_SRGB8)
  unsigned long long* raster_keys = nullptr;  // mesh producers' per-pixel visibility (drv_raster_*)
  size_t raster_keys_cap = 0;
  uint8_t* vox_corners = nullptr;  // level 0, corner-packed bytes, x fastest
  void* mips = nullptr;  // levels 1..L concatenated: float (FP32 precision) or half (BF16 precision)
  size_t mip_offset[kMaxVoxelLevels] = {};
  uint4* vox_records = nullptr;  // corner-packed mip records (voxel_sample.cuh)
  uint32_t record_offset[kMaxVoxelLevels + 1] = {};
  int record_levels = 0;
  // The voxel inputs of the light stage: without the mip records when
  // DrvTuning.plain_voxel_reads asks for it.
  VoxelInputs light_voxels() const {
    VoxelInputs v = voxels();
    if (tuning.plain_voxel_reads) {
      v.records = nullptr;
      v.record_levels = 0;
    }
    return v;
  }
  VoxelInputs voxels() const {
    return VoxelInputs{vox_corners, mips, mip_offset, vox_records, record_offset, record_levels};
  }
  int n_voxel_levels = 0;
  // RSM + VPLs per light.
  RsmChain rsm[DRV_MAX_LIGHTS];
  void* vpls[DRV_MAX_LIGHTS] = {};  // DrvVPL or DrvVPLBF16 per cfg.precision
  DrvShadowCone* cones[DRV_MAX_LIGHTS] = {};
  float4* vpl_records[DRV_MAX_LIGHTS] = {};  // the cull's plane record of every VPL (written by the extraction)
  int n_vpls[DRV_MAX_LIGHTS] = {};
  int n_cones[DRV_MAX_LIGHTS] = {};
  int interval[DRV_MAX_LIGHTS] = {};
  int n_lights = 0;
  // Scene boxes: pinned staging + device copy.
  DrvBox* h_boxes = nullptr;
  DrvBox* d_boxes = nullptr;
  int box_capacity = 0;
  int resident_boxes = -1;  // boxes currently on the device (-1: none)
  // Light-stage partial sums: [max_caches * kMaxLightChunks][27] and a ticket per cache.
  float* light_scratch = nullptr;
  uint32_t* light_tickets = nullptr;
  // Pair list of the split light stage (one allocation, carved up).
  void* pair_mem = nullptr;
  PairList pairs{};
  DrvTuning tuning{};
  // Events between the split light stage's kernels (DrvTuning.time_kernels).
  cudaEvent_t lk_events[2 * DRV_LK_COUNT] = {};  // start and end of each light-stage kernel slot
  bool lk_recorded = false;
  // Visibility surrogate: packed BF16 inference weights and their feature set.
  void* sur_weights = nullptr;
  bool sur_ready = false;
  int sur_features = DRV_SURROGATE_FEATURES_SEGMENT8;
  DrvVolumeInfo last_volume{};  // volume of the last drv_allocate_caches (cache positions refer to it)
  // Indirect specular: the envmap atlas, all levels in one allocation.
  uint32_t* spec_env = nullptr;
  uint32_t spec_off[8] = {};
  int spec_atlas = 0;
  int spec_levels = 0;
  uint2* spec_half = nullptr;  // the apply's per-cache FP16 copy (SpecView::half)
  bool spec_lit = false;       // a light stage has written the level-0 envmaps
  bool spec_ready = false;     // the envmaps were prepared after the last light stage
};

int light_chunks(int total_blocks, int max_chunks);

RayFrame make_ray_frame(const float pos[3], const float dir[3], const float up[3], double tan_x, double tan_y);

// ---- launchers (each returns cudaGetLastError() of its launch) -----------
cudaError_t launch_raycast_gbuffer(cudaStream_t s, const DrvBox* boxes, int n_boxes, RayFrame rf,
                                   const float* view_proj, int w, int h, DrvGBufferOut out);
cudaError_t launch_raycast_rsm(cudaStream_t s, const DrvBox* boxes, int n_boxes, const DrvSpotLight& L, DrvRSMOut out);
cudaError_t launch_raster_gbuffer(cudaStream_t s, const DrvMesh& mesh, RayFrame rf, const float* view_proj, int w,
                                  int h, unsigned long long* keys, DrvGBufferOut out, int num_sms);
cudaError_t launch_raster_rsm(cudaStream_t s, const DrvMesh& mesh, const DrvSpotLight& L, unsigned long long* keys,
                              DrvRSMOut out, int num_sms);
// Up to three RSM downsample passes res -> res/2 -> ... in one launch;
// fo/no/dlo[k] receive level k + 1 (F32 flux and (d, d^2), RG16I normals).
cudaError_t launch_rsm_chain(cudaStream_t s, int res, int passes, const void* flux, const int16_t* nrm,
                             const void* dls, int src_half, float* const* fo, int16_t* const* no, float* const* dlo);
cudaError_t launch_extract_vpls(cudaStream_t s, const DrvSpotLight& L, int res, const void* flux, const int16_t* nrm,
                                const void* dls, int read_half, const void* dls_shadow, int shadow_half, void* vpls,
                                DrvShadowCone* cones, int precision, float4* records);
cudaError_t launch_voxelize(cudaStream_t s, const DrvBox* boxes, int n_boxes, const DrvVolumeInfo& vol, int n,
                            uint32_t* bits);
cudaError_t launch_voxelize_triangles(cudaStream_t s, const float* positions, int n_vertices, const uint32_t* indices,
                                      int n_triangles, const DrvVolumeInfo& vol, int n, uint32_t* bits, int num_sms);
// ticket: a zeroed word of the context's (the last CTA builds the levels
// above one 32^3 block and zeroes it again).
cudaError_t launch_build_mips(cudaStream_t s, int n, const uint32_t* bits, void* mips, const size_t* offsets,
                              int n_levels, int precision, uint32_t* ticket);
cudaError_t launch_build_corners(cudaStream_t s, int n, const uint32_t* bits, uint8_t* corners);
cudaError_t launch_build_records(cudaStream_t s, int n, const void* mips, const size_t* mip_offsets, int precision,
                                 uint4* records, const uint32_t* record_offsets, int record_levels);
cudaError_t launch_allocate(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const DrvPerFrame& f,
                            const float* depth, int w, int h, uint32_t* atlas, void* entries, uint32_t entry_stride,
                            DrvCacheCounter* counter, uint32_t* ticket, uint32_t* err, const float* ndc = nullptr);
cudaError_t launch_light_caches(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                                const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                                const VoxelInputs& vox, const LightScratch& scratch, int num_sms);
// The learned visibility surrogate of a light stage: packed weights
// (nullptr: plain cones), feature set (kFeature*), confidence threshold, the
// device error word its bounded waits report to, and the timeout test hook
// (DrvTuning.surrogate_wait_test).
struct SurrogateArgs {
  const void* weights = nullptr;
  int feature_set = 0;
  float threshold = 0.5f;
  uint32_t* err = nullptr;
  int hold_commit = 0;
};

// Execution knobs of the split light stage (DrvTuning): CTAs per SM of the
// cone and gather passes (0: as many as fit), the cull's caches per pass (2,
// 4 or 8) and the gather's threads per cache (128 or 256), and the cone
// pass's measuring instance.
struct SplitKnobs {
  int cone_ctas_per_sm = 0;
  int gather_ctas_per_sm = 0;
  int cull_caches_per_pass = 4;
  int gather_threads = 512;
  int gather_wait_test = 0;  // test hook: the gather's VPL copies are withheld (its bounded wait runs out)
  bool count_voxel_reads = false;
};

// Split light stage: cull -> (cones | surrogate MLP + cones of the
// unconfident pairs) -> gather.
bool light_split_supported(const DrvConfig& cfg, const LightLaunch& ll);
cudaError_t launch_light_split(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const LightLaunch& ll,
                               const DrvCacheCounter* counter, void* entries, uint32_t entry_stride,
                               const VoxelInputs& vox, const PairList& pairs, const SurrogateArgs& sur,
                               uint32_t* err, const SplitKnobs& knobs, int num_sms, cudaEvent_t* events = nullptr,
                               cudaEvent_t voxels_ready = nullptr);
cudaError_t launch_bruteforce_rsm(cudaStream_t s, const DrvPerFrame& f, const DrvGBufferView& g,
                                  const float* rough_metal, const LightLaunch& ll, int bf16, float* out_rgb,
                                  const float* srgb);
// spec: the envmap atlas when specular is on, else nullptr.
// err: device error word (DRV_DEVERR_BOUNDS for an atlas slot past the count).
// tensor_core: BF16 entries evaluated a warp's cells at a time on the tensor
// cores instead of per pixel on the FP32 pipes (DrvTuning.tensor_core_apply).
cudaError_t launch_apply(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol, const DrvPerFrame& f,
                         const DrvGBufferView& g, const uint32_t* atlas, const void* entries, uint32_t entry_stride,
                         const DrvCacheCounter* counter, float* out_rgb, const float* srgb,
                         const SpecView* spec = nullptr, uint32_t* err = nullptr, bool tensor_core = false);
// Sets DRV_DEVERR_NUMERIC in *word when any of n values (float, or half when
// half is nonzero) is NaN or infinite.
cudaError_t launch_scan_finite(cudaStream_t s, const void* data, size_t n, int half, uint32_t* word);
// Indirect specular (k_specular.cu): the level-0 envmaps of the allocated
// caches (pairs: the split stage's pair list with its shadowing; nullptr:
// every shadow block, cones traced here), then their mips and hole fill.
SpecView make_spec_view(const DrvConfig& cfg, uint32_t* levels, const uint32_t off[8], int atlas, uint2* half,
                        const DrvPerFrame& f);
cudaError_t launch_specular_gather(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol,
                                   const LightLaunch& ll, const DrvCacheCounter* counter, void* entries,
                                   uint32_t entry_stride, const VoxelInputs& vox, const PairList* pairs,
                                   const SpecView& sv, int num_sms);
cudaError_t launch_envmap_prepare(cudaStream_t s, const SpecView& sv, const DrvCacheCounter* counter,
                                  uint32_t max_caches, int fill, int num_sms);

size_t surrogate_weights_bytes();
size_t surrogate_train_scratch_floats(int n);
cudaError_t launch_pack_surrogate_weights(cudaStream_t s, const float* params, void* weights);
cudaError_t launch_surrogate_eval(cudaStream_t s, const void* weights, const float* X, int n, float* out,
                                  uint32_t* err, int num_sms);
cudaError_t launch_surrogate_pairs(cudaStream_t s, const DrvConfig& cfg, const DrvVolumeInfo& vol,
                                   const LightLaunch& ll, const DrvCacheCounter* counter, const void* entries,
                                   uint32_t entry_stride, const VoxelInputs& vox, uint64_t seed, int n_pairs,
                                   float* features, float* targets, int feature_set);
cudaError_t launch_surrogate_train_step(cudaStream_t s, const float* X, const float* Y, int n, float* params,
                                        float* m, float* v, float* scratch, int step, float lr, float conf_tau,
                                        float weight_decay, float* loss_out);


}  // namespace drv

// The opaque handle of the C ABI is the context itself.
struct DrvContext : drv::Context {};

