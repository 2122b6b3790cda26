// api.cu — the extern "C" entry points of include/drv.h: context lifetime,
// resident buffers and the per-frame stage sequence of the reference's
// Renderer::Draw (renderer.cpp:539-594). Every entry point validates its
// arguments, enqueues work on the context stream and returns a drv_status; no
// exception crosses the ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "drv_internal.h"

using drv::Context;

namespace {

drv_status fail(DrvContext* ctx, drv_status st, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return st;
}

drv_status cuda_check(DrvContext* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return DRV_OK;
  return fail(ctx, DRV_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define DRV_TRY_CUDA(ctx, expr)                              \
  do {                                                       \
    drv_status _st = cuda_check((ctx), (expr), #expr);       \
    if (_st != DRV_OK) return _st;                           \
  } while (0)

int ilog2(int v) {
  int l = 0;
  while ((1 << (l + 1)) <= v) ++l;
  return l;
}

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

void release(Context* c) {
  cudaFree(c->entries);
  cudaFree(c->atlas);
  cudaFree(c->counter);
  cudaFree(c->voxel_bits);
  cudaFree(c->mips);
  cudaFree(c->vox_corners);
  cudaFree(c->vox_records);
  cudaFree(c->ndc);
  cudaFree(c->srgb);
  cudaFree(c->raster_keys);
  cudaFree(c->spec_env);
  cudaFree(c->spec_half);

  cudaFree(c->light_scratch);
  cudaFree(c->light_tickets);
  cudaFree(c->sur_weights);
  for (cudaEvent_t e : c->lk_events)
    if (e) cudaEventDestroy(e);
  cudaFree(c->pair_mem);
  for (int l = 0; l < DRV_MAX_LIGHTS; ++l) {
    for (int k = 1; k < drv::kMaxRsmLevels; ++k) {
      cudaFree(c->rsm[l].flux[k]);
      cudaFree(c->rsm[l].normal[k]);
      cudaFree(c->rsm[l].dls[k]);
    }
    cudaFree(c->vpls[l]);
    cudaFree(c->cones[l]);
    cudaFree(c->vpl_records[l]);
  }
  cudaFree(c->d_boxes);
  cudaFreeHost(c->h_boxes);
  for (int i = 0; i < 3; ++i) {
    if (c->side[i]) cudaStreamDestroy(c->side[i]);
    if (c->join_ev[i]) cudaEventDestroy(c->join_ev[i]);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->vox_fork_ev) cudaEventDestroy(c->vox_fork_ev);
  if (c->stream) cudaStreamDestroy(c->stream);
}

drv_status validate_config(const DrvConfig* c, std::string& why) {
  if (c->width < 1 || c->height < 1) return why = "width/height must be positive", DRV_ERR_INVALID_ARG;
  if (c->sh_order != 1 && c->sh_order != 2) return why = "sh_order must be 1 or 2", DRV_ERR_INVALID_ARG;
  if (c->n_cascades < 1 || c->n_cascades > DRV_MAX_CASCADES) return why = "n_cascades must be 1..4", DRV_ERR_INVALID_ARG;
  if (c->cav_res < 2 || c->cav_res > 256) return why = "cav_res must be 2..256", DRV_ERR_INVALID_ARG;
  if (!is_pow2(c->voxel_res) || c->voxel_res < 32 || c->voxel_res > 1024)
    return why = "voxel_res must be a power of two in 32..1024", DRV_ERR_INVALID_ARG;
  if (c->max_caches < 1) return why = "max_caches must be positive", DRV_ERR_INVALID_ARG;
  if (c->max_cone_steps < 1 || c->max_cone_steps > 4096) return why = "max_cone_steps must be 1..4096", DRV_ERR_INVALID_ARG;
  if (c->max_lights < 1 || c->max_lights > DRV_MAX_LIGHTS) return why = "max_lights must be 1..16", DRV_ERR_INVALID_ARG;
  if (!is_pow2(c->max_rsm_resolution) || c->max_rsm_resolution > 4096)
    return why = "max_rsm_resolution must be a power of two <= 4096", DRV_ERR_INVALID_ARG;
  if (c->precision != DRV_PRECISION_FP32 && c->precision != DRV_PRECISION_BF16)
    return why = "precision must be DRV_PRECISION_FP32 or DRV_PRECISION_BF16", DRV_ERR_INVALID_ARG;
  if (c->visibility != DRV_VISIBILITY_CONE && c->visibility != DRV_VISIBILITY_SURROGATE)
    return why = "visibility must be DRV_VISIBILITY_CONE or DRV_VISIBILITY_SURROGATE", DRV_ERR_INVALID_ARG;
  if (c->visibility == DRV_VISIBILITY_SURROGATE && !c->indirect_shadow)
    return why = "the visibility surrogate replaces the indirect-shadow cone: indirect_shadow must be on",
           DRV_ERR_INVALID_ARG;
  if (c->sh2_sign != DRV_SH2_SIGN_REFERENCE && c->sh2_sign != DRV_SH2_SIGN_FIXED)
    return why = "sh2_sign must be 0 or 1", DRV_ERR_INVALID_ARG;
  if (c->output_format != DRV_OUTPUT_RGB32F && c->output_format != DRV_OUTPUT_RGBA16F)
    return why = "output_format must be DRV_OUTPUT_RGB32F or DRV_OUTPUT_RGBA16F", DRV_ERR_INVALID_ARG;
  if (c->output_blend != DRV_OUTPUT_WRITE && c->output_blend != DRV_OUTPUT_ADD)
    return why = "output_blend must be DRV_OUTPUT_WRITE or DRV_OUTPUT_ADD", DRV_ERR_INVALID_ARG;
  if (c->specular_envmap_size != 0 &&
      (!is_pow2(c->specular_envmap_size) || c->specular_envmap_size < 4 || c->specular_envmap_size > 64))
    return why = "specular_envmap_size must be 0 or a power of two in 4..64", DRV_ERR_INVALID_ARG;
  if (c->specular_fill_level < 0 || (c->specular_fill_level > 0 && (c->specular_envmap_size == 0 ||
                                     (1 << c->specular_fill_level) > c->specular_envmap_size)))
    return why = "specular_fill_level must be 0..log2(specular_envmap_size)", DRV_ERR_INVALID_ARG;
  return DRV_OK;
}

// Texel arrays must be aligned to their texel's scalar (the RG16I normal is
// read as one 32-bit word per pixel).
// Chunk partials of the single-launch light stage, a ticket per cache and
// the two words of its unit counter (tickets and counter are reset by the
// kernel that consumes them, so they are zeroed once here). About 3.5 KB per
// cache with SH2, so contexts that only run the split stage never hold it.
cudaError_t ensure_single_scratch(Context* c) {
  if (c->light_scratch) return cudaSuccess;
  const size_t n = c->cfg.max_caches;
  cudaError_t e = cudaMalloc(&c->light_scratch, n * drv::kMaxLightChunks * (c->cfg.sh_order == 2 ? 27 : 12) * 4);
  if (e != cudaSuccess) return e;
  if ((e = cudaMalloc(&c->light_tickets, (n + 2) * 4)) != cudaSuccess) return e;
  return cudaMemset(c->light_tickets, 0, (n + 2) * 4);
}

// (Re)allocates the pair list for `cap` pairs (one allocation, carved up).
cudaError_t alloc_pairs(Context* c, uint64_t cap) {
  if (cap > 0xFFFFFFF0ull) return cudaErrorInvalidValue;
  if (c->pair_mem) {
    cudaError_t e = cudaStreamSynchronize(c->s());
    if (e != cudaSuccess) return e;
    cudaFree(c->pair_mem);
    c->pair_mem = nullptr;
  }
  // Every array starts on a 16-byte boundary (the unit list is read and
  // written as 8-byte vectors).
  const size_t slots = drv::gather_partial_slots(cap, c->cfg.max_caches);
  const size_t mc = c->cfg.max_caches;
  size_t bytes = 0;
  auto take = [&bytes](size_t n) {
    const size_t at = bytes;
    bytes = (bytes + n + 15) & ~(size_t)15;
    return at;
  };
  const size_t o_cache = take(cap * 4), o_block = take(cap * 4), o_shadow = take(cap * 4),
               o_order = take(cap * 4), o_info = take(mc * 8),
               o_counters = take(drv::kPairCounters * 4), o_tickets = take(mc * 4),
               o_partials = take(slots * drv::kGatherSlotFloats * 4), o_units = take(slots * sizeof(uint2)),
               o_cls = take(cap);
  cudaError_t e = cudaMalloc(&c->pair_mem, bytes);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemset(c->pair_mem, 0, bytes)) != cudaSuccess) return e;
  char* m = static_cast<char*>(c->pair_mem);
  c->pairs.cache = reinterpret_cast<uint32_t*>(m + o_cache);
  c->pairs.block = reinterpret_cast<uint32_t*>(m + o_block);
  c->pairs.shadow = reinterpret_cast<float*>(m + o_shadow);
  c->pairs.order = reinterpret_cast<uint32_t*>(m + o_order);
  c->pairs.info = reinterpret_cast<uint32_t*>(m + o_info);
  c->pairs.counters = reinterpret_cast<uint32_t*>(m + o_counters);
  c->pairs.tickets = reinterpret_cast<uint32_t*>(m + o_tickets);
  c->pairs.partials = reinterpret_cast<float*>(m + o_partials);
  c->pairs.partial_tail = (uint32_t)(cap / drv::kGatherChunk + 1);
  c->pairs.units = reinterpret_cast<uint2*>(m + o_units);
  c->pairs.cls = reinterpret_cast<uint8_t*>(m + o_cls);
  c->pairs.cap = (uint32_t)cap;
  return cudaSuccess;
}

bool views_ok(const DrvGBufferView* g, const DrvConfig& c) {
  return g && g->depth && g->normal && g->albedo && g->width == c.width && g->height == c.height &&
         (g->normal_format == DRV_NORMAL_RG16I || g->normal_format == DRV_NORMAL_F32X3) &&
         (g->albedo_format == DRV_ALBEDO_F32X3 || g->albedo_format == DRV_ALBEDO_SRGB8) &&
         reinterpret_cast<uintptr_t>(g->depth) % 4 == 0 && reinterpret_cast<uintptr_t>(g->normal) % 4 == 0 &&
         (g->albedo_format == DRV_ALBEDO_SRGB8 || reinterpret_cast<uintptr_t>(g->albedo) % 4 == 0);
}

// The apply's roughness / metallic input: needed only with specular on.
bool rough_metal_ok(const DrvGBufferView* g, const DrvConfig& c) {
  if (c.specular_envmap_size == 0) return true;
  if (!g->rough_metal) return false;
  if (g->rough_metal_format == DRV_ROUGH_METAL_RG8) return reinterpret_cast<uintptr_t>(g->rough_metal) % 2 == 0;
  return g->rough_metal_format == DRV_ROUGH_METAL_F32 && reinterpret_cast<uintptr_t>(g->rough_metal) % 8 == 0;
}

// The GL 4.5 sRGB decode (section 8.24) of the 256 byte values, evaluated in
// double and rounded to float.
void srgb_decode_table(float out[256]) {
  for (int b = 0; b < 256; ++b) {
    const double cs = b / 255.0;
    out[b] = (float)(cs <= 0.04045 ? cs / 12.92 : std::pow((cs + 0.055) / 1.055, 2.4));
  }
}

}  // namespace

extern "C" {

int drv_struct_sizes(uint32_t* out, int capacity) {
  const uint32_t s[] = {sizeof(DrvConfig),     sizeof(DrvCascade),    sizeof(DrvVolumeInfo), sizeof(DrvPerFrame),
                        sizeof(DrvSpotLight),  sizeof(DrvLightDesc),  sizeof(DrvCamera),     sizeof(DrvBox),
                        sizeof(DrvScene),      sizeof(DrvGBufferView), sizeof(DrvGBufferOut), sizeof(DrvRSMView),
                        sizeof(DrvRSMOut),     sizeof(DrvVPL),        sizeof(DrvShadowCone), sizeof(DrvCacheCounter),
                        sizeof(DrvBuffers),    sizeof(DrvTuning),     sizeof(DrvMesh)};
  int n = (int)(sizeof(s) / sizeof(s[0]));
  if (!out) return n;
  int k = capacity < n ? capacity : n;
  for (int i = 0; i < k; ++i) out[i] = s[i];
  return k;
}

drv_status drv_create(const DrvConfig* cfg, DrvContext** out) {
  if (!cfg || !out) return DRV_ERR_INVALID_ARG;
  *out = nullptr;
  std::string why;
  drv_status st = validate_config(cfg, why);
  if (st != DRV_OK) return st;
  DrvContext* c = new (std::nothrow) DrvContext();
  if (!c) return DRV_ERR_CUDA;
  c->cfg = *cfg;
  auto bail = [&](cudaError_t e) {
    release(c);
    delete c;
    (void)e;
    return DRV_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&c->device)) != cudaSuccess) return bail(e);
  if ((e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device)) != cudaSuccess) return bail(e);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
  // The side streams carry the frame's longest dependency chains (voxels,
  // RSM): highest priority, so their small launches are not queued behind
  // the allocation's CTAs.
  int least = 0, greatest = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess) return bail(e);
  for (int i = 0; i < 3; ++i) {
    if ((e = cudaStreamCreateWithPriority(&c->side[i], cudaStreamNonBlocking, greatest)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming)) != cudaSuccess) return bail(e);
  }
  if ((e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
  if ((e = cudaEventCreateWithFlags(&c->vox_fork_ev, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
  // LightCacheBuffer: 64 B (SH1) or 128 B (SH2) entries (lightcache.glsl:33-76);
  // DrvCacheEntryBF16 (64 B) in BF16 precision.
  c->entry_stride = drv::entry_stride_for(*cfg);
  if ((e = cudaMalloc(&c->entries, (size_t)cfg->max_caches * c->entry_stride)) != cudaSuccess) return bail(e);
  c->atlas_words = (size_t)cfg->n_cascades * cfg->cav_res * cfg->cav_res * cfg->cav_res;
  if ((e = cudaMalloc(&c->atlas, c->atlas_words * 4)) != cudaSuccess) return bail(e);
  // counter (16 B) + ticket + error word (cleared by every allocation, 32 B in
  // all), then the input-check word (read and cleared by drv_get_error) and
  // the opacity mips' ticket (reset by its own kernel), one allocation.
  if ((e = cudaMalloc(&c->counter, 64)) != cudaSuccess) return bail(e);
  c->scratch_words = reinterpret_cast<uint32_t*>(c->counter + 1);
  if ((e = cudaMemset(c->counter, 0, 64)) != cudaSuccess) return bail(e);
  // Voxel level 0 (bitmask) and FP32 mips.
  const int N = cfg->voxel_res;
  c->voxel_words = (size_t)N * N * N / 32;
  if ((e = cudaMalloc(&c->voxel_bits, c->voxel_words * 4)) != cudaSuccess) return bail(e);
  c->n_voxel_levels = ilog2(N) + 1;
  size_t off = 0;
  for (int l = 1; l < c->n_voxel_levels; ++l) {
    c->mip_offset[l] = off;
    size_t n = (size_t)(N >> l);
    off += n * n * n;
  }
  if ((e = cudaMalloc(&c->mips, off * 4)) != cudaSuccess) return bail(e);
  if ((e = cudaMalloc(&c->vox_corners, (size_t)N * N * N)) != cudaSuccess) return bail(e);
  {
    // NDC of every pixel column and row, computed as the kernels would
    // (2 * ((p + 0.5) / size) - 1 in binary32, no contraction): a table read
    // replaces two IEEE divisions per pixel in the allocation.
    std::vector<float> ndc((size_t)cfg->width + cfg->height);
    for (int x = 0; x < cfg->width; ++x) {
      const float t = ((float)x + 0.5f) / (float)cfg->width;
      ndc[x] = t * 2.0f - 1.0f;
    }
    for (int y = 0; y < cfg->height; ++y) {
      const float t = ((float)y + 0.5f) / (float)cfg->height;
      ndc[cfg->width + y] = t * 2.0f - 1.0f;
    }
    if ((e = cudaMalloc(&c->ndc, ndc.size() * sizeof(float))) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->ndc, ndc.data(), ndc.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail(e);
    float srgb[256];
    srgb_decode_table(srgb);
    if ((e = cudaMalloc(&c->srgb, sizeof(srgb))) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->srgb, srgb, sizeof(srgb), cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
  }
  c->record_levels = drv::record_levels_for(cfg->precision, c->n_voxel_levels);
  uint32_t records = 0;
  for (int l = 1; l <= c->record_levels; ++l) {
    c->record_offset[l] = records;
    const uint32_t n = (uint32_t)(N >> l);
    records += n * n * n;
  }
  c->record_offset[c->record_levels + 1] = records;
  if (records && (e = cudaMalloc(&c->vox_records, (size_t)records * 16)) != cudaSuccess) return bail(e);

  // The single-launch light stage's scratch, where frames need it from the
  // start (no indirect shadow); otherwise on first use (ensure_single_scratch).
  if (!cfg->indirect_shadow && (e = ensure_single_scratch(c)) != cudaSuccess) return bail(e);
  // RSM chains (levels below the caller's render-resolution level) and VPLs.
  const int R = cfg->max_rsm_resolution;
  for (int l = 0; l < cfg->max_lights; ++l) {
    for (int k = 1; (R >> k) >= 1 && k < drv::kMaxRsmLevels; ++k) {
      size_t n = (size_t)(R >> k) * (R >> k);
      if ((e = cudaMalloc(&c->rsm[l].flux[k], n * 12)) != cudaSuccess) return bail(e);
      if ((e = cudaMalloc(&c->rsm[l].normal[k], n * 4)) != cudaSuccess) return bail(e);
      if ((e = cudaMalloc(&c->rsm[l].dls[k], n * 8)) != cudaSuccess) return bail(e);
    }
    if ((e = cudaMalloc(&c->vpls[l], (size_t)R * R * sizeof(DrvVPL))) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&c->cones[l], (size_t)R * R * sizeof(DrvShadowCone))) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&c->vpl_records[l], (size_t)R * R * sizeof(float4))) != cudaSuccess) return bail(e);
  }
  if ((e = cudaMalloc(&c->sur_weights, drv::surrogate_weights_bytes())) != cudaSuccess) return bail(e);
  // Pair list of the split light stage: room for 256 contributing shadow
  // blocks per cache on average (clamped to [2^22, 2^26] pairs, 21 B each:
  // 88 MB .. 1.4 GB; DrvTuning.pair_capacity grows it); caches beyond a full
  // list are traced by the gather itself, with exact cones also when the
  // surrogate is on.
  if ((e = alloc_pairs(c, std::min<uint64_t>(std::max<uint64_t>((uint64_t)cfg->max_caches * 256u, 1ull << 22),
                                             1ull << 26))) != cudaSuccess)
    return bail(e);
  if (cfg->specular_envmap_size > 0) {
    // AllocateCacheData (renderer.cpp:253, 279-287): an atlas of side
    // 2^ceil(log2(ceil(sqrt(max_caches)) * size)) with log2(size) + 1 levels.
    const int S = cfg->specular_envmap_size;
    const uint64_t per_side = (uint64_t)std::ceil(std::sqrt((double)cfg->max_caches));
    uint64_t side = 1;
    while (side < per_side * (uint64_t)S) side <<= 1;
    if (side > 65536) return bail(cudaErrorInvalidValue);
    c->spec_atlas = (int)side;
    c->spec_levels = ilog2(S) + 1;
    uint64_t words = 0;
    for (int l = 0; l < c->spec_levels; ++l) {
      c->spec_off[l] = (uint32_t)words;
      words += (side >> l) * (side >> l);
    }
    if (words > 0xFFFFFFFFull) return bail(cudaErrorInvalidValue);
    if ((e = cudaMalloc(&c->spec_env, words * 4)) != cudaSuccess) return bail(e);
    uint64_t per_cache = 0;  // the apply's FP16 copy: every level of each cache, 8 bytes a texel
    for (int l = 0; l < c->spec_levels; ++l) per_cache += (uint64_t)(S >> l) * (S >> l);
    if ((e = cudaMalloc(&c->spec_half, (size_t)cfg->max_caches * per_cache * 8)) != cudaSuccess) return bail(e);
  }
  c->box_capacity = 512;
  if ((e = cudaMallocHost(&c->h_boxes, c->box_capacity * sizeof(DrvBox))) != cudaSuccess) return bail(e);
  if ((e = cudaMalloc(&c->d_boxes, c->box_capacity * sizeof(DrvBox))) != cudaSuccess) return bail(e);
  c->resident_boxes = -1;
  *out = c;
  return DRV_OK;
}

drv_status drv_destroy(DrvContext* ctx) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->has_user_stream) cudaStreamSynchronize(ctx->user_stream);
  release(ctx);
  delete ctx;
  return DRV_OK;
}

drv_status drv_set_stream(DrvContext* ctx, void* stream) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  ctx->user_stream = (cudaStream_t)stream;
  ctx->has_user_stream = true;
  return DRV_OK;
}

const char* drv_last_error_string(DrvContext* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

drv_status drv_get_error(DrvContext* ctx, uint32_t* bits) {
  if (!ctx || !bits) return DRV_ERR_INVALID_ARG;
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  uint32_t w[4];
  DRV_TRY_CUDA(ctx, cudaMemcpy(w, ctx->scratch_words + 1, 16, cudaMemcpyDeviceToHost));
  *bits = w[0] | w[3];
  // The input-check word is reported once: cleared once read.
  if (w[3]) DRV_TRY_CUDA(ctx, cudaMemset(ctx->input_err(), 0, 4));
  return DRV_OK;
}

drv_status drv_sync(DrvContext* ctx) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  uint32_t bits = 0;
  drv_status st = drv_get_error(ctx, &bits);
  if (st != DRV_OK) return st;
  if (bits & DRV_DEVERR_CAPACITY) return fail(ctx, DRV_ERR_CAPACITY, "more light caches requested than max_caches");
  if (bits & DRV_DEVERR_TIMEOUT) return fail(ctx, DRV_ERR_TIMEOUT, "a bounded device-side wait gave up");
  if (bits & DRV_DEVERR_BOUNDS)
    return fail(ctx, DRV_ERR_INVALID_ARG, "device-side bounds check failed: an atlas slot names a cache beyond the count");
  if (bits & DRV_DEVERR_NUMERIC) return fail(ctx, DRV_ERR_NUMERIC, "non-finite value in an input (check_inputs)");
  return DRV_OK;
}

drv_status drv_get_buffers(DrvContext* ctx, DrvBuffers* o) {
  if (!ctx || !o) return DRV_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  o->cache_entries = ctx->entries;
  o->entry_stride = ctx->entry_stride;
  o->cav_atlas = ctx->atlas;
  o->counter = ctx->counter;
  o->voxel_bits = ctx->voxel_bits;
  o->voxel_corners = ctx->vox_corners;
  for (int l = 0; l < 16; ++l)
    o->voxel_mip_records[l] = l >= 1 && l <= ctx->record_levels ? (void*)(ctx->vox_records + ctx->record_offset[l]) : nullptr;
  o->n_record_levels = ctx->record_levels;
  const size_t texel = ctx->cfg.precision == DRV_PRECISION_BF16 ? 2 : 4;
  for (int l = 1; l < ctx->n_voxel_levels && l < 16; ++l)
    o->voxel_mips[l] = static_cast<char*>(ctx->mips) + ctx->mip_offset[l] * texel;
  o->n_voxel_levels = ctx->n_voxel_levels;
  for (int l = 0; l < DRV_MAX_LIGHTS; ++l) {
    o->vpls[l] = ctx->vpls[l];
    o->cones[l] = ctx->cones[l];
    o->n_vpls[l] = ctx->n_vpls[l];
  }
  o->n_lights = ctx->n_lights;
  for (int l = 0; l < ctx->spec_levels; ++l) o->specular_envmap[l] = ctx->spec_env + ctx->spec_off[l];
  o->specular_atlas_size = ctx->spec_atlas;
  o->n_specular_levels = ctx->spec_levels;
  return DRV_OK;
}

drv_status drv_get_cache_count(DrvContext* ctx, uint32_t* out) {
  if (!ctx || !out) return DRV_ERR_INVALID_ARG;
  DrvCacheCounter h;
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  DRV_TRY_CUDA(ctx, cudaMemcpy(&h, ctx->counter, sizeof(h), cudaMemcpyDeviceToHost));
  *out = (uint32_t)(h.total_light_cache_count < 0 ? 0 : h.total_light_cache_count);
  return drv_sync(ctx);
}

drv_status drv_set_scene(DrvContext* ctx, const DrvScene* scene) {
  if (!ctx || !scene || !scene->boxes || scene->n_boxes < 1) return DRV_ERR_INVALID_ARG;
  if (scene->n_boxes > ctx->box_capacity) return fail(ctx, DRV_ERR_INVALID_ARG, "scene has more than 512 boxes");
  if (ctx->resident_boxes == scene->n_boxes &&
      std::memcmp(ctx->h_boxes, scene->boxes, scene->n_boxes * sizeof(DrvBox)) == 0)
    return DRV_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  DRV_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->s(), &cs));
  if (cs != cudaStreamCaptureStatusNone)
    return fail(ctx, DRV_ERR_INVALID_ARG, "scene changed while the stream is being captured");
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  std::memcpy(ctx->h_boxes, scene->boxes, scene->n_boxes * sizeof(DrvBox));
  DRV_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->d_boxes, ctx->h_boxes, scene->n_boxes * sizeof(DrvBox),
                                    cudaMemcpyHostToDevice, ctx->s()));
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  ctx->resident_boxes = scene->n_boxes;
  return DRV_OK;
}

drv_status drv_raycast_gbuffer(DrvContext* ctx, const DrvScene* scene, const DrvCamera* cam, const DrvPerFrame* frame,
                               int32_t w, int32_t h, const DrvGBufferOut* out) {
  if (!ctx || !scene || !cam || !frame || !out || !out->depth || !out->albedo || w < 1 || h < 1)
    return DRV_ERR_INVALID_ARG;
  drv_status st = drv_set_scene(ctx, scene);
  if (st != DRV_OK) return st;
  const double ty = std::tan(cam->fov_y_deg * (3.14159265358979323846 / 180.0) * 0.5);
  drv::RayFrame rf = drv::make_ray_frame(cam->position, cam->direction, cam->up, ty * cam->aspect, ty);
  return cuda_check(ctx, drv::launch_raycast_gbuffer(ctx->s(), ctx->d_boxes, scene->n_boxes, rf, frame->view_projection,
                                                     w, h, *out),
                    "raycast_gbuffer");
}

drv_status drv_raycast_rsm(DrvContext* ctx, const DrvScene* scene, const DrvSpotLight* light, const DrvRSMOut* out) {
  if (!ctx || !scene || !light || !out || !out->flux || !out->normal || !out->depth_lin_sq) return DRV_ERR_INVALID_ARG;
  if (light->rsm_render_resolution < 1) return DRV_ERR_INVALID_ARG;
  drv_status st = drv_set_scene(ctx, scene);
  if (st != DRV_OK) return st;
  return cuda_check(ctx, drv::launch_raycast_rsm(ctx->s(), ctx->d_boxes, scene->n_boxes, *light, *out), "raycast_rsm");
}

namespace {

bool mesh_ok(const DrvMesh* m) {
  if (!m || m->n_triangles < 0 || m->n_vertices < 0) return false;
  if (m->n_triangles > 0 && (!m->positions || m->n_vertices < 1)) return false;
  if (!m->indices && (int64_t)m->n_triangles * 3 > m->n_vertices) return false;
  for (const void* p : {(const void*)m->positions, (const void*)m->normals, (const void*)m->albedo,
                        (const void*)m->indices})
    if (reinterpret_cast<uintptr_t>(p) % 4) return false;
  return true;
}

// The visibility buffer of the mesh producers, grown to `pixels`.
drv_status ensure_raster_keys(DrvContext* ctx, size_t pixels) {
  if (ctx->raster_keys_cap >= pixels) return DRV_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  DRV_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->s(), &cs));
  if (cs != cudaStreamCaptureStatusNone)
    return fail(ctx, DRV_ERR_INVALID_ARG, "first mesh raster at this size while the stream is being captured");
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  cudaFree(ctx->raster_keys);
  ctx->raster_keys = nullptr;
  ctx->raster_keys_cap = 0;
  DRV_TRY_CUDA(ctx, cudaMalloc(&ctx->raster_keys, pixels * sizeof(unsigned long long)));
  ctx->raster_keys_cap = pixels;
  return DRV_OK;
}

}  // namespace

drv_status drv_raster_gbuffer(DrvContext* ctx, const DrvMesh* mesh, const DrvCamera* cam, const DrvPerFrame* frame,
                              int32_t w, int32_t h, const DrvGBufferOut* out) {
  if (!ctx || !cam || !frame || !out || !out->depth || !out->albedo || w < 1 || h < 1) return DRV_ERR_INVALID_ARG;
  if (!mesh_ok(mesh)) return fail(ctx, DRV_ERR_INVALID_ARG, "bad mesh");
  drv_status st = ensure_raster_keys(ctx, (size_t)w * h);
  if (st != DRV_OK) return st;
  const double ty = std::tan(cam->fov_y_deg * (3.14159265358979323846 / 180.0) * 0.5);
  const drv::RayFrame rf = drv::make_ray_frame(cam->position, cam->direction, cam->up, ty * cam->aspect, ty);
  return cuda_check(ctx,
                    drv::launch_raster_gbuffer(ctx->s(), *mesh, rf, frame->view_projection, w, h, ctx->raster_keys,
                                               *out, ctx->num_sms),
                    "raster_gbuffer");
}

drv_status drv_raster_rsm(DrvContext* ctx, const DrvMesh* mesh, const DrvSpotLight* light, const DrvRSMOut* out) {
  if (!ctx || !light || !out || !out->flux || !out->normal || !out->depth_lin_sq) return DRV_ERR_INVALID_ARG;
  if (light->rsm_render_resolution < 1) return DRV_ERR_INVALID_ARG;
  if (!mesh_ok(mesh)) return fail(ctx, DRV_ERR_INVALID_ARG, "bad mesh");
  const size_t R = (size_t)light->rsm_render_resolution;
  drv_status st = ensure_raster_keys(ctx, R * R);
  if (st != DRV_OK) return st;
  return cuda_check(ctx, drv::launch_raster_rsm(ctx->s(), *mesh, *light, ctx->raster_keys, *out, ctx->num_sms),
                    "raster_rsm");
}

// ShadowMap::PrepareRSM (renderer.cpp:1300-1339): successive 2x2 reductions,
// down to the deepest level the light reads (read lod + shadow lod).
drv_status drv_prepare_rsm(DrvContext* ctx, int32_t li, const DrvSpotLight* L, const DrvRSMView* v) {
  if (!ctx || !L || !v || !v->flux || !v->normal || !v->depth_lin_sq) return DRV_ERR_INVALID_ARG;
  if (li < 0 || li >= ctx->cfg.max_lights) return fail(ctx, DRV_ERR_INVALID_ARG, "light index out of range");
  const int R = v->resolution;
  if (!is_pow2(R) || R != L->rsm_render_resolution || R > ctx->cfg.max_rsm_resolution)
    return fail(ctx, DRV_ERR_INVALID_ARG, "RSM resolution must equal rsm_render_resolution (power of two, <= max)");
  if (L->rsm_read_resolution < 1 || R % L->rsm_read_resolution != 0)
    return fail(ctx, DRV_ERR_INVALID_ARG, "rsm_read_resolution must divide the RSM resolution");
  const int read_lod = ilog2(R / L->rsm_read_resolution);
  const int shadow_lod = (int)L->indirect_shadow_lod;
  const int deepest = read_lod + shadow_lod;
  if ((R >> deepest) < 1) return fail(ctx, DRV_ERR_INVALID_ARG, "indirect shadow lod beyond the RSM chain");
  drv::RsmChain& ch = ctx->rsm[li];
  ch.res0 = R;
  ch.n_levels = deepest + 1;
  if (v->format != DRV_RSM_F32 && v->format != DRV_RSM_F16) return fail(ctx, DRV_ERR_INVALID_ARG, "bad RSM format");
  const size_t align = v->format == DRV_RSM_F16 ? 2 : 4;
  if (reinterpret_cast<uintptr_t>(v->flux) % align || reinterpret_cast<uintptr_t>(v->depth_lin_sq) % align ||
      reinterpret_cast<uintptr_t>(v->normal) % 2)
    return fail(ctx, DRV_ERR_INVALID_ARG, "misaligned RSM view");
  ch.flux[0] = const_cast<void*>(v->flux);
  ch.normal[0] = const_cast<int16_t*>(v->normal);
  ch.dls[0] = const_cast<void*>(v->depth_lin_sq);
  ch.half0 = v->format == DRV_RSM_F16;
  if (ctx->tuning.check_inputs) {
    const size_t n = (size_t)R * R;
    DRV_TRY_CUDA(ctx, drv::launch_scan_finite(ctx->s(), v->flux, n * 3, ch.half0, ctx->input_err()));
    DRV_TRY_CUDA(ctx, drv::launch_scan_finite(ctx->s(), v->depth_lin_sq, n * 2, ch.half0, ctx->input_err()));
  }
  // The chain in launches of up to three passes each (launch_rsm_chain).
  for (int k = 0; k < deepest; k += 3) {
    const int passes = deepest - k < 3 ? deepest - k : 3;
    float* fo[3] = {};
    int16_t* no[3] = {};
    float* dlo[3] = {};
    for (int q = 0; q < passes; ++q) {
      fo[q] = static_cast<float*>(ch.flux[k + 1 + q]);
      no[q] = ch.normal[k + 1 + q];
      dlo[q] = static_cast<float*>(ch.dls[k + 1 + q]);
    }
    DRV_TRY_CUDA(ctx, drv::launch_rsm_chain(ctx->s(), R >> k, passes, ch.flux[k], ch.normal[k], ch.dls[k], ch.half(k),
                                            fo, no, dlo));
  }
  return DRV_OK;
}

drv_status drv_extract_vpls(DrvContext* ctx, int32_t li, const DrvSpotLight* L) {
  if (!ctx || !L) return DRV_ERR_INVALID_ARG;
  if (li < 0 || li >= ctx->cfg.max_lights) return fail(ctx, DRV_ERR_INVALID_ARG, "light index out of range");
  drv::RsmChain& ch = ctx->rsm[li];
  if (ch.res0 != L->rsm_render_resolution || ch.n_levels < 1)
    return fail(ctx, DRV_ERR_INVALID_ARG, "drv_prepare_rsm must run for this light first");
  const int R = L->rsm_read_resolution;
  const int read_lod = ilog2(ch.res0 / R);
  const int shadow_level = read_lod + (int)L->indirect_shadow_lod;
  if (shadow_level >= ch.n_levels) return fail(ctx, DRV_ERR_INVALID_ARG, "RSM chain too short for the shadow lod");
  if (L->indirect_shadow_sample_interval < 1) return DRV_ERR_INVALID_ARG;
  DRV_TRY_CUDA(ctx, drv::launch_extract_vpls(ctx->s(), *L, R, ch.flux[read_lod], ch.normal[read_lod], ch.dls[read_lod],
                                             ch.half(read_lod), ch.dls[shadow_level], ch.half(shadow_level),
                                             ctx->vpls[li], ctx->cones[li], ctx->cfg.precision,
                                             ctx->vpl_records[li]));
  ctx->n_vpls[li] = R * R;
  ctx->interval[li] = L->indirect_shadow_sample_interval;
  ctx->n_cones[li] = (R * R + L->indirect_shadow_sample_interval - 1) / L->indirect_shadow_sample_interval;
  if (li + 1 > ctx->n_lights) ctx->n_lights = li + 1;
  return DRV_OK;
}

drv_status drv_voxelize(DrvContext* ctx, const DrvScene* scene, const DrvVolumeInfo* vol) {
  if (!ctx || !scene || !vol) return DRV_ERR_INVALID_ARG;
  drv_status st = drv_set_scene(ctx, scene);
  if (st != DRV_OK) return st;
  return cuda_check(ctx, drv::launch_voxelize(ctx->s(), ctx->d_boxes, scene->n_boxes, *vol, ctx->cfg.voxel_res,
                                              ctx->voxel_bits),
                    "voxelize");
}

drv_status drv_voxelize_triangles(DrvContext* ctx, const float* positions, int32_t n_vertices, const uint32_t* indices,
                                  int32_t n_triangles, const DrvVolumeInfo* vol) {
  if (!ctx || !vol || n_triangles < 0 || n_vertices < 0 || (n_triangles > 0 && (!positions || n_vertices < 1)))
    return DRV_ERR_INVALID_ARG;
  if (!indices && (int64_t)n_triangles * 3 > n_vertices)
    return fail(ctx, DRV_ERR_INVALID_ARG, "without indices the triangles take 3 consecutive vertices each");
  if (reinterpret_cast<uintptr_t>(positions) % 4 || reinterpret_cast<uintptr_t>(indices) % 4)
    return fail(ctx, DRV_ERR_INVALID_ARG, "positions and indices must be 4-byte aligned");
  return cuda_check(ctx, drv::launch_voxelize_triangles(ctx->s(), positions, n_vertices, indices, n_triangles, *vol,
                                                        ctx->cfg.voxel_res, ctx->voxel_bits, ctx->num_sms),
                    "voxelize_triangles");
}

drv_status drv_build_opacity_mips(DrvContext* ctx) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  // The corner grid (side stream 2) and the mip chain + records (this
  // stream) both read only the level-0 bits: built concurrently, joined here.
  const cudaStream_t s = ctx->s();
  DRV_TRY_CUDA(ctx, cudaEventRecord(ctx->vox_fork_ev, s));
  DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->side[2], ctx->vox_fork_ev, 0));
  const drv_status corners =
      cuda_check(ctx, drv::launch_build_corners(ctx->side[2], ctx->cfg.voxel_res, ctx->voxel_bits, ctx->vox_corners),
                 "build_corners");
  drv_status st = cuda_check(ctx,
                             drv::launch_build_mips(s, ctx->cfg.voxel_res, ctx->voxel_bits, ctx->mips, ctx->mip_offset,
                                                    ctx->n_voxel_levels, ctx->cfg.precision, ctx->mips_ticket()),
                             "build_mips");
  if (st == DRV_OK)
    st = cuda_check(ctx,
                    drv::launch_build_records(s, ctx->cfg.voxel_res, ctx->mips, ctx->mip_offset, ctx->cfg.precision,
                                              ctx->vox_records, ctx->record_offset, ctx->record_levels),
                    "build_records");
  DRV_TRY_CUDA(ctx, cudaEventRecord(ctx->join_ev[2], ctx->side[2]));
  DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(s, ctx->join_ev[2], 0));
  return st != DRV_OK ? st : corners;
}

// Renderer::AllocateCaches: clear counter and atlas (renderer.cpp:968-970),
// then cacheGather.comp + cachePrepareLighting.comp in one launch.
drv_status drv_allocate_caches(DrvContext* ctx, const DrvGBufferView* g, const DrvPerFrame* f, const DrvVolumeInfo* vol) {
  if (!ctx || !f || !vol) return DRV_ERR_INVALID_ARG;
  if (!views_ok(g, ctx->cfg)) return fail(ctx, DRV_ERR_INVALID_ARG, "G-buffer view does not match the config");
  ctx->last_volume = *vol;
  if (ctx->tuning.check_inputs) {
    const size_t n = (size_t)g->width * g->height;
    DRV_TRY_CUDA(ctx, drv::launch_scan_finite(ctx->s(), g->depth, n, 0, ctx->input_err()));
    if (g->normal_format == DRV_NORMAL_F32X3)
      DRV_TRY_CUDA(ctx, drv::launch_scan_finite(ctx->s(), g->normal, n * 3, 0, ctx->input_err()));
  }
  DRV_TRY_CUDA(ctx, cudaMemsetAsync(ctx->counter, 0, 32, ctx->s()));
  DRV_TRY_CUDA(ctx, cudaMemsetAsync(ctx->atlas, 0, ctx->atlas_words * 4, ctx->s()));
  return cuda_check(ctx, drv::launch_allocate(ctx->s(), ctx->cfg, *vol, *f, g->depth, g->width, g->height, ctx->atlas,
                                              ctx->entries, ctx->entry_stride, ctx->counter, ctx->scratch_words,
                                              ctx->scratch_words + 1, ctx->ndc),
                    "allocate_caches");
}

namespace {

// The level-0 specular envmaps of the light stage just issued (pairs: its
// pair list, or nullptr after the single-launch form).
drv_status specular_gather(DrvContext* ctx, const drv::LightLaunch& ll, const DrvVolumeInfo* vol,
                           const DrvPerFrame* frame, const drv::PairList* pairs) {
  const drv::SpecView sv =
      drv::make_spec_view(ctx->cfg, ctx->spec_env, ctx->spec_off, ctx->spec_atlas, ctx->spec_half, *frame);
  ctx->spec_ready = false;  // the mips and the apply's copy are stale until drv_prepare_specular_envmaps
  drv_status st = cuda_check(ctx, drv::launch_specular_gather(ctx->s(), ctx->cfg, *vol, ll, ctx->counter, ctx->entries,
                                                              ctx->entry_stride, ctx->light_voxels(), pairs, sv,
                                                              ctx->num_sms),
                             "specular envmaps");
  if (st == DRV_OK) ctx->spec_lit = true;
  return st;
}

// The light stage. voxels_ready (drv_frame): an event the voxel build records
// on another stream; only the kernels that read the voxels wait for it.
drv_status light_caches(DrvContext* ctx, const DrvSpotLight* lights, int32_t n_lights, const DrvVolumeInfo* vol,
                        const DrvPerFrame* frame, cudaEvent_t voxels_ready) {
  if (!ctx || !lights || !vol || !frame) return DRV_ERR_INVALID_ARG;
  if (n_lights < 0 || n_lights > ctx->cfg.max_lights) return fail(ctx, DRV_ERR_INVALID_ARG, "bad light count");
  drv::LightLaunch ll{};
  ll.n_lights = n_lights;
  for (int l = 0; l < n_lights; ++l) {
    if (ctx->n_vpls[l] != lights[l].rsm_read_resolution * lights[l].rsm_read_resolution)
      return fail(ctx, DRV_ERR_INVALID_ARG, "drv_extract_vpls must run for every light first");
    ll.lights[l].vpls = ctx->vpls[l];
    ll.lights[l].cones = ctx->cones[l];
    ll.lights[l].n_vpls = ctx->n_vpls[l];
    ll.lights[l].interval = ctx->interval[l];
    ll.lights[l].records = ctx->vpl_records[l];
  }
  const bool surrogate = ctx->cfg.visibility == DRV_VISIBILITY_SURROGATE && ctx->cfg.indirect_shadow;
  if (surrogate && !ctx->sur_ready)
    return fail(ctx, DRV_ERR_INVALID_ARG, "surrogate visibility needs drv_set_surrogate_params");
  const bool split = ctx->tuning.light_path != DRV_LIGHT_PATH_SINGLE && drv::light_split_supported(ctx->cfg, ll);
  if (split) {
    drv::PairList pairs = ctx->pairs;
    if (ctx->tuning.pair_capacity) pairs.cap = std::min(pairs.cap, ctx->tuning.pair_capacity);
    cudaEvent_t* events = nullptr;
    if (ctx->tuning.time_kernels) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      DRV_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->s(), &cs));
      if (cs == cudaStreamCaptureStatusNone) {
        for (cudaEvent_t& e : ctx->lk_events)
          if (!e) DRV_TRY_CUDA(ctx, cudaEventCreate(&e));
        events = ctx->lk_events;
      }
    }
    drv::SplitKnobs knobs;
    knobs.cone_ctas_per_sm = ctx->tuning.cone_ctas_per_sm;
    knobs.gather_ctas_per_sm = ctx->tuning.gather_ctas_per_sm;
    if (ctx->tuning.cull_caches_per_pass) knobs.cull_caches_per_pass = ctx->tuning.cull_caches_per_pass;
    if (ctx->tuning.gather_threads) knobs.gather_threads = ctx->tuning.gather_threads;
    knobs.count_voxel_reads = ctx->tuning.count_voxel_reads != 0;
    knobs.gather_wait_test = ctx->tuning.gather_wait_test;
    drv::SurrogateArgs sur;
    if (surrogate) {
      sur.weights = ctx->sur_weights;
      sur.feature_set = ctx->sur_features;
      sur.threshold = ctx->cfg.surrogate_conf_threshold;
      sur.err = ctx->scratch_words + 1;
      sur.hold_commit = ctx->tuning.surrogate_wait_test;
    }
    if (ctx->tuning.per_light_dispatch && ll.n_lights > 1) {
      // One split stage per light, each adding its SH into the entries (the
      // reference's dispatch loop); the voxel wait is taken once, up front.
      if (voxels_ready) DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->s(), voxels_ready, 0));
      ctx->lk_recorded = false;
      drv_status st = DRV_OK;
      for (int l = 0; l < ll.n_lights && st == DRV_OK; ++l) {
        drv::LightLaunch one{};
        one.n_lights = 1;
        one.lights[0] = ll.lights[l];
        st = cuda_check(ctx, drv::launch_light_split(ctx->s(), ctx->cfg, *vol, one, ctx->counter, ctx->entries,
                                                     ctx->entry_stride, ctx->light_voxels(), pairs, sur,
                                                     ctx->scratch_words + 1, knobs, ctx->num_sms, nullptr, nullptr),
                        "light_caches");
      }
      if (st == DRV_OK && ctx->spec_env) st = specular_gather(ctx, ll, vol, frame, nullptr);
      return st;
    }
    drv_status st = cuda_check(ctx, drv::launch_light_split(ctx->s(), ctx->cfg, *vol, ll, ctx->counter, ctx->entries,
                                                            ctx->entry_stride, ctx->light_voxels(), pairs, sur,
                                                            ctx->scratch_words + 1, knobs, ctx->num_sms, events,
                                                            voxels_ready),
                               "light_caches");
    if (events) ctx->lk_recorded = st == DRV_OK;
    if (st == DRV_OK && ctx->spec_env) st = specular_gather(ctx, ll, vol, frame, &pairs);
    return st;
  }
  if (voxels_ready) DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->s(), voxels_ready, 0));
  if (surrogate && ctx->tuning.light_path == DRV_LIGHT_PATH_SINGLE)
    return fail(ctx, DRV_ERR_INVALID_ARG, "surrogate visibility runs on the split light stage");
  long blocks = 0;
  for (int l = 0; l < ll.n_lights; ++l) blocks += ll.lights[l].n_vpls / ll.lights[l].interval;
  if (surrogate && blocks > drv::kMaxSplitBlocks)
    return fail(ctx, DRV_ERR_INVALID_ARG, "surrogate visibility supports at most 65536 shadow blocks per frame");
  if (!ctx->light_scratch) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    DRV_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->s(), &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return fail(ctx, DRV_ERR_INVALID_ARG, "first single-launch light stage while the stream is being captured");
    DRV_TRY_CUDA(ctx, ensure_single_scratch(ctx));
  }
  const drv::LightScratch scratch{ctx->light_scratch, ctx->light_tickets, ctx->light_tickets + ctx->cfg.max_caches,
                                  drv::kMaxLightChunks};
  drv_status st = cuda_check(ctx, drv::launch_light_caches(ctx->s(), ctx->cfg, *vol, ll, ctx->counter, ctx->entries,
                                                           ctx->entry_stride, ctx->light_voxels(), scratch,
                                                           ctx->num_sms),
                             "light_caches");
  if (st == DRV_OK && ctx->spec_env) st = specular_gather(ctx, ll, vol, frame, nullptr);
  return st;
}

}  // namespace

drv_status drv_light_caches(DrvContext* ctx, const DrvSpotLight* lights, int32_t n_lights, const DrvVolumeInfo* vol,
                            const DrvPerFrame* frame) {
  return light_caches(ctx, lights, n_lights, vol, frame, nullptr);
}

drv_status drv_apply(DrvContext* ctx, const DrvGBufferView* g, const DrvPerFrame* f, const DrvVolumeInfo* vol,
                     float* out_rgb) {
  if (!ctx || !f || !vol || !out_rgb) return DRV_ERR_INVALID_ARG;
  if (!views_ok(g, ctx->cfg)) return fail(ctx, DRV_ERR_INVALID_ARG, "G-buffer view does not match the config");
  if (!rough_metal_ok(g, ctx->cfg))
    return fail(ctx, DRV_ERR_INVALID_ARG, "specular needs the G-buffer's roughness / metallic (aligned, known format)");
  if (reinterpret_cast<uintptr_t>(out_rgb) % (ctx->cfg.output_format == DRV_OUTPUT_RGBA16F ? 8 : 4))
    return fail(ctx, DRV_ERR_INVALID_ARG, "misaligned output");
  drv::SpecView sv{};
  if (ctx->spec_env) {
    if (!ctx->spec_ready)
      return fail(ctx, DRV_ERR_INVALID_ARG, "specular apply needs drv_prepare_specular_envmaps after the light stage");
    sv = drv::make_spec_view(ctx->cfg, ctx->spec_env, ctx->spec_off, ctx->spec_atlas, ctx->spec_half, *f);
  }
  if (ctx->tuning.check_inputs && g->albedo_format == DRV_ALBEDO_F32X3)
    DRV_TRY_CUDA(ctx, drv::launch_scan_finite(ctx->s(), g->albedo, (size_t)g->width * g->height * 3, 0,
                                              ctx->input_err()));
  return cuda_check(ctx, drv::launch_apply(ctx->s(), ctx->cfg, *vol, *f, *g, ctx->atlas, ctx->entries,
                                           ctx->entry_stride, ctx->counter, out_rgb, ctx->srgb,
                                           ctx->spec_env ? &sv : nullptr, ctx->scratch_words + 1,
                                           ctx->tuning.tensor_core_apply != 0),
                    "apply");
}

drv_status drv_prepare_specular_envmaps(DrvContext* ctx) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  if (!ctx->spec_env) return fail(ctx, DRV_ERR_INVALID_ARG, "specular is off (specular_envmap_size 0)");
  if (!ctx->spec_lit) return fail(ctx, DRV_ERR_INVALID_ARG, "drv_light_caches must run first");
  const DrvPerFrame none{};
  const drv::SpecView sv =
      drv::make_spec_view(ctx->cfg, ctx->spec_env, ctx->spec_off, ctx->spec_atlas, ctx->spec_half, none);
  drv_status st = cuda_check(ctx, drv::launch_envmap_prepare(ctx->s(), sv, ctx->counter, ctx->cfg.max_caches,
                                                             ctx->cfg.specular_fill_level, ctx->num_sms),
                             "specular envmap mips");
  if (st == DRV_OK) ctx->spec_ready = true;
  return st;
}

// Renderer::Draw, DYN_RADIANCE_VOLUME branch (renderer.cpp:539-594), plus the
// RSM preparation of DrawShadowMaps (renderer.cpp:801-810).
drv_status drv_frame(DrvContext* ctx, const DrvScene* scene, const DrvGBufferView* g, const DrvPerFrame* f,
                     const DrvVolumeInfo* vol, const DrvSpotLight* lights, const DrvRSMView* rsms, int32_t n_lights,
                     float* out_rgb) {
  if (!ctx || !scene || !g || !f || !vol || (n_lights > 0 && (!lights || !rsms)) || !out_rgb)
    return DRV_ERR_INVALID_ARG;
  if (ctx->cur) return fail(ctx, DRV_ERR_INVALID_ARG, "drv_frame re-entered");
  if (!views_ok(g, ctx->cfg) || !rough_metal_ok(g, ctx->cfg))
    return fail(ctx, DRV_ERR_INVALID_ARG, "G-buffer view does not match the config");
  drv_status st;
  // The box upload synchronises when the scene changed: do it on the
  // context's stream, before the fork.
  if (ctx->cfg.indirect_shadow && (st = drv_set_scene(ctx, scene)) != DRV_OK) return st;
  // Renderer::Draw's first three stages are independent: RSM/VPLs on side
  // stream 0, voxels on side stream 1, the cache allocation on the context's
  // stream; the light stage waits for all three.
  const cudaStream_t main = ctx->s();
  DRV_TRY_CUDA(ctx, cudaEventRecord(ctx->fork_ev, main));
  for (int i = 0; i < 2; ++i) DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->side[i], ctx->fork_ev, 0));
  st = DRV_OK;
  ctx->cur = ctx->side[0];
  for (int l = 0; l < n_lights && st == DRV_OK; ++l) {
    st = drv_prepare_rsm(ctx, l, &lights[l], &rsms[l]);
    if (st == DRV_OK) st = drv_extract_vpls(ctx, l, &lights[l]);
  }
  ctx->cur = ctx->side[1];
  if (st == DRV_OK && ctx->cfg.indirect_shadow) {
    st = drv_voxelize(ctx, scene, vol);
    if (st == DRV_OK) st = drv_build_opacity_mips(ctx);
  }
  ctx->cur = nullptr;
  if (st == DRV_OK) st = drv_allocate_caches(ctx, g, f, vol);
  // The light stage's cull and ordering need the VPLs and the caches; the
  // voxels are waited for only by the kernels that read them. After an error
  // both side streams are joined, so that no later call races them.
  for (int i = 0; i < 2; ++i) DRV_TRY_CUDA(ctx, cudaEventRecord(ctx->join_ev[i], ctx->side[i]));
  DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(main, ctx->join_ev[0], 0));
  if (st == DRV_OK) st = light_caches(ctx, lights, n_lights, vol, f, ctx->join_ev[1]);
  // Joined by now on success (the voxel readers waited); this also covers an
  // error or a stage that skipped the wait.
  DRV_TRY_CUDA(ctx, cudaStreamWaitEvent(main, ctx->join_ev[1], 0));
  if (st == DRV_OK && ctx->spec_env) st = drv_prepare_specular_envmaps(ctx);  // renderer.cpp:556-558
  if (st != DRV_OK) return st;
  return drv_apply(ctx, g, f, vol, out_rgb);
}

// ---- learned visibility surrogate ----------------------------------------
drv_status drv_set_surrogate_params(DrvContext* ctx, const float* params) {
  if (!ctx || !params) return DRV_ERR_INVALID_ARG;
  DRV_TRY_CUDA(ctx, drv::launch_pack_surrogate_weights(ctx->s(), params, ctx->sur_weights));
  ctx->sur_ready = true;
  return DRV_OK;
}

drv_status drv_surrogate_eval(DrvContext* ctx, const float* features, int32_t n, float* out) {
  if (!ctx || !features || !out || n < 0) return DRV_ERR_INVALID_ARG;
  if (!ctx->sur_ready) return fail(ctx, DRV_ERR_INVALID_ARG, "drv_set_surrogate_params first");
  if (n == 0) return DRV_OK;
  if (((uintptr_t)features & 15u) != 0) return fail(ctx, DRV_ERR_INVALID_ARG, "features must be 16-byte aligned");
  return cuda_check(ctx, drv::launch_surrogate_eval(ctx->s(), ctx->sur_weights, features, n, out,
                                                    ctx->scratch_words + 1, ctx->num_sms),
                    "surrogate_eval");
}

drv_status drv_set_surrogate_features(DrvContext* ctx, int32_t feature_set) {
  if (!ctx) return DRV_ERR_INVALID_ARG;
  if (feature_set != DRV_SURROGATE_FEATURES_SEGMENT8 && feature_set != DRV_SURROGATE_FEATURES_CONE4 &&
      feature_set != DRV_SURROGATE_FEATURES_CONE8)
    return fail(ctx, DRV_ERR_INVALID_ARG, "unknown surrogate feature set");
  ctx->sur_features = feature_set;
  return DRV_OK;
}

drv_status drv_get_surrogate_fallbacks(DrvContext* ctx, uint32_t* out) {
  if (!ctx || !out) return DRV_ERR_INVALID_ARG;
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  uint32_t v[2];
  DRV_TRY_CUDA(ctx, cudaMemcpy(v, ctx->pairs.counters + 3, 8, cudaMemcpyDeviceToHost));
  *out = v[0] + v[1];
  return DRV_OK;
}

drv_status drv_bruteforce_rsm(DrvContext* ctx, const DrvGBufferView* g, const float* rough_metal,
                              const DrvPerFrame* f, int32_t n_lights, float* out_rgb) {
  if (!ctx || !f || !out_rgb || n_lights < 0 || n_lights > ctx->cfg.max_lights) return DRV_ERR_INVALID_ARG;
  if (!views_ok(g, ctx->cfg)) return fail(ctx, DRV_ERR_INVALID_ARG, "G-buffer view does not match the config");
  drv::LightLaunch ll{};
  ll.n_lights = n_lights;
  for (int l = 0; l < n_lights; ++l) {
    if (ctx->n_vpls[l] < 1) return fail(ctx, DRV_ERR_INVALID_ARG, "drv_extract_vpls must run for every light first");
    ll.lights[l].vpls = ctx->vpls[l];
    ll.lights[l].n_vpls = ctx->n_vpls[l];
    ll.lights[l].interval = 1;
  }
  return cuda_check(ctx, drv::launch_bruteforce_rsm(ctx->s(), *f, *g, rough_metal, ll,
                                                    ctx->cfg.precision == DRV_PRECISION_BF16, out_rgb, ctx->srgb),
                    "bruteforce_rsm");
}

drv_status drv_set_tuning(DrvContext* ctx, const DrvTuning* t) {
  if (!ctx || !t) return DRV_ERR_INVALID_ARG;
  if (t->light_path < DRV_LIGHT_PATH_AUTO || t->light_path > DRV_LIGHT_PATH_SPLIT || t->cone_ctas_per_sm < 0 ||
      t->gather_ctas_per_sm < 0 || t->cone_ctas_per_sm > 32 || t->gather_ctas_per_sm > 32)
    return fail(ctx, DRV_ERR_INVALID_ARG, "bad tuning");
  if (t->cull_caches_per_pass != 0 && t->cull_caches_per_pass != 2 && t->cull_caches_per_pass != 4 &&
      t->cull_caches_per_pass != 8)
    return fail(ctx, DRV_ERR_INVALID_ARG, "cull_caches_per_pass must be 0, 2, 4 or 8");
  if (t->gather_threads != 0 && t->gather_threads != 256 && t->gather_threads != 512)
    return fail(ctx, DRV_ERR_INVALID_ARG, "gather_threads must be 0, 256 or 512");
  if (t->light_path == DRV_LIGHT_PATH_SINGLE) DRV_TRY_CUDA(ctx, ensure_single_scratch(ctx));
  if (t->pair_capacity > ctx->pairs.cap) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    DRV_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->s(), &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return fail(ctx, DRV_ERR_INVALID_ARG, "the pair list cannot grow while the stream is being captured");
    DRV_TRY_CUDA(ctx, alloc_pairs(ctx, t->pair_capacity));
  }
  ctx->tuning = *t;
  return DRV_OK;
}

drv_status drv_get_cone_voxel_reads(DrvContext* ctx, uint32_t reads[3]) {
  if (!ctx || !reads) return DRV_ERR_INVALID_ARG;
  if (!ctx->tuning.count_voxel_reads)
    return fail(ctx, DRV_ERR_INVALID_ARG, "set DrvTuning.count_voxel_reads before the light stage");
  uint32_t c[8];
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  DRV_TRY_CUDA(ctx, cudaMemcpy(c, ctx->pairs.counters, sizeof(c), cudaMemcpyDeviceToHost));
  reads[0] = c[1];
  reads[1] = c[2];
  reads[2] = c[7];
  return DRV_OK;
}

drv_status drv_get_light_pairs(DrvContext* ctx, uint32_t* pairs) {
  if (!ctx || !pairs) return DRV_ERR_INVALID_ARG;
  uint32_t n = 0;
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  DRV_TRY_CUDA(ctx, cudaMemcpy(&n, ctx->pairs.counters, 4, cudaMemcpyDeviceToHost));
  *pairs = n;
  return DRV_OK;
}

drv_status drv_get_light_kernel_ms(DrvContext* ctx, float ms[DRV_LK_COUNT]) {
  if (!ctx || !ms) return DRV_ERR_INVALID_ARG;
  if (!ctx->lk_recorded) return fail(ctx, DRV_ERR_INVALID_ARG, "no split light stage ran with time_kernels");
  DRV_TRY_CUDA(ctx, cudaEventSynchronize(ctx->lk_events[2 * DRV_LK_GATHER + 1]));
  for (int k = 0; k < DRV_LK_COUNT; ++k)
    DRV_TRY_CUDA(ctx, cudaEventElapsedTime(&ms[k], ctx->lk_events[2 * k], ctx->lk_events[2 * k + 1]));
  return DRV_OK;
}

drv_status drv_get_tuning(DrvContext* ctx, DrvTuning* t) {
  if (!ctx || !t) return DRV_ERR_INVALID_ARG;
  *t = ctx->tuning;
  return DRV_OK;
}

drv_status drv_get_surrogate_stats(DrvContext* ctx, uint32_t* evaluated, uint32_t* retraced) {
  if (!ctx || !evaluated || !retraced) return DRV_ERR_INVALID_ARG;
  uint32_t v[3];
  DRV_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->s()));
  DRV_TRY_CUDA(ctx, cudaMemcpy(v, ctx->pairs.counters + 3, 12, cudaMemcpyDeviceToHost));
  *retraced = v[0] + v[1];
  *evaluated = v[2];
  return DRV_OK;
}

drv_status drv_surrogate_make_pairs(DrvContext* ctx, uint64_t seed, int32_t n_pairs, float* features,
                                    float* targets) {
  if (!ctx || !features || !targets || n_pairs < 0) return DRV_ERR_INVALID_ARG;
  if (!ctx->cfg.indirect_shadow) return fail(ctx, DRV_ERR_INVALID_ARG, "pairs need the indirect-shadow cone");
  if (ctx->n_lights < 1) return fail(ctx, DRV_ERR_INVALID_ARG, "drv_extract_vpls must run first");
  if (n_pairs == 0) return DRV_OK;
  drv::LightLaunch ll{};
  ll.n_lights = ctx->n_lights;
  for (int l = 0; l < ctx->n_lights; ++l) {
    ll.lights[l].vpls = ctx->vpls[l];
    ll.lights[l].cones = ctx->cones[l];
    ll.lights[l].n_vpls = ctx->n_vpls[l];
    ll.lights[l].interval = ctx->interval[l];
  }
  return cuda_check(ctx, drv::launch_surrogate_pairs(ctx->s(), ctx->cfg, ctx->last_volume, ll, ctx->counter,
                                                     ctx->entries, ctx->entry_stride, ctx->voxels(), seed, n_pairs,
                                                     features, targets, ctx->sur_features),
                    "surrogate_make_pairs");
}

size_t drv_surrogate_train_scratch_floats(int32_t n) { return n > 0 ? drv::surrogate_train_scratch_floats(n) : 0; }

drv_status drv_surrogate_train_step(const float* features, const float* targets, int32_t n, float* params,
                                    float* adam_m, float* adam_v, float* scratch, int32_t step, float lr,
                                    float conf_tau, float weight_decay, float* loss_out, void* cuda_stream) {
  if (!features || !targets || n < 1 || !params || !adam_m || !adam_v || !scratch || step < 1 || !(lr > 0.0f))
    return DRV_ERR_INVALID_ARG;
  cudaError_t e = drv::launch_surrogate_train_step((cudaStream_t)cuda_stream, features, targets, n, params, adam_m,
                                                   adam_v, scratch, step, lr, conf_tau, weight_decay, loss_out);
  return e == cudaSuccess ? DRV_OK : DRV_ERR_CUDA;
}

}  // extern "C"
