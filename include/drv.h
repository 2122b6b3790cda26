/*
 * drv.h — C ABI of the GB300 dynamic-radiance-volume indirect-lighting path.
 *
 * The path is the per-frame stage sequence of Wumpf/DynamicRadianceVolume's
 * `Renderer::Draw` (DynamicRadianceVolume/rendering/renderer.cpp:539-594):
 *
 *   RSM downsample + VPL extraction  (downsamplersm.frag, cacheLightingRSM.comp:135-163)
 *   VoxelizeScene + opacity mips     (voxelization.cpp:90-176, voxelize.*, voxelmipmap.comp)
 *   AllocateCaches                   (renderer.cpp:951-992, cacheGather.comp, cachePrepareLighting.comp)
 *   LightCachesRSM                   (renderer.cpp:899-933, cacheLightingRSM.comp)
 *   ApplyCaches                      (renderer.cpp:1047-1079, cacheApply.frag, lightcache.glsl:137-183)
 *
 * In the reference these are private `Renderer` methods driving GLSL
 * programs; here each is an `extern "C"` entry point over plain device
 * pointers, asynchronous on the context's CUDA stream. No function throws;
 * every function returns a drv_status. Device-side failures (cache capacity
 * overflow, bounded waits that ran out) are latched into a device error word
 * and surface from drv_sync / drv_get_cache_count / drv_get_error.
 *
 * Conventions (the reference's, see each struct):
 *  - 4x4 matrices are 16 floats, row-major, applied as M * v (column vector).
 *    This equals the reference's GLSL `vec4 * mat4` with row-major ei::Mat4x4
 *    uploaded as-is (e.g. cacheGather.comp:118).
 *  - Images are row-major, x fastest; row 0 is the bottom row (GL texture
 *    origin). 3D images are x fastest, then y, then z.
 *  - Depth is reversed-Z in [0,1] (0 = cleared/far, renderer.cpp:113-117).
 */
#ifndef DRV_H_
#define DRV_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DRV_ABI_VERSION 10  /* 10: the voxel sampling copies (voxel_corners, voxel_mip_records) are x-fastest */
#define DRV_MAX_CASCADES 4   /* MAX_NUM_ADDRESS_VOLUME_CASCADES, globalubos.glsl:43 */
#define DRV_MAX_LIGHTS 16    /* maxExpectedLights, renderer.cpp:80 */
#define DRV_LIGHTING_THREADS_PER_GROUP 64 /* lightcache.glsl:95 */

typedef enum drv_status {
  DRV_OK = 0,
  DRV_ERR_INVALID_ARG = 1,
  DRV_ERR_CAPACITY = 2,   /* more caches requested than DrvConfig.max_caches */
  DRV_ERR_CUDA = 3,
  DRV_ERR_TIMEOUT = 4,    /* a bounded device-side wait gave up */
  DRV_ERR_NOT_SUPPORTED = 5,
  DRV_ERR_NUMERIC = 6     /* non-finite value found in an input */
} drv_status;

/* Device error-word bits (drv_get_error). */
#define DRV_DEVERR_CAPACITY 0x1u
#define DRV_DEVERR_TIMEOUT 0x2u
#define DRV_DEVERR_BOUNDS 0x4u   /* an atlas slot named a cache beyond the frame's count (drv_apply) */
#define DRV_DEVERR_NUMERIC 0x8u  /* a non-finite input value (DrvTuning.check_inputs) */

typedef enum drv_sh2_sign {
  /* Host constants exactly as renderer.cpp:296-300 uploads them
   * (ShCosLobeFactor2n2_p1_n1 = -sqrt(15 pi)/8). */
  DRV_SH2_SIGN_REFERENCE = 0,
  /* Mathematically correct band-2 cosine-lobe factor (+sqrt(15 pi)/8). */
  DRV_SH2_SIGN_FIXED = 1
} drv_sh2_sign;

typedef enum drv_precision {
  DRV_PRECISION_FP32 = 0,      /* FP32 storage, FP32 accumulation */
  DRV_PRECISION_BF16 = 1       /* BF16 VPL flux/normal + cache SH, FP16 mips, Kahan FP32 accumulation */
} drv_precision;

typedef enum drv_visibility {
  DRV_VISIBILITY_CONE = 0,      /* voxel cone trace, cacheLightingRSM.comp:167-232 */
  DRV_VISIBILITY_SURROGATE = 1  /* BF16 MLP surrogate with cone-trace fallback */
} drv_visibility;

typedef enum drv_normal_format {
  DRV_NORMAL_RG16I = 0,   /* PackNormal16I, utils.glsl:83-89 (reference layout) */
  DRV_NORMAL_F32X3 = 1
} drv_normal_format;

/* G-buffer diffuse: linear RGB F32, or the reference's SRGB8 target
 * (renderer.cpp:468, written with FRAMEBUFFER_SRGB on, renderer.cpp:507):
 * 3 bytes per pixel, sRGB-encoded, read back as linear through the GL sRGB
 * decode (GL 4.5 section 8.24). */
/* RSM flux and (d, d^2): F32, or F16 as the reference's RGB16F / RG16F
 * targets (renderer.cpp:1288-1297); the context's mip chain below the caller's
 * level is F32 either way. */
typedef enum drv_rsm_format {
  DRV_RSM_F32 = 0,
  DRV_RSM_F16 = 1
} drv_rsm_format;

typedef enum drv_albedo_format {
  DRV_ALBEDO_F32X3 = 0,
  DRV_ALBEDO_SRGB8 = 1
} drv_albedo_format;

/* Roughness / metallic per pixel (GBuffer_RoughnessMetalic): the
 * reference's RG8 unorm target (renderer.cpp:469, 2 bytes per pixel, read as
 * byte / 255) or RG F32. */
typedef enum drv_rough_metal_format {
  DRV_ROUGH_METAL_RG8 = 0,
  DRV_ROUGH_METAL_F32 = 1
} drv_rough_metal_format;

/* Compile-time specialisations and setters of the reference's Renderer
 * (renderer.hpp:63-142, renderer.cpp:197-246). */
typedef struct DrvConfig {
  int32_t width, height;            /* BackbufferResolution */
  int32_t sh_order;                 /* 1: INDDIFFUSE_VIA_SH1, 2: INDDIFFUSE_VIA_SH2 */
  int32_t indirect_shadow;          /* INDIRECT_SHADOW */
  int32_t max_cone_steps;           /* cone loop bound, 32 in cacheLightingRSM.comp:211 */
  float cascade_transition;         /* CAVTransitionZoneSize; <= 0 disables ADDRESSVOL_CASCADE_TRANSITIONS */
  int32_t n_cascades;               /* 1..4 */
  int32_t cav_res;                  /* AddressVolumeResolution */
  float cascade_world_size[DRV_MAX_CASCADES]; /* m_CAVCascadeWorldSize */
  int32_t voxel_res;                /* VoxelResolution (power of two) */
  uint32_t max_caches;              /* MaxNumLightCaches */
  int32_t precision;                /* drv_precision */
  int32_t visibility;               /* drv_visibility */
  float surrogate_conf_threshold;   /* confidence below which the cone tracer re-traces a pair */
  int32_t sh2_sign;                 /* drv_sh2_sign */
  int32_t max_lights;               /* lights per frame, <= DRV_MAX_LIGHTS */
  int32_t max_rsm_resolution;       /* largest RSMRenderResolution any light will use */
  int32_t output_format;            /* drv_output_format of drv_apply / drv_frame's out_rgb */
  int32_t output_blend;             /* drv_output_blend */
  /* INDIRECT_SPECULAR (renderer.cpp:200-206): 0 = off (the reference's
   * default, m_indirectSpecular false); otherwise SPECULARENVMAP_PERCACHESIZE,
   * the per-cache envmap resolution, a power of two in 4..64 (16 in the
   * reference). With it on, the light stage also fills a per-cache specular
   * envmap, skips VPLs whose flux sum is below 0.001 (for the SH too, as
   * cacheLightingRSM.comp:240-241 does), and the apply adds the specular
   * term with the G-buffer's roughness / metallic. */
  int32_t specular_envmap_size;
  int32_t specular_fill_level;      /* m_specularEnvmapMaxFillHolesLevel, 0..log2(size) (0 in the reference) */
} DrvConfig;

/* The apply's target: RGB F32 (width*height*3 floats), or the reference's
 * RGBA16F HDR back buffer (renderer.cpp:477; width*height*4 halves; alpha 1
 * when written, kept when added). */
typedef enum drv_output_format {
  DRV_OUTPUT_RGB32F = 0,
  DRV_OUTPUT_RGBA16F = 1
} drv_output_format;

/* Written, or added to what the target holds (the reference's blending,
 * glBlendFunc(GL_ONE, GL_ONE) renderer.cpp:119 with BLEND on in
 * ApplyCaches, renderer.cpp:1053: indirect light on top of the direct light;
 * an RGBA16F sum is formed in FP32 and rounded once). */
typedef enum drv_output_blend {
  DRV_OUTPUT_WRITE = 0,
  DRV_OUTPUT_ADD = 1
} drv_output_blend;

/* CAVCascade, globalubos.glsl:48-58 (std140, 64 B). */
typedef struct DrvCascade {
  float min[3];
  float world_voxel_size;
  float max[3];
  float _pad0;
  float decision_min[3];
  float _pad1;
  float decision_max[3];
  float _pad2;
} DrvCascade;

/* VolumeInfo UBO, globalubos.glsl:62-75. */
typedef struct DrvVolumeInfo {
  float volume_world_min[3];
  float voxel_size_in_world;
  float volume_world_max[3];
  float cav_transition_zone_size;
  DrvCascade cascades[DRV_MAX_CASCADES];
} DrvVolumeInfo;

/* PerFrame UBO, globalubos.glsl:33-42 (the fields the path reads). */
typedef struct DrvPerFrame {
  float view_projection[16];
  float inverse_view_projection[16];
  float camera_position[3];
  float _pad0;
  float camera_direction[3];
  float _pad1;
} DrvPerFrame;

/* SpotLight UBO, globalubos.glsl:85-110, filled by drv_prepare_light
 * (Renderer::PrepareLights, renderer.cpp:664-725). */
typedef struct DrvSpotLight {
  float intensity[3];
  float shadow_normal_offset;
  float shadow_bias;
  float position[3];
  float direction[3];
  float cos_half_angle;
  float view_projection[16];
  float inverse_view_projection[16];
  int32_t rsm_render_resolution;
  int32_t rsm_read_resolution;
  float val_area_factor;
  float indirect_shadow_lod;
  float indirect_shadow_block_size;
  int32_t indirect_shadow_sample_interval;
  float indirect_shadow_super_val_width;
  float indirect_shadow_sampling_offset;
} DrvSpotLight;

/* Light description, scene/light.hpp:8-54 (spot lights only, as the
 * reference asserts at renderer.cpp:672). */
typedef struct DrvLightDesc {
  float intensity[3];
  float position[3];
  float direction[3];
  float half_angle;                 /* radians */
  uint32_t rsm_resolution;          /* power of two */
  uint32_t rsm_read_lod;
  uint32_t indirect_shadow_lod;
  float near_plane, far_plane;      /* Light::nearPlane/farPlane, scene.cpp:6-7 */
} DrvLightDesc;

/* Camera (camera/camera.hpp:8-30). fov_y in degrees; the projection is
 * DX-style reversed-Z (far and near swapped, camera.hpp:27-28). */
typedef struct DrvCamera {
  float position[3];
  float direction[3];
  float up[3];
  float fov_y_deg;
  float aspect;
  float near_plane, far_plane;
} DrvCamera;

/* Procedural scene primitive: an axis-aligned box. `inward` boxes are rooms
 * (rays hit their inside faces, normals point inward). The reference loads
 * meshes through assimp; the procedural box scene replaces them. */
typedef struct DrvBox {
  float min[3];
  float max[3];
  float albedo[3];
  int32_t inward;
} DrvBox;

typedef struct DrvScene {
  int32_t n_boxes;
  const DrvBox* boxes;              /* host pointer */
  float aabb_min[3];                /* Scene::GetBoundingBox, scene.cpp:36-48 */
  float aabb_max[3];
} DrvScene;

/* G-buffer (renderer.cpp:466-471), device pointers, width*height texels;
 * each array 4-byte aligned (DRV_ERR_INVALID_ARG otherwise). */
typedef struct DrvGBufferView {
  int32_t width, height;
  const float* depth;               /* D32F reversed-Z */
  const void* normal;               /* drv_normal_format */
  int32_t normal_format;
  const void* albedo;               /* drv_albedo_format */
  int32_t albedo_format;
  const void* rough_metal;          /* drv_rough_metal_format; read only with specular_envmap_size > 0 */
  int32_t rough_metal_format;
} DrvGBufferView;

/* Writable G-buffer for the ray-cast producer. */
typedef struct DrvGBufferOut {
  float* depth;
  int16_t* normal_rg16i;            /* may be NULL */
  float* normal_f32;                /* may be NULL */
  float* albedo;
} DrvGBufferOut;

/* One level of a reflective shadow map (renderer.cpp:1288-1297), device
 * pointers, resolution^2 texels: flux RGB (already divided by pi), packed
 * normal RG16I, (distance, distance^2). */
typedef struct DrvRSMView {
  int32_t resolution;
  const void* flux;                 /* RGB, drv_rsm_format */
  const int16_t* normal;            /* RG16I PackNormal16I */
  const void* depth_lin_sq;         /* (d, d^2), drv_rsm_format */
  int32_t format;                   /* drv_rsm_format */
} DrvRSMView;

typedef struct DrvRSMOut {
  float* flux;
  int16_t* normal;
  float* depth_lin_sq;
} DrvRSMOut;

/* One virtual area light as the light stage consumes it (LightInfo,
 * cacheLightingRSM.comp:34-40), 48 B. */
typedef struct DrvVPL {
  float flux[3];
  float disc_area;
  float position[3];
  float _pad0;
  float normal[3];
  float _pad1;
} DrvVPL;

/* DRV_PRECISION_BF16 storage of a VPL (32 B): position and disc area stay
 * FP32 (directions are computed from them), flux and normal are BF16. */
typedef struct DrvVPLBF16 {
  float position[3];
  float disc_area;
  uint16_t flux_bf16[3];
  uint16_t normal_bf16[3];
  uint32_t _pad;
} DrvVPLBF16;

/* DRV_PRECISION_BF16 cache entry (64 B): the cell it sits on instead of an
 * FP32 position (x | y << 9 | z << 18 | cascade << 27, cascade-local corner
 * coordinates; the position is cell * WorldVoxelSize + Min as in
 * cacheGather.comp:65), then the 27 SH values in BF16, ordered coefficient-
 * major (SH00, SH1neg1, SH10, SH1pos1, SH2neg2, SH2neg1, SH20, SH2pos1,
 * SH2pos2), RGB within each; SH1 leaves the last 15 zero. */
typedef struct DrvCacheEntryBF16 {
  uint32_t cell;
  uint16_t sh_bf16[27];
  uint16_t _pad[3];
} DrvCacheEntryBF16;

/* Per-block indirect-shadow cone source (cacheLightingRSM.comp:171-192):
 * average VAL position and distToSphereRad. */
typedef struct DrvShadowCone {
  float average_val_position[3];
  float dist_to_sphere_rad;
} DrvShadowCone;

/* Counter buffer, lightcache.glsl:83-90. */
typedef struct DrvCacheCounter {
  uint32_t groups_x, groups_y, groups_z;
  int32_t total_light_cache_count;
} DrvCacheCounter;

/* Read-only views of the context's device buffers (for callers that render
 * debug views or compare results). */
typedef struct DrvBuffers {
  void* cache_entries;              /* FP32: LightCacheEntry std430, 64 B (SH1) / 128 B (SH2); BF16: DrvCacheEntryBF16 */
  uint32_t entry_stride;
  uint32_t* cav_atlas;              /* R32UI [n_cascades*res][res][res], x fastest */
  DrvCacheCounter* counter;
  uint32_t* voxel_bits;             /* level 0 as a bitmask, bit (x&31) of word ((z*N+y)*N+x)/32 */
  uint8_t* voxel_corners;           /* level 0 corner-packed: byte (x,y,z) = voxels (x+dx,y+dy,z+dz), +1 clamped,
                                       bit dx|dy<<1|dz<<2, at (z*N+y)*N+x */
  void* voxel_mips[16];             /* levels 1..L (index 1..L), float (FP32 precision) or half (BF16 precision) */
  int32_t n_voxel_levels;           /* levels including 0 */
  void* vpls[DRV_MAX_LIGHTS];       /* VPL array per light, Morton order: DrvVPL (FP32) or DrvVPLBF16 */
  DrvShadowCone* cones[DRV_MAX_LIGHTS];
  int32_t n_vpls[DRV_MAX_LIGHTS];
  int32_t n_lights;
  void* voxel_mip_records[16];      /* levels 1..n_record_levels (index 1..): corner-packed 16-byte records, record
                                       (x,y,z) = FP16 texels (x+dx,y+dy,z+dz) of the level, +1 clamped, slot
                                       dx|dy<<1|dz<<2, at (z*n+y)*n+x; FP32 precision: levels 1..3 (FP16 holds
                                       their texels k / 8^l exactly), BF16 precision: every level */
  int32_t n_record_levels;
  /* The per-cache specular envmap atlas (m_specularEnvmap, renderer.cpp:253-
   * 287): n_specular_levels levels of specular_atlas_size >> level texels
   * square, R11F_G11F_B10F packed in 32 bits (R bits 0-10, G 11-21, B 22-31),
   * rows contiguous; cache i's region at each level is the square of side
   * specular_envmap_size >> level at column i % n, row i / n (n =
   * specular_atlas_size / specular_envmap_size). Only allocated caches'
   * regions are written; NULL when specular is off. */
  uint32_t* specular_envmap[8];
  int32_t specular_atlas_size;
  int32_t n_specular_levels;
} DrvBuffers;

typedef struct DrvContext DrvContext;

/* ---- lifetime ----------------------------------------------------------
 * Replaces Renderer::Renderer / SetMaxCacheCount / SetCAVCascades /
 * Voxelization(...) resource creation (renderer.cpp:26-120, 248-288,
 * 1174-1193; voxelization.cpp:22-68). */
drv_status drv_create(const DrvConfig* cfg, DrvContext** out_ctx);
drv_status drv_destroy(DrvContext* ctx);
drv_status drv_set_stream(DrvContext* ctx, void* cuda_stream);
drv_status drv_sync(DrvContext* ctx);
const char* drv_last_error_string(DrvContext* ctx);
drv_status drv_get_error(DrvContext* ctx, uint32_t* out_bits);
drv_status drv_get_buffers(DrvContext* ctx, DrvBuffers* out);
void drv_default_config(DrvConfig* cfg);
int drv_abi_version(void);
/* sizeof of the ABI structs in the order DrvConfig, DrvCascade,
 * DrvVolumeInfo, DrvPerFrame, DrvSpotLight, DrvLightDesc, DrvCamera, DrvBox,
 * DrvScene, DrvGBufferView, DrvGBufferOut, DrvRSMView, DrvRSMOut, DrvVPL,
 * DrvShadowCone, DrvCacheCounter, DrvBuffers (for binding checks). Returns
 * the number of sizes written. */
int drv_struct_sizes(uint32_t* out, int capacity);

/* ---- host-side parameter setup ------------------------------------------
 * Renderer::UpdateVolumeUBO (renderer.cpp:346-431). */
drv_status drv_compute_volume_info(const DrvConfig* cfg, const float aabb_min[3], const float aabb_max[3],
                                   const float camera_position[3], DrvVolumeInfo* out);
/* Renderer::PrepareLights (renderer.cpp:664-725). */
drv_status drv_prepare_light(const DrvLightDesc* light, DrvSpotLight* out);
/* Renderer::UpdatePerFrameUBO (renderer.cpp:324-344) with the camera of camera/camera.hpp:27-30. */
drv_status drv_prepare_camera(const DrvCamera* cam, DrvPerFrame* out);
/* Seeded procedural scene: an inward unit-cube room plus n_boxes boxes with
 * sizes U[size_min,size_max] per axis and albedo U[albedo_min,albedo_max]. */
drv_status drv_generate_scene(uint64_t seed, int32_t n_boxes, float size_min, float size_max,
                              float albedo_min, float albedo_max, DrvBox* out_boxes /* n_boxes+1 */,
                              DrvScene* out_scene);
/* Seeded camera and spot light inside the unit room, clear of the scene's
 * boxes (scene may be NULL). */
drv_status drv_generate_camera(uint64_t seed, const DrvScene* scene, float aspect, DrvCamera* out);
drv_status drv_generate_light(uint64_t seed, const DrvScene* scene, uint32_t rsm_resolution, uint32_t rsm_read_lod,
                              uint32_t indirect_shadow_lod, DrvLightDesc* out);

/* ---- input producers (replace the reference's raster passes) -------------
 * G-buffer fill (fillgbuffer.frag, renderer.cpp:760-776) as a ray cast. */
drv_status drv_raycast_gbuffer(DrvContext* ctx, const DrvScene* scene, const DrvCamera* camera,
                               const DrvPerFrame* frame, int32_t width, int32_t height, const DrvGBufferOut* out);
/* RSM fill (fillrsm.frag:24-62) as a ray cast from the spot light. */
drv_status drv_raycast_rsm(DrvContext* ctx, const DrvScene* scene, const DrvSpotLight* light,
                           const DrvRSMOut* out);

/* A triangle mesh (device buffers): world-space positions (xyz per vertex),
 * optional vertex normals (xyz per vertex; NULL: face normals), optional
 * linear RGB albedo per triangle (NULL: 1), indices (3 per triangle; NULL:
 * consecutive vertex triples). Untextured: the reference's base-colour and
 * normal maps are not read. */
typedef struct DrvMesh {
  const float* positions;
  const float* normals;
  const float* albedo;
  const uint32_t* indices;
  int32_t n_vertices, n_triangles;
} DrvMesh;

/* The G-buffer fill (fillgbuffer.frag) and the RSM fill (fillrsm.frag:24-62)
 * of a triangle mesh: visibility by rasterising the mesh (near-plane clip,
 * pixel centres, reversed-Z nearest), then the pixel's ray against the
 * visible triangle, shaded as the box producers above (normals turned to the
 * viewer). The first call at a size allocates a 64-bit per-pixel visibility
 * buffer (not while the stream is being captured). */
drv_status drv_raster_gbuffer(DrvContext* ctx, const DrvMesh* mesh, const DrvCamera* camera,
                              const DrvPerFrame* frame, int32_t width, int32_t height, const DrvGBufferOut* out);
drv_status drv_raster_rsm(DrvContext* ctx, const DrvMesh* mesh, const DrvSpotLight* light, const DrvRSMOut* out);

/* ---- the per-frame stages ----------------------------------------------- */
/* ShadowMap::PrepareRSM + downsamplersm.frag (renderer.cpp:1300-1339): build
 * the RSM mip chain of light `light_index` from its render-resolution level
 * down to 1x1 inside the context. */
drv_status drv_prepare_rsm(DrvContext* ctx, int32_t light_index, const DrvSpotLight* light,
                           const DrvRSMView* full_res);
/* VPL extraction at RSMReadResolution (cacheLightingRSM.comp:141-158) and the
 * per-block shadow cone sources (cacheLightingRSM.comp:171-192). Requires
 * drv_prepare_rsm for the same light. */
drv_status drv_extract_vpls(DrvContext* ctx, int32_t light_index, const DrvSpotLight* light);
/* Makes the scene resident on the device (the reference keeps its meshes in
 * GL buffers). drv_voxelize / drv_raycast_* call it implicitly; a changed
 * scene is uploaded synchronously, so during CUDA-graph capture the scene must
 * already be resident. */
drv_status drv_set_scene(DrvContext* ctx, const DrvScene* scene);
/* Voxelization::VoxelizeScene (voxelization.cpp:90-142): surface voxels of the
 * scene into the level-0 bitmask. */
drv_status drv_voxelize(DrvContext* ctx, const DrvScene* scene, const DrvVolumeInfo* vol);
/* Voxelization::VoxelizeScene for a triangle mesh (voxelize.vert/.geom/.frag:
 * dominant-axis projection, half-voxel conservative raster, +-1 voxel depth
 * conservativeness): the level-0 bitmask is cleared and the triangles'
 * surface voxels set. positions: device, xyz per vertex in world space
 * (n_vertices); indices: device, 3 per triangle, or NULL for consecutive
 * vertex triples; triangles naming a vertex >= n_vertices are skipped. The
 * opacity mips follow with drv_build_opacity_mips; drv_frame voxelizes the
 * box scene it is given, so a mesh frame runs its stages one by one. */
drv_status drv_voxelize_triangles(DrvContext* ctx, const float* positions, int32_t n_vertices, const uint32_t* indices,
                                  int32_t n_triangles, const DrvVolumeInfo* vol);
/* voxelmipmap.comp + voxelization.cpp:155-172: the full opacity mip chain. */
drv_status drv_build_opacity_mips(DrvContext* ctx);
/* Renderer::AllocateCaches (renderer.cpp:951-992): clear counter + atlas,
 * cacheGather.comp, cachePrepareLighting.comp. */
drv_status drv_allocate_caches(DrvContext* ctx, const DrvGBufferView* gbuffer, const DrvPerFrame* frame,
                               const DrvVolumeInfo* vol);
/* Renderer::LightCachesRSM (renderer.cpp:899-933): all lights accumulated into
 * the cache SH (the reference dispatches once per light with `+=`). */
drv_status drv_light_caches(DrvContext* ctx, const DrvSpotLight* lights, int32_t n_lights,
                            const DrvVolumeInfo* vol, const DrvPerFrame* frame);
/* Renderer::ApplyCaches (renderer.cpp:1047-1079, cacheApply.frag): indirect
 * diffuse radiance per pixel into out_rgb (device; DrvConfig.output_format:
 * width*height*3 floats, or width*height*4 halves; DrvConfig.output_blend:
 * written, or added; pixels with depth < 1e-5 get 0, or are left as they are
 * when adding). */
drv_status drv_apply(DrvContext* ctx, const DrvGBufferView* gbuffer, const DrvPerFrame* frame,
                     const DrvVolumeInfo* vol, float* out_rgb);
/* All stages of one frame on the context stream (Renderer::Draw,
 * DYN_RADIANCE_VOLUME branch, renderer.cpp:539-594): voxelize (if indirect
 * shadow), mips, per-light RSM prepare + VPL extraction, allocate, light,
 * apply. Device pointers only; capturable in a CUDA graph. */
drv_status drv_frame(DrvContext* ctx, const DrvScene* scene, const DrvGBufferView* gbuffer,
                     const DrvPerFrame* frame, const DrvVolumeInfo* vol,
                     const DrvSpotLight* lights, const DrvRSMView* rsms, int32_t n_lights,
                     float* out_rgb);
/* Optional cache-count readback (renderer.cpp:960-966). Synchronises. */
drv_status drv_get_cache_count(DrvContext* ctx, uint32_t* out_count);

/* ---- learned visibility surrogate -----------------------------------------
 * No counterpart in the reference: an MLP (32 inputs -> 64 -> 64 -> 64 -> 2,
 * GELU in its sigmoid form x sigmoid(1.702 x); BF16 weights and activations,
 * FP32 accumulation on the tcgen05 tensor cores) predicts the indirect-shadow
 * cone's visibility of a (cache, shadow block) pair plus a confidence; with
 * DrvConfig.visibility = DRV_VISIBILITY_SURROGATE, drv_light_caches uses it and
 * re-traces pairs whose confidence is below DrvConfig.surrogate_conf_threshold
 * with the cone. Parameters are a flat FP32 array of DRV_SURROGATE_PARAMS
 * floats: W1[64][32], b1[64], W2[64][64], b2, W3[64][64], b3, W4[2][64], b4[2]
 * (weights [out][in]). Input 31 is the constant 1. */
#define DRV_SURROGATE_INPUTS 32
#define DRV_SURROGATE_PARAMS 10562
/* Uploads parameters (device FP32 array) as the context's BF16 inference weights. */
drv_status drv_set_surrogate_params(DrvContext* ctx, const float* params_device);
/* The inputs the uploaded parameters were trained on:
 *  SEGMENT8 (default): the cache and the block's cone target in normalised
 *    volume coordinates, the VPL normal, and eight trilinear opacity samples
 *    of voxel mip 3 at the midpoints of eight equal parts of the segment
 *    between them (inputs 0-16);
 *  CONE4: 27 inputs, adding the cone's aperture and length, the direction,
 *    and the cone's own first four samples and their composited occlusion
 *    (mip-3 samples over the part of the segment the cone reaches);
 *  CONE8: inputs 0-8 as SEGMENT8, then eight samples of the cone's own
 *    sampler at its level of detail at geometrically spaced marched
 *    distances, their composited occlusion, the aperture, the march length
 *    and the direction (23 inputs). */
enum { DRV_SURROGATE_FEATURES_SEGMENT8 = 0, DRV_SURROGATE_FEATURES_CONE4 = 1, DRV_SURROGATE_FEATURES_CONE8 = 2 };
drv_status drv_set_surrogate_features(DrvContext* ctx, int32_t feature_set);
/* Training pairs from the context's current frame (after drv_extract_vpls,
 * drv_build_opacity_mips and drv_allocate_caches): random (cache, shadow
 * block) pairs, features[n][32] (the context's feature set) and the
 * cone-traced visibility targets[n].
 * seed = DRV_SURROGATE_ENUMERATE lists the pairs in order instead (pair i =
 * cache i / n_blocks, block i % n_blocks, blocks of all lights in light
 * order). */
#define DRV_SURROGATE_ENUMERATE 0xFFFFFFFFFFFFFFFFull
drv_status drv_surrogate_make_pairs(DrvContext* ctx, uint64_t seed, int32_t n_pairs, float* features,
                                    float* targets);
/* Device scratch (floats) one drv_surrogate_train_step over n samples needs. */
size_t drv_surrogate_train_scratch_floats(int32_t n);
/* One optimisation step over n samples: fused forward/backward per 64-sample
 * chunk, then Adam (step >= 1) on params with moments adam_m/adam_v (all
 * device FP32, DRV_SURROGATE_PARAMS each). loss_out (device, 2 floats, may be
 * NULL) receives the summed visibility and confidence losses. */
drv_status drv_surrogate_train_step(const float* features, const float* targets, int32_t n, float* params,
                                    float* adam_m, float* adam_v, float* scratch, int32_t step, float lr,
                                    float conf_tau, float weight_decay, float* loss_out, void* cuda_stream);
/* Evaluates the context's inference weights on n feature rows (the
 * tensor-core kernel of the light stage; input 31 is taken as 1):
 * out[n][2] = (visibility, confidence). */
drv_status drv_surrogate_eval(DrvContext* ctx, const float* features, int32_t n, float* out);
/* Pairs re-traced with the cone by the last surrogate light stage. Synchronises. */
drv_status drv_get_surrogate_fallbacks(DrvContext* ctx, uint32_t* out);
/* Pairs the last surrogate light stage evaluated with the MLP (the
 * (cache, shadow block) pairs that can contribute) and of those re-traced
 * with the cone. Synchronises. */
drv_status drv_get_surrogate_stats(DrvContext* ctx, uint32_t* evaluated, uint32_t* retraced);

/* ---- execution knobs -------------------------------------------------------
 * No counterpart in the reference (its shaders have fixed work-group sizes).
 * Knobs change how the GPU is used, not what is computed: results stay the
 * same up to the order of FP32 summation. Zero fields keep the default. */
typedef struct DrvTuning {
  int32_t light_path;      /* DRV_LIGHT_PATH_*: light stage as one launch or as cull, cone, gather */
  uint32_t pair_capacity;  /* split stage: pairs the list may hold; caches that do not fit are traced
                              by the gather itself (exact cones). 0: the whole allocation; above the
                              allocation: the list grows to it (synchronises; not while capturing) */
  int32_t cone_ctas_per_sm;   /* split stage: CTAs of the cone pass per SM (0: as many as fit) */
  int32_t gather_ctas_per_sm; /* split stage: CTAs of the gather pass per SM (0: as many as fit) */
  int32_t time_kernels;       /* nonzero: the split light stage records CUDA events between its
                                 kernels (not while the stream is being captured) */
  int32_t plain_voxel_reads;  /* nonzero: the cone tracer reads the plain mip arrays instead of the
                                 corner-packed mip records; the result is the same bit for bit */
  int32_t surrogate_wait_test; /* test hook, nonzero: the surrogate pass withholds its first tensor-core
                                  commit, so its bounded wait (~10 ms here) runs out; the stage then
                                  reports DRV_ERR_TIMEOUT from drv_sync and leaves the shadowing unset */
  int32_t count_voxel_reads;   /* nonzero: the split stage's cone pass runs its measuring instance, which
                                  also counts the voxel loads of its cones (drv_get_cone_voxel_reads);
                                  results are the same bit for bit */
  int32_t check_inputs;        /* nonzero: drv_prepare_rsm, drv_allocate_caches and drv_apply (so also
                                  drv_frame) scan their float inputs (RSM flux and (d, d^2), depth, F32
                                  normals and albedo) for NaN / Inf; one found is reported once, as
                                  DRV_ERR_NUMERIC, by the next drv_sync (DRV_DEVERR_NUMERIC). A debugging
                                  aid: it reads every input once more */
  int32_t cull_caches_per_pass; /* split stage: caches the cull tests per pass against the VPL records staged
                                   in shared memory (the cull's tile: 2, 4 or 8; 0: 4) */
  int32_t gather_threads;      /* split stage: threads per CTA of the gather, one CTA per SM sharing its
                                  staged VPLs, a warp per unit of a cache's pairs (256 or 512; 0: 512) */
  int32_t tensor_core_apply;   /* nonzero: with BF16 entries (no specular) the apply evaluates a warp's
                                  cells on the tensor cores (mma.sync of per-pixel factors against a
                                  cell's corner SH) instead of each corner's SH per pixel on the FP32
                                  pipes; the same result to FP32 rounding (measured slower at 1080p:
                                  107 against 101 us) */
  int32_t per_light_dispatch;  /* nonzero: the split light stage runs once per light, each light's SH added
                                  into the entries in turn, as the reference dispatches one lighting pass
                                  per light (renderer.cpp:924-932); the same result to FP32 rounding (BF16
                                  entries are rounded once per light). Kernel timing is off, the pair and
                                  surrogate counts are the last light's, and with indirect specular the
                                  envmaps are gathered after the loop with their own cones */
  int32_t gather_wait_test;    /* test hook, nonzero: the split stage's gather waits for VPL copies it never
                                  issues, so its bounded wait (~10 ms here) runs out; the stage reports
                                  DRV_ERR_TIMEOUT from drv_sync and its caches miss their SH */
} DrvTuning;
enum { DRV_LIGHT_PATH_AUTO = 0, DRV_LIGHT_PATH_SINGLE = 1, DRV_LIGHT_PATH_SPLIT = 2 };
drv_status drv_set_tuning(DrvContext* ctx, const DrvTuning* tuning);
drv_status drv_get_tuning(DrvContext* ctx, DrvTuning* tuning);

/* (cache, shadow block) pairs the last split light stage found able to
 * contribute (each traced or evaluated once; those beyond the list's
 * capacity traced by the gather). Synchronises. */
drv_status drv_get_light_pairs(DrvContext* ctx, uint32_t* pairs);

/* Voxel loads of the last split light stage's cone pass run with
 * DrvTuning.count_voxel_reads: reads[0] level-0 corner-packed bytes (1 B each),
 * reads[1] corner-packed FP16 mip records (16 B each), reads[2] plain mip
 * texels (4 B with FP32 precision, 2 B with BF16). These are the algorithmic
 * bytes of the cone march (its L1/L2 roofline). Synchronises. No counterpart in
 * the reference. */
drv_status drv_get_cone_voxel_reads(DrvContext* ctx, uint32_t reads[3]);

/* Load throughput of this GPU from L1 (level 1: every CTA re-reads its own
 * 32 KB window; buffer >= 64 KB x SMs) or from L2 (level 2: all SMs sweep
 * `bytes` of the buffer with loads that bypass L1; a buffer below the L2 size
 * stays resident), in GB/s: the peaks the cone pass's voxel loads are held
 * against. buffer: device, 16-byte aligned, never written. Synchronises. No
 * counterpart in the reference. */
drv_status drv_measure_load_bandwidth(int32_t level, const void* buffer, size_t bytes, int32_t reps,
                                      void* cuda_stream, float* out_gbs);

/* Kernels of the split light stage, in launch order (DrvTuning.time_kernels). */
enum {
  DRV_LK_CULL = 0, DRV_LK_CLASSIFY = 1, DRV_LK_SCATTER = 2, DRV_LK_MLP = 3, DRV_LK_CONE = 4, DRV_LK_GATHER = 5,
  DRV_LK_COUNT = 6
};
/* Milliseconds of each kernel of the last split light stage launched with
 * time_kernels set (0 for kernels that stage did not run). Synchronises.
 * DRV_ERR_INVALID_ARG when no such stage ran. */
drv_status drv_get_light_kernel_ms(DrvContext* ctx, float ms[DRV_LK_COUNT]);

/* ---- indirect specular ---------------------------------------------------
 * Renderer::PrepareSpecularEnvmaps (renderer.cpp:994-1043): the mip levels
 * of every allocated cache's envmap (specularenvmap_mipmap.frag: each texel
 * the mean of the 2x2 texels below) and, with specular_fill_level > 0, the
 * hole fill from that level down to 1 (specularenvmap_fillholes.frag). Runs
 * after drv_light_caches (drv_frame calls it); DRV_ERR_INVALID_ARG when
 * specular is off. */
drv_status drv_prepare_specular_envmaps(DrvContext* ctx);

/* ---- brute-force RSM gather and image dumps --------------------------------
 * Renderer::ApplyRSMsBruteForce (renderer.cpp:851-871, bruteforcersm.frag):
 * per pixel, the unshadowed sum over every VAL (the context's extracted
 * VPLs of lights 0..n_lights-1; drv_extract_vpls must have run for each)
 * without caches: the ground truth the cache volume interpolates. out_rgb:
 * device, width*height*3. rough_metal: device RG F32 per pixel for the
 * reference BRDF (normalized Blinn-Phong + metallic, lightingfunctions.glsl),
 * or NULL for its diffuse term albedo/pi (the cache path's). Pixels with
 * depth below 1e-5 are 0. */
drv_status drv_bruteforce_rsm(DrvContext* ctx, const DrvGBufferView* gbuffer, const float* rough_metal,
                              const DrvPerFrame* frame, int32_t n_lights, float* out_rgb);
/* The reference's PFM dump (rendering/hdrimage.cpp:6-66): host RGB floats
 * (channels 3, or 4 with the 4th skipped), row 0 first. */
drv_status drv_write_pfm(const char* path, const float* rgb, int32_t width, int32_t height, int32_t channels);
/* Reads an RGB PFM written that way: width/height always, the pixels when rgb
 * is non-NULL (DRV_ERR_CAPACITY when more than capacity_pixels). */
drv_status drv_read_pfm(const char* path, float* rgb, int64_t capacity_pixels, int32_t* width, int32_t* height);

/* ---- batched frames ---------------------------------------------------------
 * No counterpart in the reference (one scene per renderer). Many scenes'
 * frames -- each its own context, inputs and sizes -- captured once into one
 * CUDA graph, the scenes dealt round-robin over n_streams concurrent branches,
 * and replayed with one launch. Every scene's drv_frame arguments are copied
 * into the graph at capture (kernel parameters by value): new cameras,
 * lights or buffers need a new batch. The scenes' contexts must not be used
 * on other streams while a batch of theirs runs. */
typedef struct DrvBatchScene {
  DrvContext* ctx;
  const DrvScene* scene;
  const DrvGBufferView* gbuffer;
  const DrvPerFrame* frame;
  const DrvVolumeInfo* volume;
  const DrvSpotLight* lights;
  const DrvRSMView* rsms;
  int32_t n_lights;
  float* out_rgb;                   /* device, width*height*3 */
} DrvBatchScene;
typedef struct DrvBatch DrvBatch;
/* cuda_stream: the stream the capture starts from and joins back to (not the
 * legacy default stream; NULL: an internal one). Each context's stream
 * setting is restored after the capture. */
drv_status drv_batch_create(const DrvBatchScene* scenes, int32_t n_scenes, int32_t n_streams, void* cuda_stream,
                            DrvBatch** out);
/* One launch of the whole batch on cuda_stream (NULL: the capture stream). */
drv_status drv_batch_launch(DrvBatch* batch, void* cuda_stream);
/* After a launch: per scene, milliseconds from the batch's start to the end
 * of that scene's frame, and the batch's total. Synchronises. */
drv_status drv_batch_times(DrvBatch* batch, float* scene_ms, float* total_ms);
drv_status drv_batch_destroy(DrvBatch* batch);

/* ---- allocation-free light stage ------------------------------------------
 * No counterpart in the reference: the reference renderer always owns its GL
 * buffers. This is the cache-lighting stage (the kernel behind
 * drv_light_caches) for callers that cannot allocate device memory — engines
 * running inside a fixed, pre-reserved GPU memory arena, plug-ins hosted by
 * them, code recorded into CUDA graphs. It needs no DrvContext and calls no
 * cudaMalloc: its scratch (per-chunk partial sums and per-cache tickets) is a
 * fixed array compiled into the library, which every GPU that loads the
 * library holds until exit (about 3.5 MB). The caller passes every input
 * (per-light VPL and cone arrays, the corner-packed level-0 voxel bytes and
 * the FP32 mips 1..L as laid out by drv_build_opacity_mips, the cache counter)
 * and the output (the cache entries: positions read, SH accumulated with +=)
 * as device pointers, and the stream to run on.
 *  - max_caches above DRV_STATIC_SCRATCH_MAX_CACHES returns DRV_ERR_CAPACITY;
 *  - specular_envmap_size > 0 returns DRV_ERR_INVALID_ARG (the envmap atlas
 *    belongs to a context);
 *  - FP32 precision only (DrvVPL inputs, FP32 mips, LightCacheEntry std430
 *    entries of 64 B for SH1 and 128 B for SH2): precision BF16 returns
 *    DRV_ERR_INVALID_ARG and launches nothing;
 *  - the first call on a device looks the array up on that device, in the
 *    context current then (use the device's primary context, as the CUDA
 *    runtime does); make it before any stream capture;
 *  - all calls share the array (it keeps the last call's contents; each call
 *    clears the tickets first): calls that overlap on the GPU race. */
#define DRV_STATIC_SCRATCH_MAX_CACHES 4096
drv_status drv_light_caches_static_scratch(const DrvConfig* cfg, const DrvVolumeInfo* vol,
                                           const DrvVPL* const* vpls, const DrvShadowCone* const* cones,
                                           const int32_t* n_vpls, const int32_t* intervals, int32_t n_lights,
                                           const uint8_t* voxel_corners, const float* voxel_mips,
                                           const DrvCacheCounter* counter, void* cache_entries, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* DRV_H_ */
