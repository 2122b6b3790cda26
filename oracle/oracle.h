/*
 * oracle.h — CPU FP64 restatement of Wumpf/DynamicRadianceVolume's
 * per-frame indirect-lighting shader math.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product links, imports or calls
 * this library; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark do, and only to check results against.
 *
 * The reference is GLSL inside a Windows/OpenGL 4.5 application; it cannot
 * run without a graphics stack, so parity is anchored on this restatement.
 * Each function names the reference lines it follows. Integer decisions
 * that the reference derives from FP32 arithmetic (which cell a pixel lands
 * in, which cascade it selects) are restated in binary32 with a fixed
 * operation order and no contraction (this library is compiled with
 * -ffp-contract=off), so that allocation is comparable bit-exactly; all
 * lighting math is FP64.
 *
 * Camera/projection helpers of the reference come from the absent `epsilon`
 * library (ei::perspectiveDX, ei::camera, ei::invert): parity unpinned there;
 * both sides share the conventions written in include/drv.h.
 */
#ifndef DRV_ORACLE_H_
#define DRV_ORACLE_H_

#include <stdint.h>
#include "../include/drv.h"

#ifdef __cplusplus
extern "C" {
#endif

/* -- small known-answer helpers --------------------------------------- */
void orc_morton_decode(uint32_t morton, uint32_t* x, uint32_t* y);
void orc_pack_normal16i(const double n[3], int16_t out[2]);
void orc_unpack_normal16i(const int16_t packed[2], double out[3]);
/* cos_lobe[5] = ShCosLobeFactor0,1,2n2_p1_n1,20,2p2; eva[5] = ShEvaFactor* */
void orc_sh_constants(int sh2_sign, double cos_lobe[5], double eva[5]);
/* SampleCacheIrradiance for a single entry (27 doubles, see orc_light_caches). */
void orc_sh_irradiance(int sh_order, int sh2_sign, const double* sh27, const double n[3], double out_rgb[3]);
/* Quadrilinear 3D texture sample (GL 4.5 textureLod, LINEAR/LINEAR/LINEAR,
 * CLAMP_TO_EDGE) of the opacity pyramid; level 0 from the bitmask. */
double orc_sample_voxels(int voxel_res, const uint32_t* bits, const double* mips, const double s[3], double lod);
/* Indirect-shadow cone (cacheLightingRSM.comp:195-230); returns shadowing. */
double orc_cone_shadow(const DrvVolumeInfo* vol, int voxel_res, const uint32_t* bits, const double* mips,
                       const double cache_pos[3], const double avg_val_pos[3], double dist_to_sphere_rad,
                       int max_steps);

/* -- host parameter setup --------------------------------------------- */
void orc_prepare_light(const DrvLightDesc* light, DrvSpotLight* out);
void orc_prepare_camera(const DrvCamera* cam, DrvPerFrame* out);
void orc_compute_volume_info(const DrvConfig* cfg, const float aabb_min[3], const float aabb_max[3],
                             const float camera_position[3], DrvVolumeInfo* out);

/* -- the benchmark's seeded procedural scenes (host-side, no reference
 *    counterpart: they replace the reference's assimp meshes). The same
 *    generator as the product's drv_generate_scene / drv_generate_camera /
 *    drv_generate_light, restated so that the CPU arm of the benchmark
 *    builds its frame without the product library; a CPU test requires both
 *    to produce identical scenes. */
void orc_generate_scene(uint64_t seed, int n_boxes, float size_min, float size_max, float albedo_min,
                        float albedo_max, DrvBox* boxes /* n_boxes + 1 */, DrvScene* scene);
void orc_generate_camera(uint64_t seed, const DrvScene* scene, float aspect, DrvCamera* out);
void orc_generate_light(uint64_t seed, const DrvScene* scene, uint32_t rsm_resolution, uint32_t rsm_read_lod,
                        uint32_t indirect_shadow_lod, DrvLightDesc* out);

/* -- input producers ---------------------------------------------------- */
void orc_raycast_gbuffer(const DrvBox* boxes, int n_boxes, const DrvPerFrame* frame, const DrvCamera* cam,
                         int width, int height, float* depth, int16_t* normal16, float* normal32, float* albedo);
void orc_raycast_rsm(const DrvBox* boxes, int n_boxes, const DrvSpotLight* light, float* flux, int16_t* normal16,
                     float* depth_lin_sq);

/* -- stages -------------------------------------------------------------- */
/* One downsamplersm.frag pass: level of size `res` -> res/2. FP64 internally,
 * outputs in the RSM storage types. */
void orc_downsample_rsm(int res, const float* flux, const int16_t* normal, const float* dls,
                        float* flux_out, int16_t* normal_out, float* dls_out);
/* VPLs at the read level (res = RSMReadResolution) in Morton order:
 * vpl_out[i*10 + 0..2] flux, 3 disc area, 4..6 position, 7..9 normal.
 * cone_out[b*4 + 0..2] average VAL position, 3 distToSphereRad, one per
 * shadow block (n = res^2 / interval). dls_shadow is the RSM (d, d^2) level
 * at read_lod + indirect_shadow_lod, of size res >> indirect_shadow_lod. */
void orc_extract_vpls(const DrvSpotLight* light, int res, const float* flux, const int16_t* normal, const float* dls,
                      const float* dls_shadow, double* vpl_out, double* cone_out);
/* Surface voxelization of the box scene into the level-0 bitmask. */
void orc_voxelize(const DrvBox* boxes, int n_boxes, const DrvVolumeInfo* vol, int voxel_res, uint32_t* bits);
// Mesh producers (nrm, alb, idx may be NULL).
void orc_raycast_gbuffer_mesh(const float* pos, const float* nrm, const float* alb, const uint32_t* idx, int n_tris,
                              const DrvPerFrame* f, const DrvCamera* cam, int W, int H, float* depth, int16_t* n16,
                              float* n32, float* albedo);
void orc_raycast_rsm_mesh(const float* pos, const float* nrm, const float* alb, const uint32_t* idx, int n_tris,
                          const DrvSpotLight* L, float* flux, int16_t* n16, float* dls);
// Triangle mesh (positions xyz per vertex; indices: 3 per triangle, or NULL for consecutive triples).
void orc_voxelize_triangles(const float* positions, const uint32_t* indices, int n_tris, const DrvVolumeInfo* vol,
                            int voxel_res, uint32_t* bits);
/* Opacity mips 1..L concatenated (level l has (N>>l)^3 doubles, x fastest). */
void orc_build_mips(int voxel_res, const uint32_t* bits, double* mips);
/* cacheGather.comp over the whole screen, tiles in row-major order, threads
 * in (x fastest) order, corners in the shader's order. atlas: cleared here.
 * positions_out: max_caches*3 floats. Returns DRV_OK or DRV_ERR_CAPACITY. */
int orc_allocate_caches(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* frame,
                        int width, int height, const float* depth, uint32_t* atlas, float* positions_out,
                        uint32_t* count_out);
/* cacheLightingRSM.comp for every cache and every light; sh_out[c*27 + k*3 + ch]
 * with k = 0 SH00, 1 SH1neg1, 2 SH10, 3 SH1pos1, 4 SH2neg2, 5 SH2neg1,
 * 6 SH20, 7 SH2pos1, 8 SH2pos2 (the stored, sign-flipped values of
 * cacheLightingRSM.comp:267-277). vpls/cones per light as orc_extract_vpls.
 * n_threads <= 0 uses all OpenMP threads; a sample of caches is lit by
 * passing a subset of positions. */
void orc_light_caches(const DrvConfig* cfg, const DrvVolumeInfo* vol, int n_caches, const float* positions,
                      int n_lights, const DrvSpotLight* lights, const double* const* vpls, const double* const* cones,
                      const int* n_vpls, const uint32_t* bits, const double* mips, double* sh_out, int n_threads);
/* orc_light_caches with INDIRECT_SPECULAR (cfg->specular_envmap_size S > 0):
 * VPLs whose flux sum is below 0.001 are skipped (cacheLightingRSM.comp:240),
 * and with cam and env_out each cache's level-0 specular envmap is written,
 * S*S texels RGB row-major per cache, FP64 before rounding
 * (cacheLightingRSM.comp:87-98, 310-335: reflected radiance into the texel of
 * the cache-local half vector, times the base level's Blinn normalisation). */
void orc_light_caches_specular(const DrvConfig* cfg, const DrvVolumeInfo* vol, int n_caches, const float* positions,
                               const float* cam, int n_lights, const DrvSpotLight* lights,
                               const double* const* vpls, const double* const* cones, const int* n_vpls,
                               const uint32_t* bits, const double* mips, double* sh_out, double* env_out,
                               int n_threads);
/* HemisphericalProjection (utils.glsl:103-170, concentric square map) of a
 * direction of the z+ hemisphere to [0, 1]^2. */
void orc_hemi_projection(const double d[3], double uv[2]);
/* R11F_G11F_B10F (GL packed float: R bits 0-10, G 11-21, B 22-31). */
uint32_t orc_encode_r11g11b10(const double rgb[3]);
void orc_encode_r11g11b10_n(const double* rgb, int64_t n, uint32_t* out);
void orc_decode_r11g11b10(uint32_t v, double rgb[3]);
/* Renderer::PrepareSpecularEnvmaps on per-cache envmaps in place (level 0
 * given, encoded): mips and the hole fill from level `fill` down to 1. Cache
 * c's levels start at c * sum_l (S >> l)^2 words. */
void orc_specular_prepare(int S, int fill, int n_caches, uint32_t* env, int n_threads);
/* The same gather with given shadowing per (cache, shadow block) pair:
 * shadow[c * total_blocks + b], blocks of all lights in light order. */
void orc_light_caches_shadowed(const DrvConfig* cfg, int n_caches, const float* positions, int n_lights,
                               const DrvSpotLight* lights, const double* const* vpls, const int* n_vpls,
                               const double* shadow, int total_blocks, double* sh_out, int n_threads);
/* Renderer::ApplyRSMsBruteForce (renderer.cpp:851-871) / bruteforcersm.frag:15-82:
 * per pixel the unshadowed sum over every VAL of every light
 * (bruteforcersm.frag:44-81), VALs as orc_extract_vpls makes them (the same
 * position / normal / flux / disc-area formulas, bruteforcersm.frag:51-73).
 * rough_metal (RG per pixel, may be NULL) selects the reference BRDF
 * (lightingfunctions.glsl:27-66: normalized Blinn-Phong + metallic mix);
 * NULL: the diffuse term albedo / pi of the cache path. Pixels with depth
 * below 1e-5 (no geometry) are 0. normal: RG16I. */
void orc_bruteforce_rsm(const DrvPerFrame* frame, int width, int height, const float* depth, const int16_t* normal16,
                        const float* albedo, const float* rough_metal, int n_lights, const double* const* vpls,
                        const int* n_vpls, double* out_rgb, int n_threads);
/* cacheApply.frag per pixel; normal is RG16I (normal_format 0) or F32x3. */
void orc_apply(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* frame, int width, int height,
               const float* depth, const void* normal, int normal_format, const float* albedo, const uint32_t* atlas,
               int n_caches, const double* sh, double* out_rgb, int n_threads);
/* orc_apply plus the INDIRECT_SPECULAR term (cfg->specular_envmap_size > 0,
 * rough_metal RG F32 per pixel and env as orc_specular_prepare lays it out;
 * either NULL: the diffuse apply). */
void orc_apply_specular(const DrvConfig* cfg, const DrvVolumeInfo* vol, const DrvPerFrame* frame, int width,
                        int height, const float* depth, const void* normal, int normal_format, const float* albedo,
                        const float* rough_metal, const uint32_t* atlas, int n_caches, const double* sh,
                        const uint32_t* env, double* out_rgb, int n_threads);
#ifdef __cplusplus
}
#endif
#endif
