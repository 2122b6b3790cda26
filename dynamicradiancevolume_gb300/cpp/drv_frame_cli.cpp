// drv_frame_cli — a C++ caller of the C ABI (include/drv.h) with no Python:
// procedural scene, camera and spot light, ray-cast G-buffer and RSM, then
// `frames` timed drv_frame calls on one stream, the cache count, and the
// final indirect radiance written as a PFM (drv_write_pfm). It is what a
// renderer's Draw() does around the library (the reference's
// Renderer::Draw, renderer.cpp:539-594), and the tests run it against the
// Python binding's frame.
//
//   drv_frame_cli W H boxes voxel_res rsm_res read_lod n_cascades cav_res
//                 cascade_size0 sh_order cone_steps transition seed frames out.pfm
//
// Prints one JSON line: {"caches": N, "ms_per_frame": T, "checksum": S}.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "drv.h"

namespace {

int fail(const char* what, DrvContext* ctx = nullptr) {
  std::fprintf(stderr, "drv_frame_cli: %s%s%s\n", what, ctx ? ": " : "", ctx ? drv_last_error_string(ctx) : "");
  return 1;
}

#define CHECK(call)                                \
  do {                                             \
    if ((call) != DRV_OK) return fail(#call, ctx); \
  } while (0)
#define CUDA(call)                                        \
  do {                                                    \
    if ((call) != cudaSuccess) return fail(#call, ctx);   \
  } while (0)

}  // namespace

int main(int argc, char** argv) {
  if (argc != 16) {
    std::fprintf(stderr,
                 "usage: %s W H boxes voxel_res rsm_res read_lod n_cascades cav_res cascade_size0 sh_order "
                 "cone_steps transition seed frames out.pfm\n",
                 argv[0]);
    return 2;
  }
  const int W = std::atoi(argv[1]), H = std::atoi(argv[2]), n_boxes = std::atoi(argv[3]);
  const int voxel_res = std::atoi(argv[4]), rsm_res = std::atoi(argv[5]), read_lod = std::atoi(argv[6]);
  const int n_cascades = std::atoi(argv[7]), cav_res = std::atoi(argv[8]);
  const float cascade0 = (float)std::atof(argv[9]);
  const int sh_order = std::atoi(argv[10]), steps = std::atoi(argv[11]);
  const float transition = (float)std::atof(argv[12]);
  const uint64_t seed = std::strtoull(argv[13], nullptr, 10);
  const int frames = std::atoi(argv[14]);
  const char* out_path = argv[15];
  DrvContext* ctx = nullptr;

  DrvConfig cfg;
  drv_default_config(&cfg);
  cfg.width = W;
  cfg.height = H;
  cfg.sh_order = sh_order;
  cfg.indirect_shadow = 1;
  cfg.max_cone_steps = steps;
  cfg.cascade_transition = transition;
  cfg.n_cascades = n_cascades;
  cfg.cav_res = cav_res;
  for (int c = 0; c < DRV_MAX_CASCADES; ++c) cfg.cascade_world_size[c] = cascade0 * (float)(1 << c);
  cfg.voxel_res = voxel_res;
  cfg.max_caches = 262144;
  cfg.max_lights = 1;
  cfg.max_rsm_resolution = rsm_res;

  // Scene, camera, light and volume (host).
  std::vector<DrvBox> boxes(n_boxes + 1);
  DrvScene scene;
  CHECK(drv_generate_scene(seed, n_boxes, 0.05f, 0.3f, 0.2f, 0.9f, boxes.data(), &scene));
  DrvCamera cam;
  CHECK(drv_generate_camera(seed, &scene, (float)W / (float)H, &cam));
  DrvPerFrame frame;
  CHECK(drv_prepare_camera(&cam, &frame));
  DrvLightDesc desc;
  CHECK(drv_generate_light(seed * 31, &scene, (uint32_t)rsm_res, (uint32_t)read_lod, 0, &desc));
  DrvSpotLight light;
  CHECK(drv_prepare_light(&desc, &light));
  DrvVolumeInfo vol;
  CHECK(drv_compute_volume_info(&cfg, scene.aabb_min, scene.aabb_max, cam.position, &vol));

  CHECK(drv_create(&cfg, &ctx));
  cudaStream_t stream;
  CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  CHECK(drv_set_stream(ctx, stream));

  // Device G-buffer, RSM and output.
  const size_t px = (size_t)W * H, tx = (size_t)rsm_res * rsm_res;
  float *depth, *albedo, *normal32, *out, *flux, *dls;
  int16_t *normal16, *rsm_normal;
  CUDA(cudaMalloc(&depth, px * 4));
  CUDA(cudaMalloc(&normal16, px * 4));
  CUDA(cudaMalloc(&normal32, px * 12));
  CUDA(cudaMalloc(&albedo, px * 12));
  CUDA(cudaMalloc(&out, px * 12));
  CUDA(cudaMalloc(&flux, tx * 12));
  CUDA(cudaMalloc(&rsm_normal, tx * 4));
  CUDA(cudaMalloc(&dls, tx * 8));
  const DrvGBufferOut gout{depth, normal16, normal32, albedo};
  CHECK(drv_raycast_gbuffer(ctx, &scene, &cam, &frame, W, H, &gout));
  const DrvRSMOut rout{flux, rsm_normal, dls};
  CHECK(drv_raycast_rsm(ctx, &scene, &light, &rout));

  DrvGBufferView gview{};
  gview.width = W;
  gview.height = H;
  gview.depth = depth;
  gview.normal = normal16;
  gview.normal_format = DRV_NORMAL_RG16I;
  gview.albedo = albedo;
  gview.albedo_format = DRV_ALBEDO_F32X3;
  DrvRSMView rsm{};
  rsm.resolution = rsm_res;
  rsm.flux = flux;
  rsm.normal = rsm_normal;
  rsm.depth_lin_sq = dls;
  rsm.format = DRV_RSM_F32;

  // One frame makes the scene resident, then `frames` timed frames.
  CHECK(drv_frame(ctx, &scene, &gview, &frame, &vol, &light, &rsm, 1, out));
  CHECK(drv_sync(ctx));
  cudaEvent_t a, b;
  CUDA(cudaEventCreate(&a));
  CUDA(cudaEventCreate(&b));
  CUDA(cudaEventRecord(a, stream));
  for (int f = 0; f < frames; ++f) CHECK(drv_frame(ctx, &scene, &gview, &frame, &vol, &light, &rsm, 1, out));
  CUDA(cudaEventRecord(b, stream));
  CHECK(drv_sync(ctx));
  float ms = 0.0f;
  CUDA(cudaEventElapsedTime(&ms, a, b));

  uint32_t caches = 0;
  CHECK(drv_get_cache_count(ctx, &caches));
  std::vector<float> rgb(px * 3);
  CUDA(cudaMemcpy(rgb.data(), out, px * 12, cudaMemcpyDeviceToHost));
  double sum = 0.0;
  for (float v : rgb) sum += v;
  CHECK(drv_write_pfm(out_path, rgb.data(), W, H, 3));
  std::printf("{\"caches\": %u, \"ms_per_frame\": %.4f, \"checksum\": %.9g}\n", caches,
              frames > 0 ? ms / frames : 0.0f, sum);

  for (void* p : {(void*)depth, (void*)normal16, (void*)normal32, (void*)albedo, (void*)out, (void*)flux,
                  (void*)rsm_normal, (void*)dls})
    cudaFree(p);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  drv_destroy(ctx);
  cudaStreamDestroy(stream);
  return 0;
}
