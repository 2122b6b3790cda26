// light_static.cu — the cache-lighting stage for callers that may not allocate
// device memory.
//
// drv_light_caches keeps its per-chunk partial sums and per-cache tickets in
// buffers that drv_create obtains with cudaMalloc. Some hosts cannot allocate
// at all once they are running: engines that hand the GPU a fixed,
// pre-reserved memory arena and forbid driver allocations during a frame,
// plug-ins loaded into such engines, and code that must stay safe to record
// into a CUDA graph. For them, drv_light_caches_static_scratch runs the same
// kernel with its scratch in a fixed-size array compiled into this library:
// every GPU that loads the library holds that array (about 3.5 MB) until the
// process exits, and no call allocates anything.
//
// Rules a caller must know:
//  - the first call on a device looks the array up on that device
//    (cudaGetSymbolAddress, with the device current); make that first call
//    before capturing a stream into a CUDA graph;
//  - all calls share the one array and it keeps the last call's contents:
//    each call clears the per-cache tickets and the unit counter before its
//    kernel runs, and calls that overlap on the GPU (different streams, no
//    ordering) race on it;
//  - at most DRV_STATIC_SCRATCH_MAX_CACHES caches; a config with a larger
//    max_caches is rejected with DRV_ERR_CAPACITY;
//  - FP32 precision only: the inputs are DrvVPL arrays and FP32 mips, the
//    entries LightCacheEntry std430 (64 B for SH1, 128 B for SH2). A BF16
//    config is rejected with DRV_ERR_INVALID_ARG before anything is launched;
//  - the array's device address is looked up once per device ordinal, in the
//    context current at that first call: callers use the device's primary
//    context (the runtime API's, as torch and most engines do).
#include <mutex>

#include "drv_internal.h"

namespace {

constexpr int kStaticChunks = 8;  // chunks per cache (the context path allows more)
constexpr size_t kPartialFloats = (size_t)DRV_STATIC_SCRATCH_MAX_CACHES * kStaticChunks * 27;
constexpr size_t kTicketWords = DRV_STATIC_SCRATCH_MAX_CACHES + 2;

// Partial sums first, then one ticket per cache and the two words of the
// dynamic unit counter (reinterpreted as uint32).
static __device__ __align__(256) float g_light_static_scratch[kPartialFloats + kTicketWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float* g_scratch_ptr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Per-device set-up: the device address of the array and the SM count.
drv_status device_scratch(float** ptr, int* num_sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DRV_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_light_static_scratch) != cudaSuccess || !p) return DRV_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
      return DRV_ERR_CUDA;
    g_num_sms[dev] = sms;
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *ptr = g_scratch_ptr[dev];
  *num_sms = g_num_sms[dev];
  return DRV_OK;
}

}  // namespace

extern "C" drv_status drv_light_caches_static_scratch(const DrvConfig* cfg, const DrvVolumeInfo* vol,
                                                      const DrvVPL* const* vpls, const DrvShadowCone* const* cones,
                                                      const int32_t* n_vpls, const int32_t* intervals,
                                                      int32_t n_lights, const uint8_t* voxel_corners,
                                                      const float* voxel_mips, const DrvCacheCounter* counter,
                                                      void* cache_entries, void* cuda_stream) {
  if (!cfg || !vol || !counter || !cache_entries || n_lights < 0 || n_lights > DRV_MAX_LIGHTS)
    return DRV_ERR_INVALID_ARG;
  if (n_lights > 0 && (!vpls || !n_vpls || !intervals)) return DRV_ERR_INVALID_ARG;
  if (cfg->indirect_shadow && (!cones || !voxel_corners || !voxel_mips)) return DRV_ERR_INVALID_ARG;
  if (cfg->sh_order != 1 && cfg->sh_order != 2) return DRV_ERR_INVALID_ARG;
  // The declared inputs are FP32 (DrvVPL, float mips) and so are the entries:
  // a BF16 config would make the kernel read DrvVPLBF16 / half mips and
  // address entries with another stride than the caller's buffer.
  if (cfg->precision != DRV_PRECISION_FP32) return DRV_ERR_INVALID_ARG;
  if (cfg->specular_envmap_size != 0) return DRV_ERR_INVALID_ARG;  // the envmap atlas belongs to a context
  if (cfg->voxel_res < 32 || cfg->voxel_res > 1024 || (cfg->voxel_res & (cfg->voxel_res - 1)))
    return DRV_ERR_INVALID_ARG;
  if (cfg->max_caches > DRV_STATIC_SCRATCH_MAX_CACHES) return DRV_ERR_CAPACITY;
  drv::LightLaunch ll{};
  ll.n_lights = n_lights;
  for (int l = 0; l < n_lights; ++l) {
    if (!vpls[l] || n_vpls[l] < 1 || intervals[l] < 1 || n_vpls[l] % intervals[l] != 0) return DRV_ERR_INVALID_ARG;
    if (cfg->indirect_shadow && !cones[l]) return DRV_ERR_INVALID_ARG;
    ll.lights[l].vpls = vpls[l];
    ll.lights[l].cones = cfg->indirect_shadow ? cones[l] : nullptr;
    ll.lights[l].n_vpls = n_vpls[l];
    ll.lights[l].interval = intervals[l];
  }
  float* scratch = nullptr;
  int num_sms = 0;
  drv_status st = device_scratch(&scratch, &num_sms);
  if (st != DRV_OK) return st;
  uint32_t* tickets = reinterpret_cast<uint32_t*>(scratch + kPartialFloats);
  const drv::LightScratch ls{scratch, tickets, tickets + DRV_STATIC_SCRATCH_MAX_CACHES, kStaticChunks};
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (cudaMemsetAsync(tickets, 0, kTicketWords * sizeof(uint32_t), s) != cudaSuccess) return DRV_ERR_CUDA;
  // Offsets of mip levels 1..L inside the concatenated FP32 pyramid.
  size_t offsets[drv::kMaxVoxelLevels] = {};
  size_t off = 0;
  for (int l = 1; l < drv::kMaxVoxelLevels && (cfg->voxel_res >> l) >= 1; ++l) {
    offsets[l] = off;
    const size_t n = (size_t)(cfg->voxel_res >> l);
    off += n * n * n;
  }
  const uint32_t stride = drv::entry_stride_for(*cfg);
  const drv::VoxelInputs vox{voxel_corners, voxel_mips, offsets};
  cudaError_t e = drv::launch_light_caches(s, *cfg, *vol, ll, counter, cache_entries, stride, vox, ls, num_sms);
  return e == cudaSuccess ? DRV_OK : DRV_ERR_CUDA;
}
