// batch.cu — many scenes' frames as one CUDA graph (drv_batch_*).
//
// A batch captures drv_frame of every scene once. The capture starts on one
// stream, forks to n_streams side streams through an event, deals the scenes
// round-robin over them (each scene's context is pointed at its side stream
// for the capture, then restored), records an external timing event after
// each scene and joins every side stream back. The instantiated graph runs
// the whole batch with one launch; the scenes on different branches run
// concurrently, so small scenes that cannot fill 152 SMs alone share the GPU,
// and no frame pays host launch overhead per kernel.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/drv.h"
#include "drv_internal.h"

struct DrvBatch {
  cudaStream_t origin = nullptr;
  bool own_origin = false;
  std::vector<cudaStream_t> streams;
  cudaEvent_t fork = nullptr, start = nullptr, end = nullptr;
  std::vector<cudaEvent_t> joins, done;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool launched = false;
};

namespace {

void release(DrvBatch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  for (cudaEvent_t e : b->done) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->start) cudaEventDestroy(b->start);
  if (b->end) cudaEventDestroy(b->end);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  if (b->own_origin && b->origin) cudaStreamDestroy(b->origin);
  delete b;
}

}  // namespace

extern "C" drv_status drv_batch_create(const DrvBatchScene* scenes, int32_t n_scenes, int32_t n_streams,
                                       void* cuda_stream, DrvBatch** out) {
  if (!scenes || n_scenes < 1 || n_streams < 1 || !out) return DRV_ERR_INVALID_ARG;
  for (int i = 0; i < n_scenes; ++i)
    if (!scenes[i].ctx) return DRV_ERR_INVALID_ARG;
  DrvBatch* b = new DrvBatch();
  auto bail = [&](drv_status st) {
    release(b);
    return st;
  };
  const int S = n_streams < n_scenes ? n_streams : n_scenes;
  b->origin = static_cast<cudaStream_t>(cuda_stream);
  if (!b->origin) {
    if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess) return bail(DRV_ERR_CUDA);
    b->own_origin = true;
  }
  b->streams.resize(S, nullptr);
  b->joins.resize(S, nullptr);
  b->done.resize(n_scenes, nullptr);
  for (int s = 0; s < S; ++s) {
    if (cudaStreamCreateWithFlags(&b->streams[s], cudaStreamNonBlocking) != cudaSuccess) return bail(DRV_ERR_CUDA);
    if (cudaEventCreateWithFlags(&b->joins[s], cudaEventDisableTiming) != cudaSuccess) return bail(DRV_ERR_CUDA);
  }
  for (int i = 0; i < n_scenes; ++i)
    if (cudaEventCreate(&b->done[i]) != cudaSuccess) return bail(DRV_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->start) != cudaSuccess || cudaEventCreate(&b->end) != cudaSuccess)
    return bail(DRV_ERR_CUDA);

  if (cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return bail(DRV_ERR_CUDA);
  drv_status st = DRV_OK;
  bool ok = cudaEventRecordWithFlags(b->start, b->origin, cudaEventRecordExternal) == cudaSuccess &&
            cudaEventRecord(b->fork, b->origin) == cudaSuccess;
  for (int s = 0; ok && s < S; ++s) ok = cudaStreamWaitEvent(b->streams[s], b->fork, 0) == cudaSuccess;
  for (int i = 0; ok && st == DRV_OK && i < n_scenes; ++i) {
    const DrvBatchScene& sc = scenes[i];
    drv::Context* c = sc.ctx;
    const cudaStream_t user = c->user_stream;
    const bool has_user = c->has_user_stream;
    c->user_stream = b->streams[i % S];
    c->has_user_stream = true;
    st = drv_frame(sc.ctx, sc.scene, sc.gbuffer, sc.frame, sc.volume, sc.lights, sc.rsms, sc.n_lights, sc.out_rgb);
    c->user_stream = user;
    c->has_user_stream = has_user;
    if (st == DRV_OK) ok = cudaEventRecordWithFlags(b->done[i], b->streams[i % S], cudaEventRecordExternal) == cudaSuccess;
  }
  for (int s = 0; s < S; ++s) {
    // Join every branch, also after a failure, so that the capture can end.
    cudaEventRecord(b->joins[s], b->streams[s]);
    cudaStreamWaitEvent(b->origin, b->joins[s], 0);
  }
  if (ok && st == DRV_OK) ok = cudaEventRecordWithFlags(b->end, b->origin, cudaEventRecordExternal) == cudaSuccess;
  const cudaError_t ce = cudaStreamEndCapture(b->origin, &b->graph);
  if (st != DRV_OK) return bail(st);
  if (!ok || ce != cudaSuccess) return bail(DRV_ERR_CUDA);
  // Node priorities: the frames' high-priority side streams (RSM, voxels) keep theirs.
  if (cudaGraphInstantiate(&b->exec, b->graph, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess)
    return bail(DRV_ERR_CUDA);
  *out = b;
  return DRV_OK;
}

extern "C" drv_status drv_batch_launch(DrvBatch* b, void* cuda_stream) {
  if (!b || !b->exec) return DRV_ERR_INVALID_ARG;
  cudaStream_t s = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : b->origin;
  if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return DRV_ERR_CUDA;
  b->launched = true;
  return DRV_OK;
}

extern "C" drv_status drv_batch_times(DrvBatch* b, float* scene_ms, float* total_ms) {
  if (!b || !b->launched) return DRV_ERR_INVALID_ARG;
  if (cudaEventSynchronize(b->end) != cudaSuccess) return DRV_ERR_CUDA;
  for (size_t i = 0; scene_ms && i < b->done.size(); ++i)
    if (cudaEventElapsedTime(&scene_ms[i], b->start, b->done[i]) != cudaSuccess) return DRV_ERR_CUDA;
  if (total_ms && cudaEventElapsedTime(total_ms, b->start, b->end) != cudaSuccess) return DRV_ERR_CUDA;
  return DRV_OK;
}

extern "C" drv_status drv_batch_destroy(DrvBatch* b) {
  if (!b) return DRV_ERR_INVALID_ARG;
  release(b);
  return DRV_OK;
}
