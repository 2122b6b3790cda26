"""Batched multi-scene frames: many independent seeded scenes of uneven sizes
rendered by one CUDA-graph launch (drv_batch_*), against the same scenes run
one by one; plus the autotuner that picks the batch's stream count and the
light stage's grid and tile knobs.

    python -m dynamicradiancevolume_gb300.batch --scenes 64 --reps 10

prints one JSON line: batch and one-by-one totals, scenes/s and caches lit/s,
per-scene latency p50/p99, the tuned knobs.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics
import sys
import time
from dataclasses import dataclass

import numpy as np

from . import abi, check, load, pipeline, surrogate

# Size menus of the batch (log-spaced where the range is wide).
RESOLUTIONS = (256, 384, 512, 768, 1024)
VOXELS = (64, 128, 256)
LIGHTS_LOD = ((2, 5), (1, 4), (2, 4), (1, 3), (2, 3))  # (lights, RSM read lod of 512^2): 512 ... 8192 VPLs
CAV_RES = (32, 64)


def batch_workloads(n: int, seed0: int = 0, precision: int = abi.PRECISION_BF16,
                    visibility: int = abi.VISIBILITY_SURROGATE) -> list[tuple[pipeline.Workload, int]]:
    """n scenes with sizes drawn from the menus by the scene's seed."""
    out = []
    for i in range(n):
        seed = seed0 + i
        r = np.random.default_rng(1000 + seed)
        res = int(r.choice(RESOLUTIONS))
        lights, lod = LIGHTS_LOD[int(r.integers(len(LIGHTS_LOD)))]
        w = pipeline.Workload(f"batch_{seed}", res, res, int(r.integers(16, 65)), int(r.choice(VOXELS)), lights, 512,
                              lod, 0, 4, 0.25, int(r.choice(CAV_RES)), 2, 32, 65536, precision=precision,
                              visibility=visibility)
        out.append((w, seed))
    return out


@dataclass
class Scene:
    pipe: pipeline.Pipeline
    caches: int
    vpls: int


def make_scenes(specs, threshold: float = 0.5, params=None, device: str = "cuda") -> list[Scene]:
    """Contexts, inputs (ray-cast once) and one ordinary frame per scene, so
    that every scene's boxes are resident before a capture."""
    scenes = []
    for w, seed in specs:
        hf = pipeline.host_frame(w, seed)
        hf.config.surrogate_conf_threshold = threshold
        p = pipeline.Pipeline(hf, device=device)
        if w.visibility == abi.VISIBILITY_SURROGATE:
            surrogate.upload(p, params if params is not None else surrogate.load_params(),
                             "segment8" if params is not None else surrogate.load_features())
        p.raycast_inputs()
        p.frame()
        p.sync()
        # The pair list sized to this scene's contributing pairs (+25%): grown
        # where the default is too small, so that no cache falls back to the
        # gather's own cones.
        p.set_tuning(pair_capacity=min(int(p.light_pairs() * 1.25) + 4096, 1 << 28))
        p.frame()
        p.sync()
        scenes.append(Scene(p, p.cache_count(), w.n_vpls))
    return scenes


def _batch_table(scenes: list[Scene]):
    tab = (abi.DrvBatchScene * len(scenes))()
    for i, s in enumerate(scenes):
        p = s.pipe
        tab[i] = abi.DrvBatchScene(p.ctx.value, C.addressof(p.hf.scene), C.addressof(p.gview),
                                   C.addressof(p.hf.frame), C.addressof(p.hf.volume), C.addressof(p.hf.lights),
                                   C.addressof(p.rsm_views), p.hf.workload.n_lights, p.out.data_ptr())
    return tab


class Batch:
    """One captured graph over `scenes`, dealt over `streams` branches. A
    launch waits for nothing: inputs written on other streams must be
    complete (synchronised) first."""

    def __init__(self, scenes: list[Scene], streams: int, stream=None):
        self.lib = load()
        self.scenes = scenes
        self.table = _batch_table(scenes)
        self.handle = C.c_void_p()
        self.stream = stream
        check(self.lib.drv_batch_create(self.table, len(scenes), streams,
                                        C.c_void_p(stream.cuda_stream) if stream is not None else None,
                                        C.byref(self.handle)))

    def launch(self, stream=None) -> None:
        """One launch on `stream` (default: the stream it was captured from);
        returns without waiting."""
        check(self.lib.drv_batch_launch(self.handle, C.c_void_p(stream.cuda_stream) if stream is not None else None))

    def run(self) -> tuple[float, np.ndarray]:
        """One launch; (total ms, per-scene completion ms from the start)."""
        check(self.lib.drv_batch_launch(self.handle, None))
        ms = (C.c_float * len(self.scenes))()
        total = C.c_float()
        check(self.lib.drv_batch_times(self.handle, ms, C.byref(total)))
        return total.value, np.array(ms, dtype=np.float64)

    def close(self):
        if self.handle:
            self.lib.drv_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# The light stage's knobs the autotuner searches, each with its menu: the cone
# and gather passes' CTAs per SM (0: as many as fit), the cull's tile (caches
# tested per pass against the VPL records staged in shared memory) and the
# gather's tile (threads per cache, i.e. pairs a thread sums).
KNOB_MENUS = {"cone_ctas_per_sm": (0, 4, 2), "gather_ctas_per_sm": (0, 2, 1), "cull_caches_per_pass": (4, 2, 8),
              "gather_threads": (512, 256)}


def set_knobs(scenes: list[Scene], **knobs) -> None:
    for s in scenes:
        s.pipe.set_tuning(**knobs)


def time_batch(scenes, streams: int, reps: int, warmup: int = 2):
    b = Batch(scenes, streams)
    for _ in range(warmup):
        b.run()
    totals, per = [], []
    for _ in range(reps):
        t, ms = b.run()
        totals.append(t)
        per.append(ms)
    b.close()
    return statistics.median(totals), np.median(np.stack(per), axis=0)


def time_one_by_one(scenes, reps: int, warmup: int = 2):
    """Each scene alone (its frame as a one-scene graph), one after the other:
    per-scene latency = its own frame time; total = their sum."""
    lat = []
    for s in scenes:
        b = Batch([s], 1)
        for _ in range(warmup):
            b.run()
        lat.append(statistics.median(b.run()[0] for _ in range(reps)))
        b.close()
    lat = np.array(lat)
    return float(lat.sum()), lat


def time_reference_form(scenes, reps: int, warmup: int = 2):
    """The reference's unbatched form: each scene alone, its frame issued
    kernel by kernel from the host (drv_frame, no graph) with one lighting
    pass per light (renderer.cpp:899-933, DrvTuning.per_light_dispatch);
    per-scene latency = its own frame time; total = their sum."""
    import torch
    lat = []
    for s in scenes:
        p = s.pipe
        p.set_tuning(per_light_dispatch=1)
        for _ in range(warmup):
            p.frame()
        times = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(p.stream)
            p.frame()
            b.record(p.stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        p.set_tuning(per_light_dispatch=0)
        lat.append(statistics.median(times))
    lat = np.array(lat)
    return float(lat.sum()), lat


def autotune(scenes, reps: int = 3, streams_menu=(1, 2, 4, 8, 16, 32), knob_menus=None, log=print):
    """Stream count first (default knobs), then each light-stage knob in turn
    over its menu with the others held at their best (coordinate descent);
    returns the best setting and every trial."""
    knob_menus = knob_menus or KNOB_MENUS
    best_knobs = {k: menu[0] for k, menu in knob_menus.items()}
    set_knobs(scenes, **best_knobs)
    trials, best = [], None
    for s in streams_menu:
        if s > len(scenes):
            continue
        t, _ = time_batch(scenes, s, reps, warmup=1)
        trials.append({"streams": s, **best_knobs, "ms": t})
        log(f"  streams {s:2d}: {t:.3f} ms")
        if best is None or t < best[0]:
            best = (t, s)
    best_ms, streams = best
    for name, menu in knob_menus.items():
        for v in menu[1:]:
            trial = dict(best_knobs, **{name: v})
            set_knobs(scenes, **trial)
            t, _ = time_batch(scenes, streams, reps, warmup=1)
            trials.append({"streams": streams, **trial, "ms": t})
            log(f"  streams {streams:2d} {name} {v}: {t:.3f} ms")
            if t < best_ms:
                best_ms, best_knobs = t, trial
    set_knobs(scenes, **best_knobs)
    return {"streams": streams, **best_knobs, "ms": best_ms}, trials


def run_batch(n_scenes: int, reps: int, threshold: float = 0.5, fp32_cone: bool = False, log=None,
              tune_reps: int = 3) -> dict:
    """Builds n seeded scenes, autotunes, times the batch and the scenes one
    by one; returns the report (scenes/s, caches lit/s, latency p50/p99)."""
    prec = abi.PRECISION_FP32 if fp32_cone else abi.PRECISION_BF16
    vis = abi.VISIBILITY_CONE if fp32_cone else abi.VISIBILITY_SURROGATE
    log = log or (lambda s: print(s, file=sys.stderr, flush=True))
    t0 = time.time()
    specs = batch_workloads(n_scenes, precision=prec, visibility=vis)
    scenes = make_scenes(specs, threshold)
    setup_s = time.time() - t0
    tuned, trials = autotune(scenes, reps=tune_reps, log=log)
    batch_ms, batch_lat = time_batch(scenes, tuned["streams"], reps)
    seq_ms, seq_lat = time_one_by_one(scenes, reps)
    ref_ms, ref_lat = time_reference_form(scenes, reps)
    caches = np.array([s.caches for s in scenes])
    px = np.array([s.pipe.hf.workload.width * s.pipe.hf.workload.height for s in scenes])
    line = {
        "scenes": n_scenes, "precision": "bf16" if prec == abi.PRECISION_BF16 else "f32",
        "visibility": "surrogate" if vis == abi.VISIBILITY_SURROGATE else "cone",
        "threshold": threshold if vis == abi.VISIBILITY_SURROGATE else None,
        "sizes": {"pixels": [int(px.min()), int(px.max())], "caches": [int(caches.min()), int(caches.max())],
                  "vpls": [int(min(s.vpls for s in scenes)), int(max(s.vpls for s in scenes))],
                  "voxels": sorted({s.pipe.hf.workload.voxel_res for s in scenes})},
        "tuned": tuned,
        "batch": {"ms": batch_ms, "scenes_per_s": n_scenes / (batch_ms / 1e3),
                  "caches_per_s": float(caches.sum()) / (batch_ms / 1e3),
                  "latency_ms_p50": float(np.percentile(batch_lat, 50)),
                  "latency_ms_p99": float(np.percentile(batch_lat, 99))},
        "one_by_one": {"ms": seq_ms, "scenes_per_s": n_scenes / (seq_ms / 1e3),
                       "caches_per_s": float(caches.sum()) / (seq_ms / 1e3),
                       "latency_ms_p50": float(np.percentile(seq_lat, 50)),
                       "latency_ms_p99": float(np.percentile(seq_lat, 99))},
        "reference_form": {"ms": ref_ms, "scenes_per_s": n_scenes / (ref_ms / 1e3),
                           "caches_per_s": float(caches.sum()) / (ref_ms / 1e3),
                           "latency_ms_p50": float(np.percentile(ref_lat, 50)),
                           "latency_ms_p99": float(np.percentile(ref_lat, 99)),
                           "form": "each scene alone, drv_frame issued from the host (no graph), "
                                   "one lighting pass per light"},
        "speedup": seq_ms / batch_ms,
        "speedup_vs_reference_form": ref_ms / batch_ms,
        # the tenth of the scenes with the longest frames alone: their share of
        # the one-by-one total bounds what any schedule of the batch can save
        "largest_tenth": {"scenes": max(1, n_scenes // 10),
                          "alone_ms": float(np.sort(seq_lat)[::-1][:max(1, n_scenes // 10)].sum()),
                          "share_of_one_by_one": float(np.sort(seq_lat)[::-1][:max(1, n_scenes // 10)].sum()
                                                       / max(seq_ms, 1e-9))},
        "per_scene": [{"pixels": int(px[i]), "voxels": s.pipe.hf.workload.voxel_res, "vpls": s.vpls,
                       "caches": s.caches, "cav_res": s.pipe.hf.workload.cav_res, "alone_ms": float(seq_lat[i]),
                       "reference_form_ms": float(ref_lat[i]), "batch_done_ms": float(batch_lat[i])} for i, s in enumerate(scenes)],
        "trials": trials,
        "setup_s": setup_s,
    }
    for s in scenes:
        s.pipe.close()
    return line


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--threshold", type=float, default=0.5)
    ap.add_argument("--fp32-cone", action="store_true", help="FP32 storage and cone visibility instead")
    args = ap.parse_args(argv)
    print(json.dumps(run_batch(args.scenes, args.reps, args.threshold, args.fp32_cone)), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
