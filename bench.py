#!/usr/bin/env python
"""Benchmark: caches lit/s and ms/frame of the per-frame indirect-lighting
path at 1080p with 4096 VPLs (the production workload with one spot light).

A step is the cache-lighting stage (SH gather of every VPL into every cache
with a cone-traced shadow per pair) over one frame's VPLs, voxel pyramid and
caches, resident in HBM; `value` = caches lit per second of that stage (all
ranks) and `ms_per_frame` = the whole frame (RSM mips + VPL extraction,
voxelization + opacity mips, cache allocation, cache lighting, apply).
`e2e` = caches lit per second of whole frames through the C-ABI calls with
host buffers in the reference's render-target formats, the H2D copy of the
G-buffer and RSM and the D2H copy of the radiance inside the timed region.

--impl reference times the reference's CPU implementation of the path: the
reference itself is GLSL inside an OpenGL 4.5 Windows application that cannot
run here (no graphics stack), so its CPU arm is the FP64 restatement of its
shader math, on all host cores, with the product library never loaded.

Multi-GPU: replicas only (each rank renders its own frame; no collective on
the data path); `value` sums the ranks' caches over the max of their times.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "caches lit/s and ms/frame at 1080p: plain vs surrogate, at ≤1% rel-L2 vs FP64"
UNIT = "caches/s"

# DRAM bytes (read + write) per launch of the light stage's top kernel at
# ns_1080p_4096 (BF16), from one `ncu --set full --clock-control none`
# capture (cold caches) of the second frame's launch of
# `python -m dynamicradiancevolume_gb300.pipeline ns_1080p_4096 --precision bf16 --frames 2`.
NCU_TRAFFIC = {"cone_kernel": 16_459_008}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="ns_1080p_4096")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-workloads", action="store_true",
                    help="measure only --workload (by default the 1080p line also measures c2_production)")
    ap.add_argument("--batch-scenes", type=int, default=64,
                    help="scenes of the batched multi-scene measurement (0: none)")
    ap.add_argument("--thresholds", type=float, nargs="*", default=[0.5, 0.8],
                    help="surrogate confidence thresholds to measure")
    return ap.parse_args()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3] not in ("[N/A]", ""))
                if any(r[3] not in ("[N/A]", "") for r in rows) else None}


# ---------------------------------------------------------------- helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# Frames in flight of the end-to-end measurement: contexts taking the steps
# in turn, each step's copies overlapping the other frames' kernels (a
# renderer's triple-buffered swap chain).
E2E_FRAMES_IN_FLIGHT = 3

# BF16 tensor flops of one surrogate MLP evaluation (32 -> 64 -> 64 -> 64 -> 2).
MLP_FLOPS_PER_PAIR = 2 * (32 * 64 + 64 * 64 + 64 * 64 + 64 * 2)


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "sm_max_mhz": d.get("sm_max_mhz", 2070.0),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0,
            "source": "fallback"}


def sh_flops_per_pair(sh_order: int) -> int:
    # Frozen from the light kernel's per-pair arithmetic (FMA = 2, rsqrt/rcp = 1):
    # geometry 24 + SH1 27 (+ SH2 43).
    return 51 if sh_order == 1 else 94


def light_stage_launches(w, surrogate: bool = False) -> int:
    # split stage: cull, classify, scatter, cone, gather; with the surrogate
    # the MLP runs between the cull and the classify pass (which then sorts
    # only the re-traced pairs); without indirect shadow: the single kernel.
    if not w.indirect_shadow:
        return 1
    return 6 if surrogate else 5


def kernel_launches_per_frame(w, surrogate: bool = False) -> int:
    # per light: (read_lod + shadow_lod) downsample passes + 1 extraction;
    # voxelize 1 + mips (1, +1 tail above 32^3) + mip records 1 + corner grid
    # 1; allocate 2 (allocation, dispatch size); the light stage; apply 1.
    n = w.n_lights * (w.rsm_read_lod + w.shadow_lod + 1)
    if w.indirect_shadow:
        n += 1 + (2 if w.voxel_res > 32 else 1) + 1 + 1
        n += light_stage_launches(w, surrogate)
    else:
        n += 1
    return n + 3


def reduce_over_ranks(light_ms: float, frame_ms: float, e2e_ms: float, caches: float, device=None):
    """Replicas: the slowest rank's times and the caches of all ranks
    (no collective on the data path, only this one for the report)."""
    import torch
    import torch.distributed as dist
    vals = torch.tensor([light_ms, frame_ms, e2e_ms, caches], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        mx, tot = vals.clone(), vals.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        return mx[0].item(), mx[1].item(), mx[2].item(), tot[3].item()
    return light_ms, frame_ms, e2e_ms, float(caches)


# ---------------------------------------------------------------- CPU arm
def workload_config(w) -> dict:
    """The `config` object of both arms' JSON lines: the workload alone."""
    return {"workload": w.name, "width": w.width, "height": w.height, "n_vpls": w.n_vpls, "n_lights": w.n_lights,
            "voxel_res": w.voxel_res, "cascades": f"{w.n_cascades}x{w.cav_res}^3", "sh_order": w.sh_order,
            "cone_steps": w.max_cone_steps,
            "l2": "GPU arm: flushed between steps (256 MiB write); CPU arm: host caches, not flushed"}


def product_library_mapped() -> bool:
    """True when this process has mapped libdrv_gb300.so (Linux /proc)."""
    try:
        return "libdrv_gb300.so" in Path("/proc/self/maps").read_text()
    except OSError:
        return False


def oracle_inputs(hf, w):
    """The frame's G-buffer and RSMs, ray-cast by the oracle (not timed)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O
    depth, n16, n32, alb = O.raycast_gbuffer(hf.boxes, hf.scene.n_boxes, hf.frame, hf.camera, w.width, w.height)
    rsms = [O.raycast_rsm(hf.boxes, hf.scene.n_boxes, hf.lights[l]) for l in range(w.n_lights)]
    return depth, n16, alb, rsms


def cpu_frame(w, hf, inputs, n_threads: int, cache_sample: int | None = None):
    """One FP64 oracle frame on the host over ray-cast inputs. Every cache is
    lit unless cache_sample is given (then a spread sample, extrapolated
    linearly and labelled so). Returns (caches, frame s, light s, note)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import oracle_py as O
    depth, n16, alb, rsms = inputs
    t0 = time.perf_counter()
    vp, cones = [], []
    for l in range(w.n_lights):
        chain = O.rsm_chain(*rsms[l], w.rsm_read_lod + w.shadow_lod)
        v, c = O.extract_vpls(hf.lights[l], *chain[w.rsm_read_lod], chain[w.rsm_read_lod + w.shadow_lod][2])
        vp.append(v)
        cones.append(c)
    bits = O.voxelize(hf.boxes, hf.scene.n_boxes, hf.volume, w.voxel_res)
    mips = O.build_mips(w.voxel_res, bits)
    st, atlas, pos, count = O.allocate_caches(hf.config, hf.volume, hf.frame, depth)
    t_fixed = time.perf_counter() - t0
    n = pos.shape[0]
    sample = n if not cache_sample or cache_sample >= n else cache_sample
    idx = np.linspace(0, n - 1, sample).astype(int) if sample < n else np.arange(n)
    t1 = time.perf_counter()
    sh_s = O.light_caches(hf.config, hf.volume, pos[idx], hf.lights, vp, cones, bits, mips, n_threads=n_threads)
    t_light = (time.perf_counter() - t1) * (n / sample)
    sh = np.zeros((n, 27))
    sh[idx] = sh_s
    t2 = time.perf_counter()
    O.apply(hf.config, hf.volume, hf.frame, depth, n16, 0, alb, atlas, sh, n_threads=n_threads)
    t_apply = time.perf_counter() - t2
    note = (f"FP64 oracle frame on {n_threads} host threads; light stage on {sample} of {n} caches"
            + (" (extrapolated linearly)" if sample < n else " (all caches, every step)"))
    return n, t_fixed + t_light + t_apply, t_light, note


def run_reference(args):
    """The CPU arm: the FP64 oracle alone (scene, inputs, every stage), on all
    host cores; the product library is never loaded in this process."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O
    from dynamicradiancevolume_gb300 import pipeline  # workload table only (pure Python)
    w = pipeline.WORKLOADS[args.workload]
    hf = O.host_frame(w)
    inputs = oracle_inputs(hf, w)
    threads = os.cpu_count() or 1
    frames, lights, caches, note = [], [], 0, ""
    for i in range(args.warmup + args.steps):
        caches, t_frame, t_light, note = cpu_frame(w, hf, inputs, threads)
        if i >= args.warmup:
            frames.append(t_frame)
            lights.append(t_light)
    t, tf = statistics.mean(lights), statistics.mean(frames)
    value = caches / t
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "ms_per_frame": tf * 1e3, "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded procedural box room)",
            "config": workload_config(w), "caches": caches, "variant": "fp64_oracle",
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": note},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "product_library_loaded": product_library_mapped()}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm
def oracle_frame_from(pipe):
    """FP64 oracle frame from a pipeline's own G-buffer and RSM inputs."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O
    w, hf = pipe.hf.workload, pipe.hf
    depth, n16, alb = (t.cpu().numpy() for t in (pipe.depth, pipe.normal16, pipe.albedo))
    vp, cones = [], []
    for l in range(w.n_lights):
        rsm = tuple(t.cpu().numpy() for t in (pipe.rsm_flux[l], pipe.rsm_normal[l], pipe.rsm_dls[l]))
        chain = O.rsm_chain(*rsm, w.rsm_read_lod + w.shadow_lod)
        v, c = O.extract_vpls(hf.lights[l], *chain[w.rsm_read_lod], chain[w.rsm_read_lod + w.shadow_lod][2])
        vp.append(v)
        cones.append(c)
    bits = O.voxelize(hf.boxes, hf.scene.n_boxes, hf.volume, w.voxel_res)
    mips = O.build_mips(w.voxel_res, bits)
    cfg = type(hf.config).from_buffer_copy(hf.config)
    cfg.precision, cfg.visibility = 0, 0
    st, atlas, pos, count = O.allocate_caches(cfg, hf.volume, hf.frame, depth)
    sh = O.light_caches(cfg, hf.volume, pos, hf.lights, vp, cones, bits, mips)
    out = O.apply(cfg, hf.volume, hf.frame, depth, n16, 0, alb, atlas, sh)  # 0: RG16I normals
    return out, pos[:count], sh[:count]


def errors_vs_fp64(pipe, count, out, reference) -> dict:
    """Per-result errors against the FP64 oracle frame: the caches' SH
    (matched by position: the allocation is bit-exact, its order is the
    atomics') and the final radiance, rel-L2 and max |difference|."""
    import numpy as np
    ref_out, ref_pos, ref_sh = reference
    e = {"rel_l2_vs_fp64": rel_l2(out, ref_out), "radiance_max_abs_vs_fp64": float(np.max(np.abs(out - ref_out)))}
    pos, sh = pipe.read_entries_decoded(count)
    if pos.shape == ref_pos.shape:
        a, b = np.lexsort(pos.T[::-1]), np.lexsort(ref_pos.T[::-1])
        if np.array_equal(pos[a], ref_pos[b]):
            nk = 27 if pipe.hf.workload.sh_order == 2 else 12
            g, r = sh[a][:, :nk], ref_sh[b][:, :nk]
            e["sh_rel_l2_vs_fp64"] = rel_l2(g, r)
            e["sh_max_abs_vs_fp64"] = float(np.max(np.abs(g - r)))
    return e


def rel_l2(a, b) -> float:
    import numpy as np
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def measure(pipe, steps, warmup, flush, clocks=None):
    """Per-stage CUDA-event times of `steps` frames (L2 flushed between them)."""
    import torch
    stream = pipe.stream
    names = ["rsm+vpl", "voxelize+mips", "allocate", "light", "apply"]

    def staged(ev):
        ev[0].record(stream)
        pipe.prepare_and_extract()
        ev[1].record(stream)
        pipe.voxelize()
        ev[2].record(stream)
        pipe.allocate()
        ev[3].record(stream)
        pipe.light()
        ev[4].record(stream)
        pipe.apply()
        ev[5].record(stream)

    for _ in range(warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        staged([torch.cuda.Event(enable_timing=True) for _ in range(6)])
    pipe.sync()
    torch.cuda.synchronize(pipe.device)
    events = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush between timed steps (outside the events)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        staged(ev)
        events.append(ev)
    torch.cuda.synchronize(pipe.device)
    pipe.sync()
    stage_ms = {n: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in events) for i, n in enumerate(names)}
    frame_ms = statistics.mean(e[0].elapsed_time(e[5]) for e in events)
    return frame_ms, stage_ms


def measure_graph(pipe, steps, warmup, flush):
    """Mean ms of `steps` replays of one frame captured as a CUDA graph
    (every replay runs every stage; L2 flushed between replays, outside the
    timed events)."""
    import torch
    stream = pipe.stream
    out = torch.zeros_like(pipe.out)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        pipe.frame(out)
    for _ in range(warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
            g.replay()
    torch.cuda.synchronize(pipe.device)
    ev = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            g.replay()
            b.record(stream)
        ev.append((a, b))
    torch.cuda.synchronize(pipe.device)
    return statistics.mean(a.elapsed_time(b) for a, b in ev)


def measure_light_graph(pipe, steps, warmup, flush):
    """Mean ms of `steps` replays of the light stage (drv_light_caches)
    captured as a CUDA graph, over the frame's own VPLs, voxels and caches
    (each replay relights every cache; its SH accumulates, as per-light
    dispatches do). L2 flushed between replays, outside the timed events."""
    import torch
    stream = pipe.stream
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        pipe.light()
    for _ in range(warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
            g.replay()
    torch.cuda.synchronize(pipe.device)
    ev = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            g.replay()
            b.record(stream)
        ev.append((a, b))
    torch.cuda.synchronize(pipe.device)
    return statistics.mean(a.elapsed_time(b) for a, b in ev)


def measure_cache_peaks(dev) -> dict:
    """L1 and L2 load throughput of this GPU (drv_measure_load_bandwidth),
    GB/s: the denominators of the cone pass's memory roofline."""
    import ctypes as C
    import torch
    from dynamicradiancevolume_gb300 import load
    lib = load()
    buf = torch.randint(0, 2**31 - 1, (16 * 1024 * 1024,), dtype=torch.int32, device=dev)  # 64 MB < L2
    stream = torch.cuda.current_stream(dev)
    out = {}
    for level, reps in ((1, 200), (2, 20)):
        g = C.c_float()
        st = lib.drv_measure_load_bandwidth(level, C.c_void_p(buf.data_ptr()), buf.numel() * 4, reps,
                                            C.c_void_p(stream.cuda_stream), C.byref(g))
        out[f"l{level}_gbs"] = g.value if st == 0 else None
    out["method"] = ("drv_measure_load_bandwidth: 16-byte loads, L1 = every CTA re-reading its own 32 KB window "
                     "(2 CTAs per SM), L2 = all SMs sweeping a 64 MB buffer with L1-bypassing loads")
    return out


def measure_workload(w, args, dev, flush, rank, weights, features, full: bool) -> dict:
    """Everything the JSON line reports for one workload: its variants
    (plain FP32 cone, BF16 precision, surrogate thresholds), the headline
    variant (fastest within 1% rel-L2 of the FP64 oracle frame), its e2e
    through the C ABI with host buffers, per-kernel light-stage times and the
    voxel loads of its cone pass. `full`: also the specular cost, the
    drv_frame / one-context / F32-target e2e forms."""
    import ctypes as C
    import numpy as np
    import torch
    from dynamicradiancevolume_gb300 import abi, pipeline, surrogate
    from dynamicradiancevolume_gb300 import batch as batch_mod

    plan = [("plain_fp32", w, None), ("precision_bf16", pipeline.scaled(w, precision=abi.PRECISION_BF16), None)]
    if weights is not None:
        for thr in args.thresholds:
            plan.append((f"surrogate_t{thr:g}", pipeline.scaled(w, visibility=abi.VISIBILITY_SURROGATE), thr))
    variants, pipes, reference = {}, {}, None
    for name, wv, thr in plan:
        hf = pipeline.host_frame(wv)
        if thr is not None:
            hf.config.surrogate_conf_threshold = thr
        pipe = pipeline.Pipeline(hf, device=str(dev))
        if thr is not None:
            surrogate.upload(pipe, weights, features)
        pipe.raycast_inputs()
        pipe.frame()
        pipe.sync()
        count = pipe.cache_count()
        frame_ms, stage_ms = measure(pipe, args.steps, args.warmup, flush)
        graph_ms = measure_graph(pipe, args.steps, args.warmup, flush)
        light_ms = measure_light_graph(pipe, args.steps, args.warmup, flush)
        pipe.frame()
        pipe.sync()
        # errors of this frame's SH and radiance (read before the extra light
        # stage below, whose SH would add onto the frame's)
        out = pipe.out.cpu().numpy()
        if reference is None and rank == 0:
            reference = oracle_frame_from(pipe)
        errors = errors_vs_fp64(pipe, count, out, reference) if rank == 0 else {}
        pipe.light()  # one eager light stage: its pair count and surrogate statistics
        info = {"caches_lit_per_s": count / (light_ms / 1e3), "light_ms": light_ms, "frame_ms": graph_ms,
                "live_pairs": pipe.light_pairs(), "frame_ms_stream": frame_ms, "stage_ms": stage_ms,
                "caches": count, "caches_per_s_of_frame": count / (graph_ms / 1e3)}
        if w.n_lights > 1:
            # the reference's form: one lighting pass per light, each adding
            # into the entries (renderer.cpp:924-932)
            pipe.set_tuning(per_light_dispatch=1)
            info["light_ms_per_light_dispatch"] = measure_light_graph(pipe, args.steps, args.warmup, flush)
            pipe.set_tuning(per_light_dispatch=0)
        if thr is not None:
            # per-kernel times of this variant's light stage (events between its
            # kernels, L2 flushed before each stage) and the MLP's tensor rate
            pipe.set_tuning(time_kernels=1)
            kern = {k: [] for k in abi.LIGHT_KERNELS}
            for i in range(args.warmup + args.steps):
                with torch.cuda.stream(pipe.stream):
                    flush.zero_()
                pipe.light()
                if i >= args.warmup:
                    for k, v in pipe.light_kernel_ms().items():
                        kern[k].append(v)
            pipe.set_tuning(time_kernels=0)
            info["light_kernel_ms"] = {k: statistics.mean(v) for k, v in kern.items()}
            ev, fb = C.c_uint32(), C.c_uint32()
            pipe.lib.drv_get_surrogate_stats(pipe.ctx, C.byref(ev), C.byref(fb))
            mlp_s = info["light_kernel_ms"]["mlp"] / 1e3
            tf = ev.value * MLP_FLOPS_PER_PAIR / mlp_s / 1e12 if mlp_s > 0 else None
            info["mlp_tensor"] = {"flops_per_pair": MLP_FLOPS_PER_PAIR, "tflops": tf,
                                  "frac_of_bf16_peak": tf / peaks()["bf16_tflops"] if tf else None,
                                  "peak_source": peaks()["source"] + " (bf16_tflops, burst)"}
            blocks = sum(pipe.buffers().n_vpls[l] // hf.lights[l].indirect_shadow_sample_interval
                         for l in range(w.n_lights))
            info.update({"threshold": thr, "features": features, "shadow_blocks": blocks,
                         "evaluated_pairs": ev.value, "retraced_pairs": fb.value,
                         "evaluated_share_of_pairs": ev.value / max(count * blocks, 1),
                         "retraced_share_of_evaluated": fb.value / max(ev.value, 1)})
        info.update(errors)
        variants[name] = info
        pipes[name] = pipe
    specular = None
    if full:
        # INDIRECT_SPECULAR with the reference's 16x16 per-cache envmaps on
        # the BF16 frame: its cost (the envmap pass inside the light stage,
        # the mips and the specular apply inside the frame). Not a headline
        # candidate: the specular frame is another image.
        hf = pipeline.host_frame(pipeline.scaled(w, precision=abi.PRECISION_BF16, specular_envmap_size=16))
        sp = pipeline.Pipeline(hf, device=str(dev))
        rm = np.random.default_rng(11).integers(0, 256, (w.height, w.width, 2), dtype=np.uint8)
        sp.rough_metal.copy_(torch.from_numpy(rm).to(dev))
        torch.cuda.synchronize(dev)
        sp.raycast_inputs()
        sp.frame()
        sp.sync()
        specular = {"envmap_size": 16, "precision": "bf16", "caches": sp.cache_count(),
                    "light_ms": measure_light_graph(sp, args.steps, args.warmup, flush),
                    "frame_ms": measure_graph(sp, args.steps, args.warmup, flush),
                    "light_ms_without": variants["precision_bf16"]["light_ms"],
                    "frame_ms_without": variants["precision_bf16"]["frame_ms"]}
        sp.close()
    ok = {n: v for n, v in variants.items() if v.get("rel_l2_vs_fp64", 1.0) <= 0.01}
    head = max(ok, key=lambda n: ok[n]["caches_lit_per_s"]) if ok else "plain_fp32"
    pipe = pipes[head]
    stream = pipe.stream
    hv = variants[head]
    for n, p in pipes.items():
        if n != head:
            p.close()

    # ---- e2e through the C ABI with host buffers (pinned), H2D + D2H inside the region.
    # E2E_FRAMES_IN_FLIGHT contexts on their own streams take the steps in
    # turn (a renderer's swap chain: frame k+1 uploads while frame k renders):
    # every step copies its G-buffer and RSM from pinned host memory, runs the
    # frame and copies its radiance back; the copies of one step overlap the
    # kernels of the others, and frames overlap where one leaves SMs idle. The headline uses the reference's own render targets (D32F depth,
    # RG16I normal, SRGB8 diffuse, RGB16F / RG16I / RG16F RSM, RGBA16F output
    # with additive blending, renderer.cpp:119, 468-480, 1288-1290); the same
    # steps over F32 targets are reported beside it.
    wv_head = next(wv for name, wv, thr in plan if name == head)
    g_ref, rsm_ref = pipeline.reference_format_inputs(pipe)

    def e2e_pipes(formats, n):
        out = []
        for _ in range(n):
            hf2 = pipeline.host_frame(wv_head)
            if head.startswith("surrogate"):
                hf2.config.surrogate_conf_threshold = hv["threshold"]
            if formats == "reference":
                hf2.config.output_format, hf2.config.output_blend = abi.OUTPUT_RGBA16F, abi.OUTPUT_ADD
                q = pipeline.Pipeline(hf2, device=str(dev), albedo_format=abi.ALBEDO_SRGB8, rsm_format=abi.RSM_F16)
            else:
                q = pipeline.Pipeline(hf2, device=str(dev))
            if head.startswith("surrogate"):
                surrogate.upload(q, weights, features)
            out.append(q)
        return out

    def run_e2e(formats, graph, n_ctx=E2E_FRAMES_IN_FLIGHT):
        """Mean ms per step with n_ctx contexts taking the steps in turn, each
        on its own stream (n_ctx frames in flight; 1: one step at a time);
        (h2d, d2h) bytes per step."""
        qs = e2e_pipes(formats, n_ctx)
        if formats == "reference":
            host_in = [torch.from_numpy(a).pin_memory() for a in g_ref]
            host_rsm = [[torch.from_numpy(a).pin_memory() for a in r] for r in rsm_ref]
            dev_in = lambda q: [q.depth, q.normal16, q.albedo8]
            dev_rsm = lambda q, l: (q.rsm_flux16[l], q.rsm_normal[l], q.rsm_dls16[l])
        else:
            host_in = [t.cpu().pin_memory() for t in (pipe.depth, pipe.normal16, pipe.albedo)]
            host_rsm = [[t.cpu().pin_memory() for t in (pipe.rsm_flux[l], pipe.rsm_normal[l], pipe.rsm_dls[l])]
                        for l in range(w.n_lights)]
            dev_in = lambda q: [q.depth, q.normal16, q.albedo]
            dev_rsm = lambda q, l: (q.rsm_flux[l], q.rsm_normal[l], q.rsm_dls[l])
        host_out = [torch.empty(q.out.shape, dtype=q.out.dtype).pin_memory() for q in qs]
        h2d = sum(t.numel() * t.element_size() for t in host_in) + sum(
            t.numel() * t.element_size() for r in host_rsm for t in r)
        d2h = host_out[0].numel() * host_out[0].element_size()
        # one eager frame per context first (the scene's boxes become
        # resident: a capture cannot include their upload)
        for q in qs:
            with torch.cuda.stream(q.stream):
                for d, h in zip(dev_in(q), host_in):
                    d.copy_(h, non_blocking=True)
                for l in range(w.n_lights):
                    for d, h in zip(dev_rsm(q, l), host_rsm[l]):
                        d.copy_(h, non_blocking=True)
            q.frame()
            q.sync()
        graphs = [batch_mod.Batch([batch_mod.Scene(q, 0, 0)], 1, stream=q.stream) for q in qs] if graph else None

        def step(k):
            i = k % n_ctx
            q = qs[i]
            with torch.cuda.stream(q.stream):
                for d, h in zip(dev_in(q), host_in):
                    d.copy_(h, non_blocking=True)
                for l in range(w.n_lights):
                    for d, h in zip(dev_rsm(q, l), host_rsm[l]):
                        d.copy_(h, non_blocking=True)
            if graph:
                graphs[i].launch(q.stream)
            else:
                q.frame()
            with torch.cuda.stream(q.stream):
                host_out[i].copy_(q.out, non_blocking=True)

        for k in range(max(args.warmup, n_ctx)):  # every context's graph warmed
            step(k)
        torch.cuda.synchronize(dev)
        a = qs[0]
        with torch.cuda.stream(a.stream):
            flush.zero_()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if n_ctx > 1:
            start.record(a.stream)
            for q in qs[1:]:
                q.stream.wait_event(start)
            for k in range(args.steps):
                step(k)
            for q in qs[1:]:
                a.stream.wait_stream(q.stream)
            end.record(a.stream)
            end.synchronize()
            ms = start.elapsed_time(end) / args.steps
        else:
            serial = []
            for k in range(args.steps):
                with torch.cuda.stream(a.stream):
                    flush.zero_()
                start.record(a.stream)
                step(0)
                end.record(a.stream)
                end.synchronize()
                serial.append(start.elapsed_time(end))
            ms = statistics.mean(serial)
        torch.cuda.synchronize(dev)
        for g in graphs or []:
            g.close()
        for q in qs:
            q.close()
        return ms, h2d, d2h

    count = hv["caches"]
    e2e_ms, h2d, d2h = run_e2e("reference", graph=True)
    e2e = {"value": count / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "ms_per_step": e2e_ms,
           "formats": "the reference's render targets: D32F depth, RG16I normal, SRGB8 diffuse; RSM RGB16F flux, "
                      "RG16I normal, RG16F (d, d^2); radiance added into an RGBA16F HDR buffer",
           "scope": "whole frame per step: G-buffer and RSM copied from pinned host memory, the frame replayed as "
                    "a CUDA graph (drv_batch_launch of a one-scene batch captured once per context), radiance "
                    f"copied back, all inside the timed region; {E2E_FRAMES_IN_FLIGHT} contexts on their own "
                    "streams take the steps in turn (frames in flight, as a renderer's swap chain)",
           "frames_in_flight": E2E_FRAMES_IN_FLIGHT}
    if full:
        e2e["ms_per_step_by_frames_in_flight"] = {
            str(n): (e2e_ms if n == E2E_FRAMES_IN_FLIGHT else run_e2e("reference", graph=True, n_ctx=n)[0])
            for n in (1, 2, 3, 4)}
        e2e["ms_per_step_drv_frame"], _, _ = run_e2e("reference", graph=False)
        e2e["ms_per_step_one_context"], _, _ = run_e2e("reference", graph=False, n_ctx=1)
        f32_ms, h2d_f32, d2h_f32 = run_e2e("f32", graph=True)
        e2e["f32_formats"] = {"ms_per_step": f32_ms, "h2d_bytes_per_step": h2d_f32, "d2h_bytes_per_step": d2h_f32,
                              "value": count / (f32_ms / 1e3)}
        e2e["scope"] += ("; ms_per_step_by_frames_in_flight: the graph steps with 1-4 contexts in turn; "
                         "ms_per_step_drv_frame: the same steps calling drv_frame (kernels launched one by one); "
                         "ms_per_step_one_context: drv_frame steps on one context, one at a time; f32_formats: the "
                         "graph steps with F32 diffuse, F32 RSM and an RGB F32 output")

    # ---- per-kernel times of the headline light stage (non-graph, events between its kernels)
    pipe.set_tuning(time_kernels=1)
    kern = {k: [] for k in abi.LIGHT_KERNELS}
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        pipe.light()
        if i >= args.warmup:
            for k, v in pipe.light_kernel_ms().items():
                kern[k].append(v)
    pipe.set_tuning(time_kernels=0)
    kernel_ms = {k: statistics.mean(v) for k, v in kern.items()}
    # ---- the voxel loads of one cone pass (its measuring instance, outside the timed regions)
    pipe.set_tuning(count_voxel_reads=1)
    pipe.light()
    reads = (C.c_uint32 * 3)()
    pipe._c(pipe.lib.drv_get_cone_voxel_reads(pipe.ctx, reads))
    pipe.set_tuning(count_voxel_reads=0)
    traced = hv.get("retraced_pairs") if head.startswith("surrogate") else hv["live_pairs"]
    pipe.close()
    return {"w": w, "head": head, "variants": variants, "specular": specular, "e2e": e2e, "kernel_ms": kernel_ms,
            "voxel_reads": list(reads), "traced_pairs": traced, "hv": hv, "count": count}


def cone_roofline(r, cache_peaks, pk, w_name) -> dict:
    """The light stage's dominant kernel against its bound. The cone pass
    reads its voxel pyramid from L1/L2 (16 MiB corner grid + mip records,
    L2-resident): algorithmic bytes = the counted voxel loads (level-0 corner
    bytes x 1 B, FP16 mip records x 16 B, plain mip texels x 4 B FP32 / 2 B
    BF16) + 16 B per traced pair (its order index, cache and block indices,
    the shadowing written), over the kernel's live event time, against the
    measured L2 load throughput; L1 and HBM figures beside it."""
    kernel_ms, hv = r["kernel_ms"], r["hv"]
    top = max(kernel_ms, key=kernel_ms.get)
    top_ms = kernel_ms[top]
    if top == "mlp":
        n_pairs = hv.get("evaluated_pairs") or 0
        flop = n_pairs * 20736  # 2 (32*64 + 64*64 + 64*64 + 64*2) per evaluated pair
        achieved = flop / (top_ms / 1e3) / 1e12
        return {"bound": "tensor", "kernel": "mlp_tc_kernel", "achieved": achieved, "peak": pk["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"], "traffic": None,
                "peak_source": pk["source"] + " (bf16_tflops, burst)",
                "algorithmic": f"{n_pairs} evaluated pairs x 20736 flop"}
    l0, rec, tex = r["voxel_reads"]
    tex_bytes = 2 if r["head"] in ("precision_bf16",) or r["head"].startswith("surrogate") else 4
    traced = r["traced_pairs"] or 0
    voxel_bytes = l0 * 1 + rec * 16 + tex * tex_bytes
    nbytes = voxel_bytes + traced * 16
    achieved = nbytes / (top_ms / 1e3) / 1e9
    l2 = cache_peaks.get("l2_gbs") or float("nan")
    l1 = cache_peaks.get("l1_gbs") or float("nan")
    return {"bound": "l2", "kernel": f"{top}_kernel", "achieved": achieved, "peak": l2, "unit": "GB/s",
            "frac": achieved / l2,
            "traffic": NCU_TRAFFIC.get(f"{top}_kernel") if w_name == "ns_1080p_4096" else None,
            "peak_source": "measured on this GPU by drv_measure_load_bandwidth (L2, 16-byte loads)",
            "algorithmic": (f"{l0} level-0 corner bytes x 1 B + {rec} mip records x 16 B + {tex} mip texels x "
                            f"{tex_bytes} B + {traced} traced pairs x 16 B = {nbytes} B per launch"),
            "l1": {"peak_gbs": l1, "frac": achieved / l1},
            "hbm": {"peak_gbs": pk["hbm_gbs"], "frac": achieved / pk["hbm_gbs"],
                    "peak_source": pk["source"] + " (hbm_gbs)",
                    "note": "the voxel pyramid is L2-resident; one ncu capture of this pass read 16.5 MB "
                            "from DRAM per launch (profiles/)"},
            "note": "the cone pass is bound by issue and load latency (67% issue active, ALU pipe 43%, 23 of 32 "
                    "lanes active, long_scoreboard the top stall): its loads are a small share of either cache's "
                    "throughput",
            "gather": gather_roofline(r, pk)}


def stage_rooflines(w, bf16: bool, caches: int, stage_ms: dict, pk) -> dict:
    """The HBM-bound stages against the measured copy bandwidth: algorithmic
    bytes of one frame's stage (every input read once, every output written
    once, gathered per-cache data counted once per cache) over the stage's
    stream-timed duration. RSM texels: RGB F32 flux + RG16I normal + RG F32
    (d, d^2) = 24 B; G-buffer: F32 depth, RG16I normal, RGB F32 albedo; output
    RGB F32."""
    px = w.width * w.height
    R, K = w.rsm_resolution, w.rsm_read_lod + w.shadow_lod
    levels = [(R >> k) ** 2 * 24 for k in range(K + 1)]
    n_vpl = (R >> w.rsm_read_lod) ** 2
    vpl_out = n_vpl * ((32 if bf16 else 48) + 16 + 16)  # VPL, shadow cone, cull record
    # level 0 read, levels 1..K written (the chain keeps the levels between
    # its passes on chip), the VPL level and the shadow level read by the
    # extraction
    extract_reads = levels[w.rsm_read_lod] + (levels[K] if K > w.rsm_read_lod else 0)
    rsm = w.n_lights * (levels[0] + sum(levels[1:]) + extract_reads + vpl_out)
    N = w.voxel_res
    L = N.bit_length() - 1
    mip_texels = sum((N >> l) ** 3 for l in range(1, L + 1))
    rec_levels = L if bf16 else min(L, 3)
    rec_texels = sum((N >> l) ** 3 for l in range(1, rec_levels + 1))
    vox = (N ** 3 // 8 * 3  # bit grid written once, read by the mip and corner passes
           + mip_texels * (2 if bf16 else 4) * 2  # mip texels written, read back for the records
           + N ** 3  # corner-packed level 0 written
           + rec_texels * 16)  # mip records written
    entry = 64 if bf16 else (128 if w.sh_order == 2 else 64)
    atlas = w.n_cascades * w.cav_res ** 3 * 4
    alloc = px * 4 + atlas + caches * entry
    apply = px * (4 + 4 + 12 + 12) + atlas + caches * entry
    out = {}
    for name, nbytes in (("rsm+vpl", rsm), ("voxelize+mips", vox), ("allocate", alloc), ("apply", apply)):
        ms = stage_ms.get(name) or 0.0
        gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else None
        out[name] = {"bytes": int(nbytes), "ms": ms, "achieved_gbs": gbs,
                     "frac_of_hbm": gbs / pk["hbm_gbs"] if gbs else None}
    out["peak_gbs"] = pk["hbm_gbs"]
    out["peak_source"] = pk["source"] + " (hbm_gbs)"
    out["note"] = ("stream-timed stages of one frame, L2 flushed before the frame; these stages are latency- or "
                   "issue-bound (profiles/): their HBM fractions are low by that measure")
    return out


def gather_roofline(r, pk) -> dict:
    """The gather pass against the FP32 pipe: the algorithmic flops of the SH
    sum per gathered pair (sh_flops_per_pair; the BF16 variant's Kahan
    compensation is not counted) over its live event time, against the
    nominal FP32 rate of this GPU (SMs x 128 FP32 lanes x 2 flop x max SM
    clock)."""
    import torch
    g_ms = r["kernel_ms"].get("gather") or 0.0
    pairs = r["hv"].get("live_pairs") or 0
    per = sh_flops_per_pair(r["w"].sh_order)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = sms * 128 * 2 * pk["sm_max_mhz"] * 1e6 / 1e12
    achieved = pairs * per / (g_ms / 1e3) / 1e12 if g_ms > 0 else None
    return {"kernel": "gather_kernel", "bound": "fp32 pipe", "flops_per_pair": per, "pairs": pairs,
            "achieved_tflops": achieved, "peak_tflops": peak, "frac": achieved / peak if achieved else None,
            "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 flop x {pk['sm_max_mhz']:.0f} MHz"}


def cpu_baseline_of(w, threads) -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py as O
    hf_cpu = O.host_frame(w)
    caches, t_frame, t_light, note = cpu_frame(w, hf_cpu, oracle_inputs(hf_cpu, w), threads)
    return {"value": caches / t_light, "unit": UNIT, "cores": threads, "kind": "port", "sample": note + " (one frame)",
            "ms_per_frame": t_frame * 1e3}


def run_ours(args):
    import torch
    import torch.distributed as dist
    from dynamicradiancevolume_gb300 import abi, pipeline, surrogate

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = pipeline.WORKLOADS[args.workload]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > 129 MB L2
    if ws > 1:
        dist.barrier()
    weights, features, surrogate_note = None, "segment8", None
    if surrogate.DEFAULT_WEIGHTS.with_suffix(".bin").exists():
        try:
            weights, features = surrogate.load_params(), surrogate.load_features()
        except ValueError as e:  # a checkpoint of another model layout: no surrogate variants
            surrogate_note = str(e)
    extra = ([] if args.no_extra_workloads or args.workload != "ns_1080p_4096"
             else ["c2_production", "ns_1080p_4096_cav128"])
    with ClockSampler(local) as clk:
        r = measure_workload(w, args, dev, flush, rank, weights, features, full=True)
        others = {name: measure_workload(pipeline.WORKLOADS[name], args, dev, flush, rank, None, features,
                                         full=False) for name in extra}
        cache_peaks = measure_cache_peaks(dev)
        batch = None
        if args.batch_scenes > 0 and args.workload == "ns_1080p_4096" and rank == 0:
            from dynamicradiancevolume_gb300 import batch as batch_mod
            batch = batch_mod.run_batch(args.batch_scenes, reps=5, log=lambda m: None, tune_reps=2)
    clocks = clk.summary()
    pk = peaks()
    hv, head, count = r["hv"], r["head"], r["count"]

    # ---- max over ranks (replicas)
    light_ms_all, frame_ms_all, e2e_ms_all, caches_all = reduce_over_ranks(hv["light_ms"], hv["frame_ms"],
                                                                           r["e2e"]["ms_per_step"], float(count),
                                                                           device=dev)
    e2e = dict(r["e2e"])
    e2e.update({"value": caches_all / (e2e_ms_all / 1e3), "ms_per_step": e2e_ms_all})
    line = {
        "metric": METRIC, "value": caches_all / (light_ms_all / 1e3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": light_ms_all, "ms_per_frame": frame_ms_all,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if head != "plain_fp32" else "f32",
        "data": "synthetic (seeded procedural box room)",
        "config": workload_config(w), "variant": head, "caches": count,
        "step": "the light stage (drv_light_caches) over the frame's VPLs, voxels and caches, captured once as "
                "a CUDA graph and replayed; ms_per_frame = the whole frame (drv_frame) replayed the same way",
        "rel_l2_vs_fp64": hv.get("rel_l2_vs_fp64"),
        "errors_vs_fp64": {k: hv.get(k) for k in ("rel_l2_vs_fp64", "radiance_max_abs_vs_fp64", "sh_rel_l2_vs_fp64",
                                                  "sh_max_abs_vs_fp64")},
        "stage_ms": hv["stage_ms"],
        "light_kernel_ms": r["kernel_ms"],
        "variants": r["variants"],
        "specular": r["specular"],
        "roofline": cone_roofline(r, cache_peaks, pk, w.name),
        "cache_peaks": cache_peaks,
        "stage_roofline": stage_rooflines(w, head != "plain_fp32", count, hv["stage_ms"], pk),
        "e2e": e2e,
        "gpu_launches": light_stage_launches(w, head.startswith("surrogate")) * args.steps,
        "clocks": clocks,
    }
    if surrogate_note:
        line["surrogate_skipped"] = surrogate_note
    if batch is not None:
        # config 5: many seeded scenes of uneven sizes, BF16 storage, surrogate
        # visibility; one CUDA-graph launch against the scenes one by one (each
        # scene's frame alone as a graph) and against the reference's form
        # (each scene alone, host-issued kernels, one lighting pass per light)
        line["batch"] = {k: batch[k] for k in ("scenes", "precision", "visibility", "threshold", "sizes", "tuned",
                                               "batch", "one_by_one", "reference_form", "speedup",
                                               "speedup_vs_reference_form", "largest_tenth")}
        line["batch"]["trials"] = len(batch["trials"])
        # the stream-count sweep at default knobs: 1 stream = the scenes back
        # to back inside one graph (no host gaps, no concurrency)
        line["batch"]["ms_by_streams"] = {str(t["streams"]): t["ms"] for t in batch["trials"]
                                          if all(t.get(k) == m[0] for k, m in batch_mod.KNOB_MENUS.items())}
    threads = os.cpu_count() or 1
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_of(w, threads)
    if others:
        line["workloads"] = {}
        for name, o in others.items():
            ov = o["hv"]
            entry = {"config": workload_config(o["w"]), "variant": o["head"], "caches": o["count"],
                     "value": o["count"] / (ov["light_ms"] / 1e3), "unit": UNIT, "ms_per_step": ov["light_ms"],
                     "ms_per_frame": ov["frame_ms"], "rel_l2_vs_fp64": ov.get("rel_l2_vs_fp64"),
                     "errors_vs_fp64": {k: ov.get(k) for k in ("rel_l2_vs_fp64", "radiance_max_abs_vs_fp64",
                                                               "sh_rel_l2_vs_fp64", "sh_max_abs_vs_fp64")},
                     "light_kernel_ms": o["kernel_ms"], "variants": o["variants"],
                     "roofline": cone_roofline(o, cache_peaks, pk, name), "e2e": o["e2e"]}
            if rank == 0 and not args.no_cpu_baseline:
                entry["cpu_baseline"] = cpu_baseline_of(o["w"], threads)
            line["workloads"][name] = entry
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
