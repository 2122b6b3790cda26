"""Visibility surrogate: training data, training, checkpoints.

The surrogate (csrc/surrogate.cuh) predicts the indirect-shadow cone's
visibility for a (cache, shadow block) pair. This module drives the C-ABI
kernels that generate cone-traced training pairs on seeded scenes
(drv_surrogate_make_pairs), train the MLP (drv_surrogate_train_step: fused
forward/backward + Adam), and evaluate it (drv_surrogate_eval). Torch only
holds device buffers and shuffles sample indices.

Checkpoint = a flat little-endian BF16 blob of the DRV_SURROGATE_PARAMS
parameters (W1[64][32], b1, W2[64][64], b2, W3[64][64], b3, W4[2][64], b4)
plus a JSON header describing the layout, the input feature set and how the
weights were trained. A training run can also save its Adam state
(`<out>.adam.npz`: FP32 parameters, both moments, the step) and resume from
it (`--resume`).

    python -m dynamicradiancevolume_gb300.surrogate train --out weights/visibility_mlp
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

from . import abi, check, load, pipeline

PKG = Path(__file__).resolve().parent
DEFAULT_WEIGHTS = PKG / "weights" / "visibility_mlp"
N_IN, N_H, N_OUT = abi.SURROGATE_INPUTS, 64, 2
LAYOUT = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("W3", (N_H, N_H)),
          ("b3", (N_H,)), ("W4", (N_OUT, N_H)), ("b4", (N_OUT,))]

# Scenes the pairs come from: the production generator (64 boxes, 256^3
# voxels, 4 cascades, one 512^2 RSM read at 64^2), at half resolution.
TRAIN_WORKLOAD = pipeline.scaled(pipeline.WORKLOADS["ns_1080p_4096"], name="surrogate_train", width=960, height=540)


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def init_params(seed: int = 0):
    """Glorot-uniform weights, zero biases (FP32, numpy)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in LAYOUT:
        if name.startswith("W"):
            fan_out, fan_in = shape
            lim = math.sqrt(6.0 / (fan_in + fan_out))
            parts.append(rng.uniform(-lim, lim, size=shape).astype(np.float32).ravel())
        else:
            parts.append(np.zeros(shape, np.float32))
    p = np.concatenate(parts)
    assert p.size == abi.SURROGATE_PARAMS
    return p


def save(params: np.ndarray, path: Path, meta: dict, features: str = "segment8") -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    p = np.asarray(params, np.float32)
    bits = p.view(np.uint32)
    # round to nearest even BF16
    bf16 = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype("<u2")
    path.with_suffix(".bin").write_bytes(bf16.tobytes())
    header = {"format": "bf16-le", "n_params": int(p.size), "layout": [[n, list(s)] for n, s in LAYOUT],
              "inputs": N_IN, "hidden": N_H, "outputs": N_OUT, "activation": "gelu-sigmoid: x sigmoid(1.702 x)",
              "features": features,
              "outputs_meaning": ["visibility logit", "confidence logit"], **meta}
    path.with_suffix(".json").write_text(json.dumps(header, indent=2) + "\n")


def load_params(path: Path = DEFAULT_WEIGHTS) -> np.ndarray:
    path = Path(path)
    header = json.loads(path.with_suffix(".json").read_text())
    raw = np.frombuffer(path.with_suffix(".bin").read_bytes(), "<u2")
    if raw.size != header["n_params"] or raw.size != abi.SURROGATE_PARAMS:
        raise ValueError(f"{path}: expected {abi.SURROGATE_PARAMS} parameters, found {raw.size}")
    if not header.get("activation", "").startswith("gelu-sigmoid"):
        raise ValueError(f"{path}: trained with another activation ({header.get('activation')})")
    return (raw.astype(np.uint32) << 16).view(np.float32).copy()


def load_features(path: Path = DEFAULT_WEIGHTS) -> str:
    """The input feature set a checkpoint was trained on."""
    return json.loads(Path(path).with_suffix(".json").read_text()).get("features", "segment8")


def set_features(pipe: "pipeline.Pipeline", features: str) -> None:
    check(pipe.lib.drv_set_surrogate_features(pipe.ctx, abi.SURROGATE_FEATURE_NAMES[features]), pipe.ctx)


def upload(pipe: "pipeline.Pipeline", params: np.ndarray, features: str = "segment8") -> None:
    """Loads FP32 parameters (host) as the pipeline context's inference
    weights, trained on the given feature set."""
    torch = pipe.torch
    set_features(pipe, features)
    dev = torch.from_numpy(np.asarray(params, np.float32)).to(pipe.device)
    check(pipe.lib.drv_set_surrogate_params(pipe.ctx, _ptr(dev)), pipe.ctx)
    pipe.stream.synchronize()


def generate_pairs(seeds, pairs_per_scene: int, workload=TRAIN_WORKLOAD, device="cuda", log=print,
                   features: str = "segment8"):
    """Cone-traced (features, visibility) pairs from each seeded scene."""
    import torch
    lib = load()
    n = len(seeds) * pairs_per_scene
    X = torch.empty((n, N_IN), dtype=torch.float32, device=device)
    Y = torch.empty((n,), dtype=torch.float32, device=device)
    t0 = time.time()
    pipe = None
    for k, seed in enumerate(seeds):
        hf = pipeline.host_frame(workload, seed)
        if pipe is None:
            pipe = pipeline.Pipeline(hf, device=device)
            set_features(pipe, features)
        else:
            pipe.set_frame(hf)
        pipe.raycast_inputs()
        pipe.prepare_and_extract()
        pipe.voxelize()
        pipe.allocate()
        off = k * pairs_per_scene
        check(lib.drv_surrogate_make_pairs(pipe.ctx, 1000003 * seed + 17, pairs_per_scene,
                                           C.c_void_p(X.data_ptr() + off * N_IN * 4),
                                           C.c_void_p(Y.data_ptr() + off * 4)), pipe.ctx)
        if log and (k + 1) % 50 == 0:
            pipe.sync()
            log(f"pairs: {k + 1}/{len(seeds)} scenes, {time.time() - t0:.1f} s")
    pipe.sync()
    pipe.close()
    return X, Y


def save_state(path: Path, params, m, v, step: int, epoch: int) -> None:
    """Adam state of a training run (FP32 parameters, both moments, the step
    count and finished epochs), for resuming it."""
    np.savez(Path(path).with_suffix(".adam.npz"), params=np.asarray(params, np.float32),
             m=np.asarray(m, np.float32), v=np.asarray(v, np.float32), step=np.int64(step), epoch=np.int64(epoch))


def load_state(path: Path) -> dict:
    z = np.load(Path(path).with_suffix(".adam.npz"))
    return {"params": z["params"], "m": z["m"], "v": z["v"], "step": int(z["step"]), "epoch": int(z["epoch"])}


def train(X, Y, epochs=6, batch=4096, lr=2e-3, conf_tau=0.03, weight_decay=0.0, seed=0, log=print, state=None,
          checkpoint: Path | None = None):
    """Adam on the hand-written training kernels; returns FP32 numpy params.
    state: a load_state() dict to resume from (its finished epochs are
    skipped, the learning-rate schedule continues where it stopped);
    checkpoint: where to save the Adam state after every epoch."""
    import torch
    lib = load()
    dev = X.device
    if state is not None:
        params = torch.from_numpy(state["params"]).to(dev)
        m = torch.from_numpy(state["m"]).to(dev)
        v = torch.from_numpy(state["v"]).to(dev)
        step, first_epoch = state["step"], state["epoch"]
    else:
        params = torch.from_numpy(init_params(seed)).to(dev)
        m = torch.zeros_like(params)
        v = torch.zeros_like(params)
        step, first_epoch = 0, 0
    scratch = torch.empty(lib.drv_surrogate_train_scratch_floats(batch), dtype=torch.float32, device=dev)
    loss = torch.zeros(2, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    n = X.shape[0]
    steps_per_epoch = n // batch
    total = steps_per_epoch * epochs
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    for _ in range(first_epoch):  # the permutations of the finished epochs
        torch.randperm(n, device=dev, generator=g)
    t0 = time.time()
    for ep in range(first_epoch, epochs):
        perm = torch.randperm(n, device=dev, generator=g)
        Xs, Ys = X.index_select(0, perm), Y.index_select(0, perm)
        acc = torch.zeros(2, dtype=torch.float64, device=dev)
        for b in range(steps_per_epoch):
            step += 1
            lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * (step - 1) / total))  # cosine decay
            st = lib.drv_surrogate_train_step(C.c_void_p(Xs.data_ptr() + b * batch * N_IN * 4),
                                              C.c_void_p(Ys.data_ptr() + b * batch * 4), batch, _ptr(params),
                                              _ptr(m), _ptr(v), _ptr(scratch), step, lr_t, conf_tau, weight_decay,
                                              _ptr(loss), C.c_void_p(stream.cuda_stream))
            if st != abi.OK:
                raise RuntimeError(f"drv_surrogate_train_step failed: {abi.STATUS_NAMES.get(st, st)}")
            acc += loss.double()
        torch.cuda.synchronize(dev)
        if checkpoint is not None:
            save_state(checkpoint, params.cpu().numpy(), m.cpu().numpy(), v.cpu().numpy(), step, ep + 1)
        if log:
            l = (acc / (steps_per_epoch * batch)).tolist()
            log(f"epoch {ep + 1}/{epochs}: visibility BCE {l[0]:.4f}, confidence BCE {l[1]:.4f}, "
                f"{time.time() - t0:.1f} s")
    return params.cpu().numpy()


def evaluate(pipe, X, Y, threshold: float):
    """Surrogate accuracy on pairs: MAE overall, share confident, MAE on the
    confident pairs."""
    import torch
    out = torch.empty((X.shape[0], 2), dtype=torch.float32, device=X.device)
    check(pipe.lib.drv_surrogate_eval(pipe.ctx, _ptr(X), X.shape[0], _ptr(out)), pipe.ctx)
    pipe.stream.synchronize()
    vis, conf = out[:, 0], out[:, 1]
    err = (vis - Y).abs()
    confident = conf >= threshold
    return {"mae": float(err.mean()), "confident_share": float(confident.float().mean()),
            "mae_confident": float(err[confident].mean()) if bool(confident.any()) else None,
            "p99_err_confident": float(err[confident].quantile(0.99)) if bool(confident.any()) else None}


def frame_error(params, seeds, threshold: float, workload=None, device="cuda", features: str = "segment8"):
    """Final indirect radiance of full frames with surrogate visibility
    against the same frames with cone visibility (both on the GPU): relative
    L2 per seed, the share of contributing pairs re-traced, and the light
    stage's time in both forms (graph replays, not L2-flushed)."""
    import torch
    workload = workload or pipeline.WORKLOADS["ns_1080p_4096"]
    out = []
    for seed in seeds:
        hf_c = pipeline.host_frame(workload, seed)
        cone = pipeline.Pipeline(hf_c, device=device)
        cone.raycast_inputs()
        cone.frame()
        cone.sync()
        ref = cone.out.clone()
        t_cone = _light_ms(cone)
        cone.close()
        hf_s = pipeline.host_frame(pipeline.scaled(workload, visibility=abi.VISIBILITY_SURROGATE), seed)
        hf_s.config.surrogate_conf_threshold = threshold
        sur = pipeline.Pipeline(hf_s, device=device)
        upload(sur, params, features)
        sur.raycast_inputs()
        sur.frame()
        sur.sync()
        evaluated, retraced = sur.surrogate_stats()
        err = float(torch.linalg.vector_norm((sur.out - ref).double()) / torch.linalg.vector_norm(ref.double()))
        t_sur = _light_ms(sur)
        out.append({"seed": seed, "rel_l2_vs_cone": err, "retraced_share": retraced / max(evaluated, 1),
                    "light_ms_cone": t_cone, "light_ms_surrogate": t_sur})
        sur.close()
    return out


def _light_ms(pipe, reps: int = 20) -> float:
    """Mean ms of the light stage replayed as a CUDA graph."""
    import torch
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=pipe.stream):
        pipe.light()
    for _ in range(3):
        g.replay()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(pipe.stream):
        a.record(pipe.stream)
        for _ in range(reps):
            g.replay()
        b.record(pipe.stream)
    b.synchronize()
    return a.elapsed_time(b) / reps


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--scenes", type=int, default=200)
    t.add_argument("--pairs", type=int, default=100_000)
    t.add_argument("--epochs", type=int, default=6)
    t.add_argument("--batch", type=int, default=4096)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--tau", type=float, default=0.03)
    t.add_argument("--features", choices=sorted(abi.SURROGATE_FEATURE_NAMES), default="segment8")
    t.add_argument("--out", type=Path, default=DEFAULT_WEIGHTS)
    t.add_argument("--resume", action="store_true", help="continue from <out>.adam.npz")
    t.add_argument("--eval-scenes", type=int, default=10)
    t.add_argument("--thresholds", type=float, nargs="*", default=[0.0, 0.5, 0.8])
    args = ap.parse_args(argv)
    dev = torch.device("cuda")
    t0 = time.time()
    X, Y = generate_pairs(list(range(args.scenes)), args.pairs, device=dev, features=args.features)
    gen_s = time.time() - t0
    print(f"{X.shape[0]} pairs ({args.features}) in {gen_s:.1f} s; mean visibility {float(Y.mean()):.3f}")
    t1 = time.time()
    state = load_state(args.out) if args.resume else None
    params = train(X, Y, epochs=args.epochs, batch=args.batch, lr=args.lr, conf_tau=args.tau, state=state,
                   checkpoint=args.out)
    train_s = time.time() - t1
    del X, Y
    Xe, Ye = generate_pairs(list(range(1000, 1000 + args.eval_scenes)), args.pairs, device=dev,
                            features=args.features)
    hf = pipeline.host_frame(TRAIN_WORKLOAD, 1000)
    pipe = pipeline.Pipeline(hf)
    upload(pipe, params, args.features)
    stats = evaluate(pipe, Xe, Ye, threshold=0.5)
    pipe.close()
    print("held-out pairs:", json.dumps(stats))
    frames = {}
    for thr in args.thresholds:
        fe = frame_error(params, list(range(1000, 1000 + args.eval_scenes)), thr, features=args.features)
        frames[str(thr)] = fe
        print(f"held-out frames, threshold {thr}:", json.dumps(fe))
    stats["frames"] = frames
    save(params, args.out, {"trained_on": {"workload": TRAIN_WORKLOAD.name, "scene_seeds": [0, args.scenes - 1],
                                           "pairs": args.scenes * args.pairs, "epochs": args.epochs,
                                           "batch": args.batch, "lr": args.lr, "conf_tau": args.tau,
                                           "pair_generation_s": round(gen_s, 1), "training_s": round(train_s, 1)},
                             "held_out": {"scene_seeds": [1000, 1000 + args.eval_scenes - 1], **stats}},
         features=args.features)
    print(f"saved {args.out}.bin / .json")


if __name__ == "__main__":
    main()
