"""Host logic without a GPU: the batch autotuner's coordinate descent over a
synthetic cost, the bench's launch count and per-stage algorithmic bytes."""
import numpy as np
import pytest

import bench
from dynamicradiancevolume_gb300 import abi, batch, pipeline


class _FakePipe:
    def __init__(self):
        self.knobs = {}

    def set_tuning(self, **knobs):
        self.knobs.update(knobs)


class _FakeScene:
    def __init__(self):
        self.pipe = _FakePipe()


def test_autotune_descends_each_knob_and_leaves_the_best_set(monkeypatch):
    scenes = [_FakeScene() for _ in range(16)]
    menus = {"a": (0, 1, 2), "b": (4, 2, 8)}

    def cost(streams, knobs):
        # minimum at 4 streams, a = 2, b = 8; each term independent
        return abs(np.log2(streams) - 2) + abs(knobs["a"] - 2) + abs(knobs["b"] - 8) / 2 + 10.0

    def fake_time_batch(sc, streams, reps, warmup=2):
        return cost(streams, sc[0].pipe.knobs), None

    monkeypatch.setattr(batch, "time_batch", fake_time_batch)
    best, trials = batch.autotune(scenes, streams_menu=(1, 2, 4, 8, 32, 64), knob_menus=menus, log=lambda m: None)
    assert (best["streams"], best["a"], best["b"]) == (4, 2, 8)
    assert best["ms"] == pytest.approx(10.0)
    assert all(s.pipe.knobs == {"a": 2, "b": 8} for s in scenes)
    assert all(t["streams"] <= len(scenes) for t in trials)  # 32 and 64 streams exceed the scenes: skipped
    assert len(trials) == 4 + 2 + 2


def test_light_stage_launch_count():
    ns = pipeline.WORKLOADS["ns_1080p_4096"]
    assert bench.light_stage_launches(ns) == 5  # cull, classify, scatter, cone, gather
    assert bench.light_stage_launches(ns, surrogate=True) == 6  # cull, MLP, classify, scatter, cone, gather
    assert bench.light_stage_launches(pipeline.scaled(ns, indirect_shadow=0)) == 1


def test_stage_roofline_bytes_of_the_headline():
    ns = pipeline.WORKLOADS["ns_1080p_4096"]
    pk = {"hbm_gbs": 1000.0, "source": "test"}
    r = bench.stage_rooflines(ns, True, 1814, {"rsm+vpl": 0.01, "voxelize+mips": 0.01, "allocate": 0.01,
                                               "apply": 0.01}, pk)
    px, atlas = 1920 * 1080, 4 * 32 ** 3 * 4
    assert r["apply"]["bytes"] == px * 32 + atlas + 1814 * 64
    assert r["allocate"]["bytes"] == px * 4 + atlas + 1814 * 64
    # RSM chain: 512^2 read, levels 1..3 written once, level 3 (VPLs and shadow blocks) read by the extraction
    lv = [(512 >> k) ** 2 * 24 for k in range(4)]
    assert r["rsm+vpl"]["bytes"] == lv[0] + sum(lv[1:]) + lv[3] + 4096 * (32 + 16 + 16)
    # voxels: bit grid x3, FP16 mips written + read, corner grid, every level's records
    texels = sum((256 >> l) ** 3 for l in range(1, 9))
    assert r["voxelize+mips"]["bytes"] == 256 ** 3 // 8 * 3 + texels * 2 * 2 + 256 ** 3 + texels * 16
    assert r["apply"]["achieved_gbs"] == pytest.approx(r["apply"]["bytes"] / 1e-5 / 1e9)
    assert r["apply"]["frac_of_hbm"] == pytest.approx(r["apply"]["achieved_gbs"] / 1000.0)
