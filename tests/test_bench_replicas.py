"""The benchmark's multi-GPU mode is replicas: each rank renders its own
frame, and only the report is reduced (slowest rank's times, all ranks'
caches). Checked with two gloo ranks on the CPU; a reference-arm rank other
than 0 exits without work, and rank 0 prints the CPU arm's line."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: light 1+r ms, frame 2+r ms, e2e 3+r ms, 100*(r+1) caches
        out[rank] = bench.reduce_over_ranks(1.0 + rank, 2.0 + rank, 3.0 + rank, 100.0 * (rank + 1))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_time_and_total_caches():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        assert res[r] == pytest.approx((2.0, 3.0, 4.0, 300.0))


def test_single_process_reduction_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_over_ranks(1.5, 2.5, 3.5, 7) == (1.5, 2.5, 3.5, 7.0)


def test_reference_arm_rank_one_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""


def test_reference_arm_line_on_the_small_workload():
    """The CPU arm's one JSON line on the small workload: the FP64 oracle
    alone (the product library never mapped into the process), the
    workload's config, and its own cpu_baseline and e2e objects."""
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "c1_small",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    d = json.loads(p.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["product_library_loaded"] is False
    assert d["config"]["workload"] == "c1_small" and d["dtype"] == "f64"
    assert d["unit"] == "caches/s" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "caches/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
