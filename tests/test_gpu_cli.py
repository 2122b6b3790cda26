"""The C++ caller (drv_frame_cli, C ABI only, no Python in the process)
renders the same frame as the Python binding: the same cache count and the
same radiance, bit for bit (written through drv_write_pfm)."""
import json
import subprocess

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import build, pipeline

pytestmark = pytest.mark.gpu


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4")
    return data.reshape(h, w, 3)


def test_cli_frame_equals_python_frame(lib, cuda, tmp_path):
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], name="cli", seed=11)
    cli = build.build_cli()
    out = tmp_path / "frame.pfm"
    args = [str(cli), str(w.width), str(w.height), str(w.n_boxes), str(w.voxel_res), str(w.rsm_resolution),
            str(w.rsm_read_lod), str(w.n_cascades), str(w.cav_res), repr(w.cascade_world_size0), str(w.sh_order),
            str(w.max_cone_steps), repr(w.cascade_transition), str(w.seed), "3", str(out)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    p = pipeline.Pipeline(pipeline.host_frame(pipeline.scaled(w, max_caches=262144)))
    p.raycast_inputs()
    p.frame()
    p.sync()
    assert line["caches"] == p.cache_count()
    img = read_pfm(out)
    assert np.array_equal(img, p.out.cpu().numpy())
    assert line["ms_per_frame"] > 0
    p.close()
