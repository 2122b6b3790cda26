"""The CUDA path on the golden frame's own inputs (tests/golden, the FP64
oracle's G-buffer and RSM) against the oracle's outputs for every stage."""
from pathlib import Path

import numpy as np
import pytest

from test_gpu_parity import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).with_name("golden")


def test_cuda_path_on_golden_inputs(cuda, lib):
    import sys
    import torch
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    from dynamicradiancevolume_gb300 import pipeline
    g = dict(np.load(GOLDEN / "tiny_frame.npz"))
    p = pipeline.Pipeline(pipeline.host_frame(make_golden.TINY, make_golden.SEED))
    for t, k in ((p.depth, "depth"), (p.normal16, "normal16"), (p.albedo, "albedo"), (p.rsm_flux[0], "rsm_flux"),
                 (p.rsm_normal[0], "rsm_normal16"), (p.rsm_dls[0], "rsm_dls")):
        t.copy_(torch.from_numpy(g[k]))
    torch.cuda.synchronize()
    p.frame()
    p.sync()
    # VPLs (flux 0:3, area 3, position 4:7, normal 7:10 in the oracle's layout)
    v = p.read_vpls(0).cpu().numpy()
    gv = g["vpls"]
    assert np.allclose(v[:, 0:3], gv[:, 0:3], rtol=1e-5, atol=1e-12)
    assert np.allclose(v[:, 4:7], gv[:, 4:7], rtol=0, atol=1e-5)
    # voxels bit-exact, the allocated cache set exact
    assert np.array_equal(p.read_voxel_bits().cpu().numpy().view(np.uint32), g["voxel_bits"])
    n = p.cache_count()
    assert n == int(g["cache_count"])
    pos, sh = p.read_entries_decoded(n)
    order = np.lexsort(pos.T[::-1])
    assert np.array_equal(pos[order], g["cache_positions"].astype(np.float32))
    assert rel_l2(sh[order], g["cache_sh"]) < 1e-3
    assert rel_l2(p.out.cpu().numpy(), g["radiance"]) < 1e-3
    p.close()
