"""drv_frame is capture-safe: captured once into a CUDA graph on the
context's stream and replayed, it gives the frame drv_frame gives (the
per-cache gather runs in a fixed order, so the frame is bitwise
reproducible), with plain and surrogate visibility."""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline, surrogate
from test_gpu_parity import REDUCED

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("visibility", [abi.VISIBILITY_CONE, abi.VISIBILITY_SURROGATE], ids=["cone", "surrogate"])
def test_captured_frame_replays_drv_frame(visibility, cuda, lib):
    import torch
    w = pipeline.scaled(REDUCED, visibility=visibility)
    hf = pipeline.host_frame(w, 12)
    hf.config.surrogate_conf_threshold = 0.5
    p = pipeline.Pipeline(hf)
    if visibility == abi.VISIBILITY_SURROGATE:
        surrogate.upload(p, surrogate.init_params(2))
    p.raycast_inputs()
    p.frame()
    p.sync()
    direct = p.out.clone()
    out = torch.zeros_like(p.out)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=p.stream):
        p.frame(out)
    for _ in range(3):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(out, direct)
    p.close()
