"""The reference's G-buffer diffuse format (SRGB8, renderer.cpp:468, read
back through the GL sRGB decode): apply and the brute-force gather over an
SRGB8 G-buffer equal, bit for bit, the same passes over the linear F32
values the decode gives."""
import ctypes as C

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import REDUCED

pytestmark = pytest.mark.gpu


def srgb_decode(b):
    """GL 4.5 section 8.24, in double, rounded to float."""
    cs = np.asarray(b, np.float64) / 255.0
    return np.where(cs <= 0.04045, cs / 12.92, ((cs + 0.055) / 1.055) ** 2.4).astype(np.float32)


def srgb_encode(lin):
    lin = np.clip(np.asarray(lin, np.float64), 0.0, 1.0)
    cs = np.where(lin <= 0.0031308, lin * 12.92, 1.055 * lin ** (1 / 2.4) - 0.055)
    return np.clip(np.rint(cs * 255.0), 0, 255).astype(np.uint8)


def test_decode_table_known_values():
    t = srgb_decode(np.arange(256))
    assert t[0] == 0.0 and t[255] == 1.0
    assert t[10] == np.float32(10 / 255 / 12.92)  # the linear segment
    assert np.all(np.diff(t) > 0)


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["c1_small"], REDUCED], ids=["c1", "c2r"])
def test_srgb8_albedo_equals_its_linear_decode(w, lib, cuda):
    torch = pytest.importorskip("torch")
    p = pipeline.Pipeline(pipeline.host_frame(w, 4))
    p.raycast_inputs()
    p.frame()
    p.sync()
    H, W = w.height, w.width
    alb = p.albedo.cpu().numpy()
    b8 = srgb_encode(alb)
    dev8 = torch.from_numpy(b8.reshape(-1)).to(p.device)
    p.albedo.copy_(torch.from_numpy(srgb_decode(b8)).to(p.device))
    torch.cuda.synchronize()
    ref = torch.zeros_like(p.out)
    p.apply(ref)
    brute_ref = p.bruteforce()
    p.sync()
    v8 = abi.DrvGBufferView(W, H, p.depth.data_ptr(), p.gview.normal, p.gview.normal_format, dev8.data_ptr(),
                            abi.ALBEDO_SRGB8)
    out8 = torch.zeros_like(p.out)
    assert lib.drv_apply(p.ctx, C.byref(v8), C.byref(p.hf.frame), C.byref(p.hf.volume),
                         C.c_void_p(out8.data_ptr())) == abi.OK
    keep = p.gview
    p.gview = v8
    brute8 = p.bruteforce()
    p.gview = keep
    p.sync()
    assert torch.equal(out8, ref)
    assert torch.equal(brute8, brute_ref)
    assert float(ref.abs().sum()) > 0
    # an unknown format is rejected
    bad = abi.DrvGBufferView(W, H, p.depth.data_ptr(), p.gview.normal, p.gview.normal_format, dev8.data_ptr(), 7)
    assert lib.drv_apply(p.ctx, C.byref(bad), C.byref(p.hf.frame), C.byref(p.hf.volume),
                         C.c_void_p(out8.data_ptr())) == abi.ERR_INVALID_ARG
    p.close()
