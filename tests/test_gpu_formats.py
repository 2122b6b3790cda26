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


srgb_encode = pipeline.srgb_encode


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


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["c1_small"], REDUCED], ids=["c1", "c2r"])
def test_f16_rsm_equals_its_f32_widening(w, lib, cuda):
    """RGB16F flux and RG16F (d, d^2), the reference's RSM targets: the VPLs
    and shadow-cone sources equal those of an F32 RSM holding the same
    values, bit for bit (the chain below the caller's level is F32)."""
    torch = pytest.importorskip("torch")
    p = pipeline.Pipeline(pipeline.host_frame(w, 6))
    p.raycast_inputs()
    p.sync()
    n = w.n_lights
    halves = [(p.rsm_flux[l].half().contiguous(), p.rsm_dls[l].half().contiguous()) for l in range(n)]
    for l in range(n):  # the F32 RSM now holds the F16-rounded values
        p.rsm_flux[l].copy_(halves[l][0].float())
        p.rsm_dls[l].copy_(halves[l][1].float())
    torch.cuda.synchronize()
    p.prepare_and_extract()
    p.sync()
    nc = [p.buffers().n_vpls[l] // p.hf.lights[l].indirect_shadow_sample_interval for l in range(n)]
    ref = [(p.read_vpls(l).cpu().clone(), p.read_cones(l, nc[l]).cpu().clone()) for l in range(n)]
    R = w.rsm_resolution
    views = (abi.DrvRSMView * n)()
    for l in range(n):
        views[l] = abi.DrvRSMView(R, halves[l][0].data_ptr(), p.rsm_normal[l].data_ptr(), halves[l][1].data_ptr(),
                                  abi.RSM_F16)
        assert lib.drv_prepare_rsm(p.ctx, l, C.byref(p.hf.lights[l]), C.byref(views[l])) == abi.OK
        assert lib.drv_extract_vpls(p.ctx, l, C.byref(p.hf.lights[l])) == abi.OK
    p.sync()
    for l in range(n):
        assert torch.equal(p.read_vpls(l).cpu(), ref[l][0])
        assert torch.equal(p.read_cones(l, nc[l]).cpu(), ref[l][1])
    bad = abi.DrvRSMView(R, halves[0][0].data_ptr(), p.rsm_normal[0].data_ptr(), halves[0][1].data_ptr(), 5)
    assert lib.drv_prepare_rsm(p.ctx, 0, C.byref(p.hf.lights[0]), C.byref(bad)) == abi.ERR_INVALID_ARG
    p.close()


@pytest.mark.parametrize("fmt,blend", [(abi.OUTPUT_RGB32F, abi.OUTPUT_ADD), (abi.OUTPUT_RGBA16F, abi.OUTPUT_WRITE),
                                       (abi.OUTPUT_RGBA16F, abi.OUTPUT_ADD)])
def test_output_targets(fmt, blend, lib, cuda):
    """RGBA16F target and additive blending (the reference's HDR back buffer
    with glBlendFunc(ONE, ONE)) against the RGB F32 written result: the same
    FP32 radiance, added in FP32 and rounded once to FP16."""
    torch = pytest.importorskip("torch")
    w = pipeline.WORKLOADS["c1_small"]
    hf = pipeline.host_frame(w, 8)
    p = pipeline.Pipeline(hf)  # RGB32F, written
    p.raycast_inputs()
    p.frame()
    p.sync()
    ref = p.out.clone()
    p.close()
    hf2 = pipeline.host_frame(w, 8)
    hf2.config.output_format, hf2.config.output_blend = fmt, blend
    q = pipeline.Pipeline(hf2)
    q.raycast_inputs()
    H, W = w.height, w.width
    g = torch.Generator(device="cpu").manual_seed(3)
    if fmt == abi.OUTPUT_RGBA16F:
        base = (torch.rand((H, W, 4), generator=g) * 4).half().to(q.device)
    else:
        base = (torch.rand((H, W, 3), generator=g) * 4).to(q.device)
    out = base.clone() if blend == abi.OUTPUT_ADD else torch.full_like(base, 7.0)
    torch.cuda.synchronize()
    q.frame(out)
    q.sync()
    r = ref.cpu().numpy()
    o = out.cpu().numpy()
    b = base.cpu().numpy()
    if fmt == abi.OUTPUT_RGB32F:
        assert np.array_equal(o, b + r)
    else:
        exp_rgb = ((b[..., :3].astype(np.float32) + r) if blend == abi.OUTPUT_ADD else r).astype(np.float16)
        assert np.array_equal(o[..., :3], exp_rgb)
        exp_a = b[..., 3] if blend == abi.OUTPUT_ADD else np.ones((H, W), np.float16)
        assert np.array_equal(o[..., 3], exp_a)
    q.close()
