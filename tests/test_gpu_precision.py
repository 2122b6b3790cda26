"""The precision variant (BF16 VPL flux/normal and cache SH, FP16 opacity
mips, FP32 Kahan-compensated accumulation) against the FP64 oracle.

Bars: allocation stays bit-exact (positions rebuilt from the entries' cell
keys); stored values are within their storage format's rounding of FP64;
final indirect radiance within 1% relative L2 of the FP64 oracle frame.
"""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import Run, _key_set, oracle_frame, rel_l2

pytestmark = pytest.mark.gpu

BF16_REL = 2.0 ** -8   # round-to-nearest relative error bound of BF16
FP16_REL = 2.0 ** -11


@pytest.fixture(scope="module")
def c3(lib, oracle, cuda):
    return Run(pipeline.WORKLOADS["c3_precision"], oracle)


@pytest.fixture(scope="module")
def c3_sh2(lib, oracle, cuda):
    w = pipeline.scaled(pipeline.WORKLOADS["c3_precision"], name="c3_sh2", sh_order=2, n_boxes=24, seed=5)
    return Run(w, oracle, seed=5)


def test_entries_are_bf16_layout(c3):
    assert c3.pipe.buffers().entry_stride == 64


@pytest.mark.parametrize("case", ["c3", "c3_sh2"])
def test_allocation_bit_exact_from_cell_keys(case, request, oracle):
    r = request.getfixturevalue(case)
    st, atlas, pos, count = oracle.allocate_caches(r.hf.config, r.hf.volume, r.hf.frame, r.depth)
    assert r.count == count
    assert _key_set(r.positions) == _key_set(pos)
    assert np.array_equal(r.atlas != 0, atlas != 0)


@pytest.mark.parametrize("case", ["c3", "c3_sh2"])
def test_vpls_within_bf16_rounding(case, request):
    r = request.getfixturevalue(case)
    for (ov, _), gv in zip(r.oracle_vpls(), r.gpu_vpls_f64()):
        assert np.all(np.abs(gv[:, 0:3] - ov[:, 0:3]) <= BF16_REL * np.abs(ov[:, 0:3]) + 1e-12)
        assert np.allclose(gv[:, 4:7], ov[:, 4:7], atol=1e-5)  # positions stay FP32
        assert np.max(np.abs(gv[:, 7:10] - ov[:, 7:10])) < 2e-3 + BF16_REL


@pytest.mark.parametrize("case", ["c3", "c3_sh2"])
def test_mips_are_fp16(case, request, oracle):
    r = request.getfixturevalue(case)
    mips = oracle.build_mips(r.w.voxel_res, r.bits)
    for l, g in enumerate(r.mips, start=1):
        ref = oracle.mip_level(mips, r.w.voxel_res, l)
        assert np.all(np.abs(g - ref) <= 2 * FP16_REL * np.abs(ref) + 1e-7)
        if l <= 3:  # count / 8^l with 8^l <= 512 is exact in FP16
            assert np.array_equal(g.astype(np.float64), ref)


@pytest.mark.parametrize("case", ["c3"])
def test_mip_records_are_fp16_texels(case, request):
    """BF16 precision: every mip level gets corner-packed records of its FP16
    texels."""
    from test_gpu_parity import device_records, expected_records
    r = request.getfixturevalue(case)
    b = r.pipe.buffers()
    assert b.n_record_levels == len(r.mips)
    for l in range(1, b.n_record_levels + 1):
        g, n = device_records(r, l)
        assert np.array_equal(g, expected_records(r.mips[l - 1], n))


@pytest.mark.parametrize("case", ["c3", "c3_sh2"])
def test_light_sh_error_is_storage_rounding(case, request, oracle):
    """With Kahan-compensated FP32 accumulation the SH error against FP64 (on
    the GPU's own BF16 VPLs) is dominated by the final BF16 rounding."""
    r = request.getfixturevalue(case)
    mips = oracle.build_mips(r.w.voxel_res, r.bits)
    sh = oracle.light_caches(r.hf.config, r.hf.volume, r.positions, r.hf.lights, r.gpu_vpls_f64(),
                             [c.astype(np.float64) for c in r.cones], r.bits, mips)
    g = r.gpu_sh()
    nk = 27 if r.w.sh_order == 2 else 12
    assert rel_l2(g[:, :nk], sh[:, :nk]) < 1e-2
    band0 = np.abs(g[:, 0:3] - sh[:, 0:3]) / np.maximum(np.abs(sh[:, 0:3]), 1e-30)
    assert np.percentile(band0, 99) < 2 * BF16_REL


@pytest.mark.parametrize("case", ["c3", "c3_sh2"])
def test_precision_frame_within_one_percent_of_fp64(case, request, oracle):
    r = request.getfixturevalue(case)
    ref = oracle_frame(r, oracle)
    err = rel_l2(r.out, ref)
    assert err < 1e-2, err


@pytest.mark.parametrize("sh_order", [1, 2])
def test_tensor_core_apply_equals_per_pixel_apply(sh_order, lib, cuda):
    """With BF16 entries the apply's tensor-core form (DrvTuning.
    tensor_core_apply: a warp's cells at a time, F split into BF16 hi + lo
    parts, FP32 accumulation) gives the same radiance as the per-pixel FP32
    form to FP32 rounding, on a production-shaped frame with four cascades and
    transitions."""
    from test_gpu_parity import REDUCED
    w = pipeline.scaled(REDUCED, name=f"tc_apply_sh{sh_order}", sh_order=sh_order, precision=abi.PRECISION_BF16)
    p = pipeline.Pipeline(pipeline.host_frame(w, 4))
    p.raycast_inputs()
    p.frame()
    p.sync()
    scalar = p.out.cpu().numpy().copy()
    p.set_tuning(tensor_core_apply=1)
    p.apply()
    p.sync()
    tc = p.out.cpu().numpy()
    assert np.abs(scalar).max() > 0
    assert rel_l2(tc, scalar) < 1e-5
    assert np.max(np.abs(tc - scalar)) <= 1e-4 * np.abs(scalar).max()
    p.close()
