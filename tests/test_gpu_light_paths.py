"""The light stage's two execution forms — one launch (warp per cache chunk)
and cull -> cone -> gather over a compacted pair list — give the same SH up
to FP32 summation order; a pair list too small for the frame makes the gather
trace the caches that did not fit, with the same result to FP32 rounding; the
split form is deterministic run to run; reading the corner-packed mip records
instead of the plain mip arrays leaves the result unchanged bit for bit."""
import ctypes as C

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import REDUCED, rel_l2

pytestmark = pytest.mark.gpu


def _lit(w, seed, **knobs):
    p = pipeline.Pipeline(pipeline.host_frame(w, seed))
    if knobs:
        p.set_tuning(**knobs)
    p.raycast_inputs()
    p.prepare_and_extract()
    p.voxelize()
    p.allocate()
    p.light()
    p.sync()
    n = p.cache_count()
    pos, sh = p.read_entries_decoded(n)
    order = np.lexsort(pos.T[::-1])  # allocation order is atomic order
    return p, pos[order], sh[order]


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["c1_small"], REDUCED], ids=["c1", "c2r"])
def test_single_launch_equals_split(w, cuda, lib):
    p1, pos1, sh1 = _lit(w, 5, light_path=abi.LIGHT_PATH_SINGLE)
    p2, pos2, sh2 = _lit(w, 5, light_path=abi.LIGHT_PATH_SPLIT)
    assert np.array_equal(pos1, pos2)
    assert rel_l2(sh2, sh1) < 1e-5
    p1.close()
    p2.close()


def test_split_is_deterministic(cuda, lib):
    p1, _, sh1 = _lit(REDUCED, 9)
    p2, _, sh2 = _lit(REDUCED, 9)
    assert np.array_equal(sh1, sh2)
    p1.close()
    p2.close()


@pytest.mark.parametrize("cap", [1, 777, 20000])
def test_full_pair_list_is_traced_by_the_gather(cap, cuda, lib):
    # caches that do not fit are traced by the gather, the k-th live block on
    # lane k mod 32 as its listed pair would be, in one unit (a listed cache
    # of more than 512 pairs sums several units' partials); the cone code is
    # inlined into two kernels, whose FMA contraction may differ, so the SH
    # agree to FP32 rounding
    p1, _, sh1 = _lit(REDUCED, 4)
    p2, _, sh2 = _lit(REDUCED, 4, pair_capacity=cap)
    print("overflow cap %d: bitwise %s, rel-L2 %.3e" % (cap, np.array_equal(sh1, sh2), rel_l2(sh2, sh1)))
    assert rel_l2(sh2, sh1) < 1e-6
    p1.close()
    p2.close()


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["ns_1080p_4096"], REDUCED,
                               pipeline.scaled(REDUCED, precision=abi.PRECISION_BF16)], ids=["ns", "c2r", "c2r_bf16"])
@pytest.mark.parametrize("path", [abi.LIGHT_PATH_SPLIT, abi.LIGHT_PATH_SINGLE], ids=["split", "single"])
def test_plain_voxel_reads_give_the_same_sh(w, path, cuda, lib):
    p1, pos1, sh1 = _lit(w, 3, light_path=path)
    p2, pos2, sh2 = _lit(w, 3, light_path=path, plain_voxel_reads=1)
    assert np.array_equal(pos1, pos2)
    assert np.array_equal(sh1, sh2)
    p1.close()
    p2.close()


def test_tuning_knobs_are_validated(cuda, lib):
    p = pipeline.Pipeline(pipeline.host_frame(pipeline.WORKLOADS["c1_small"]))
    t = abi.DrvTuning()
    t.light_path = 3
    assert lib.drv_set_tuning(p.ctx, C.byref(t)) == abi.ERR_INVALID_ARG
    t.light_path = abi.LIGHT_PATH_SPLIT
    t.cone_ctas_per_sm = 2
    assert lib.drv_set_tuning(p.ctx, C.byref(t)) == abi.OK
    back = abi.DrvTuning()
    assert lib.drv_get_tuning(p.ctx, C.byref(back)) == abi.OK
    assert (back.light_path, back.cone_ctas_per_sm) == (abi.LIGHT_PATH_SPLIT, 2)
    p.close()


def test_cta_knobs_keep_results(cuda, lib):
    p1, _, sh1 = _lit(REDUCED, 6)
    p2, _, sh2 = _lit(REDUCED, 6, cone_ctas_per_sm=1, gather_ctas_per_sm=1)
    assert np.array_equal(sh1, sh2)  # the gather's order is fixed per cache
    p1.close()
    p2.close()


def test_kernel_timing_keeps_results_and_reports_each_kernel(cuda, lib):
    p1, _, sh1 = _lit(REDUCED, 8)
    p2, _, sh2 = _lit(REDUCED, 8, time_kernels=1)
    assert np.array_equal(sh1, sh2)
    ms = p2.light_kernel_ms()
    assert set(ms) == set(abi.LIGHT_KERNELS)
    assert ms["cull"] > 0 and ms["cone"] > 0 and ms["gather"] > 0 and ms["classify"] > 0
    assert ms["mlp"] == pytest.approx(0.0, abs=0.05)  # no surrogate: the slot is empty
    p1.close()
    p2.close()


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["c1_small"], REDUCED], ids=["c1", "c2r"])
def test_counting_cone_pass_is_bitwise_the_same(w, cuda, lib):
    """The cone pass's measuring instance (DrvTuning.count_voxel_reads) traces
    the same cones: same SH bit for bit; it reads at least one voxel sample per
    traced cone and no more than its step limit allows (a step reads at most
    two samples: level-0 bytes, mip records, or eight plain texels each)."""
    p1, pos1, sh1 = _lit(w, 9, light_path=abi.LIGHT_PATH_SPLIT)
    p2, pos2, sh2 = _lit(w, 9, light_path=abi.LIGHT_PATH_SPLIT, count_voxel_reads=1)
    assert np.array_equal(pos1, pos2) and np.array_equal(sh1, sh2)
    reads = (C.c_uint32 * 3)()
    assert lib.drv_get_cone_voxel_reads(p2.ctx, reads) == abi.OK
    l0, rec, tex = list(reads)
    pairs = p2.light_pairs()
    assert pairs > 0
    assert l0 + rec + tex // 8 >= pairs
    assert l0 + rec + tex / 8 <= 2 * pairs * w.max_cone_steps
    # without the knob the counts are not available
    assert lib.drv_get_cone_voxel_reads(p1.ctx, reads) == abi.ERR_INVALID_ARG
    p1.close()
    p2.close()


def test_load_bandwidth_probe(cuda, lib):
    """L1- and L2-resident load throughput, in GB/s (the cone pass's roofline
    denominators): positive and within what a GPU can do; bad arguments refused."""
    import torch
    buf = torch.zeros(16 * 1024 * 1024, dtype=torch.int32, device=cuda)  # 64 MB
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = C.c_float()
    for level in (1, 2):
        assert lib.drv_measure_load_bandwidth(level, C.c_void_p(buf.data_ptr()), buf.numel() * 4, 10, s,
                                              C.byref(g)) == abi.OK
        assert 100.0 < g.value < 1e6
    assert lib.drv_measure_load_bandwidth(3, C.c_void_p(buf.data_ptr()), buf.numel() * 4, 10, s,
                                          C.byref(g)) == abi.ERR_INVALID_ARG
    assert lib.drv_measure_load_bandwidth(1, C.c_void_p(buf.data_ptr()), 1024, 10, s,
                                          C.byref(g)) == abi.ERR_INVALID_ARG
    assert int(buf.abs().sum()) == 0  # never written


@pytest.mark.parametrize("w", [pipeline.WORKLOADS["c1_small"], REDUCED], ids=["c1", "c2r"])
def test_tile_knobs_keep_the_result(w, cuda, lib):
    """The cull's caches per pass only change which caches share a pass (each
    cache's pair run stays in block order), and the gather's threads per CTA
    only how many of its warp units share a CTA: the SH are the same bit for
    bit."""
    p0, pos0, sh0 = _lit(w, 13, light_path=abi.LIGHT_PATH_SPLIT)
    for k in (2, 8):
        p1, pos1, sh1 = _lit(w, 13, light_path=abi.LIGHT_PATH_SPLIT, cull_caches_per_pass=k)
        assert np.array_equal(pos1, pos0) and np.array_equal(sh1, sh0)
        p1.close()
    p2, pos2, sh2 = _lit(w, 13, light_path=abi.LIGHT_PATH_SPLIT, gather_threads=256)
    assert np.array_equal(pos2, pos0) and np.array_equal(sh2, sh0)
    p2.close()
    p0.close()


W_MULTI_UNIT = pipeline.scaled(pipeline.WORKLOADS["c1_small"], name="c1_4096_vpls", rsm_resolution=64)


def test_multi_unit_caches_are_deterministic_and_match_single_launch(cuda, lib):
    """With 4096 VPLs in one 2 m cascade the caches average more than one
    gather unit (512 pairs) of contributing blocks: each unit's partial sums
    are combined in unit order by whichever unit finishes last, so runs agree
    bit for bit, whatever the CTA size or grid, and equal the single-launch
    form to FP32 summation order."""
    p1, pos1, sh1 = _lit(W_MULTI_UNIT, 2, light_path=abi.LIGHT_PATH_SPLIT)
    assert p1.light_pairs() > 512 * p1.cache_count()  # so some cache has several units
    p2, pos2, sh2 = _lit(W_MULTI_UNIT, 2, light_path=abi.LIGHT_PATH_SPLIT, gather_threads=256,
                         gather_ctas_per_sm=1)
    assert np.array_equal(pos1, pos2) and np.array_equal(sh1, sh2)
    p3, pos3, sh3 = _lit(W_MULTI_UNIT, 2, light_path=abi.LIGHT_PATH_SINGLE)
    assert np.array_equal(pos1, pos3)
    assert rel_l2(sh3, sh1) < 1e-5
    # twice on one context: each stage starts from zeroed tickets
    p1.light()
    p1.sync()
    pos_b, sh_b = p1.read_entries_decoded(p1.cache_count())
    assert rel_l2(sh_b[np.lexsort(pos_b.T[::-1])], 2 * sh1) < 1e-6
    for p in (p1, p2, p3):
        p.close()


@pytest.mark.parametrize("prec", [abi.PRECISION_FP32, abi.PRECISION_BF16], ids=["f32", "bf16"])
def test_per_light_dispatch_equals_one_pass(prec, cuda, lib):
    """The reference's dispatch loop (DrvTuning.per_light_dispatch: one split
    stage per light, each adding into the entries) against one pass over every
    light's pairs: the same SH to FP32 rounding; BF16 entries are rounded once
    per light instead of once, so they agree to BF16 rounding."""
    w = pipeline.scaled(REDUCED, precision=prec)
    assert w.n_lights > 1
    p1, pos1, sh1 = _lit(w, 7)
    p2, pos2, sh2 = _lit(w, 7, per_light_dispatch=1)
    assert np.array_equal(pos1, pos2)
    err = rel_l2(sh2, sh1)
    print("per-light dispatch: rel-L2 %.3e" % err)
    assert err < (1e-5 if prec == abi.PRECISION_FP32 else 1e-2)
    assert np.abs(sh1).max() > 0
    p1.close()
    p2.close()


def test_gather_copy_timeout_is_reported_and_context_recovers(cuda, lib):
    """The gather's wait for its staged VPLs is bounded: with the test hook
    the copies are withheld, every CTA's wait runs out (about 10 ms), the
    stage latches DRV_DEVERR_TIMEOUT and drv_sync reports DRV_ERR_TIMEOUT.
    The same context, allocated and lit again without the hook, gives the
    SH of a context that never timed out, bit for bit: no cache is left
    with a count of finished units from the stage that stopped."""
    import dynamicradiancevolume_gb300 as drv
    ref_p, ref_pos, ref_sh = _lit(W_MULTI_UNIT, 2, light_path=abi.LIGHT_PATH_SPLIT)
    p = pipeline.Pipeline(pipeline.host_frame(W_MULTI_UNIT, 2))
    p.set_tuning(light_path=abi.LIGHT_PATH_SPLIT)
    p.raycast_inputs()
    p.prepare_and_extract()
    p.voxelize()
    p.allocate()
    p.set_tuning(gather_wait_test=1)
    p.light()
    with pytest.raises(drv.DrvError) as e:
        p.sync()
    assert e.value.status == abi.ERR_TIMEOUT
    p.set_tuning(gather_wait_test=0)
    p.allocate()
    p.light()
    p.sync()
    pos, sh = p.read_entries_decoded(p.cache_count())
    order = np.lexsort(pos.T[::-1])
    assert np.array_equal(pos[order], ref_pos)
    assert np.array_equal(sh[order], ref_sh)
    p.close()
    ref_p.close()
