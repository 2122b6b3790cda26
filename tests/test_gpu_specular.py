"""Indirect specular (INDIRECT_SPECULAR): the per-cache envmaps the light
stage fills, their mips and hole fill, and the apply's specular term, each
against the FP64 oracle on the GPU's own inputs, and the whole frame against
the oracle's own chain; the single-launch stage and a full pair list give the
same envmaps; the envmaps are deterministic; bad configurations and missing
inputs are rejected."""
import ctypes as C

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import REDUCED, Run, rel_l2

pytestmark = pytest.mark.gpu

# The reference's default envmap size (16) on the small case; the reduced
# production case (SH2, two lights, shadow blocks of 4 VPLs, cascade
# transitions) with 8x8 envmaps and the hole fill from level 2.
SPEC_C1 = pipeline.scaled(pipeline.WORKLOADS["c1_small"], name="c1_specular", specular_envmap_size=16)
SPEC_C2R = pipeline.scaled(REDUCED, name="c2_reduced_specular", specular_envmap_size=8, specular_fill_level=2)


@pytest.fixture(scope="module")
def s1(lib, oracle, cuda):
    return Run(SPEC_C1, oracle)


@pytest.fixture(scope="module")
def s2(lib, oracle, cuda):
    return Run(SPEC_C2R, oracle, seed=3)


def _level0(r, oracle, env):
    S = r.w.specular_envmap_size
    return oracle.decode_r11g11b10(env[:, :S * S]).reshape(-1, S, S, 3)


@pytest.mark.parametrize("case", ["s1", "s2"])
def test_light_stage_sh_and_envmaps_match_fp64(case, request, oracle):
    """SH (with the specular path's flux threshold) and level-0 envmaps from
    the GPU's VPLs, cones and voxels vs FP64."""
    r = request.getfixturevalue(case)
    mips = oracle.build_mips(r.w.voxel_res, r.bits)
    cones = [c.astype(np.float64) for c in r.cones]
    sh, env = oracle.light_caches_specular(r.hf.config, r.hf.volume, r.positions.copy(), r.hf.frame.camera_position[:],
                                           r.hf.lights, r.gpu_vpls_f64(), cones, r.bits, mips)
    nk = 27 if r.w.sh_order == 2 else 12
    assert rel_l2(r.gpu_sh()[:, :nk], sh[:, :nk]) < 1e-3
    g0 = _level0(r, oracle, r.env_lit)
    # R11F_G11F_B10F keeps 6 (blue 5) mantissa bits: up to 2^-7 (2^-6) relative per texel
    err = rel_l2(g0, env)
    print("%s: %d caches, envmap rel-L2 %.3e, energy %.6g vs %.6g" % (case, env.shape[0], err, g0.sum(), env.sum()))
    assert err < 1e-2
    # the energy per cache does not depend on which texel a VPL lands in
    assert rel_l2(g0.sum(axis=(1, 2)), env.sum(axis=(1, 2))) < 5e-3
    # rounded once from the exact sum: the oracle's rounding of the FP64 sum
    # gives the same words except across a rounding or texel boundary
    same = np.mean(oracle.encode_r11g11b10(env).reshape(env.shape[0], -1) == r.env_lit[:, :env[0, ..., 0].size])
    assert same > 0.95, same
    assert env.sum() > 0


@pytest.mark.parametrize("case", ["s1", "s2"])
def test_envmap_mips_and_hole_fill_match_oracle(case, request, oracle):
    """drv_prepare_specular_envmaps on the GPU's level 0 = the oracle's
    mips (the 2x2 means, exact in FP32) and hole fill."""
    r = request.getfixturevalue(case)
    S, fill = r.w.specular_envmap_size, r.w.specular_fill_level
    ref = oracle.specular_prepare(S, fill, r.env_lit)
    if fill == 0:
        assert np.array_equal(r.env[:, S * S:], ref[:, S * S:])
        assert np.array_equal(r.env[:, :S * S], r.env_lit[:, :S * S])  # level 0 untouched
    else:
        same = np.mean(r.env == ref)
        assert same > 0.999, same
        assert rel_l2(oracle.decode_r11g11b10(r.env), oracle.decode_r11g11b10(ref)) < 1e-4
        # the fill changed level 0 (some holes were filled)
        assert not np.array_equal(r.env[:, :S * S], r.env_lit[:, :S * S])


@pytest.mark.parametrize("case", ["s1", "s2"])
def test_specular_apply_matches_fp64(case, request, oracle):
    """The apply with the specular term on the GPU's atlas, SH and envmaps vs FP64."""
    r = request.getfixturevalue(case)
    ref = oracle.apply_specular(r.hf.config, r.hf.volume, r.hf.frame, r.depth, r.n16, abi.NORMAL_RG16I, r.albedo,
                                r.rough_metal, r.atlas, r.gpu_sh(), r.env)
    err = rel_l2(r.out, ref)
    print("%s: apply rel-L2 %.3e" % (case, err))
    assert err < 1e-4


@pytest.mark.parametrize("case", ["s1", "s2"])
def test_specular_frame_within_one_percent_of_fp64(case, request, oracle):
    """The oracle's own chain (VPLs, voxels, allocation, FP64 SH and envmaps
    rounded once, mips and fill, specular apply) on the same G-buffer and RSM."""
    r = request.getfixturevalue(case)
    cfg = r.hf.config
    vp = r.oracle_vpls()
    bits = oracle.voxelize(r.hf.boxes, r.hf.scene.n_boxes, r.hf.volume, r.w.voxel_res)
    mips = oracle.build_mips(r.w.voxel_res, bits)
    st, atlas, pos, count = oracle.allocate_caches(cfg, r.hf.volume, r.hf.frame, r.depth)
    sh, env = oracle.light_caches_specular(cfg, r.hf.volume, pos, r.hf.frame.camera_position[:], r.hf.lights,
                                           [v for v, _ in vp], [c for _, c in vp], bits, mips)
    S, fill = r.w.specular_envmap_size, r.w.specular_fill_level
    words = oracle.specular_levels(S)[-1]
    e = np.zeros((env.shape[0], words), np.uint32)
    e[:, :S * S] = oracle.encode_r11g11b10(env).reshape(env.shape[0], S * S)
    e = oracle.specular_prepare(S, fill, e)
    ref = oracle.apply_specular(cfg, r.hf.volume, r.hf.frame, r.depth, r.n16, abi.NORMAL_RG16I, r.albedo,
                                r.rough_metal, atlas, sh, e)
    err = rel_l2(r.out, ref)
    diffuse = oracle.apply(cfg, r.hf.volume, r.hf.frame, r.depth, r.n16, abi.NORMAL_RG16I, r.albedo, atlas, sh)
    print("%s: frame rel-L2 %.3e (specular changes the frame by %.3f)" % (case, err, rel_l2(ref, diffuse)))
    assert err < 1e-2
    assert rel_l2(ref, diffuse) > 0.02  # the specular term is not negligible


def _sorted_env(r):
    order = np.lexsort(r.positions.T[::-1])  # cache order is the allocation's atomic order
    return r.positions[order], r.env[order]


def test_stage_forms_give_the_same_envmaps(lib, oracle, cuda):
    """Split stage (pair list), single launch (cones traced by the specular
    pass) and a full pair list (the overflowing caches' cones traced there):
    the same envmaps up to FP32 rounding of the cones."""
    base = Run(SPEC_C1, oracle, seed=4)
    p0, e0 = _sorted_env(base)
    for knobs in (dict(light_path=abi.LIGHT_PATH_SINGLE), dict(pair_capacity=777)):
        r = Run(SPEC_C1, oracle, seed=4, tuning=knobs)
        p1, e1 = _sorted_env(r)
        assert np.array_equal(p0, p1)
        same = np.mean(e0 == e1)
        print(knobs, "words equal %.6f" % same)
        assert same > 0.999
        assert rel_l2(oracle.decode_r11g11b10(e1), oracle.decode_r11g11b10(e0)) < 1e-4


def test_envmaps_are_deterministic(lib, oracle, cuda):
    a = Run(SPEC_C2R, oracle, seed=6)
    b = Run(SPEC_C2R, oracle, seed=6)
    pa, ea = _sorted_env(a)
    pb, eb = _sorted_env(b)
    assert np.array_equal(pa, pb)
    assert np.array_equal(ea, eb)
    assert np.array_equal(a.out, b.out)


def test_specular_config_and_inputs_are_checked(lib, cuda):
    for size, fill in [(3, 0), (2, 0), (128, 0), (16, 5), (0, 1), (8, -1)]:
        cfg = pipeline.make_config(pipeline.scaled(SPEC_C1, specular_envmap_size=size, specular_fill_level=fill))
        ctx = C.c_void_p()
        assert lib.drv_create(C.byref(cfg), C.byref(ctx)) == abi.ERR_INVALID_ARG, (size, fill)
    # specular off: no envmaps, and the prepare entry point refuses
    p = pipeline.Pipeline(pipeline.host_frame(pipeline.WORKLOADS["c1_small"]))
    assert p.buffers().specular_envmap[0] is None and p.buffers().n_specular_levels == 0
    assert lib.drv_prepare_specular_envmaps(p.ctx) == abi.ERR_INVALID_ARG
    p.close()
    # specular on: prepare before any light stage, and an apply without the
    # roughness / metallic target, are refused
    q = pipeline.Pipeline(pipeline.host_frame(SPEC_C1))
    b = q.buffers()
    assert b.n_specular_levels == 5 and b.specular_atlas_size >= 16
    assert lib.drv_prepare_specular_envmaps(q.ctx) == abi.ERR_INVALID_ARG
    q.raycast_inputs()
    q.prepare_and_extract()
    q.voxelize()
    q.allocate()
    q.light()
    q.prepare_specular()
    g = abi.DrvGBufferView.from_buffer_copy(q.gview)
    g.rough_metal = None
    assert lib.drv_apply(q.ctx, C.byref(g), C.byref(q.hf.frame), C.byref(q.hf.volume),
                         C.c_void_p(q.out.data_ptr())) == abi.ERR_INVALID_ARG
    g.rough_metal, g.rough_metal_format = q.rough_metal.data_ptr(), 7
    assert lib.drv_apply(q.ctx, C.byref(g), C.byref(q.hf.frame), C.byref(q.hf.volume),
                         C.c_void_p(q.out.data_ptr())) == abi.ERR_INVALID_ARG
    q.apply()
    q.sync()
    q.close()


def test_rough_metal_f32_equals_rg8(lib, oracle, cuda):
    """The roughness / metallic target as RG F32 holding byte / 255 gives the
    frame the reference's RG8 target gives, bit for bit."""
    torch = pytest.importorskip("torch")
    r = Run(SPEC_C1, oracle, seed=2)
    q = r.pipe
    rm32 = torch.from_numpy(r.rough_metal.copy()).to(q.device)
    torch.cuda.synchronize()
    g = abi.DrvGBufferView.from_buffer_copy(q.gview)
    g.rough_metal, g.rough_metal_format = rm32.data_ptr(), abi.ROUGH_METAL_F32
    out = torch.zeros_like(q.out)
    assert lib.drv_apply(q.ctx, C.byref(g), C.byref(q.hf.frame), C.byref(q.hf.volume),
                         C.c_void_p(out.data_ptr())) == abi.OK
    q.sync()
    assert np.array_equal(out.cpu().numpy(), r.out)


def test_bf16_specular_frame_within_one_percent_of_fp64(lib, oracle, cuda):
    """BF16 storage with the specular path: the frame against the FP64 chain."""
    r = Run(pipeline.scaled(SPEC_C1, precision=abi.PRECISION_BF16), oracle, seed=5)
    cfg = r.hf.config
    vp = r.oracle_vpls()
    bits = oracle.voxelize(r.hf.boxes, r.hf.scene.n_boxes, r.hf.volume, r.w.voxel_res)
    mips = oracle.build_mips(r.w.voxel_res, bits)
    c32 = abi.DrvConfig.from_buffer_copy(cfg)
    c32.precision = abi.PRECISION_FP32
    st, atlas, pos, count = oracle.allocate_caches(c32, r.hf.volume, r.hf.frame, r.depth)
    sh, env = oracle.light_caches_specular(c32, r.hf.volume, pos, r.hf.frame.camera_position[:], r.hf.lights,
                                           [v for v, _ in vp], [c for _, c in vp], bits, mips)
    S = r.w.specular_envmap_size
    e = np.zeros((env.shape[0], oracle.specular_levels(S)[-1]), np.uint32)
    e[:, :S * S] = oracle.encode_r11g11b10(env).reshape(env.shape[0], S * S)
    e = oracle.specular_prepare(S, r.w.specular_fill_level, e)
    ref = oracle.apply_specular(c32, r.hf.volume, r.hf.frame, r.depth, r.n16, abi.NORMAL_RG16I, r.albedo,
                                r.rough_metal, atlas, sh, e)
    err = rel_l2(r.out, ref)
    print("bf16 specular frame rel-L2 %.3e" % err)
    assert err < 1e-2
