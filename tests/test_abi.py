"""The C-ABI library loads and exports every symbol include/drv.h declares;
host-side parameter setup agrees with the oracle's restatement of the
reference's UBO fills. No GPU work here."""
import ctypes as C

import numpy as np
import pytest

import dynamicradiancevolume_gb300 as drv
from dynamicradiancevolume_gb300 import abi, pipeline


def test_library_exports_every_declared_symbol(lib):
    declared = abi.header_functions(drv.HEADER)
    assert len(declared) > 20
    missing = [name for name in declared if not hasattr(lib, name)]
    assert missing == []
    # and the Python prototypes cover the declared surface
    assert set(abi.PROTOTYPES) <= set(declared)


def test_struct_sizes_match_c(lib):
    n = lib.drv_struct_sizes(None, 0)
    assert n == len(abi.STRUCT_ORDER)
    sizes = (C.c_uint32 * n)()
    lib.drv_struct_sizes(sizes, n)
    assert [C.sizeof(s) for s in abi.STRUCT_ORDER] == list(sizes)
    assert C.sizeof(abi.DrvCascade) == 64  # std140 CAVCascade
    assert C.sizeof(abi.DrvVPL) == 48


def test_abi_version(lib):
    assert lib.drv_abi_version() == 10


@pytest.mark.parametrize("name", list(pipeline.WORKLOADS))
def test_host_params_match_oracle(lib, oracle, name):
    w = pipeline.WORKLOADS[name]
    hf = pipeline.host_frame(w)
    vol = oracle.compute_volume_info(hf.config, list(hf.scene.aabb_min), list(hf.scene.aabb_max),
                                     list(hf.camera.position))
    assert bytes(vol) == bytes(hf.volume)
    assert bytes(oracle.prepare_camera(hf.camera)) == bytes(hf.frame)
    for l in range(w.n_lights):
        assert bytes(oracle.prepare_light(hf.light_descs[l])) == bytes(hf.lights[l])


def test_volume_info_reference_semantics(lib):
    cfg = pipeline.make_config(pipeline.WORKLOADS["c2_production"])
    vol = abi.DrvVolumeInfo()
    amin, amax = (C.c_float * 3)(0, 0, 0), (C.c_float * 3)(1, 2, 0.5)
    cam = (C.c_float * 3)(0.3, 0.4, 0.2)
    assert lib.drv_compute_volume_info(C.byref(cfg), amin, amax, cam, C.byref(vol)) == abi.OK
    # cubified around the largest extent (renderer.cpp:351-356)
    ext = [vol.volume_world_max[i] - vol.volume_world_min[i] for i in range(3)]
    assert max(ext) - min(ext) < 1e-6
    for c in range(cfg.n_cascades):
        k = vol.cascades[c]
        size = cfg.cascade_world_size[c]
        assert k.world_voxel_size == pytest.approx(size / cfg.cav_res)
        for i in range(3):
            # snapped to the cell, decision box shrunk by 1.5 cells (renderer.cpp:373-379)
            assert (k.min[i] + size / 2) / k.world_voxel_size == pytest.approx(round(cam[i] / k.world_voxel_size))
            assert k.decision_max[i] - k.decision_min[i] == pytest.approx(size - 3 * k.world_voxel_size, rel=1e-5)


def test_light_params_reference_semantics(lib):
    d = abi.DrvLightDesc()
    assert lib.drv_generate_light(3, None, 1000, 4, 2, C.byref(d)) == abi.OK
    L = abi.DrvSpotLight()
    assert lib.drv_prepare_light(C.byref(d), C.byref(L)) == abi.OK
    assert L.rsm_render_resolution == 1024  # next power of two (renderer.cpp:694)
    assert L.rsm_read_resolution == 64      # 1024 / 2^4
    assert L.indirect_shadow_sample_interval == 16
    assert L.indirect_shadow_sampling_offset == pytest.approx(0.5 + 2 ** 0.5 * 4 / 2)
    vaf = (np.sin(d.half_angle) * d.near_plane * 2) ** 2 / (d.near_plane ** 2 * 64 ** 2)
    assert L.val_area_factor == pytest.approx(vaf, rel=1e-6)
    assert L.indirect_shadow_super_val_width == pytest.approx(np.sqrt(vaf) * 4, rel=1e-6)
    # the light's VP maps its own position to w = 0 and its direction to the RSM centre
    M = np.array(L.view_projection).reshape(4, 4)
    p = np.array(list(L.position) + [1.0])
    assert abs((M @ p)[3]) < 1e-5
    q = np.array([L.position[i] + L.direction[i] for i in range(3)] + [1.0])
    c = M @ q
    assert abs(c[0] / c[3]) < 1e-5 and abs(c[1] / c[3]) < 1e-5


def test_scene_generation_is_deterministic(lib):
    w = pipeline.WORKLOADS["c2_production"]
    a, b = pipeline.host_frame(w, seed=5), pipeline.host_frame(w, seed=5)
    assert bytes(a.boxes) == bytes(b.boxes) and bytes(a.lights) == bytes(b.lights)
    assert bytes(a.camera) == bytes(b.camera)
    c = pipeline.host_frame(w, seed=6)
    assert bytes(a.boxes) != bytes(c.boxes)
    for i in range(1, w.n_boxes + 1):
        bx = a.boxes[i]
        for k in range(3):
            assert 0.0 <= bx.min[k] < bx.max[k] <= 1.0
            assert 0.05 - 1e-6 <= bx.max[k] - bx.min[k] <= 0.3 + 1e-6


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    assert lib.drv_create(None, None) == abi.ERR_INVALID_ARG
    cfg = abi.DrvConfig()
    lib.drv_default_config(C.byref(cfg))
    ctx = C.c_void_p()
    bad = abi.DrvConfig.from_buffer_copy(cfg)
    bad.sh_order = 3
    assert lib.drv_create(C.byref(bad), C.byref(ctx)) == abi.ERR_INVALID_ARG
    bad = abi.DrvConfig.from_buffer_copy(cfg)
    bad.voxel_res = 100
    assert lib.drv_create(C.byref(bad), C.byref(ctx)) == abi.ERR_INVALID_ARG
    bad = abi.DrvConfig.from_buffer_copy(cfg)
    bad.n_cascades = 5
    assert lib.drv_create(C.byref(bad), C.byref(ctx)) == abi.ERR_INVALID_ARG
    d = abi.DrvLightDesc()
    L = abi.DrvSpotLight()
    assert lib.drv_prepare_light(C.byref(d), C.byref(L)) == abi.ERR_INVALID_ARG
    assert lib.drv_sync(None) == abi.ERR_INVALID_ARG


@pytest.mark.parametrize("channels", [3, 4])
def test_pfm_round_trip_and_header(lib, tmp_path, channels):
    # rendering/hdrimage.cpp: "PF\n<w> <h>\n-1.000000\n" then RGB floats, row 0 first
    import ctypes as C
    w, h = 5, 3
    img = np.random.default_rng(channels).random((h, w, channels)).astype(np.float32)
    path = str(tmp_path / "x.pfm").encode()
    assert lib.drv_write_pfm(path, img.ctypes.data_as(C.POINTER(C.c_float)), w, h, channels) == 0
    raw = open(path, "rb").read()
    header = b"PF\n5 3\n-1.000000\n"
    assert raw.startswith(header) and len(raw) == len(header) + w * h * 12
    ww, hh = C.c_int32(), C.c_int32()
    assert lib.drv_read_pfm(path, None, 0, C.byref(ww), C.byref(hh)) == 0 and (ww.value, hh.value) == (w, h)
    back = np.zeros((h, w, 3), np.float32)
    assert lib.drv_read_pfm(path, back.ctypes.data_as(C.POINTER(C.c_float)), 2, C.byref(ww), C.byref(hh)) == 2
    assert lib.drv_read_pfm(path, back.ctypes.data_as(C.POINTER(C.c_float)), w * h, C.byref(ww), C.byref(hh)) == 0
    assert np.array_equal(back, img[..., :3])


def test_static_scratch_refuses_bf16_before_any_device_call(lib):
    """No GPU needed: the precision check comes before any CUDA call, so the
    dummy (never dereferenced) pointers below are not touched."""
    hf = pipeline.host_frame(pipeline.scaled(pipeline.WORKLOADS["c1_small"], sh_order=2, max_caches=1024,
                                             precision=abi.PRECISION_BF16))
    dummy = C.c_void_p(16)
    ptrs = (C.c_void_p * 1)(16)
    n_vpls = (C.c_int32 * 1)(1024)
    intervals = (C.c_int32 * 1)(1)
    st = lib.drv_light_caches_static_scratch(C.byref(hf.config), C.byref(hf.volume), ptrs, ptrs, n_vpls, intervals,
                                             1, dummy, dummy, dummy, dummy, None)
    assert st == abi.ERR_INVALID_ARG


@pytest.mark.parametrize("name", list(pipeline.WORKLOADS))
def test_oracle_host_frame_equals_product_host_frame(lib, oracle, name):
    """The benchmark's CPU arm builds its frame with the oracle alone; it must
    be the frame the GPU arm renders: same config, boxes, camera, lights and
    volume, byte for byte."""
    w = pipeline.WORKLOADS[name]
    a, b = pipeline.host_frame(w), oracle.host_frame(w)
    assert bytes(a.config) == bytes(b.config)
    assert bytes(a.boxes) == bytes(b.boxes)
    assert bytes(a.camera) == bytes(b.camera)
    assert bytes(a.frame) == bytes(b.frame)
    assert bytes(a.lights) == bytes(b.lights)
    assert all(bytes(x) == bytes(y) for x, y in zip(a.light_descs, b.light_descs))
    assert bytes(a.volume) == bytes(b.volume)


def test_missing_library_is_not_supported_not_a_fallback(tmp_path):
    """Without the built library every entry point raises DRV_ERR_NOT_SUPPORTED
    (there is no CPU fallback)."""
    import subprocess
    import sys
    code = ("import dynamicradiancevolume_gb300 as d, pathlib\n"
            "d.LIB_PATH = pathlib.Path(r'%s') / 'libdrv_gb300.so'\n"
            "try:\n    d.load()\nexcept d.DrvError as e:\n    print('status', e.status)\n" % tmp_path)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=str(drv.HEADER.parents[1]))
    assert f"status {abi.ERR_NOT_SUPPORTED}" in r.stdout, r.stdout + r.stderr
