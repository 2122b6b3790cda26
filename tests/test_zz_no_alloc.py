"""The allocation-free light stage (drv_light_caches_static_scratch) against
the regular one (drv_light_caches).

The allocation-free variant exists for callers that are not allowed to
allocate device memory (engines that run inside a fixed, pre-reserved GPU
arena, their plug-ins, graph-recorded code): it takes every buffer from the
caller and keeps its scratch in a fixed array inside the library. Here both
entry points light the same freshly allocated caches, through the C ABI, and
the static-scratch one is called twice in a row, since its array keeps the
previous call's contents.
"""
import ctypes as C

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline

pytestmark = pytest.mark.gpu


def _device_floats(torch, ptr, numel, device):
    """A writable float32 view of `numel` floats at a device address."""

    class _View:
        __cuda_array_interface__ = {"shape": (numel,), "typestr": "<f4", "data": (int(ptr), False), "version": 3,
                                    "strides": None}

    return torch.as_tensor(_View(), device=device)


def _rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("sh_order", [1, 2])
def test_static_scratch_light_matches_regular_light(sh_order, lib, cuda):
    import torch
    # 1024 VPLs in one-VPL shadow blocks: two chunks per cache, so the
    # chunk partials and tickets in the static array are exercised.
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], sh_order=sh_order, max_caches=abi.STATIC_SCRATCH_MAX_CACHES)
    hf = pipeline.host_frame(w)
    p = pipeline.Pipeline(hf)
    p.raycast_inputs()
    p.prepare_and_extract()
    p.voxelize()
    p.allocate()
    p.sync()
    count = p.cache_count()
    assert 0 < count <= abi.STATIC_SCRATCH_MAX_CACHES
    b = p.buffers()
    entries = _device_floats(torch, b.cache_entries, count * (b.entry_stride // 4), p.device)
    fresh = entries.clone()  # positions + zeroed SH, as the allocation left them
    p.light()
    p.sync()
    expected = entries.clone().cpu().numpy()
    assert np.abs(expected).sum() > 0

    vpls = (C.c_void_p * 1)(b.vpls[0])
    cones = (C.c_void_p * 1)(b.cones[0])
    n_vpls = (C.c_int32 * 1)(b.n_vpls[0])
    intervals = (C.c_int32 * 1)(hf.lights[0].indirect_shadow_sample_interval)
    for _ in range(2):
        entries.copy_(fresh)
        torch.cuda.synchronize()
        st = lib.drv_light_caches_static_scratch(C.byref(hf.config), C.byref(hf.volume), vpls, cones, n_vpls,
                                                 intervals, 1, b.voxel_corners, b.voxel_mips[1], b.counter,
                                                 b.cache_entries, C.c_void_p(p.stream.cuda_stream))
        assert st == abi.OK
        p.stream.synchronize()
        got = entries.clone().cpu().numpy()
        assert _rel_l2(got, expected) < 1e-5

    # Beyond the array's fixed capacity the call is refused, and nothing runs.
    big = abi.DrvConfig.from_buffer_copy(hf.config)
    big.max_caches = abi.STATIC_SCRATCH_MAX_CACHES + 1
    st = lib.drv_light_caches_static_scratch(C.byref(big), C.byref(hf.volume), vpls, cones, n_vpls, intervals, 1,
                                             b.voxel_corners, b.voxel_mips[1], b.counter, b.cache_entries,
                                             C.c_void_p(p.stream.cuda_stream))
    assert st == abi.ERR_CAPACITY
    p.close()


def test_static_scratch_refuses_bf16_and_launches_nothing(lib, cuda):
    """The entry point's inputs are FP32 (DrvVPL, FP32 mips, std430 entries):
    a BF16 config, whose entries are 64 B even with SH2, is refused before
    anything runs, so the caller's entries stay as they were."""
    import torch
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], sh_order=2, max_caches=abi.STATIC_SCRATCH_MAX_CACHES,
                        precision=abi.PRECISION_BF16)
    hf = pipeline.host_frame(w)
    p = pipeline.Pipeline(hf)
    p.raycast_inputs()
    p.prepare_and_extract()
    p.voxelize()
    p.allocate()
    p.sync()
    count = p.cache_count()
    b = p.buffers()
    assert b.entry_stride == 64
    entries = _device_floats(torch, b.cache_entries, count * (b.entry_stride // 4), p.device)
    before = entries.clone().cpu().numpy()
    vpls = (C.c_void_p * 1)(b.vpls[0])
    cones = (C.c_void_p * 1)(b.cones[0])
    n_vpls = (C.c_int32 * 1)(b.n_vpls[0])
    intervals = (C.c_int32 * 1)(hf.lights[0].indirect_shadow_sample_interval)
    st = lib.drv_light_caches_static_scratch(C.byref(hf.config), C.byref(hf.volume), vpls, cones, n_vpls, intervals,
                                             1, b.voxel_corners, b.voxel_mips[1], b.counter, b.cache_entries,
                                             C.c_void_p(p.stream.cuda_stream))
    assert st == abi.ERR_INVALID_ARG
    p.stream.synchronize()
    assert np.array_equal(entries.clone().cpu().numpy(), before)
    p.close()
