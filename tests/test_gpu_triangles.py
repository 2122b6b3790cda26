"""Triangle-mesh voxelization (drv_voxelize_triangles): the GPU bitmask
equals the oracle's bit for bit on random triangle soups (every orientation,
sizes from a sub-voxel sliver to the whole volume, vertices outside the
volume, degenerate triangles) and on indexed meshes; a box scene given as
triangles voxelizes exactly as the box voxelizer."""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import pipeline
from test_oracle_known_answers import _box_triangles

pytestmark = pytest.mark.gpu


def _soup(rng, vol, N, n):
    vm = np.array(vol.volume_world_min[:3], np.float64)
    ext = vol.voxel_size_in_world * N
    tris = []
    for k in range(n):
        kind = k % 5
        c = vm + rng.uniform(-0.05, 1.05, 3) * ext  # some centres outside the volume
        scale = [0.002, 0.01, 0.05, 0.3, 1.2][kind] * ext
        t = c + rng.normal(0, scale, (3, 3))
        if k % 37 == 0:
            t[2] = t[0] + 0.5 * (t[1] - t[0])  # degenerate (collinear)
        if k % 41 == 0:
            t[:, k % 3] = t[0, k % 3]  # exactly axis-aligned
        tris.append(t)
    return np.array(tris, np.float32).reshape(-1, 3)


@pytest.fixture(scope="module", params=["c1_small", "c2r"])
def pipe(request, lib, cuda):
    w = pipeline.WORKLOADS["c1_small"] if request.param == "c1_small" else pipeline.scaled(
        pipeline.WORKLOADS["c2_production"], width=480, height=272)
    p = pipeline.Pipeline(pipeline.host_frame(w, 2))
    yield p
    p.close()


def _gpu_bits(p, positions, indices=None):
    torch = p.torch
    pos = torch.from_numpy(positions).to(p.device)
    idx = None if indices is None else torch.from_numpy(indices.astype(np.int32)).to(p.device)
    p.voxelize_triangles(pos, idx, mips=False)
    p.sync()
    N = p.hf.workload.voxel_res
    b = p.buffers()
    return p._dev_tensor(b.voxel_bits, N ** 3 // 32, torch.int32).cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("seed", [0, 1])
def test_triangle_soup_bit_exact(pipe, oracle, seed):
    rng = np.random.default_rng(seed)
    N = pipe.hf.workload.voxel_res
    pos = _soup(rng, pipe.hf.volume, N, 3000)
    g = _gpu_bits(pipe, pos)
    o = oracle.voxelize_triangles(pos, None, pipe.hf.volume, N)
    assert g.any()
    assert np.array_equal(g, o)


def test_indexed_mesh_and_box_scene(pipe, oracle):
    hf = pipe.hf
    N = hf.workload.voxel_res
    tris = np.concatenate([_box_triangles(hf.boxes[i].min[:3], hf.boxes[i].max[:3]) for i in range(hf.scene.n_boxes)])
    uniq, inv = np.unique(tris, axis=0, return_inverse=True)
    g = _gpu_bits(pipe, np.ascontiguousarray(uniq, np.float32), inv.reshape(-1, 3))
    assert np.array_equal(g, oracle.voxelize(hf.boxes, hf.scene.n_boxes, hf.volume, N))
    # the box voxelizer of the library itself
    pipe.voxelize()
    pipe.sync()
    b = pipe.buffers()
    box = pipe._dev_tensor(b.voxel_bits, N ** 3 // 32, pipe.torch.int32).cpu().numpy().view(np.uint32)
    assert np.array_equal(g, box)


def test_bad_arguments(pipe, lib):
    import ctypes as C
    from dynamicradiancevolume_gb300 import abi
    vol = C.byref(pipe.hf.volume)
    # 4 triangles need 12 vertices without indices
    assert lib.drv_voxelize_triangles(pipe.ctx, C.c_void_p(pipe.out.data_ptr()), 6, None, 4, vol) == abi.ERR_INVALID_ARG
    assert lib.drv_voxelize_triangles(pipe.ctx, None, 3, None, 1, vol) == abi.ERR_INVALID_ARG
    assert lib.drv_voxelize_triangles(pipe.ctx, None, 0, None, 0, vol) == abi.OK  # empty mesh: cleared grid
