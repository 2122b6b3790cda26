"""Triangle-mesh input producers (drv_raster_gbuffer / drv_raster_rsm):
the box scene given as a mesh reproduces the box ray casters away from
silhouette and coplanar ties, with no pixel left uncovered inside the closed
room (watertight edges); a random mesh with vertex normals, some of it inside
the light's near plane, matches the FP64 oracle's mesh ray caster, which
clips at the near plane as the raster does; a whole frame runs from a mesh
(raster G-buffer and RSM, triangle voxelization)."""
import ctypes as C

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_oracle_known_answers import _box_triangles

pytestmark = pytest.mark.gpu


def _box_mesh(hf):
    boxes = [hf.boxes[i] for i in range(hf.scene.n_boxes)]
    tris = np.concatenate([_box_triangles(b.min[:3], b.max[:3]) for b in boxes])
    alb = np.repeat(np.array([b.albedo[:3] for b in boxes], np.float32), 12, axis=0)
    return tris, alb


class Mesh:
    def __init__(self, torch, device, positions, normals=None, albedo=None, indices=None):
        t = lambda a, dt: None if a is None else torch.from_numpy(np.ascontiguousarray(a, dt)).to(device)
        self.pos, self.nrm, self.alb = t(positions, np.float32), t(normals, np.float32), t(albedo, np.float32)
        self.idx = t(indices, np.int32)
        ptr = lambda x: None if x is None else x.data_ptr()
        nt = len(positions) // 3 if indices is None else len(indices)
        self.c = abi.DrvMesh(ptr(self.pos), ptr(self.nrm), ptr(self.alb), ptr(self.idx), len(positions), nt)


def _raster_inputs(p, lib, mesh):
    hf, w = p.hf, p.hf.workload
    out = abi.DrvGBufferOut(p.depth.data_ptr(), p.normal16.data_ptr(), p.normal32.data_ptr(), p.albedo.data_ptr())
    assert lib.drv_raster_gbuffer(p.ctx, C.byref(mesh.c), C.byref(hf.camera), C.byref(hf.frame), w.width, w.height,
                                  C.byref(out)) == abi.OK
    for l in range(w.n_lights):
        r = abi.DrvRSMOut(p.rsm_flux[l].data_ptr(), p.rsm_normal[l].data_ptr(), p.rsm_dls[l].data_ptr())
        assert lib.drv_raster_rsm(p.ctx, C.byref(mesh.c), C.byref(hf.lights[l]), C.byref(r)) == abi.OK
    p.sync()


def _snapshot(p):
    return {k: getattr(p, k).cpu().numpy().copy() for k in ("depth", "normal16", "albedo")}, \
        [(p.rsm_flux[l].cpu().numpy().copy(), p.rsm_normal[l].cpu().numpy().copy(), p.rsm_dls[l].cpu().numpy().copy())
         for l in range(p.hf.workload.n_lights)]


def test_box_scene_as_mesh_matches_box_ray_caster(lib, cuda):
    torch = pytest.importorskip("torch")
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], rsm_resolution=64)
    p = pipeline.Pipeline(pipeline.host_frame(w, 5))
    p.raycast_inputs()
    p.sync()
    g0, r0 = _snapshot(p)
    tris, alb = _box_mesh(p.hf)
    mesh = Mesh(torch, p.device, tris, None, alb)
    _raster_inputs(p, lib, mesh)
    g1, r1 = _snapshot(p)
    # the camera and the lights are inside the room: every ray hits a face
    assert (g0["depth"] != 0).all() and (g1["depth"] != 0).all()
    assert all((d[..., 0] > 0).all() for _, _, d in r1)
    same_depth = np.abs(g0["depth"] - g1["depth"]) <= 1e-5 * np.maximum(np.abs(g0["depth"]), 1e-6)
    assert same_depth.mean() > 0.99
    assert np.all(g0["normal16"] == g1["normal16"], -1)[same_depth].mean() > 0.999
    assert np.all(g0["albedo"] == g1["albedo"], -1)[same_depth].mean() > 0.99
    for (f0, n0, d0), (f1, n1, d1) in zip(r0, r1):
        ok = np.abs(d0[..., 0] - d1[..., 0]) <= 1e-5 * np.maximum(d0[..., 0], 1e-6)
        assert ok.mean() > 0.99
        # the spot falloff (cos - cos_half) cancels at the cone's edge, where a
        # few-ulp difference of the hit point is a large relative one: the
        # absolute part of the tolerance is scaled to the brightest texel
        assert np.allclose(f0[ok], f1[ok], rtol=1e-4, atol=1e-4 * f0.max())
        assert np.all(n0 == n1, -1)[ok].mean() > 0.999
    p.close()


def test_random_mesh_matches_oracle(lib, cuda, oracle):
    torch = pytest.importorskip("torch")
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], width=160, height=120, rsm_resolution=64)
    hf = pipeline.host_frame(w, 7)
    p = pipeline.Pipeline(hf)
    rng = np.random.default_rng(2)
    tris, alb = _box_mesh(hf)  # the room and boxes, plus a cloud of random triangles with vertex normals
    lo, hi = np.array(hf.scene.aabb_min[:]), np.array(hf.scene.aabb_max[:])
    c = lo + rng.uniform(0.2, 0.8, (300, 3)) * (hi - lo)
    extra = (c[:, None, :] + rng.normal(0, 0.06, (300, 3, 3))).reshape(-1, 3).astype(np.float32)
    pos = np.concatenate([tris, extra]).astype(np.float32)
    nrm = rng.normal(0, 1, pos.shape).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    albedo = np.concatenate([alb, rng.uniform(0.1, 0.9, (300, 3)).astype(np.float32)])
    mesh = Mesh(torch, p.device, pos, nrm, albedo)
    _raster_inputs(p, lib, mesh)
    g, r = _snapshot(p)
    d0, n0, _, a0 = oracle.raycast_gbuffer_mesh(pos, nrm, albedo, None, hf.frame, hf.camera, w.width, w.height)
    same = np.abs(d0 - g["depth"]) <= 1e-4 * np.maximum(np.abs(d0), 1e-6)
    assert same.mean() > 0.98
    assert np.all(a0 == g["albedo"], -1)[same].mean() > 0.99
    un = lambda q: np.stack([oracle.unpack_normal16i(v) for v in q.reshape(-1, 2)[::7]])
    dots = np.sum(un(n0) * un(g["normal16"]), -1)[same.reshape(-1)[::7]]
    assert np.mean(dots > 0.999) > 0.99
    f0, m0, l0 = oracle.raycast_rsm_mesh(pos, nrm, albedo, None, hf.lights[0])
    ok = np.abs(l0[..., 0] - r[0][2][..., 0]) <= 1e-4 * np.maximum(l0[..., 0], 1e-6)
    assert ok.mean() > 0.98
    assert np.allclose(f0[ok], r[0][0][ok], rtol=1e-3, atol=1e-4 * f0.max())
    p.close()


def test_frame_from_a_mesh(lib, cuda, oracle):
    """Mesh inputs end to end: raster G-buffer and RSM, triangle voxels, then
    the per-frame stages; against the FP64 oracle on the same inputs."""
    torch = pytest.importorskip("torch")
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], rsm_resolution=64)
    hf = pipeline.host_frame(w, 5)
    p = pipeline.Pipeline(hf)
    tris, alb = _box_mesh(hf)
    mesh = Mesh(torch, p.device, tris, None, alb)
    _raster_inputs(p, lib, mesh)
    p.prepare_and_extract()
    p.voxelize_triangles(mesh.pos)
    p.allocate()
    p.light()
    p.apply()
    p.sync()
    assert p.cache_count() > 0
    out = p.out.cpu().numpy()
    assert np.isfinite(out).all() and out.sum() > 0
    # the box-scene frame from the ray casters: the same to the silhouette
    # pixels. The box ray casters have no near plane while the raster clips
    # at it, so the comparison needs a light with no surface closer than its
    # near plane (this seed's nearest RSM texel is twice as far).
    q = pipeline.Pipeline(pipeline.host_frame(w, 5))
    q.raycast_inputs()
    q.frame()
    q.sync()
    for l in range(w.n_lights):
        assert q.rsm_dls[l][..., 0].min().item() > hf.light_descs[l].near_plane
    ref = q.out.cpu().numpy()
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 0.05
    p.close()
    q.close()


def test_indexed_mesh_equals_triangle_soup(lib, cuda, oracle):
    """The same triangles given once as a soup and once as shared vertices +
    indices rasterise to the same G-buffer and RSM, bit for bit; the F32
    normal target holds the normal the RG16I target packs."""
    torch = pytest.importorskip("torch")
    oracle_unpack = oracle.unpack_normal16i
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], rsm_resolution=64)
    p = pipeline.Pipeline(pipeline.host_frame(w, 3))
    tris, alb = _box_mesh(p.hf)
    _raster_inputs(p, lib, Mesh(torch, p.device, tris, None, alb))
    g0, r0 = _snapshot(p)
    n32 = p.normal32.cpu().numpy()
    uniq, inv = np.unique(tris.reshape(-1, 3), axis=0, return_inverse=True)
    _raster_inputs(p, lib, Mesh(torch, p.device, uniq, None, alb, indices=inv.reshape(-1, 3)))
    g1, r1 = _snapshot(p)
    for k in g0:
        assert np.array_equal(g0[k], g1[k]), k
    for a, b in zip(r0, r1):
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
    live = g0["depth"] != 0
    np.testing.assert_allclose(np.linalg.norm(n32[live], axis=-1), 1.0, atol=1e-6)
    un = np.stack([oracle_unpack(v) for v in g0["normal16"][live][::53]])
    assert np.all(np.sum(un * n32[live][::53], -1) > 0.9999)
    p.close()
