"""Known-answer tests that pin the FP64 oracle (the reference ships no tests,
golden images or fixtures, so these are the anchors of parity)."""
import math

import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi

KSHADER_PI = 3.14159265358979  # the shaders' PI (globalubos.glsl)


def test_morton_decode_matches_bitwise_definition(oracle):
    # cacheLightingRSM.comp:46-62: x takes the even bits, y the odd bits.
    rng = np.random.default_rng(0)
    for m in list(range(0, 4096)) + [int(v) for v in rng.integers(0, 2**32, 2000)]:
        x = sum(((m >> (2 * i)) & 1) << i for i in range(16))
        y = sum(((m >> (2 * i + 1)) & 1) << i for i in range(16))
        assert oracle.morton_decode(m) == (x, y)


@pytest.mark.parametrize("n,packed", [
    ((1, 0, 0), (0, 0)), ((-1, 0, 0), (32767, 0)), ((0, 1, 0), (16384, 0)), ((0, -1, 0), (-16384, 0)),
    ((0, 0, 1), (0, 32767)), ((0, 0, -1), (0, -32768)),
])
def test_pack_normal16i_axis_aligned(oracle, n, packed):
    # utils.glsl:61-89 with the saturating int16 conversion
    assert oracle.pack_normal16i(n) == packed
    u = oracle.unpack_normal16i(packed)
    assert np.allclose(u, n, atol=1e-2)


def test_pack_unpack_roundtrip(oracle):
    rng = np.random.default_rng(1)
    v = rng.normal(size=(500, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for n in v:
        u = oracle.unpack_normal16i(oracle.pack_normal16i(n))
        # (atan2, z) quantisation loses precision near the poles (dz = 1/32768)
        assert np.linalg.norm(u - n) < 1e-3


def _sh_of_single_vpl(oracle, direction, radiance=1.0):
    """SH coefficients (27) that cacheLightingRSM.comp:267-277 stores for a
    single VPL of unit radianceIn arriving from `direction`."""
    _, ev = oracle.sh_constants(0)
    x, y, z = direction
    basis = [ev[0], -ev[1] * y, ev[1] * z, -ev[1] * x, -ev[2] * x * y, ev[2] * y * z, ev[3] * (3 * z * z - 1),
             ev[2] * x * z, ev[4] * (x * x - y * y)]
    return np.repeat(np.array(basis)[:, None] * radiance, 3, axis=1).ravel()


def test_sh_projection_single_vpl_on_z_axis(oracle):
    # A single VPL on +z: SH00 = Y0, SH10 = Y1, the rest 0 (SH1);
    # irradiance at n = +z is Y0*c0 + Y1*c1.
    cl, ev = oracle.sh_constants(0)
    sh = _sh_of_single_vpl(oracle, (0.0, 0.0, 1.0))
    e = oracle.sh_irradiance(1, 0, sh, (0.0, 0.0, 1.0))
    assert np.allclose(e, ev[0] * cl[0] + ev[1] * cl[1], rtol=0, atol=1e-15)


def _funk_hecke(omega, n, lmax):
    # Exact l <= lmax clamped-cosine response: sum_l A_l (2l+1)/(4 pi) P_l(w.n)
    # with A_0 = pi, A_1 = 2 pi / 3, A_2 = pi / 4.
    t = float(np.dot(omega, n))
    P = [1.0, t, 0.5 * (3 * t * t - 1)]
    A = [math.pi, 2 * math.pi / 3, math.pi / 4]
    return sum(A[l] * (2 * l + 1) / (4 * math.pi) * P[l] for l in range(lmax + 1))


def test_sh_cosine_lobe_funk_hecke_both_sign_modes(oracle):
    rng = np.random.default_rng(2)
    d = rng.normal(size=(1000, 2, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    err_ref, err_fix, err_sh1 = 0.0, 0.0, 0.0
    for omega, n in d:
        sh = _sh_of_single_vpl(oracle, omega)
        exact2 = _funk_hecke(omega, n, 2)
        exact1 = _funk_hecke(omega, n, 1)
        # The apply clamps at 0; compare only where the exact response is positive.
        e_fix = oracle.sh_irradiance(2, 1, sh, n)[0]
        e_ref = oracle.sh_irradiance(2, 0, sh, n)[0]
        e_sh1 = oracle.sh_irradiance(1, 0, sh, n)[0]
        if exact2 > 0:
            err_fix = max(err_fix, abs(e_fix - exact2))
        if exact1 > 0:
            err_sh1 = max(err_sh1, abs(e_sh1 - exact1))
        err_ref = max(err_ref, abs(e_ref - max(exact2, 0.0)))
    assert err_fix < 1e-12          # corrected band-2 sign matches Funk-Hecke
    assert err_sh1 < 1e-12          # SH1 is correct with the reference constants
    assert err_ref > 0.3            # renderer.cpp:298's negative factor flips the mixed band-2 terms


def test_sh2_reference_mode_flips_exactly_the_mixed_terms(oracle):
    cl_ref, _ = oracle.sh_constants(0)
    cl_fix, _ = oracle.sh_constants(1)
    assert cl_ref[2] == -cl_fix[2]
    assert np.array_equal(np.delete(cl_ref, 2), np.delete(cl_fix, 2))


def _volume(abi, N=8, vmin=0.0, size=1.0):
    vol = abi.DrvVolumeInfo()
    for i in range(3):
        vol.volume_world_min[i] = vmin
        vol.volume_world_max[i] = vmin + size
    vol.voxel_size_in_world = size / N
    return vol


def test_mips_of_checkerboard_are_half(oracle):
    N = 32
    idx = np.arange(N ** 3)
    x, y, z = idx % N, (idx // N) % N, idx // (N * N)
    on = ((x + y + z) & 1).astype(np.uint32)
    bits = np.zeros(N ** 3 // 32, np.uint32)
    for w in range(bits.size):
        bits[w] = int(sum(int(on[w * 32 + b]) << b for b in range(32)))
    mips = oracle.build_mips(N, bits)
    assert np.all(mips == 0.5)


def test_cone_empty_volume_is_unshadowed(oracle):
    from dynamicradiancevolume_gb300 import abi
    N = 32
    vol = _volume(abi, N)
    bits = np.zeros(N ** 3 // 32, np.uint32)
    mips = oracle.build_mips(N, bits)
    s = oracle.cone_shadow(vol, N, bits, mips, (0.2, 0.5, 0.5), (0.8, 0.5, 0.5), 0.05, 32)
    assert s == 1.0


def test_cone_solid_slab_blocks(oracle):
    from dynamicradiancevolume_gb300 import abi
    N = 32
    vol = _volume(abi, N)
    idx = np.arange(N ** 3)
    x = idx % N
    on = ((x >= 14) & (x <= 17)).astype(np.uint64)
    bits = np.zeros(N ** 3 // 32, np.uint32)
    for w in range(bits.size):
        bits[w] = int(sum(int(on[w * 32 + b]) << b for b in range(32)))
    mips = oracle.build_mips(N, bits)
    s = oracle.cone_shadow(vol, N, bits, mips, (0.2, 0.5, 0.5), (0.8, 0.5, 0.5), 0.02, 32)
    assert s < 1e-3


def test_quadrilinear_filter_semantics(oracle):
    # Magnification at lod <= 0 samples level 0 trilinearly; at integer lods
    # exactly one level is used; lod beyond the chain clamps to the last level.
    N = 32
    bits = np.zeros(N ** 3 // 32, np.uint32)
    bits[0] = 1  # voxel (0,0,0)
    mips = oracle.build_mips(N, bits)
    c = (0.5 / N, 0.5 / N, 0.5 / N)  # centre of voxel (0,0,0)
    assert oracle.sample_voxels(N, bits, mips, c, -3.0) == 1.0
    assert oracle.sample_voxels(N, bits, mips, c, 0.0) == 1.0
    assert oracle.sample_voxels(N, bits, mips, (1.0 / N,) * 3, 0.0) == pytest.approx(0.125)
    assert oracle.sample_voxels(N, bits, mips, c, 1.0) == pytest.approx(0.125)  # level 1 texel (0,0,0) = 1/8
    assert oracle.sample_voxels(N, bits, mips, c, 0.5) == pytest.approx(0.5 * 1.0 + 0.5 * 0.125)
    assert oracle.sample_voxels(N, bits, mips, c, 99.0) == pytest.approx(1.0 / N ** 3)


def test_allocation_flat_wall_predictable(oracle):
    """A wall parallel to the image plane at a known depth allocates exactly
    the 8 corners of every cell its pixels land in, minus the cells whose
    only pixels sit in row 0 / column 0 of a 16x16 tile (the reference's
    dedupe compares those threads with themselves, cacheGather.comp:141-147)."""
    from dynamicradiancevolume_gb300 import abi
    W = H = 64
    cfg = abi.DrvConfig(width=W, height=H, sh_order=1, n_cascades=1, cav_res=8, voxel_res=32, max_caches=4096,
                        max_lights=1, max_rsm_resolution=32)
    cfg.cascade_world_size[0] = 2.0
    cfg.cascade_transition = 0.0
    # Orthographic-like inverse VP: x_world = ndc.x * 0.5 + 0.5 (+ same for y), z = depth.
    frame = abi.DrvPerFrame()
    M = [0.5, 0, 0, 0.5, 0, 0.5, 0, 0.5, 0, 0, 1, 0, 0, 0, 0, 1]
    for i, v in enumerate(M):
        frame.inverse_view_projection[i] = v
    vol = abi.DrvVolumeInfo()
    k = vol.cascades[0]
    k.world_voxel_size = 0.25
    for i in range(3):
        k.min[i] = -0.5
        k.max[i] = 1.5
        k.decision_min[i] = -10
        k.decision_max[i] = 10
    depth = np.full((H, W), 0.3, np.float32)
    st, atlas, pos, count = oracle.allocate_caches(cfg, vol, frame, depth)
    assert st == 0
    # Expected: pixel (x, y) -> world ((x+.5)/64, (y+.5)/64, 0.3) -> cell ((w+0.5)/0.25)
    expected = set()
    for ty in range(0, H, 16):
        for tx in range(0, W, 16):
            cells = {}
            for ly in range(16):
                for lx in range(16):
                    px, py = tx + lx, ty + ly
                    cx = int(((px + 0.5) / W + 0.5) / 0.25)
                    cy = int(((py + 0.5) / H + 0.5) / 0.25)
                    cz = int((0.3 + 0.5) / 0.25)
                    cells.setdefault((cx, cy, cz), []).append((lx, ly))
            for cell, pix in cells.items():
                sel = set(pix)
                if any(((lx, ly) == (0, 0)) or (lx >= 1 and ly >= 1 and (lx, ly - 1) not in sel and
                       (lx - 1, ly) not in sel and (lx - 1, ly - 1) not in sel) for lx, ly in pix):
                    for o in range(8):
                        expected.add((cell[0] + (o >> 2), cell[1] + (o & 1), cell[2] + ((o >> 1) & 1)))
    got = {tuple(map(int, np.round((p - (-0.5)) / 0.25))) for p in pos}
    assert got == expected
    assert count == len(expected)
    # Published atlas slots hold index + 1 of an entry at that corner.
    zs, ys, xs = np.nonzero(atlas)
    for z, y, x in zip(zs, ys, xs):
        p = pos[atlas[z, y, x] - 1]
        assert np.allclose(p, np.array([x, y, z]) * 0.25 - 0.5)


def _unit_frame(oracle, cam_pos=(0.0, 0.0, 2.5)):
    f = abi.DrvPerFrame()
    for k in range(4):
        f.inverse_view_projection[5 * k] = 1.0  # identity: world = (ndc.x, ndc.y, depth)
        f.view_projection[5 * k] = 1.0
    f.camera_position[:] = cam_pos
    return f


def test_bruteforce_single_val_facing_the_pixel(oracle):
    # 1x1 image: the pixel sits at world (0, 0, 0.5) with normal +z; one VAL
    # straight above at distance 1, facing down, unit flux, zero area.
    f = _unit_frame(oracle)
    depth = np.array([[0.5]], np.float32)
    n16 = np.array([oracle.pack_normal16i((0.0, 0.0, 1.0))], np.int16).reshape(1, 1, 2)
    alb = np.array([[[0.5, 0.25, 1.0]]], np.float32)
    a64 = alb[0, 0].astype(np.float64)
    v = np.zeros((1, 10))
    v[0, 0:3] = 1.0          # flux
    v[0, 3] = 0.0            # disc area
    v[0, 4:7] = (0, 0, 1.5)  # position
    v[0, 7:10] = (0, 0, -1)  # normal
    nz = oracle.unpack_normal16i(n16[0, 0])[2]  # +z packs to within 2^-15 of the axis
    out = oracle.bruteforce_rsm(f, depth, n16, alb, [v])
    assert np.allclose(out[0, 0], a64 / KSHADER_PI * nz, rtol=1e-12)
    # reference BRDF, roughness 1, metallic 0, camera straight above: the
    # half vector is +z, so Blinn-Phong is (e + 8) / (8 pi) * (n.z)^e
    rm = np.array([[[1.0, 0.0]]], np.float32)
    e = 2.0 / (1.0 + 0.0005)
    spec = (e + 8.0) / (8.0 * KSHADER_PI) * nz ** e * 0.04
    out = oracle.bruteforce_rsm(f, depth, n16, alb, [v], rough_metal=rm)
    assert np.allclose(out[0, 0], (a64 / KSHADER_PI + spec) * nz, rtol=1e-6)
    # a VAL facing away (or below the surface) adds nothing; no geometry -> 0
    v2 = v.copy()
    v2[0, 7:10] = (0, 0, 1)
    assert np.all(oracle.bruteforce_rsm(f, depth, n16, alb, [v2]) == 0.0)
    assert np.all(oracle.bruteforce_rsm(f, np.zeros((1, 1), np.float32), n16, alb, [v]) == 0.0)


def _box_triangles(lo, hi):
    """The 12 triangles of an axis-aligned box (float32 [36, 3])."""
    c = np.array([[hi[0] if i & 1 else lo[0], hi[1] if i & 2 else lo[1], hi[2] if i & 4 else lo[2]] for i in range(8)],
                 np.float32)
    faces = [(0, 2, 6, 4), (1, 5, 7, 3), (0, 4, 5, 1), (2, 3, 7, 6), (0, 1, 3, 2), (4, 6, 7, 5)]
    return np.array([c[k] for a, b, cc, d in faces for k in (a, b, cc, a, cc, d)], np.float32)


def test_triangle_voxelization_of_box_faces_equals_the_box_rule(oracle):
    """Axis-aligned faces as triangles: the conservative raster (half-voxel
    L1 dilation, grown AABB) covers exactly the voxels whose square touches
    the face, the box voxelizer's closed rule; the depth gradient is 0."""
    from dynamicradiancevolume_gb300 import pipeline
    w = pipeline.WORKLOADS["c1_small"]
    hf = pipeline.host_frame(w, 3)
    tris = np.concatenate([_box_triangles(hf.boxes[i].min[:3], hf.boxes[i].max[:3]) for i in range(hf.scene.n_boxes)])
    a = oracle.voxelize_triangles(tris, None, hf.volume, w.voxel_res)
    b = oracle.voxelize(hf.boxes, hf.scene.n_boxes, hf.volume, w.voxel_res)
    assert np.array_equal(a, b)
    # indexed: shared vertices give the same voxels
    verts = tris.reshape(-1, 3)
    uniq, inv = np.unique(verts, axis=0, return_inverse=True)
    c = oracle.voxelize_triangles(uniq, inv.reshape(-1, 3).astype(np.uint32), hf.volume, w.voxel_res)
    assert np.array_equal(c, b)


def test_triangle_voxelization_known_answer(oracle):
    """A triangle in the plane z = 10.25 voxels with corners at voxel
    coordinates (4, 4), (12, 4), (4, 12): the pixel centres within half a
    voxel (L1) of it — voxel columns x, y in [3, 12], x + y <= 16 + 1 — at
    voxel z = 10."""
    N = 32
    vol = _volume(abi, N)
    vs, vm = vol.voxel_size_in_world, np.array(vol.volume_world_min[:3])
    tri = (np.array([[4, 4, 10.25], [12, 4, 10.25], [4, 12, 10.25]]) * vs + vm).astype(np.float32)
    bits = oracle.voxelize_triangles(tri, None, vol, N)
    v = np.unpackbits(bits.view(np.uint8), bitorder="little").reshape(N, N, N)  # [z][y][x]
    zs, ys, xs = np.nonzero(v)
    assert set(zs.tolist()) == {10}
    exp = {(x, y) for x in range(N) for y in range(N)
           if x + 0.5 >= 3.5 and y + 0.5 >= 3.5 and x + 0.5 <= 12.5 and y + 0.5 <= 12.5 and (x + 0.5) + (y + 0.5) <= 17.0}
    assert set(zip(xs.tolist(), ys.tolist())) == exp


def test_triangle_voxelization_depth_conservative(oracle):
    """A steep triangle (depth slope 1 voxel per voxel): each covered column
    also gets the voxels above and below the centre depth where the depth
    changes by a voxel within the pixel (voxelize.frag:39-55)."""
    N = 32
    vol = _volume(abi, N)
    vs, vm = vol.voxel_size_in_world, np.array(vol.volume_world_min[:3])
    # plane z = 8 + 0.9 x (dominant axis z: |n_z| > |n_x|)
    pts = np.array([[4, 4, 8 + 0.9 * 4], [20, 4, 8 + 0.9 * 20], [4, 20, 8 + 0.9 * 4]])
    bits = oracle.voxelize_triangles((pts * vs + vm).astype(np.float32), None, vol, N)
    v = np.unpackbits(bits.view(np.uint8), bitorder="little").reshape(N, N, N)
    col = v[:, 10, 10]  # column at x = 10, y = 10
    assert col.sum() >= 2  # more than the single voxel of the centre depth


def test_r11g11b10_codec_known_answers(oracle):
    """The GL packed-float texel of the specular envmaps (GL 4.5 sections
    2.3.4.3-4): 5-bit exponent with bias 15, 6 (blue 5) mantissa bits, round
    to nearest, negatives to 0, large values to the largest finite one."""
    one = (15 << 6) | ((15 << 6) << 11) | ((15 << 5) << 22)
    assert int(oracle.encode_r11g11b10(np.array([1.0, 1.0, 1.0]))) == one
    w = oracle.encode_r11g11b10(np.array([[65024.0, 1e9, 64512.0], [-1.0, 0.0, -np.inf], [np.inf, 2.0 ** -20, 0.5]]))
    assert list(oracle.decode_r11g11b10(w[0])) == [65024.0, 65024.0, 64512.0]
    assert list(oracle.decode_r11g11b10(w[1])) == [0.0, 0.0, 0.0]
    r, g, b = oracle.decode_r11g11b10(w[2])
    assert np.isinf(r) and g == 2.0 ** -20 and b == 0.5  # 2^-20 is the smallest red/green subnormal
    # ties go to the even mantissa: 1 + 1/128 -> 1, 1 + 3/128 -> 1 + 2/64
    t = oracle.decode_r11g11b10(oracle.encode_r11g11b10(np.array([[1 + 1 / 128, 1 + 3 / 128, 1 + 1 / 64]])))[0]
    assert list(t) == [1.0, 1.0 + 2 / 64, 1.0]  # blue: 1 + 1/64 is a tie at 5 bits
    # every finite code of each channel decodes and encodes back to itself
    for shift, mb in ((0, 6), (11, 6), (22, 5)):
        codes = np.arange(0, 31 << mb, dtype=np.uint32)
        vals = oracle.decode_r11g11b10(codes << shift)
        assert np.array_equal(oracle.encode_r11g11b10(vals), codes << shift)


def test_specular_prepare_known_answer(oracle):
    """Mips are the 2x2 means (exact here); the hole fill gives zero texels
    their parent's colour and rescales the four so that their mean keeps the
    parent's value (up to the 1e-5 guard and the texel rounding)."""
    S = 8
    off = oracle.specular_levels(S)
    rng = np.random.default_rng(5)
    lvl0 = np.zeros((S, S, 3))
    lvl0[rng.random((S, S)) < 0.3] = rng.choice([0.25, 0.5, 1.0, 2.0, 4.0], size=(1, 3))
    e = np.zeros((1, off[-1]), np.uint32)
    e[0, :S * S] = oracle.encode_r11g11b10(lvl0.reshape(-1, 3))
    m = oracle.specular_prepare(S, 0, e)
    for l in range(1, len(off) - 1):
        side = S >> l
        below = oracle.decode_r11g11b10(m[0, off[l - 1]:off[l]]).reshape(2 * side, 2 * side, 3)
        mean = below.reshape(side, 2, side, 2, 3).mean(axis=(1, 3))
        assert np.array_equal(oracle.encode_r11g11b10(mean.reshape(-1, 3)), m[0, off[l]:off[l + 1]])
    f = oracle.specular_prepare(S, 2, e)
    assert np.array_equal(f[0, off[2]:], m[0, off[2]:])  # the fill leaves levels 2.. as the mips made them
    for l in (1, 0):  # levels the fill wrote (from level 2 down)
        side = S >> (l + 1)
        parent = oracle.decode_r11g11b10(f[0, off[l + 1]:off[l + 2]]).reshape(side, side, 3)
        kids = oracle.decode_r11g11b10(f[0, off[l]:off[l + 1]]).reshape(side, 2, side, 2, 3)
        live = parent.sum(-1) >= 1e-4
        assert np.all(kids.sum(-1).min(axis=(1, 3))[live] > 0)  # no holes under a lit parent
        np.testing.assert_allclose(kids.mean(axis=(1, 3))[live], parent[live], rtol=2e-2)


def test_mesh_ray_caster_equals_box_caster_on_box_scenes(oracle):
    """The box scene given as triangles (12 per box): the FP64 mesh ray
    caster reproduces the box ray caster exactly, G-buffer and RSM, when no
    surface is closer to the light than its near plane."""
    from dynamicradiancevolume_gb300 import pipeline
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], width=96, height=64, rsm_resolution=32)
    hf = pipeline.host_frame(w, 5)
    boxes = [hf.boxes[i] for i in range(hf.scene.n_boxes)]
    tris = np.concatenate([_box_triangles(b.min[:3], b.max[:3]) for b in boxes])
    alb = np.repeat(np.array([b.albedo[:3] for b in boxes], np.float32), 12, axis=0)
    d0, n0, m0, a0 = oracle.raycast_gbuffer(hf.boxes, hf.scene.n_boxes, hf.frame, hf.camera, w.width, w.height)
    d1, n1, m1, a1 = oracle.raycast_gbuffer_mesh(tris, None, alb, None, hf.frame, hf.camera, w.width, w.height)
    assert np.array_equal(n0, n1) and np.array_equal(a0, a1)
    np.testing.assert_allclose(d1, d0, rtol=1e-6, atol=0)
    f0, r0, l0 = oracle.raycast_rsm(hf.boxes, hf.scene.n_boxes, hf.lights[0])
    f1, r1, l1 = oracle.raycast_rsm_mesh(tris, None, alb, None, hf.lights[0])
    assert l0[..., 0].min() > hf.light_descs[0].near_plane
    assert np.array_equal(r0, r1)
    np.testing.assert_allclose(l1, l0, rtol=1e-6, atol=0)
    np.testing.assert_allclose(f1, f0, rtol=1e-5, atol=1e-12)


def test_mesh_ray_caster_clips_at_the_near_plane(oracle):
    """A light with a box inside its near plane: the rasteriser (and the mesh
    caster) clip that surface and see what lies behind it, the box caster
    (no near plane) sees the box."""
    from dynamicradiancevolume_gb300 import pipeline
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], rsm_resolution=32)
    hf = pipeline.host_frame(w, 9)
    near = hf.light_descs[0].near_plane
    boxes = [hf.boxes[i] for i in range(hf.scene.n_boxes)]
    tris = np.concatenate([_box_triangles(b.min[:3], b.max[:3]) for b in boxes])
    _, _, l0 = oracle.raycast_rsm(hf.boxes, hf.scene.n_boxes, hf.lights[0])
    _, _, l1 = oracle.raycast_rsm_mesh(tris, None, None, None, hf.lights[0])
    assert l0[..., 0].min() < near  # the box caster sees a surface inside the near plane
    assert l1[..., 0][l1[..., 0] > 0].min() >= near  # the mesh caster never does
    closer = l0[..., 0] < near
    assert np.all(l1[..., 0][closer] > l0[..., 0][closer])  # it sees what lies behind instead


def test_hemispherical_projection_known_answers(oracle):
    """The concentric square map (utils.glsl:103-170): the pole to the centre,
    the horizon's axis directions to the edge midpoints, the diagonal to the
    corner's direction; a direction and its mirror image are mirrored."""
    pts = {(0, 0, 1): (0.5, 0.5), (1, 0, 0): (1.0, 0.5), (0, 1, 0): (0.5, 1.0), (-1, 0, 0): (0.0, 0.5),
           (0, -1, 0): (0.5, 0.0)}
    for d, uv in pts.items():
        assert np.allclose(oracle.hemi_projection(d), uv, atol=1e-12), d
    s = math.sqrt(0.5)
    u, v = oracle.hemi_projection((s, s, 0.0))  # phi = 1: the corner of the square's right edge
    assert np.allclose((u, v), (1.0, 1.0), atol=1e-12)
    rng = np.random.default_rng(1)
    for _ in range(50):
        d = rng.normal(size=3)
        d[2] = abs(d[2])
        d /= np.linalg.norm(d)
        u, v = oracle.hemi_projection(d)
        um, vm = oracle.hemi_projection((-d[0], d[1], d[2]))
        assert 0.0 <= u <= 1.0 and 0.0 <= v <= 1.0
        assert abs(um - (1.0 - u)) < 1e-9 and abs(vm - v) < 1e-9


def test_specular_envmap_of_one_vpl_known_answer(oracle):
    """One cache, one VPL, no shadow: the level-0 envmap holds one texel, at
    the concentric projection of the cache-local half vector, with
    flux * saturate(n . -l) / (d^2 + area) * saturate(h . l) * (S^2 + 7) / (8 pi)
    (cacheLightingRSM.comp:234-335); the SH are unchanged by the specular
    path when the flux passes its 0.001 threshold."""
    S = 16
    cfg = abi.DrvConfig()
    cfg.sh_order, cfg.indirect_shadow, cfg.voxel_res, cfg.max_cone_steps = 2, 0, 32, 4
    cfg.specular_envmap_size = S
    vol = _volume(abi, 32)
    L = (abi.DrvSpotLight * 1)()
    L[0].indirect_shadow_sample_interval = 1
    c = np.array([[0.3, 0.4, 0.5]], np.float32)
    cam = np.array([0.9, 0.7, 0.1], np.float32)
    p, n = np.array([0.6, 0.2, 0.9]), np.array([-0.6, 0.3, -0.74])
    n = n / np.linalg.norm(n)
    vpl = np.array([[0.5, 0.25, 0.125, 0.01, *p, *n]])
    bits = np.zeros(32 ** 3 // 32, np.uint32)
    mips = np.zeros(oracle.n_mip_values(32))
    sh, env = oracle.light_caches_specular(cfg, vol, c, cam, L, [vpl], [np.zeros((1, 4))], bits, mips)
    # independent restatement
    cc, camd = c[0].astype(np.float64), cam.astype(np.float64)
    z = (camd - cc) / np.linalg.norm(camd - cc)
    x = np.array([z[2], 0.0, -z[0]]) / np.linalg.norm([z[2], 0.0, -z[0]])
    y = np.cross(z, x)
    t = p - cc
    d2 = t @ t
    l = t / math.sqrt(d2)
    g = max(0.0, min(1.0, -(n @ l))) / (d2 + 0.01)
    ll = np.array([l @ x, l @ y, l @ z])
    h = ll + np.array([0.0, 0.0, 1.0])
    h /= np.linalg.norm(h)
    r = math.sqrt(max(0.0, 1.0 - h[2])) * 0.5
    phi = math.atan2(h[1], h[0]) * 4.0 / 3.14159265358979
    if phi < -1:
        phi += 8
    if phi < 1:
        uv = (r, phi * r)
    elif phi < 3:
        uv = (-(phi - 2) * r, r)
    elif phi < 5:
        uv = (-r, -(phi - 4) * r)
    else:
        uv = ((phi - 6) * r, -r)
    tx, ty = (min(max(int((q + 0.5) * S + 0.5), 0), S - 1) for q in uv)
    k = g * max(0.0, min(1.0, h @ ll)) * (S * S + 7) / (8 * 3.14159265358979)
    nz = np.argwhere(env[0].sum(-1) > 0)
    assert nz.tolist() == [[ty, tx]]
    np.testing.assert_allclose(env[0, ty, tx], vpl[0, :3] * k, rtol=1e-12)
    # the SH of the same VPL without the specular path are the same (flux sum 0.875 >= 0.001)
    cfg0 = abi.DrvConfig.from_buffer_copy(cfg)
    cfg0.specular_envmap_size = 0
    sh0 = oracle.light_caches(cfg0, vol, c, L, [vpl], [np.zeros((1, 4))], bits, mips)
    np.testing.assert_allclose(sh, sh0, rtol=0, atol=0)
    # a VPL below the threshold adds nothing with specular on
    dim = vpl.copy()
    dim[0, :3] = 0.0003
    sh_dim, env_dim = oracle.light_caches_specular(cfg, vol, c, cam, L, [dim], [np.zeros((1, 4))], bits, mips)
    assert not sh_dim.any() and not env_dim.any()


def test_specular_apply_of_a_constant_envmap(oracle):
    """Zero SH and the same constant envmap in every cache (all levels): every
    lit pixel's radiance is that constant times the specular colour,
    0.04 (1 - metallic) + albedo * metallic (lightingfunctions.glsl:41-49),
    times the weight of its live corners, whatever its lookup and lod. The
    weight (1 where all 8 corners are allocated; less where the reference's
    tile dedupe or the atlas edge left some out; blended across a cascade
    transition) is the diffuse apply's output for unit irradiance and an
    albedo of pi."""
    from dynamicradiancevolume_gb300 import pipeline
    w = pipeline.scaled(pipeline.WORKLOADS["c1_small"], width=64, height=48, specular_envmap_size=8)
    hf = pipeline.host_frame(w, 5)
    depth, n16, _, albedo = oracle.raycast_gbuffer(hf.boxes, hf.scene.n_boxes, hf.frame, hf.camera, w.width,
                                                   w.height)
    st, atlas, pos, count = oracle.allocate_caches(hf.config, hf.volume, hf.frame, depth)
    E = np.array([0.75, 0.5, 0.25])
    words = oracle.specular_levels(8)[-1]
    env = np.full((count, words), int(oracle.encode_r11g11b10(E)), np.uint32)
    sh = np.zeros((count, 27))
    rng = np.random.default_rng(3)
    rm = (rng.integers(0, 256, (w.height, w.width, 2)).astype(np.float32) / np.float32(255.0))
    out = oracle.apply_specular(hf.config, hf.volume, hf.frame, depth, n16, abi.NORMAL_RG16I, albedo, rm, atlas, sh,
                                env)
    lit = depth >= 1e-5
    # corner weights: unit irradiance (SH00 = 1 / its cosine-lobe response), albedo pi
    f0 = oracle.sh_irradiance(2, 0, np.eye(1, 27).ravel(), (0.0, 0.0, 1.0))[0]
    unit = np.zeros((count, 27))
    unit[:, 0:3] = 1.0 / f0
    wsum = oracle.apply(hf.config, hf.volume, hf.frame, depth, n16, abi.NORMAL_RG16I,
                        np.full_like(albedo, np.float32(3.14159265358979)), atlas, unit)[..., 0:1]
    m = rm[..., 1:2].astype(np.float64)
    expect = wsum * E * (0.04 * (1.0 - m) + albedo.astype(np.float64) * m)
    np.testing.assert_allclose(out[lit], expect[lit], rtol=1e-6, atol=1e-12)
    assert np.mean(np.abs(wsum[lit] - 1.0) < 1e-6) > 0.9  # most pixels have all 8 corners (pi passed in binary32)
    assert not out[~lit].any()


def test_rsm_downsample_known_answers(oracle):
    """downsamplersm.frag:15-33 on an 8 x 8 RSM: flux is the sum of the 2 x 2
    children (textureGather), (d, d^2) their mean (the linear sample at the
    shared corner), the normal the normalised sum of the unpacked children,
    repacked; three levels chain."""
    R = 8
    rng = np.random.default_rng(5)
    flux = rng.integers(0, 64, size=(R, R, 3)).astype(np.float32) / 8.0  # exact in FP32 sums
    dls = np.stack([rng.integers(0, 64, size=(R, R)) / 4.0, rng.integers(0, 64, size=(R, R)) / 2.0],
                   axis=-1).astype(np.float32)
    up = oracle.pack_normal16i((0.0, 0.0, 1.0))
    n16 = np.empty((R, R, 2), np.int16)
    n16[...] = up
    # block (1, 1) of level 1: two children face +x, two +y: their mean
    # direction is (1, 1, 0) / sqrt(2)
    n16[2, 2] = n16[2, 3] = oracle.pack_normal16i((1.0, 0.0, 0.0))
    n16[3, 2] = n16[3, 3] = oracle.pack_normal16i((0.0, 1.0, 0.0))
    fo, no, do = oracle.downsample_rsm(flux, n16, dls)
    blocks = lambda a: a.reshape(R // 2, 2, R // 2, 2, *a.shape[2:])
    assert np.array_equal(fo, blocks(flux).sum(axis=(1, 3)))
    assert np.array_equal(do, blocks(dls).mean(axis=(1, 3)).astype(np.float32))
    d = oracle.unpack_normal16i(tuple(no[1, 1]))
    assert np.allclose(d, (math.sqrt(0.5), math.sqrt(0.5), 0.0), atol=2e-4)
    mask = np.ones((R // 2, R // 2), bool)
    mask[1, 1] = False
    assert np.all(no[mask] == np.array(up, np.int16))
    chain = oracle.rsm_chain(flux, n16, dls, 3)
    assert [c[0].shape[0] for c in chain] == [8, 4, 2, 1]
    assert np.array_equal(chain[3][0].reshape(3), flux.reshape(-1, 3).sum(axis=0))
    assert np.allclose(chain[3][2].reshape(2), dls.reshape(-1, 2).mean(axis=0), rtol=1e-6)


def test_vpl_extraction_known_answers(oracle):
    """cacheLightingRSM.comp:141-158 and 168-192 on a constant RSM: VPL i is
    RSM texel morton_decode(i), at the RSM depth d along its texel's ray from
    the light (inside the spot cone), with area d^2 * ValAreaFactor and the
    texel's flux and unpacked normal; a shadow block's cone source is at the
    same depth along its sample ray, and with zero depth variance its spread
    is the super-VAL width."""
    d = abi.DrvLightDesc()
    d.intensity[:] = (1.0, 1.0, 1.0)
    d.position[:] = (0.5, 0.5, 0.9)
    d.direction[:] = (0.0, 0.0, -1.0)
    d.half_angle, d.rsm_resolution, d.rsm_read_lod, d.indirect_shadow_lod = 0.5, 32, 0, 1
    d.near_plane, d.far_plane = 0.05, 5.0
    L = oracle.prepare_light(d)
    R = L.rsm_read_resolution
    assert R == 32
    depth = 0.75
    rng = np.random.default_rng(6)
    flux = rng.random((R, R, 3)).astype(np.float32)
    normal = oracle.pack_normal16i((0.0, 0.6, 0.8))
    n16 = np.empty((R, R, 2), np.int16)
    n16[...] = normal
    dls = np.empty((R, R, 2), np.float32)
    dls[...] = (depth, depth * depth)
    shadow = dls[::2, ::2].copy()  # level 1 of a constant RSM
    vpl, cones = oracle.extract_vpls(L, flux, n16, dls, shadow)
    lp = np.array(L.position, np.float64)
    un = oracle.unpack_normal16i(normal)
    for i in range(R * R):
        x, y = oracle.morton_decode(i)
        np.testing.assert_array_equal(vpl[i, 0:3], flux[y, x].astype(np.float64))
        assert vpl[i, 3] == pytest.approx(depth * depth * L.val_area_factor, rel=1e-12)
        off = vpl[i, 4:7] - lp
        assert np.linalg.norm(off) == pytest.approx(depth, rel=1e-9)
        # inside the square RSM frustum around the light's axis
        assert math.acos(-off[2] / depth) <= 0.5 * math.sqrt(2) + 1e-6
        np.testing.assert_allclose(vpl[i, 7:10], un, atol=0)
    # texels mirrored through the RSM centre look in mirrored directions
    i0 = next(i for i in range(R * R) if oracle.morton_decode(i) == (3, 5))
    i1 = next(i for i in range(R * R) if oracle.morton_decode(i) == (R - 4, R - 6))
    a, b = vpl[i0, 4:7] - lp, vpl[i1, 4:7] - lp
    assert a[0] + b[0] == pytest.approx(0, abs=1e-9) and a[1] + b[1] == pytest.approx(0, abs=1e-9)
    assert a[2] == pytest.approx(b[2], rel=1e-9)
    n_blocks = (R * R + L.indirect_shadow_sample_interval - 1) // L.indirect_shadow_sample_interval
    assert cones.shape == (n_blocks, 4)
    assert np.allclose(np.linalg.norm(cones[:, 0:3] - lp, axis=1), depth, rtol=1e-6)
    assert np.allclose(cones[:, 3], L.indirect_shadow_super_val_width, rtol=1e-6)
