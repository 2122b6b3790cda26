"""ctypes binding of the FP64 oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
CPU-baseline leg of bench.py, to check results against. Arrays are numpy; layouts are
those of include/drv.h.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _abi():
    import sys
    sys.path.insert(0, str(HERE.parent))
    from dynamicradiancevolume_gb300 import abi  # struct layouts only (pure ctypes, no library load)
    return abi


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    abi = _abi()
    lib = C.CDLL(str(LIB))
    P, VP, I, D = C.POINTER, C.c_void_p, C.c_int, C.c_double
    sig = {
        "orc_morton_decode": (None, [C.c_uint32, P(C.c_uint32), P(C.c_uint32)]),
        "orc_pack_normal16i": (None, [P(D), P(C.c_int16)]),
        "orc_unpack_normal16i": (None, [P(C.c_int16), P(D)]),
        "orc_sh_constants": (None, [I, P(D), P(D)]),
        "orc_sh_irradiance": (None, [I, I, P(D), P(D), P(D)]),
        "orc_sample_voxels": (D, [I, VP, VP, P(D), D]),
        "orc_cone_shadow": (D, [P(abi.DrvVolumeInfo), I, VP, VP, P(D), P(D), D, I]),
        "orc_prepare_light": (None, [P(abi.DrvLightDesc), P(abi.DrvSpotLight)]),
        "orc_prepare_camera": (None, [P(abi.DrvCamera), P(abi.DrvPerFrame)]),
        "orc_compute_volume_info": (None, [P(abi.DrvConfig), P(C.c_float), P(C.c_float), P(C.c_float),
                                           P(abi.DrvVolumeInfo)]),
        "orc_raycast_gbuffer": (None, [P(abi.DrvBox), I, P(abi.DrvPerFrame), P(abi.DrvCamera), I, I, VP, VP, VP, VP]),
        "orc_raycast_rsm": (None, [P(abi.DrvBox), I, P(abi.DrvSpotLight), VP, VP, VP]),
        "orc_downsample_rsm": (None, [I, VP, VP, VP, VP, VP, VP]),
        "orc_extract_vpls": (None, [P(abi.DrvSpotLight), I, VP, VP, VP, VP, VP, VP]),
        "orc_voxelize": (None, [P(abi.DrvBox), I, P(abi.DrvVolumeInfo), I, VP]),
        "orc_voxelize_triangles": (None, [VP, VP, I, P(abi.DrvVolumeInfo), I, VP]),
        "orc_raycast_gbuffer_mesh": (None, [VP, VP, VP, VP, I, P(abi.DrvPerFrame), P(abi.DrvCamera), I, I, VP, VP,
                                            VP, VP]),
        "orc_raycast_rsm_mesh": (None, [VP, VP, VP, VP, I, P(abi.DrvSpotLight), VP, VP, VP]),
        "orc_build_mips": (None, [I, VP, VP]),
        "orc_allocate_caches": (I, [P(abi.DrvConfig), P(abi.DrvVolumeInfo), P(abi.DrvPerFrame), I, I, VP, VP, VP,
                                    P(C.c_uint32)]),
        "orc_light_caches": (None, [P(abi.DrvConfig), P(abi.DrvVolumeInfo), I, VP, I, P(abi.DrvSpotLight),
                                    P(VP), P(VP), P(I), VP, VP, VP, I]),
        "orc_light_caches_shadowed": (None, [P(abi.DrvConfig), I, VP, I, P(abi.DrvSpotLight), P(VP), P(I), VP, I, VP,
                                             I]),
        "orc_apply": (None, [P(abi.DrvConfig), P(abi.DrvVolumeInfo), P(abi.DrvPerFrame), I, I, VP, VP, I, VP, VP, I,
                             VP, VP, I]),
        "orc_bruteforce_rsm": (None, [P(abi.DrvPerFrame), I, I, VP, VP, VP, VP, I, P(VP), P(I), VP, I]),
        "orc_light_caches_specular": (None, [P(abi.DrvConfig), P(abi.DrvVolumeInfo), I, VP, VP, I,
                                             P(abi.DrvSpotLight), P(VP), P(VP), P(I), VP, VP, VP, VP, I]),
        "orc_hemi_projection": (None, [P(D), P(D)]),
        "orc_encode_r11g11b10": (C.c_uint32, [P(D)]),
        "orc_encode_r11g11b10_n": (None, [VP, C.c_int64, VP]),
        "orc_decode_r11g11b10": (None, [C.c_uint32, P(D)]),
        "orc_specular_prepare": (None, [I, I, I, VP, I]),
        "orc_apply_specular": (None, [P(abi.DrvConfig), P(abi.DrvVolumeInfo), P(abi.DrvPerFrame), I, I, VP, VP, I,
                                      VP, VP, VP, I, VP, VP, VP, I]),
        "orc_generate_scene": (None, [C.c_uint64, I, C.c_float, C.c_float, C.c_float, C.c_float, P(abi.DrvBox),
                                      P(abi.DrvScene)]),
        "orc_generate_camera": (None, [C.c_uint64, P(abi.DrvScene), C.c_float, P(abi.DrvCamera)]),
        "orc_generate_light": (None, [C.c_uint64, P(abi.DrvScene), C.c_uint32, C.c_uint32, C.c_uint32,
                                      P(abi.DrvLightDesc)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def n_mip_values(N: int) -> int:
    s, l = 0, 1
    while (N >> l) >= 1:
        s += (N >> l) ** 3
        l += 1
    return s


def mip_level(mips: np.ndarray, N: int, level: int) -> np.ndarray:
    off = sum((N >> l) ** 3 for l in range(1, level))
    n = N >> level
    return mips[off:off + n ** 3].reshape(n, n, n)


# -- wrappers ---------------------------------------------------------------
def morton_decode(m: int):
    x, y = C.c_uint32(), C.c_uint32()
    load().orc_morton_decode(m, C.byref(x), C.byref(y))
    return x.value, y.value


def pack_normal16i(n) -> tuple:
    a = (C.c_double * 3)(*n)
    o = (C.c_int16 * 2)()
    load().orc_pack_normal16i(a, o)
    return o[0], o[1]


def unpack_normal16i(p) -> np.ndarray:
    a = (C.c_int16 * 2)(*p)
    o = (C.c_double * 3)()
    load().orc_unpack_normal16i(a, o)
    return np.array(o[:])


def sh_constants(sh2_sign: int):
    cl, ev = (C.c_double * 5)(), (C.c_double * 5)()
    load().orc_sh_constants(sh2_sign, cl, ev)
    return np.array(cl[:]), np.array(ev[:])


def sh_irradiance(sh_order: int, sh2_sign: int, sh27, n) -> np.ndarray:
    sh = (C.c_double * 27)(*np.asarray(sh27, dtype=np.float64).ravel())
    nn = (C.c_double * 3)(*n)
    o = (C.c_double * 3)()
    load().orc_sh_irradiance(sh_order, sh2_sign, sh, nn, o)
    return np.array(o[:])


def prepare_light(desc):
    abi = _abi()
    o = abi.DrvSpotLight()
    load().orc_prepare_light(C.byref(desc), C.byref(o))
    return o


def prepare_camera(cam):
    abi = _abi()
    o = abi.DrvPerFrame()
    load().orc_prepare_camera(C.byref(cam), C.byref(o))
    return o


def compute_volume_info(cfg, amin, amax, cam_pos):
    abi = _abi()
    o = abi.DrvVolumeInfo()
    f3 = C.c_float * 3
    load().orc_compute_volume_info(C.byref(cfg), f3(*amin), f3(*amax), f3(*cam_pos), C.byref(o))
    return o


def raycast_gbuffer(boxes, n_boxes, frame, cam, W, H):
    depth = np.zeros((H, W), np.float32)
    n16 = np.zeros((H, W, 2), np.int16)
    n32 = np.zeros((H, W, 3), np.float32)
    alb = np.zeros((H, W, 3), np.float32)
    load().orc_raycast_gbuffer(boxes, n_boxes, C.byref(frame), C.byref(cam), W, H, _p(depth), _p(n16), _p(n32),
                               _p(alb))
    return depth, n16, n32, alb


def raycast_rsm(boxes, n_boxes, light):
    R = light.rsm_render_resolution
    flux = np.zeros((R, R, 3), np.float32)
    n16 = np.zeros((R, R, 2), np.int16)
    dls = np.zeros((R, R, 2), np.float32)
    load().orc_raycast_rsm(boxes, n_boxes, C.byref(light), _p(flux), _p(n16), _p(dls))
    return flux, n16, dls


def downsample_rsm(flux, n16, dls):
    R = flux.shape[0]
    h = R // 2
    fo = np.zeros((h, h, 3), np.float32)
    no = np.zeros((h, h, 2), np.int16)
    do = np.zeros((h, h, 2), np.float32)
    load().orc_downsample_rsm(R, _p(np.ascontiguousarray(flux)), _p(np.ascontiguousarray(n16)),
                              _p(np.ascontiguousarray(dls)), _p(fo), _p(no), _p(do))
    return fo, no, do


def rsm_chain(flux, n16, dls, levels: int):
    chain = [(flux, n16, dls)]
    for _ in range(levels):
        chain.append(downsample_rsm(*chain[-1]))
    return chain


def extract_vpls(light, flux, n16, dls, dls_shadow):
    R = flux.shape[0]
    n = R * R
    interval = light.indirect_shadow_sample_interval
    vpl = np.zeros((n, 10), np.float64)
    cones = np.zeros(((n + interval - 1) // interval, 4), np.float64)
    load().orc_extract_vpls(C.byref(light), R, _p(np.ascontiguousarray(flux)), _p(np.ascontiguousarray(n16)),
                            _p(np.ascontiguousarray(dls)), _p(np.ascontiguousarray(dls_shadow)), _p(vpl), _p(cones))
    return vpl, cones


def voxelize(boxes, n_boxes, vol, N):
    bits = np.zeros(N ** 3 // 32, np.uint32)
    load().orc_voxelize(boxes, n_boxes, C.byref(vol), N, _p(bits))
    return bits


def voxelize_triangles(positions, indices, vol, N):
    """positions: float32 [V, 3] world space; indices: uint32 [T, 3] or None
    (consecutive triples). Returns the level-0 bitmask (uint32 words)."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    idx = None if indices is None else np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
    n = len(pos) // 3 if idx is None else len(idx)
    bits = np.zeros(N ** 3 // 32, np.uint32)
    load().orc_voxelize_triangles(_p(pos), None if idx is None else _p(idx), n, C.byref(vol), N, _p(bits))
    return bits


def _mesh_args(positions, normals, albedo, indices):
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    alb = None if albedo is None else np.ascontiguousarray(albedo, dtype=np.float32).reshape(-1, 3)
    idx = None if indices is None else np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
    n = len(pos) // 3 if idx is None else len(idx)
    keep = (pos, nrm, alb, idx)
    return keep, [_p(pos), None if nrm is None else _p(nrm), None if alb is None else _p(alb),
                  None if idx is None else _p(idx), n]


def raycast_gbuffer_mesh(positions, normals, albedo, indices, frame, cam, W, H):
    keep, args = _mesh_args(positions, normals, albedo, indices)
    depth = np.zeros((H, W), np.float32)
    n16 = np.zeros((H, W, 2), np.int16)
    n32 = np.zeros((H, W, 3), np.float32)
    alb = np.zeros((H, W, 3), np.float32)
    load().orc_raycast_gbuffer_mesh(*args, C.byref(frame), C.byref(cam), W, H, _p(depth), _p(n16), _p(n32), _p(alb))
    return depth, n16, n32, alb


def raycast_rsm_mesh(positions, normals, albedo, indices, light):
    keep, args = _mesh_args(positions, normals, albedo, indices)
    R = light.rsm_render_resolution
    flux = np.zeros((R, R, 3), np.float32)
    n16 = np.zeros((R, R, 2), np.int16)
    dls = np.zeros((R, R, 2), np.float32)
    load().orc_raycast_rsm_mesh(*args, C.byref(light), _p(flux), _p(n16), _p(dls))
    return flux, n16, dls


def build_mips(N, bits):
    mips = np.zeros(n_mip_values(N), np.float64)
    load().orc_build_mips(N, _p(np.ascontiguousarray(bits, dtype=np.uint32)), _p(mips))
    return mips


def sample_voxels(N, bits, mips, s, lod) -> float:
    return load().orc_sample_voxels(N, _p(bits), _p(mips), (C.c_double * 3)(*s), lod)


def cone_shadow(vol, N, bits, mips, cache_pos, avg, dsr, max_steps) -> float:
    return load().orc_cone_shadow(C.byref(vol), N, _p(bits), _p(mips), (C.c_double * 3)(*cache_pos),
                                  (C.c_double * 3)(*avg), dsr, max_steps)


def allocate_caches(cfg, vol, frame, depth):
    H, W = depth.shape
    atlas = np.zeros((cfg.cav_res, cfg.cav_res, cfg.n_cascades * cfg.cav_res), np.uint32)
    pos = np.zeros((cfg.max_caches, 3), np.float32)
    count = C.c_uint32()
    st = load().orc_allocate_caches(C.byref(cfg), C.byref(vol), C.byref(frame), W, H,
                                    _p(np.ascontiguousarray(depth, dtype=np.float32)), _p(atlas), _p(pos),
                                    C.byref(count))
    n = min(count.value, cfg.max_caches)
    return st, atlas, pos[:n].copy(), count.value


def light_caches(cfg, vol, positions, lights, vpls, cones, bits, mips, n_threads=0):
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    n = positions.shape[0]
    L = len(vpls)
    sh = np.zeros((n, 27), np.float64)
    vp = (C.c_void_p * L)(*[v.ctypes.data for v in vpls])
    cp = (C.c_void_p * L)(*[c.ctypes.data for c in cones])
    nv = (C.c_int * L)(*[v.shape[0] for v in vpls])
    load().orc_light_caches(C.byref(cfg), C.byref(vol), n, _p(positions), L, lights, vp, cp, nv, _p(bits), _p(mips),
                            _p(sh), n_threads)
    return sh


def light_caches_specular(cfg, vol, positions, cam, lights, vpls, cones, bits, mips, n_threads=0):
    """SH [n, 27] and level-0 specular envmaps [n, S, S, 3] (FP64, not rounded)."""
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    n = positions.shape[0]
    L = len(vpls)
    S = cfg.specular_envmap_size
    sh = np.zeros((n, 27), np.float64)
    env = np.zeros((n, S, S, 3), np.float64)
    vp = (C.c_void_p * L)(*[v.ctypes.data for v in vpls])
    cp = (C.c_void_p * L)(*[c.ctypes.data for c in cones])
    nv = (C.c_int * L)(*[v.shape[0] for v in vpls])
    cam = np.ascontiguousarray(cam, dtype=np.float32)
    load().orc_light_caches_specular(C.byref(cfg), C.byref(vol), n, _p(positions), _p(cam), L, lights, vp, cp, nv,
                                     _p(bits), _p(mips), _p(sh), _p(env), n_threads)
    return sh, env


def hemi_projection(d) -> tuple:
    out = (C.c_double * 2)()
    load().orc_hemi_projection((C.c_double * 3)(*d), out)
    return out[0], out[1]


def encode_r11g11b10(rgb) -> np.ndarray:
    """[..., 3] float64 -> uint32 R11F_G11F_B10F words (the GL rules, nearest)."""
    a = np.ascontiguousarray(rgb, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(a.shape[0], np.uint32)
    load().orc_encode_r11g11b10_n(_p(a), a.shape[0], _p(out))
    return out.reshape(np.shape(rgb)[:-1])


def decode_r11g11b10(words) -> np.ndarray:
    """uint32 R11F_G11F_B10F words -> [..., 3] float64 (vectorised)."""
    w = np.asarray(words, dtype=np.uint32)

    def uf(v, mb):
        e = (v >> mb).astype(np.int64)
        m = (v & ((1 << mb) - 1)).astype(np.float64)
        normal = np.ldexp(1.0 + m / (1 << mb), e - 15)
        sub = np.ldexp(m, -14 - mb)
        out = np.where(e == 0, sub, normal)
        return np.where(e == 31, np.where(m > 0, np.nan, np.inf), out)

    return np.stack([uf(w & 0x7FF, 6), uf((w >> 11) & 0x7FF, 6), uf(w >> 22, 5)], -1)


def specular_levels(S: int) -> list:
    """Word offsets of the levels of one per-cache envmap, and the total."""
    off, o, l = [], 0, 0
    while (S >> l) >= 1:
        off.append(o)
        o += (S >> l) ** 2
        l += 1
    return off + [o]


def specular_prepare(S: int, fill: int, env_words, n_threads=0) -> np.ndarray:
    """Mips + hole fill of per-cache envmaps [n, words] (level 0 given) in a copy."""
    e = np.ascontiguousarray(env_words, dtype=np.uint32).copy()
    load().orc_specular_prepare(S, fill, e.shape[0], _p(e), n_threads)
    return e


def apply_specular(cfg, vol, frame, depth, normal, normal_format, albedo, rough_metal, atlas, sh, env, n_threads=0):
    H, W = depth.shape
    out = np.zeros((H, W, 3), np.float64)
    sh = np.ascontiguousarray(sh, dtype=np.float64)
    rm = np.ascontiguousarray(rough_metal, dtype=np.float32)
    env = np.ascontiguousarray(env, dtype=np.uint32)
    load().orc_apply_specular(C.byref(cfg), C.byref(vol), C.byref(frame), W, H, _p(np.ascontiguousarray(depth)),
                              _p(np.ascontiguousarray(normal)), normal_format, _p(np.ascontiguousarray(albedo)),
                              _p(rm), _p(np.ascontiguousarray(atlas, dtype=np.uint32)), sh.shape[0], _p(sh), _p(env),
                              _p(out), n_threads)
    return out


def light_caches_shadowed(cfg, positions, lights, vpls, shadow, n_threads=0):
    """SH gather with per-(cache, block) shadowing [n_caches, total_blocks]."""
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    shadow = np.ascontiguousarray(shadow, dtype=np.float64)
    n = positions.shape[0]
    L = len(vpls)
    sh = np.zeros((n, 27), np.float64)
    vp = (C.c_void_p * L)(*[v.ctypes.data for v in vpls])
    nv = (C.c_int * L)(*[v.shape[0] for v in vpls])
    load().orc_light_caches_shadowed(C.byref(cfg), n, _p(positions), L, lights, vp, nv, _p(shadow), shadow.shape[1],
                                     _p(sh), n_threads)
    return sh


def apply(cfg, vol, frame, depth, normal, normal_format, albedo, atlas, sh, n_threads=0):
    H, W = depth.shape
    out = np.zeros((H, W, 3), np.float64)
    sh = np.ascontiguousarray(sh, dtype=np.float64)
    load().orc_apply(C.byref(cfg), C.byref(vol), C.byref(frame), W, H, _p(np.ascontiguousarray(depth)),
                     _p(np.ascontiguousarray(normal)), normal_format, _p(np.ascontiguousarray(albedo)),
                     _p(np.ascontiguousarray(atlas, dtype=np.uint32)), sh.shape[0], _p(sh), _p(out), n_threads)
    return out


def bruteforce_rsm(frame, depth, normal16, albedo, vpls, rough_metal=None, n_threads=0):
    """Unshadowed per-pixel gather over every VAL (bruteforcersm.frag)."""
    H, W = depth.shape
    out = np.zeros((H, W, 3), np.float64)
    L = len(vpls)
    keep = [np.ascontiguousarray(v, dtype=np.float64) for v in vpls]
    vp = (C.c_void_p * L)(*[v.ctypes.data for v in keep])
    nv = (C.c_int * L)(*[v.shape[0] for v in keep])
    rm = None if rough_metal is None else np.ascontiguousarray(rough_metal, dtype=np.float32)
    load().orc_bruteforce_rsm(C.byref(frame), W, H, _p(np.ascontiguousarray(depth, dtype=np.float32)),
                              _p(np.ascontiguousarray(normal16, dtype=np.int16)),
                              _p(np.ascontiguousarray(albedo, dtype=np.float32)), None if rm is None else _p(rm), L,
                              vp, nv, _p(out), n_threads)
    return out



# ---------------------------------------------------------------- host frames
def make_config(w):
    """DrvConfig of a workload (a `pipeline.Workload`), field by field as the
    product's drv_default_config + pipeline.make_config set it, without the
    product library."""
    abi = _abi()
    cfg = abi.DrvConfig()
    cfg.width, cfg.height = w.width, w.height
    cfg.sh_order = w.sh_order
    cfg.indirect_shadow = w.indirect_shadow
    cfg.max_cone_steps = w.max_cone_steps
    cfg.cascade_transition = w.cascade_transition
    cfg.n_cascades = w.n_cascades
    cfg.cav_res = w.cav_res
    for c in range(abi.MAX_CASCADES):
        cfg.cascade_world_size[c] = w.cascade_world_size0 * (2.0 ** c)
    cfg.voxel_res = w.voxel_res
    cfg.max_caches = w.max_caches
    cfg.precision = w.precision
    cfg.visibility = w.visibility
    cfg.surrogate_conf_threshold = 0.5
    cfg.sh2_sign = 0
    cfg.max_lights = w.n_lights
    cfg.max_rsm_resolution = w.rsm_resolution
    cfg.output_format = 0
    cfg.output_blend = 0
    cfg.specular_envmap_size = w.specular_envmap_size
    cfg.specular_fill_level = w.specular_fill_level
    return cfg


def host_frame(w, seed=None):
    """The seeded frame description of a workload (scene, camera, lights,
    UBO mirrors) built by the oracle alone: the same values the product's
    pipeline.host_frame produces, for the benchmark's CPU arm."""
    from types import SimpleNamespace
    abi = _abi()
    lib = load()
    seed = w.seed if seed is None else seed
    cfg = make_config(w)
    boxes = (abi.DrvBox * (w.n_boxes + 1))()
    scene = abi.DrvScene()
    lib.orc_generate_scene(seed, w.n_boxes, w.box_size[0], w.box_size[1], w.albedo[0], w.albedo[1], boxes,
                           C.byref(scene))
    cam = abi.DrvCamera()
    lib.orc_generate_camera(seed, C.byref(scene), w.width / w.height, C.byref(cam))
    frame = abi.DrvPerFrame()
    lib.orc_prepare_camera(C.byref(cam), C.byref(frame))
    descs = []
    lights = (abi.DrvSpotLight * w.n_lights)()
    for l in range(w.n_lights):
        d = abi.DrvLightDesc()
        lib.orc_generate_light(seed * 31 + l, C.byref(scene), w.rsm_resolution, w.rsm_read_lod, w.shadow_lod,
                               C.byref(d))
        lib.orc_prepare_light(C.byref(d), C.byref(lights[l]))
        descs.append(d)
    vol = abi.DrvVolumeInfo()
    lib.orc_compute_volume_info(C.byref(cfg), scene.aabb_min, scene.aabb_max, cam.position, C.byref(vol))
    return SimpleNamespace(workload=w, config=cfg, boxes=boxes, scene=scene, camera=cam, frame=frame,
                           light_descs=descs, lights=lights, volume=vol)
