"""Workloads and a thin host driver over the C ABI.

`Workload` names a synthetic, seeded scene configuration (the reference's
assimp scenes are replaced by a procedural box room). `Pipeline` owns one
DrvContext plus the device buffers of one frame's inputs (G-buffer, RSMs) and
output, and calls the stage entry points in the order of the reference's
Renderer::Draw. Device memory is allocated through torch (plumbing only);
every computation is a kernel of libdrv_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, replace

from . import abi, check, load


@dataclass(frozen=True)
class Workload:
    name: str
    width: int
    height: int
    n_boxes: int
    voxel_res: int
    n_lights: int
    rsm_resolution: int
    rsm_read_lod: int
    shadow_lod: int
    n_cascades: int
    cascade_world_size0: float
    cav_res: int
    sh_order: int
    max_cone_steps: int
    max_caches: int
    cascade_transition: float = 2.0
    indirect_shadow: int = 1
    seed: int = 1
    box_size: tuple = (0.05, 0.3)
    albedo: tuple = (0.2, 0.9)
    precision: int = abi.PRECISION_FP32
    visibility: int = abi.VISIBILITY_CONE
    specular_envmap_size: int = 0  # INDIRECT_SPECULAR off; else the per-cache envmap side (16 in the reference)
    specular_fill_level: int = 0

    @property
    def n_vpls(self) -> int:
        r = self.rsm_resolution >> self.rsm_read_lod
        return self.n_lights * r * r


WORKLOADS = {
    # Plain method, small: 256^2 G-buffer, 12 boxes, 64^3 voxels, one spot
    # light with a 32^2 RSM (1024 VPLs), one 32^3 cascade, SH1, 16 cone steps.
    "c1_small": Workload("c1_small", 256, 256, 12, 64, 1, 32, 0, 0, 1, 2.0, 32, 1, 16, 65536,
                         cascade_transition=0.0),
    # Plain method at production size: 1920x1080, 64 boxes, 256^3 voxels,
    # 3 lights x 512^2 RSM read at 64^2 (12288 VPLs), 4 cascades of 32^3, SH2,
    # up to 32 cone steps, one cone per VPL-cache pair.
    "c2_production": Workload("c2_production", 1920, 1080, 64, 256, 3, 512, 3, 0, 4, 0.25, 32, 2, 32, 262144),
    # The headline case: C2 with one light (4096 VPLs) at 1080p.
    "ns_1080p_4096": Workload("ns_1080p_4096", 1920, 1080, 64, 256, 1, 512, 3, 0, 4, 0.25, 32, 2, 32, 262144),
    # The headline scene with 128^3 cascades of the same sizes: ~22k caches
    # (cells of 2 mm at cascade 0), toward the tens of thousands of caches
    # the configuration text expects; 8.3 M contributing pairs.
    "ns_1080p_4096_cav128": Workload("ns_1080p_4096_cav128", 1920, 1080, 64, 256, 1, 512, 3, 0, 4, 0.25, 128, 2, 32,
                                     262144),
    # Precision variant of the small configuration: BF16 VPL flux/normal and
    # cache SH, FP16 opacity mips, FP32 Kahan-compensated accumulation.
    "c3_precision": Workload("c3_precision", 256, 256, 12, 64, 1, 32, 0, 0, 1, 2.0, 32, 1, 16, 65536,
                             cascade_transition=0.0, precision=abi.PRECISION_BF16),
}


def make_config(w: Workload) -> abi.DrvConfig:
    lib = load()
    cfg = abi.DrvConfig()
    lib.drv_default_config(C.byref(cfg))
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
    cfg.max_lights = w.n_lights
    cfg.max_rsm_resolution = w.rsm_resolution
    cfg.precision = w.precision
    cfg.visibility = w.visibility
    cfg.specular_envmap_size = w.specular_envmap_size
    cfg.specular_fill_level = w.specular_fill_level
    return cfg


@dataclass
class HostFrame:
    """Host-side description of one frame: scene, camera, lights, UBO mirrors."""
    workload: Workload
    config: abi.DrvConfig
    boxes: C.Array
    scene: abi.DrvScene
    camera: abi.DrvCamera
    frame: abi.DrvPerFrame
    light_descs: list
    lights: C.Array
    volume: abi.DrvVolumeInfo


def host_frame(w: Workload, seed: int | None = None) -> HostFrame:
    lib = load()
    seed = w.seed if seed is None else seed
    cfg = make_config(w)
    boxes = (abi.DrvBox * (w.n_boxes + 1))()
    scene = abi.DrvScene()
    check(lib.drv_generate_scene(seed, w.n_boxes, w.box_size[0], w.box_size[1], w.albedo[0], w.albedo[1], boxes,
                                 C.byref(scene)))
    cam = abi.DrvCamera()
    check(lib.drv_generate_camera(seed, C.byref(scene), w.width / w.height, C.byref(cam)))
    frame = abi.DrvPerFrame()
    check(lib.drv_prepare_camera(C.byref(cam), C.byref(frame)))
    descs = []
    lights = (abi.DrvSpotLight * w.n_lights)()
    for l in range(w.n_lights):
        d = abi.DrvLightDesc()
        check(lib.drv_generate_light(seed * 31 + l, C.byref(scene), w.rsm_resolution, w.rsm_read_lod, w.shadow_lod,
                                     C.byref(d)))
        check(lib.drv_prepare_light(C.byref(d), C.byref(lights[l])))
        descs.append(d)
    vol = abi.DrvVolumeInfo()
    check(lib.drv_compute_volume_info(C.byref(cfg), scene.aabb_min, scene.aabb_max, cam.position, C.byref(vol)))
    return HostFrame(w, cfg, boxes, scene, cam, frame, descs, lights, vol)


class Pipeline:
    """One DrvContext + device buffers for one frame of a workload."""

    def __init__(self, hf: HostFrame, device: str = "cuda", normal_format: int = abi.NORMAL_RG16I,
                 albedo_format: int = abi.ALBEDO_F32X3, rsm_format: int = abi.RSM_F32):
        """albedo_format / rsm_format: the G-buffer view's diffuse target and
        the RSM views' flux and (d, d^2) targets (F32, or the reference's
        SRGB8 / RGB16F + RG16F: then `albedo8`, `rsm_flux16` and `rsm_dls16`
        are the buffers the views read, and the ray casters' F32 buffers are
        only their sources). The output's shape follows the config's
        output_format (RGB F32, or RGBA16F)."""
        import torch
        self.torch = torch
        self.lib = load()
        self.hf = hf
        w = hf.workload
        self.device = torch.device(device)
        self.ctx = C.c_void_p()
        check(self.lib.drv_create(C.byref(hf.config), C.byref(self.ctx)))
        # A dedicated stream: every stage of this pipeline is ordered on it, and
        # callers time it with events recorded on the same stream.
        self.stream = torch.cuda.Stream(self.device)
        check(self.lib.drv_set_stream(self.ctx, C.c_void_p(self.stream.cuda_stream)), self.ctx)
        H, W = w.height, w.width
        dev = self.device
        self.depth = torch.zeros((H, W), dtype=torch.float32, device=dev)
        self.normal16 = torch.zeros((H, W, 2), dtype=torch.int16, device=dev)
        self.normal32 = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        self.albedo = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        if hf.config.output_format == abi.OUTPUT_RGBA16F:
            self.out = torch.zeros((H, W, 4), dtype=torch.float16, device=dev)
        else:
            self.out = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        R = w.rsm_resolution
        self.rsm_flux = [torch.zeros((R, R, 3), dtype=torch.float32, device=dev) for _ in range(w.n_lights)]
        self.rsm_normal = [torch.zeros((R, R, 2), dtype=torch.int16, device=dev) for _ in range(w.n_lights)]
        self.rsm_dls = [torch.zeros((R, R, 2), dtype=torch.float32, device=dev) for _ in range(w.n_lights)]
        # GBuffer_RoughnessMetalic (RG8 unorm), read by the specular apply.
        self.rough_metal = torch.zeros((H, W, 2), dtype=torch.uint8, device=dev)
        self.normal_format = normal_format
        self.albedo8 = torch.zeros((H, W, 3), dtype=torch.uint8, device=dev) if albedo_format == abi.ALBEDO_SRGB8 \
            else None
        self.gview = abi.DrvGBufferView(W, H, self.depth.data_ptr(),
                                        (self.normal16 if normal_format == abi.NORMAL_RG16I else self.normal32).data_ptr(),
                                        normal_format, (self.albedo8 if self.albedo8 is not None else self.albedo).data_ptr(),
                                        albedo_format, self.rough_metal.data_ptr(), abi.ROUGH_METAL_RG8)
        half = rsm_format == abi.RSM_F16
        self.rsm_flux16 = [torch.zeros((R, R, 3), dtype=torch.float16, device=dev) for _ in range(w.n_lights)] \
            if half else None
        self.rsm_dls16 = [torch.zeros((R, R, 2), dtype=torch.float16, device=dev) for _ in range(w.n_lights)] \
            if half else None
        self.rsm_views = (abi.DrvRSMView * w.n_lights)()
        for l in range(w.n_lights):
            flux = self.rsm_flux16[l] if half else self.rsm_flux[l]
            dls = self.rsm_dls16[l] if half else self.rsm_dls[l]
            self.rsm_views[l] = abi.DrvRSMView(R, flux.data_ptr(), self.rsm_normal[l].data_ptr(), dls.data_ptr(),
                                               rsm_format)
        # torch's pooled streams do not wait for its current stream, where the
        # buffers above were zeroed: finish that before any stage runs.
        torch.cuda.current_stream(self.device).synchronize()

    def set_frame(self, hf: HostFrame) -> None:
        """Switches to another frame of the same workload (scene, camera,
        lights); the context and buffers are reused."""
        w0, w1 = self.hf.workload, hf.workload
        if (w0.width, w0.height, w0.n_lights, w0.rsm_resolution) != (w1.width, w1.height, w1.n_lights,
                                                                     w1.rsm_resolution):
            raise ValueError("set_frame needs a frame of the same dimensions")
        self.hf = hf

    def close(self):
        if self.ctx:
            self.lib.drv_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st):
        check(st, self.ctx)

    # -- input producers (the reference's raster passes) --------------------
    def raycast_inputs(self):
        hf, lib = self.hf, self.lib
        out = abi.DrvGBufferOut(self.depth.data_ptr(), self.normal16.data_ptr(), self.normal32.data_ptr(),
                                self.albedo.data_ptr())
        self._c(lib.drv_raycast_gbuffer(self.ctx, C.byref(hf.scene), C.byref(hf.camera), C.byref(hf.frame),
                                        hf.workload.width, hf.workload.height, C.byref(out)))
        for l in range(hf.workload.n_lights):
            ro = abi.DrvRSMOut(self.rsm_flux[l].data_ptr(), self.rsm_normal[l].data_ptr(), self.rsm_dls[l].data_ptr())
            self._c(lib.drv_raycast_rsm(self.ctx, C.byref(hf.scene), C.byref(hf.lights[l]), C.byref(ro)))

    # -- stages ---------------------------------------------------------------
    def prepare_and_extract(self):
        for l in range(self.hf.workload.n_lights):
            self._c(self.lib.drv_prepare_rsm(self.ctx, l, C.byref(self.hf.lights[l]), C.byref(self.rsm_views[l])))
            self._c(self.lib.drv_extract_vpls(self.ctx, l, C.byref(self.hf.lights[l])))

    def voxelize(self):
        self._c(self.lib.drv_voxelize(self.ctx, C.byref(self.hf.scene), C.byref(self.hf.volume)))
        self._c(self.lib.drv_build_opacity_mips(self.ctx))

    def voxelize_triangles(self, positions, indices=None, mips: bool = True):
        """Voxelizes a triangle mesh instead of the box scene: positions is a
        device float32 tensor [V, 3] (world space), indices a device int32 /
        uint32 tensor [T, 3] or None (consecutive triples)."""
        torch = self.torch
        pos = positions.contiguous()
        assert pos.dtype == torch.float32 and pos.is_cuda
        idx = None if indices is None else indices.contiguous()
        n_tris = (pos.shape[0] // 3) if idx is None else idx.shape[0]
        cur = torch.cuda.current_stream(self.device)
        self.stream.wait_stream(cur)  # the mesh may have been written on the current stream
        self._c(self.lib.drv_voxelize_triangles(self.ctx, C.c_void_p(pos.data_ptr()), pos.shape[0],
                                                None if idx is None else C.c_void_p(idx.data_ptr()), n_tris,
                                                C.byref(self.hf.volume)))
        if mips:
            self._c(self.lib.drv_build_opacity_mips(self.ctx))

    def allocate(self):
        self._c(self.lib.drv_allocate_caches(self.ctx, C.byref(self.gview), C.byref(self.hf.frame),
                                             C.byref(self.hf.volume)))

    def light(self):
        self._c(self.lib.drv_light_caches(self.ctx, self.hf.lights, self.hf.workload.n_lights,
                                          C.byref(self.hf.volume), C.byref(self.hf.frame)))

    def apply(self, out=None):
        out = self.out if out is None else out
        self._c(self.lib.drv_apply(self.ctx, C.byref(self.gview), C.byref(self.hf.frame), C.byref(self.hf.volume),
                                   C.c_void_p(out.data_ptr())))

    def bruteforce(self, out=None, rough_metal=None):
        """Unshadowed per-pixel gather over every VPL (no caches) into `out`
        (a new tensor when None); rough_metal: (H, W, 2) device tensor for the
        reference BRDF, None for its diffuse term."""
        out = self.torch.zeros_like(self.out) if out is None else out
        # the caller's tensors were written on torch's current stream
        self.stream.wait_stream(self.torch.cuda.current_stream(self.device))
        rm = C.c_void_p(rough_metal.data_ptr()) if rough_metal is not None else None
        self._c(self.lib.drv_bruteforce_rsm(self.ctx, C.byref(self.gview), rm, C.byref(self.hf.frame),
                                            self.hf.workload.n_lights, C.c_void_p(out.data_ptr())))
        # `out` is handed back to work on torch's current stream
        self.torch.cuda.current_stream(self.device).wait_stream(self.stream)
        return out

    def frame(self, out=None):
        out = self.out if out is None else out
        self._c(self.lib.drv_frame(self.ctx, C.byref(self.hf.scene), C.byref(self.gview), C.byref(self.hf.frame),
                                   C.byref(self.hf.volume), self.hf.lights, self.rsm_views, self.hf.workload.n_lights,
                                   C.c_void_p(out.data_ptr())))

    def sync(self):
        self._c(self.lib.drv_sync(self.ctx))

    def set_tuning(self, **knobs) -> abi.DrvTuning:
        """Sets execution knobs (DrvTuning field names); the others keep their value."""
        t = abi.DrvTuning()
        self._c(self.lib.drv_get_tuning(self.ctx, C.byref(t)))
        for k, v in knobs.items():
            setattr(t, k, v)
        self._c(self.lib.drv_set_tuning(self.ctx, C.byref(t)))
        return t

    def light_pairs(self) -> int:
        """Contributing (cache, block) pairs of the last split light stage."""
        n = C.c_uint32()
        self._c(self.lib.drv_get_light_pairs(self.ctx, C.byref(n)))
        return n.value

    def light_kernel_ms(self) -> dict:
        """Per-kernel milliseconds of the last split light stage run with
        time_kernels set (see set_tuning)."""
        ms = (C.c_float * len(abi.LIGHT_KERNELS))()
        self._c(self.lib.drv_get_light_kernel_ms(self.ctx, ms))
        return dict(zip(abi.LIGHT_KERNELS, list(ms)))

    def surrogate_stats(self) -> tuple[int, int]:
        """(pairs the MLP evaluated, pairs re-traced) of the last light stage."""
        ev, rt = C.c_uint32(), C.c_uint32()
        self._c(self.lib.drv_get_surrogate_stats(self.ctx, C.byref(ev), C.byref(rt)))
        return ev.value, rt.value

    def cache_count(self) -> int:
        n = C.c_uint32()
        self._c(self.lib.drv_get_cache_count(self.ctx, C.byref(n)))
        return n.value

    def buffers(self) -> abi.DrvBuffers:
        b = abi.DrvBuffers()
        self._c(self.lib.drv_get_buffers(self.ctx, C.byref(b)))
        return b

    # -- device buffer readback (tests) -------------------------------------
    def _dev_tensor(self, ptr: int, numel: int, dtype):
        """Copies `numel` elements at device address `ptr` into a new tensor."""
        torch = self.torch
        typestr = {torch.float32: "<f4", torch.int32: "<i4", torch.int16: "<i2", torch.uint8: "|u1"}[dtype]

        class _View:
            __cuda_array_interface__ = {"shape": (numel,), "typestr": typestr, "data": (int(ptr), False),
                                        "version": 3, "strides": None}

        torch.cuda.synchronize(self.device)
        return torch.as_tensor(_View(), device=self.device).clone()

    def read_entries(self, count: int):
        b = self.buffers()
        floats = b.entry_stride // 4
        return self._dev_tensor(b.cache_entries, count * floats, self.torch.float32).view(count, floats)

    def read_entries_decoded(self, count: int):
        """(positions [n,3] float32, sh [n,27] float64 in (coefficient, rgb) order)
        for either entry layout."""
        import numpy as np
        raw = self.read_entries(count).cpu().numpy()
        if self.hf.config.precision == abi.PRECISION_BF16:
            key = raw[:, 0].view(np.uint32)
            cell = np.stack([key & 511, (key >> 9) & 511, (key >> 18) & 511], 1).astype(np.float32)
            casc = (key >> 27).astype(np.int64)
            vol = self.hf.volume
            size = np.array([vol.cascades[c].world_voxel_size for c in range(4)], np.float32)[casc]
            mins = np.array([list(vol.cascades[c].min) for c in range(4)], np.float32)[casc]
            pos = (cell * size[:, None]).astype(np.float32) + mins
            bf = raw.view(np.uint16)[:, 2:29].astype(np.uint32) << 16
            sh = bf.view(np.float32).astype(np.float64)
            return pos.astype(np.float32), sh
        off = {0: [7, 11, 15], 1: [4, 5, 6], 2: [8, 9, 10], 3: [12, 13, 14], 4: [16, 17, 18], 5: [20, 21, 22],
               6: [19, 23, 27], 7: [24, 25, 26], 8: [28, 29, 30]}
        nk = 9 if self.hf.config.sh_order == 2 else 4
        sh = np.zeros((raw.shape[0], 27))
        for k in range(nk):
            sh[:, 3 * k:3 * k + 3] = raw[:, off[k]]
        return raw[:, 0:3].copy(), sh

    def read_atlas(self):
        w = self.hf.workload
        b = self.buffers()
        n = w.n_cascades * w.cav_res ** 3
        return self._dev_tensor(b.cav_atlas, n, self.torch.int32).view(w.cav_res, w.cav_res, w.n_cascades * w.cav_res)

    def prepare_specular(self):
        self._c(self.lib.drv_prepare_specular_envmaps(self.ctx))

    def read_specular(self, n_caches: int):
        """The allocated caches' specular envmaps as numpy uint32 words
        [n_caches, sum of levels], each cache's levels row-major one after the
        other (the oracle's per-cache layout), gathered from the atlas."""
        import numpy as np
        b = self.buffers()
        S, T, L = self.hf.config.specular_envmap_size, b.specular_atlas_size, b.n_specular_levels
        per_row = T // S
        out = []
        for l in range(L):
            side, t = S >> l, T >> l
            lv = self._dev_tensor(b.specular_envmap[l], t * t, self.torch.int32).cpu().numpy().view(np.uint32)
            lv = lv.reshape(t // side, side, t // side, side).transpose(0, 2, 1, 3).reshape(-1, side * side)
            out.append(lv[:n_caches])  # atlas cell (row, col) = cache row * per_row + col
        assert per_row == T // S
        return np.concatenate(out, axis=1)

    def read_voxel_bits(self):
        N = self.hf.workload.voxel_res
        return self._dev_tensor(self.buffers().voxel_bits, N ** 3 // 32, self.torch.int32)

    def read_mip(self, level: int):
        N = self.hf.workload.voxel_res
        n = N >> level
        if self.hf.config.precision == abi.PRECISION_BF16:
            import numpy as np
            words = (n ** 3 + 1) // 2
            raw = self._dev_tensor(self.buffers().voxel_mips[level], words, self.torch.float32).cpu().numpy()
            half = raw.view(np.float16)[:n ** 3]
            return self.torch.from_numpy(half.astype(np.float32)).view(n, n, n)
        return self._dev_tensor(self.buffers().voxel_mips[level], n ** 3, self.torch.float32).view(n, n, n)

    def read_vpls(self, light: int):
        """VPLs as [n, 12] float32 in the DrvVPL layout (BF16 storage widened)."""
        b = self.buffers()
        if self.hf.config.precision == abi.PRECISION_BF16:
            import numpy as np
            raw = self._dev_tensor(b.vpls[light], b.n_vpls[light] * 8, self.torch.float32).cpu().numpy()
            raw = raw.reshape(-1, 8)
            h = raw.view(np.uint16).reshape(-1, 16)[:, 8:14].astype(np.uint32) << 16
            wide = h.view(np.float32)
            out = np.zeros((raw.shape[0], 12), np.float32)
            out[:, 0:3], out[:, 3], out[:, 4:7], out[:, 8:11] = wide[:, 0:3], raw[:, 3], raw[:, 0:3], wide[:, 3:6]
            return self.torch.from_numpy(out)
        return self._dev_tensor(b.vpls[light], b.n_vpls[light] * 12, self.torch.float32).view(-1, 12)

    def read_cones(self, light: int, n: int):
        b = self.buffers()
        return self._dev_tensor(b.cones[light], n * 4, self.torch.float32).view(-1, 4)


def scaled(w: Workload, **kw) -> Workload:
    return replace(w, **kw)


def srgb_encode(lin):
    """Linear [0, 1] -> SRGB8 bytes, the GL sRGB encoding (GL 4.5 section
    17.3.9) rounded to the nearest byte: what an SRGB8 render target stores."""
    import numpy as np
    lin = np.clip(np.asarray(lin, np.float64), 0.0, 1.0)
    cs = np.where(lin <= 0.0031308, lin * 12.92, 1.055 * lin ** (1 / 2.4) - 0.055)
    return np.clip(np.rint(cs * 255.0), 0, 255).astype(np.uint8)


def reference_format_inputs(p: "Pipeline"):
    """A pipeline's ray-cast inputs (F32 buffers) as the reference's render
    targets hold them: depth D32F, normal RG16I, diffuse SRGB8, and per light
    the RSM's RGB16F flux, RG16I normal and RG16F (d, d^2) (numpy arrays)."""
    import numpy as np
    g = (p.depth.cpu().numpy(), p.normal16.cpu().numpy(), srgb_encode(p.albedo.cpu().numpy()))
    rsm = [(p.rsm_flux[l].cpu().numpy().astype(np.float16), p.rsm_normal[l].cpu().numpy(),
            p.rsm_dls[l].cpu().numpy().astype(np.float16)) for l in range(p.hf.workload.n_lights)]
    return g, rsm


def main(argv=None) -> int:
    """Runs whole frames (drv_frame) of a named workload on cuda:0: ray-cast
    inputs once, then --frames frames; prints the cache and pair counts.
    `python -m dynamicradiancevolume_gb300.pipeline ns_1080p_4096 --precision bf16 --frames 4`."""
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("workload", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", choices=["fp32", "bf16"], default="fp32")
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--max-caches", type=int, default=None, help="capacity (the pair list scales with it)")
    ap.add_argument("--surrogate", default=None, help="surrogate visibility with this checkpoint (path stem)")
    ap.add_argument("--threshold", type=float, default=0.5, help="surrogate confidence threshold")
    a = ap.parse_args(argv)
    w = scaled(WORKLOADS[a.workload], precision=abi.PRECISION_BF16 if a.precision == "bf16" else abi.PRECISION_FP32)
    if a.max_caches:
        w = scaled(w, max_caches=a.max_caches)
    if a.surrogate:
        w = scaled(w, visibility=abi.VISIBILITY_SURROGATE)
    hf = host_frame(w, a.seed)
    hf.config.surrogate_conf_threshold = a.threshold
    p = Pipeline(hf)
    if a.surrogate:
        from . import surrogate
        surrogate.upload(p, surrogate.load_params(a.surrogate), surrogate.load_features(a.surrogate))
    p.raycast_inputs()
    for _ in range(a.frames):
        p.frame()
    p.sync()
    print("workload %s (%s): %d caches, %d lit pairs" % (w.name, a.precision, p.cache_count(), p.light_pairs()))
    if a.surrogate:
        print("surrogate: %d pairs evaluated, %d re-traced" % p.surrogate_stats())
    p.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
