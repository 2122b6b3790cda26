"""ctypes mirror of include/drv.h (structs, enums and function prototypes).

The layout of every struct is checked against the C library's own sizeof at
load time (drv_struct_sizes), so a drifting header fails loudly.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

MAX_CASCADES = 4
MAX_LIGHTS = 16

# drv_status
OK, ERR_INVALID_ARG, ERR_CAPACITY, ERR_CUDA, ERR_TIMEOUT, ERR_NOT_SUPPORTED, ERR_NUMERIC = range(7)
STATUS_NAMES = {0: "DRV_OK", 1: "DRV_ERR_INVALID_ARG", 2: "DRV_ERR_CAPACITY", 3: "DRV_ERR_CUDA",
                4: "DRV_ERR_TIMEOUT", 5: "DRV_ERR_NOT_SUPPORTED", 6: "DRV_ERR_NUMERIC"}
DEVERR_CAPACITY, DEVERR_TIMEOUT, DEVERR_BOUNDS, DEVERR_NUMERIC = 0x1, 0x2, 0x4, 0x8
SH2_SIGN_REFERENCE, SH2_SIGN_FIXED = 0, 1
PRECISION_FP32, PRECISION_BF16 = 0, 1
VISIBILITY_CONE, VISIBILITY_SURROGATE = 0, 1
NORMAL_RG16I, NORMAL_F32X3 = 0, 1
ALBEDO_F32X3, ALBEDO_SRGB8 = 0, 1
ROUGH_METAL_RG8, ROUGH_METAL_F32 = 0, 1
RSM_F32, RSM_F16 = 0, 1
OUTPUT_RGB32F, OUTPUT_RGBA16F = 0, 1
OUTPUT_WRITE, OUTPUT_ADD = 0, 1

f3 = C.c_float * 3
f16 = C.c_float * 16


class DrvConfig(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("sh_order", C.c_int32),
                ("indirect_shadow", C.c_int32), ("max_cone_steps", C.c_int32),
                ("cascade_transition", C.c_float), ("n_cascades", C.c_int32), ("cav_res", C.c_int32),
                ("cascade_world_size", C.c_float * MAX_CASCADES), ("voxel_res", C.c_int32),
                ("max_caches", C.c_uint32), ("precision", C.c_int32), ("visibility", C.c_int32),
                ("surrogate_conf_threshold", C.c_float), ("sh2_sign", C.c_int32), ("max_lights", C.c_int32),
                ("max_rsm_resolution", C.c_int32), ("output_format", C.c_int32), ("output_blend", C.c_int32),
                ("specular_envmap_size", C.c_int32), ("specular_fill_level", C.c_int32)]


class DrvCascade(C.Structure):
    _fields_ = [("min", f3), ("world_voxel_size", C.c_float), ("max", f3), ("_pad0", C.c_float),
                ("decision_min", f3), ("_pad1", C.c_float), ("decision_max", f3), ("_pad2", C.c_float)]


class DrvVolumeInfo(C.Structure):
    _fields_ = [("volume_world_min", f3), ("voxel_size_in_world", C.c_float), ("volume_world_max", f3),
                ("cav_transition_zone_size", C.c_float), ("cascades", DrvCascade * MAX_CASCADES)]


class DrvPerFrame(C.Structure):
    _fields_ = [("view_projection", f16), ("inverse_view_projection", f16), ("camera_position", f3),
                ("_pad0", C.c_float), ("camera_direction", f3), ("_pad1", C.c_float)]


class DrvSpotLight(C.Structure):
    _fields_ = [("intensity", f3), ("shadow_normal_offset", C.c_float), ("shadow_bias", C.c_float),
                ("position", f3), ("direction", f3), ("cos_half_angle", C.c_float), ("view_projection", f16),
                ("inverse_view_projection", f16), ("rsm_render_resolution", C.c_int32),
                ("rsm_read_resolution", C.c_int32), ("val_area_factor", C.c_float),
                ("indirect_shadow_lod", C.c_float), ("indirect_shadow_block_size", C.c_float),
                ("indirect_shadow_sample_interval", C.c_int32), ("indirect_shadow_super_val_width", C.c_float),
                ("indirect_shadow_sampling_offset", C.c_float)]


class DrvLightDesc(C.Structure):
    _fields_ = [("intensity", f3), ("position", f3), ("direction", f3), ("half_angle", C.c_float),
                ("rsm_resolution", C.c_uint32), ("rsm_read_lod", C.c_uint32),
                ("indirect_shadow_lod", C.c_uint32), ("near_plane", C.c_float), ("far_plane", C.c_float)]


class DrvCamera(C.Structure):
    _fields_ = [("position", f3), ("direction", f3), ("up", f3), ("fov_y_deg", C.c_float), ("aspect", C.c_float),
                ("near_plane", C.c_float), ("far_plane", C.c_float)]


class DrvBox(C.Structure):
    _fields_ = [("min", f3), ("max", f3), ("albedo", f3), ("inward", C.c_int32)]


class DrvScene(C.Structure):
    _fields_ = [("n_boxes", C.c_int32), ("boxes", C.POINTER(DrvBox)), ("aabb_min", f3), ("aabb_max", f3)]


class DrvGBufferView(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("depth", C.c_void_p), ("normal", C.c_void_p),
                ("normal_format", C.c_int32), ("albedo", C.c_void_p), ("albedo_format", C.c_int32),
                ("rough_metal", C.c_void_p), ("rough_metal_format", C.c_int32)]


class DrvGBufferOut(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("normal_rg16i", C.c_void_p), ("normal_f32", C.c_void_p),
                ("albedo", C.c_void_p)]


class DrvMesh(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("albedo", C.c_void_p), ("indices", C.c_void_p),
                ("n_vertices", C.c_int32), ("n_triangles", C.c_int32)]


class DrvRSMView(C.Structure):
    _fields_ = [("resolution", C.c_int32), ("flux", C.c_void_p), ("normal", C.c_void_p),
                ("depth_lin_sq", C.c_void_p), ("format", C.c_int32)]


class DrvRSMOut(C.Structure):
    _fields_ = [("flux", C.c_void_p), ("normal", C.c_void_p), ("depth_lin_sq", C.c_void_p)]


class DrvVPL(C.Structure):
    _fields_ = [("flux", f3), ("disc_area", C.c_float), ("position", f3), ("_pad0", C.c_float), ("normal", f3),
                ("_pad1", C.c_float)]


class DrvShadowCone(C.Structure):
    _fields_ = [("average_val_position", f3), ("dist_to_sphere_rad", C.c_float)]


class DrvCacheCounter(C.Structure):
    _fields_ = [("groups_x", C.c_uint32), ("groups_y", C.c_uint32), ("groups_z", C.c_uint32),
                ("total_light_cache_count", C.c_int32)]


class DrvBuffers(C.Structure):
    _fields_ = [("cache_entries", C.c_void_p), ("entry_stride", C.c_uint32), ("cav_atlas", C.c_void_p),
                ("counter", C.c_void_p), ("voxel_bits", C.c_void_p), ("voxel_corners", C.c_void_p),
                ("voxel_mips", C.c_void_p * 16),
                ("n_voxel_levels", C.c_int32), ("vpls", C.c_void_p * MAX_LIGHTS),
                ("cones", C.c_void_p * MAX_LIGHTS), ("n_vpls", C.c_int32 * MAX_LIGHTS), ("n_lights", C.c_int32),
                ("voxel_mip_records", C.c_void_p * 16), ("n_record_levels", C.c_int32),
                ("specular_envmap", C.c_void_p * 8), ("specular_atlas_size", C.c_int32),
                ("n_specular_levels", C.c_int32)]


class DrvTuning(C.Structure):
    _fields_ = [("light_path", C.c_int32), ("pair_capacity", C.c_uint32), ("cone_ctas_per_sm", C.c_int32),
                ("gather_ctas_per_sm", C.c_int32), ("time_kernels", C.c_int32),
                ("plain_voxel_reads", C.c_int32), ("surrogate_wait_test", C.c_int32),
                ("count_voxel_reads", C.c_int32), ("check_inputs", C.c_int32),
                ("cull_caches_per_pass", C.c_int32), ("gather_threads", C.c_int32),
                ("tensor_core_apply", C.c_int32),
                ("per_light_dispatch", C.c_int32), ("gather_wait_test", C.c_int32)]


LIGHT_KERNELS = ("cull", "classify", "scatter", "mlp", "cone", "gather")


class DrvBatchScene(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("scene", C.c_void_p), ("gbuffer", C.c_void_p), ("frame", C.c_void_p),
                ("volume", C.c_void_p), ("lights", C.c_void_p), ("rsms", C.c_void_p), ("n_lights", C.c_int32),
                ("out_rgb", C.c_void_p)]


LIGHT_PATH_AUTO, LIGHT_PATH_SINGLE, LIGHT_PATH_SPLIT = 0, 1, 2

STRUCT_ORDER = [DrvConfig, DrvCascade, DrvVolumeInfo, DrvPerFrame, DrvSpotLight, DrvLightDesc, DrvCamera, DrvBox,
                DrvScene, DrvGBufferView, DrvGBufferOut, DrvRSMView, DrvRSMOut, DrvVPL, DrvShadowCone,
                DrvCacheCounter, DrvBuffers, DrvTuning, DrvMesh]

P = C.POINTER
VP = C.c_void_p
PROTOTYPES = {
    "drv_abi_version": (C.c_int, []),
    "drv_struct_sizes": (C.c_int, [P(C.c_uint32), C.c_int]),
    "drv_default_config": (None, [P(DrvConfig)]),
    "drv_create": (C.c_int, [P(DrvConfig), P(VP)]),
    "drv_destroy": (C.c_int, [VP]),
    "drv_set_stream": (C.c_int, [VP, VP]),
    "drv_sync": (C.c_int, [VP]),
    "drv_last_error_string": (C.c_char_p, [VP]),
    "drv_get_error": (C.c_int, [VP, P(C.c_uint32)]),
    "drv_get_buffers": (C.c_int, [VP, P(DrvBuffers)]),
    "drv_compute_volume_info": (C.c_int, [P(DrvConfig), P(C.c_float), P(C.c_float), P(C.c_float),
                                          P(DrvVolumeInfo)]),
    "drv_prepare_light": (C.c_int, [P(DrvLightDesc), P(DrvSpotLight)]),
    "drv_prepare_camera": (C.c_int, [P(DrvCamera), P(DrvPerFrame)]),
    "drv_generate_scene": (C.c_int, [C.c_uint64, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float,
                                     P(DrvBox), P(DrvScene)]),
    "drv_generate_camera": (C.c_int, [C.c_uint64, P(DrvScene), C.c_float, P(DrvCamera)]),
    "drv_generate_light": (C.c_int, [C.c_uint64, P(DrvScene), C.c_uint32, C.c_uint32, C.c_uint32, P(DrvLightDesc)]),
    "drv_raycast_gbuffer": (C.c_int, [VP, P(DrvScene), P(DrvCamera), P(DrvPerFrame), C.c_int32, C.c_int32,
                                      P(DrvGBufferOut)]),
    "drv_raycast_rsm": (C.c_int, [VP, P(DrvScene), P(DrvSpotLight), P(DrvRSMOut)]),
    "drv_raster_gbuffer": (C.c_int, [VP, P(DrvMesh), P(DrvCamera), P(DrvPerFrame), C.c_int32, C.c_int32,
                                     P(DrvGBufferOut)]),
    "drv_raster_rsm": (C.c_int, [VP, P(DrvMesh), P(DrvSpotLight), P(DrvRSMOut)]),
    "drv_prepare_rsm": (C.c_int, [VP, C.c_int32, P(DrvSpotLight), P(DrvRSMView)]),
    "drv_extract_vpls": (C.c_int, [VP, C.c_int32, P(DrvSpotLight)]),
    "drv_set_scene": (C.c_int, [VP, P(DrvScene)]),
    "drv_voxelize": (C.c_int, [VP, P(DrvScene), P(DrvVolumeInfo)]),
    "drv_voxelize_triangles": (C.c_int, [VP, VP, C.c_int32, VP, C.c_int32, P(DrvVolumeInfo)]),
    "drv_build_opacity_mips": (C.c_int, [VP]),
    "drv_allocate_caches": (C.c_int, [VP, P(DrvGBufferView), P(DrvPerFrame), P(DrvVolumeInfo)]),
    "drv_light_caches": (C.c_int, [VP, P(DrvSpotLight), C.c_int32, P(DrvVolumeInfo), P(DrvPerFrame)]),
    "drv_apply": (C.c_int, [VP, P(DrvGBufferView), P(DrvPerFrame), P(DrvVolumeInfo), VP]),
    "drv_frame": (C.c_int, [VP, P(DrvScene), P(DrvGBufferView), P(DrvPerFrame), P(DrvVolumeInfo),
                            P(DrvSpotLight), P(DrvRSMView), C.c_int32, VP]),
    "drv_get_cache_count": (C.c_int, [VP, P(C.c_uint32)]),
    "drv_set_surrogate_params": (C.c_int, [VP, VP]),
    "drv_set_surrogate_features": (C.c_int, [VP, C.c_int32]),
    "drv_get_cone_voxel_reads": (C.c_int, [VP, P(C.c_uint32)]),
    "drv_measure_load_bandwidth": (C.c_int, [C.c_int32, VP, C.c_size_t, C.c_int32, VP, P(C.c_float)]),
    "drv_surrogate_make_pairs": (C.c_int, [VP, C.c_uint64, C.c_int32, VP, VP]),
    "drv_surrogate_train_scratch_floats": (C.c_size_t, [C.c_int32]),
    "drv_surrogate_train_step": (C.c_int, [VP, VP, C.c_int32, VP, VP, VP, VP, C.c_int32, C.c_float, C.c_float,
                                           C.c_float, VP, VP]),
    "drv_surrogate_eval": (C.c_int, [VP, VP, C.c_int32, VP]),
    "drv_get_surrogate_fallbacks": (C.c_int, [VP, P(C.c_uint32)]),
    "drv_get_surrogate_stats": (C.c_int, [VP, P(C.c_uint32), P(C.c_uint32)]),
    "drv_set_tuning": (C.c_int, [VP, P(DrvTuning)]),
    "drv_get_tuning": (C.c_int, [VP, P(DrvTuning)]),
    "drv_get_light_kernel_ms": (C.c_int, [VP, P(C.c_float)]),
    "drv_get_light_pairs": (C.c_int, [VP, P(C.c_uint32)]),
    "drv_bruteforce_rsm": (C.c_int, [VP, P(DrvGBufferView), VP, P(DrvPerFrame), C.c_int32, VP]),
    "drv_prepare_specular_envmaps": (C.c_int, [VP]),
    "drv_write_pfm": (C.c_int, [C.c_char_p, P(C.c_float), C.c_int32, C.c_int32, C.c_int32]),
    "drv_read_pfm": (C.c_int, [C.c_char_p, P(C.c_float), C.c_int64, P(C.c_int32), P(C.c_int32)]),
    "drv_batch_create": (C.c_int, [P(DrvBatchScene), C.c_int32, C.c_int32, VP, P(VP)]),
    "drv_batch_launch": (C.c_int, [VP, VP]),
    "drv_batch_times": (C.c_int, [VP, P(C.c_float), P(C.c_float)]),
    "drv_batch_destroy": (C.c_int, [VP]),
    "drv_light_caches_static_scratch": (C.c_int, [P(DrvConfig), P(DrvVolumeInfo), P(VP), P(VP), P(C.c_int32),
                                                  P(C.c_int32), C.c_int32, VP, VP, VP, VP, VP]),
}
STATIC_SCRATCH_MAX_CACHES = 4096
SURROGATE_INPUTS = 32
SURROGATE_PARAMS = 10562
SURROGATE_ENUMERATE = 0xFFFFFFFFFFFFFFFF
SURROGATE_FEATURES_SEGMENT8 = 0  # the configuration's 17 inputs
SURROGATE_FEATURES_CONE4 = 1     # 27 inputs with the cone's first four samples
SURROGATE_FEATURES_CONE8 = 2     # 23 inputs with eight samples of the cone's own sampler
SURROGATE_FEATURE_NAMES = {"segment8": SURROGATE_FEATURES_SEGMENT8, "cone4": SURROGATE_FEATURES_CONE4,
                           "cone8": SURROGATE_FEATURES_CONE8}


def header_functions(header: Path) -> list[str]:
    """Names of every function declared in a C header (for export checks)."""
    import re
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(drv_[a-z0-9_]+)\s*\(", text)))


def bind(lib: C.CDLL) -> C.CDLL:
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    n = lib.drv_struct_sizes(None, 0)
    sizes = (C.c_uint32 * n)()
    lib.drv_struct_sizes(sizes, n)
    for st, sz in zip(STRUCT_ORDER, sizes):
        if C.sizeof(st) != sz:
            raise RuntimeError(f"ABI mismatch: sizeof({st.__name__}) is {sz} in C, {C.sizeof(st)} in Python")
    return lib
