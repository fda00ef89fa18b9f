"""ctypes mirror of include/luxgi_ddgi.h and include/luxgi_scene.h.

The libraries are loaded from luxgi_gb300/lib/ (built in-tree by
luxgi_gb300.build).  There is no fallback: if a library is missing the
import raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint16, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"

# status codes
LUXGI_OK = 0
LUXGI_EINVAL = -1
LUXGI_ENOMEM = -2
LUXGI_ECUDA = -3
LUXGI_ETIMEOUT = -4
LUXGI_ENOTBOUND = -5
LUXGI_EUNSUPPORTED = -6
LUXGI_ESCRATCH = -7

STORAGE_FP32 = 0
STORAGE_FP16 = 1
LIGHT_CACHE = 0
LIGHT_PER_HIT = 1
LIGHT_DIRECTIONAL = 0
LIGHT_SPOT = 1
LIGHT_POINT = 2
MAX_LIGHTS = 32
BLEND_FP32 = 0
BLEND_TENSOR = 1
COLOR_RGBA16F = 0
COLOR_R11G11B10F = 1
GBUFFER_RGBA32F = 0
GBUFFER_RGBA16F = 1


class DDGIUniform(ctypes.Structure):
    """DDGIUniform (Shaders/DDGI/DDGICommon.glsl:11-31), 96 bytes."""
    _fields_ = [
        ("start_position", c_float * 4), ("step", c_float * 4), ("probe_counts", c_int32 * 4),
        ("max_distance", c_float), ("sharpness", c_float), ("hysteresis", c_float), ("normal_bias", c_float),
        ("ddgi_gamma", c_float), ("irradiance_probe_side", c_int32), ("irradiance_width", c_int32),
        ("irradiance_height", c_int32), ("depth_probe_side", c_int32), ("depth_width", c_int32),
        ("depth_height", c_int32), ("rays_per_probe", c_int32),
    ]


class SdfData(ctypes.Structure):
    """GlobalSDFData (Shaders/SDF/GlobalSDFData.glsl), 96 bytes."""
    _fields_ = [("cascade_pos_distance", (c_float * 4) * 4), ("cascade_voxel_size", c_float * 4),
                ("cascades_count", c_uint32), ("resolution", c_float), ("near_plane", c_float), ("far_plane", c_float)]


class SurfaceData(ctypes.Structure):
    """GlobalSurfaceAtlasData (Shaders/SDF/AtlasCommon.glsl:8-16), 32 bytes."""
    _fields_ = [("camera_pos", c_float * 3), ("chunk_size", c_float), ("culled_objects_capacity", c_uint32),
                ("resolution", c_uint32), ("objects_count", c_uint32), ("padding", c_uint32)]


class SurfaceObject(ctypes.Structure):
    _fields_ = [("object_bounds", c_float * 4), ("tile_offset", c_uint32 * 6), ("padding", c_int32 * 2),
                ("transform", c_float * 16), ("extends", c_float * 4)]


class SurfaceTile(ctypes.Structure):
    _fields_ = [("extends", c_float * 4), ("transform", c_float * 16), ("object_bounds", c_float * 4)]


class SdfDesc(ctypes.Structure):
    _fields_ = [("data", SdfData), ("format", c_int32), ("resolution", c_int32), ("mip_resolution", c_int32),
                ("reserved", c_int32), ("sdf", c_void_p), ("mip", c_void_p)]


class SurfaceDesc(ctypes.Structure):
    _fields_ = [("data", SurfaceData), ("num_objects", c_int32), ("num_tiles", c_int32), ("objects", c_void_p),
                ("tiles", c_void_p), ("chunks", c_void_p), ("culled_objects", c_void_p), ("light_cache", c_void_p),
                ("depth", c_void_p), ("direct_light", c_void_p), ("albedo", c_void_p), ("gbuffer0", c_void_p),
                ("gbuffer1", c_void_p), ("pbr", c_void_p), ("emissive", c_void_p), ("light_format", c_int32),
                ("gbuffer_format", c_int32)]


class Light(ctypes.Structure):
    _fields_ = [("color", c_float * 4), ("position", c_float * 4), ("direction", c_float * 4), ("intensity", c_float),
                ("radius", c_float), ("type", c_float), ("angle", c_float)]


class SurfaceLighting(ctypes.Structure):
    _fields_ = [("lights", c_void_p), ("num_lights", c_int32), ("num_tiles", c_int32), ("tiles", c_void_p),
                ("light_masks", c_void_p), ("camera_pos", c_float * 3), ("shadow_bias", c_float),
                ("copy_emissive", c_int32), ("max_steps", c_int32), ("reserved", c_int32 * 2)]


class MeshSdf(ctypes.Structure):
    _fields_ = [("aabb_min", c_float * 3), ("aabb_max", c_float * 3), ("local_to_uvw_add", c_float * 3),
                ("local_to_uvw_mul", c_float * 3), ("max_distance", c_float), ("size", c_int32 * 3),
                ("mip_count", c_int32), ("reserved", c_int32), ("mips", c_void_p * 3)]


class SdfObject(ctypes.Structure):
    _fields_ = [("world", c_float * 16), ("mesh", c_int32), ("reserved", c_int32 * 3)]


class SdfBuildDesc(ctypes.Structure):
    _fields_ = [("gi_distance", c_float), ("global_scale", c_float), ("min_object_radius", c_float),
                ("resolution", c_int32), ("cascades", c_int32), ("format", c_int32), ("near_plane", c_float),
                ("far_plane", c_float)]


class SdfRasterObject(ctypes.Structure):
    _fields_ = [("world_to_volume", c_float * 16), ("volume_to_world", c_float * 16), ("volume_to_uvw_mul", c_float * 3),
                ("mip_offset", c_float), ("volume_to_uvw_add", c_float * 3), ("decode_mul", c_float),
                ("volume_local_bounds_extent", c_float * 3), ("decode_add", c_float)]


SDF_CHUNK = 32
SDF_CHUNK_MODELS = 28


class SdfChunk(ctypes.Structure):
    _fields_ = [("coord", c_int32 * 3), ("count", c_int32), ("models", c_uint32 * SDF_CHUNK_MODELS)]


class MeshSdfFile(ctypes.Structure):
    _fields_ = [("size", c_int32 * 3), ("mip_count", c_int32), ("mip_offset", ctypes.c_uint64 * 3),
                ("mip_bytes", ctypes.c_uint64 * 3)]


class VolumeDesc(ctypes.Structure):
    _fields_ = [("uniform", DDGIUniform), ("storage", c_int32), ("light_mode", c_int32), ("blend", c_int32),
                ("max_steps", c_int32), ("infinite_bounce", c_int32), ("intensity", c_float),
                ("sky_radiance", c_float * 3), ("march_variant", c_int32), ("shade_variant", c_int32),
                ("ray_order", c_int32), ("march_budget", c_int32), ("shade_order", c_int32), ("shade_split", c_int32),
                ("reserved", c_int32 * 2)]


class Atlases(ctypes.Structure):
    _fields_ = [("irradiance", c_void_p), ("distance", c_void_p), ("prev_irradiance", c_void_p),
                ("prev_distance", c_void_p), ("irradiance_width", c_int32), ("irradiance_height", c_int32),
                ("depth_width", c_int32), ("depth_height", c_int32), ("storage", c_int32), ("frames", c_int32)]


class Rays(ctypes.Structure):
    _fields_ = [("directions", c_void_p), ("radiance", c_void_p), ("hit_info", c_void_p), ("probes", c_int32),
                ("rays", c_int32), ("storage", c_int32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("march_variant", c_int32), ("march_threads", c_int32), ("shade_variant", c_int32),
                ("blend_probes", c_int32), ("use_graph", c_int32), ("march_budget", c_int32), ("shade_order", c_int32),
                ("reserved", c_int32 * 1), ("frame_ms", c_float)]


class ServerDesc(ctypes.Structure):
    _fields_ = [("memory_budget", c_uint64), ("executor", c_int32), ("max_group", c_int32),
                ("max_inflight", c_int32), ("reserved0", c_int32), ("tuning", BatchTuning), ("sim_rate", ctypes.c_double),
                ("sim_admit_s", ctypes.c_double), ("sim_evict_s", c_float), ("reserved", c_int32 * 3)]


class SessionScene(ctypes.Structure):
    _fields_ = [("sdf", SdfDesc), ("surface", SurfaceDesc), ("atlas_resolution", c_int32), ("reserved", c_int32 * 3)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, c_uint64) for n in ("submitted", "completed", "pending", "inflight_groups", "admissions",
                                        "evictions", "rejected", "resident_sessions", "resident_bytes",
                                        "peak_resident_bytes", "groups", "probe_rays", "max_overlap")] + \
               [(n, ctypes.c_double) for n in ("mean_group", "latency_ms_p50", "latency_ms_p95", "latency_ms_p99",
                                               "latency_ms_mean", "latency_ms_max", "wall_s")]


SERVE_EXEC_CUDA = 0
SERVE_EXEC_SIM = 1


class SceneConfig(ctypes.Structure):
    _fields_ = [("seed", c_uint64), ("room_size", c_float), ("wall_thickness", c_float), ("num_primitives", c_int32),
                ("sphere_radius", c_float * 2), ("box_half_extent", c_float * 2), ("sdf_resolution", c_int32),
                ("cascades", c_int32), ("sdf_format", c_int32), ("atlas_resolution", c_int32),
                ("albedo_range", c_float * 2), ("sun_direction", c_float * 3), ("sun_color", c_float * 3),
                ("tile_resolution", c_int32), ("reserved", c_int32 * 4)]


class ScenePrimitive(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("center", c_float * 3), ("half_extent", c_float * 3), ("albedo", c_float * 3)]


class SceneView(ctypes.Structure):
    _fields_ = [("sdf_data", SdfData), ("sdf_format", c_int32), ("sdf_resolution", c_int32),
                ("mip_resolution", c_int32), ("cascades", c_int32), ("sdf", c_void_p), ("sdf_bytes", c_int64),
                ("surface_data", SurfaceData), ("num_objects", c_int32), ("num_tiles", c_int32), ("objects", c_void_p),
                ("tiles", c_void_p), ("atlas_resolution", c_int32), ("direct_light", c_void_p), ("depth", c_void_p),
                ("albedo", c_void_p), ("gbuffer0", c_void_p), ("gbuffer1", c_void_p), ("num_primitives", c_int32),
                ("primitives", c_void_p), ("sun_direction", c_float * 3), ("sun_color", c_float * 3),
                ("pbr", c_void_p), ("emissive", c_void_p)]


assert ctypes.sizeof(DDGIUniform) == 96
assert ctypes.sizeof(SdfData) == 96
assert ctypes.sizeof(SurfaceData) == 32
assert ctypes.sizeof(SurfaceObject) == 128
assert ctypes.sizeof(SurfaceTile) == 96
assert ctypes.sizeof(Light) == 64
assert ctypes.sizeof(MeshSdf) == 96
assert ctypes.sizeof(SdfObject) == 80
assert ctypes.sizeof(SdfRasterObject) == 176
assert ctypes.sizeof(SdfChunk) == 128
assert ctypes.sizeof(SurfaceLighting) == 64

# (name, restype, argtypes) of every exported entry point, as declared in
# include/luxgi_ddgi.h
DDGI_API = [
    ("luxgi_ddgi_derive_uniform", c_int, [POINTER(DDGIUniform)]),
    ("luxgi_ddgi_rotation", c_int, [POINTER(c_float), c_float, POINTER(c_float)]),
    ("luxgi_ddgi_frame_rotation", c_int, [c_uint64, c_uint32, POINTER(c_float)]),
    ("luxgi_ddgi_create", c_int, [POINTER(VolumeDesc), POINTER(c_void_p)]),
    ("luxgi_ddgi_destroy", c_int, [c_void_p]),
    ("luxgi_ddgi_bind_scene", c_int, [c_void_p, POINTER(SdfDesc), POINTER(SurfaceDesc)]),
    ("luxgi_ddgi_trace", c_int, [c_void_p, POINTER(c_float), c_void_p]),
    ("luxgi_ddgi_probe_update", c_int, [c_void_p, c_void_p]),
    ("luxgi_ddgi_border_update", c_int, [c_void_p, c_void_p]),
    ("luxgi_ddgi_end_frame", c_int, [c_void_p]),
    ("luxgi_ddgi_update", c_int, [c_void_p, POINTER(c_float), c_void_p]),
    ("luxgi_ddgi_update_batch", c_int, [POINTER(c_void_p), c_int, POINTER(c_float), c_void_p]),
    ("luxgi_ddgi_batch_create", c_int, [POINTER(c_void_p), c_int, POINTER(BatchTuning), POINTER(c_void_p)]),
    ("luxgi_ddgi_batch_update", c_int, [c_void_p, POINTER(c_float), c_void_p]),
    ("luxgi_ddgi_batch_autotune", c_int, [c_void_p, c_int, c_void_p, POINTER(BatchTuning)]),
    ("luxgi_ddgi_batch_get_tuning", c_int, [c_void_p, POINTER(BatchTuning)]),
    ("luxgi_ddgi_batch_set_tuning", c_int, [c_void_p, POINTER(BatchTuning)]),
    ("luxgi_ddgi_batch_destroy", c_int, [c_void_p]),
    ("luxgi_ddgi_set_stage_timing", c_int, [c_void_p, c_int]),
    ("luxgi_ddgi_stage_times", c_int, [c_void_p, POINTER(c_float)]),
    ("luxgi_ddgi_get_atlases", c_int, [c_void_p, POINTER(Atlases)]),
    ("luxgi_ddgi_get_rays", c_int, [c_void_p, POINTER(Rays)]),
    ("luxgi_ddgi_check_status", c_int, [c_void_p, c_void_p]),
    ("luxgi_ddgi_set_debug_rays", c_int, [c_void_p, c_int]),
    ("luxgi_ddgi_set_blend_wait_test", c_int, [c_void_p, c_int64, c_int]),
    ("luxgi_ddgi_load_atlases", c_int, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p]),
    ("luxgi_ddgi_inject_indirect", c_int, [c_void_p, c_void_p]),
    ("luxgi_ddgi_save_atlases", c_int, [c_void_p, c_void_p, c_void_p, POINTER(c_int32), c_void_p]),
    ("luxgi_ddgi_sample_probe_image", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, POINTER(c_float),
                                              POINTER(c_float), c_void_p, c_void_p]),
    ("luxgi_ddgi_sample_irradiance", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("luxgi_sdf_build_mip", c_int, [POINTER(SdfDesc), c_void_p, c_void_p, c_void_p]),
    ("luxgi_sdf_build_mip_noalloc", c_int, [POINTER(SdfDesc), c_void_p, c_void_p]),
    ("luxgi_surface_cull", c_int, [POINTER(SurfaceDesc), c_void_p, c_void_p, c_uint32, c_void_p]),
    ("luxgi_surface_light", c_int, [POINTER(SdfDesc), POINTER(SurfaceDesc), POINTER(SurfaceLighting), c_void_p,
                                    c_void_p]),
    ("luxgi_sdf_cascade_layout", c_int, [POINTER(SdfBuildDesc), POINTER(SdfData)]),
    ("luxgi_sdf_build_plan", c_int, [POINTER(SdfBuildDesc), c_void_p, c_int, c_void_p, c_int, c_int, c_void_p, c_int,
                                     POINTER(c_int), c_void_p, c_void_p, c_int, POINTER(c_int)]),
    ("luxgi_sdf_build", c_int, [POINTER(SdfBuildDesc), c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                POINTER(SdfData), c_void_p]),
    ("luxgi_mesh_sdf_parse", c_int, [c_void_p, ctypes.c_uint64, POINTER(MeshSdfFile)]),
    ("luxgi_strerror", ctypes.c_char_p, [c_int]),
    ("luxgi_launch_count", c_uint64, []),
]

SERVE_API = [
    ("luxgi_server_create", c_int, [POINTER(ServerDesc), POINTER(c_void_p)]),
    ("luxgi_server_destroy", c_int, [c_void_p]),
    ("luxgi_server_add_session", c_int, [c_void_p, POINTER(VolumeDesc), POINTER(SessionScene), POINTER(c_int32)]),
    ("luxgi_server_session_bytes", c_int, [c_void_p, c_int32, POINTER(c_uint64)]),
    ("luxgi_server_submit", c_int, [c_void_p, c_int32, POINTER(c_float), POINTER(c_uint64)]),
    ("luxgi_server_drain", c_int, [c_void_p, ctypes.c_double]),
    ("luxgi_server_run_poisson", c_int, [c_void_p, POINTER(c_int32), c_int, ctypes.c_double, ctypes.c_double,
                                         c_uint64]),
    ("luxgi_server_stats_get", c_int, [c_void_p, POINTER(ServerStats), c_int]),
    ("luxgi_server_touch", c_int, [c_void_p, c_int32]),
    ("luxgi_server_session_atlases", c_int, [c_void_p, c_int32, POINTER(Atlases)]),
    ("luxgi_server_session_state", c_int, [c_void_p, c_int32, POINTER(c_int32), POINTER(c_int32)]),
]

SCENE_API = [
    ("luxgi_scene_build", c_int, [POINTER(SceneConfig), POINTER(c_void_p)]),
    ("luxgi_scene_view_get", c_int, [c_void_p, POINTER(SceneView)]),
    ("luxgi_scene_destroy", c_int, [c_void_p]),
    ("luxgi_scene_distance", c_float, [c_void_p, POINTER(c_float)]),
    ("luxgi_float_to_half", c_uint16, [c_float]),
    ("luxgi_half_to_float", c_float, [c_uint16]),
]


def _load(name: str, api) -> ctypes.CDLL:
    path = LIB_DIR / name
    if not path.exists():
        raise ImportError(f"{path} is missing: build it with luxgi_gb300.build.build_all() "
                          "(the DDGI path has no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for fname, res, args in api:
        fn = getattr(lib, fname)
        fn.restype = res
        fn.argtypes = args
    return lib


_ddgi = None
_scene = None


def ddgi() -> ctypes.CDLL:
    global _ddgi
    if _ddgi is None:
        _ddgi = _load("libluxgi_ddgi.so", DDGI_API + SERVE_API)
    return _ddgi


def scene_lib() -> ctypes.CDLL:
    global _scene
    if _scene is None:
        _scene = _load("libluxgi_scene.so", SCENE_API)
    return _scene


class LuxgiError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        msg = ddgi().luxgi_strerror(status).decode() if _ddgi is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})")


def check(status: int, what: str) -> None:
    if status != LUXGI_OK:
        raise LuxgiError(status, what)


def floats(vals) -> ctypes.Array:
    arr = (c_float * len(vals))(*[float(v) for v in vals])
    return arr
