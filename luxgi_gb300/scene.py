"""Seeded synthetic workloads of the DDGI probe-update path.

A workload is one DDGI volume (probe grid, rays, atlas sides, blend and
storage switches) plus the scene it traces (global SDF + surface cache).
The scene is generated on the host by libluxgi_scene (deterministic for a
seed); DeviceScene uploads it and runs the path's set-up stages on the GPU
(SDF mip, chunk culling) through the C ABI.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import _native as N


@dataclass(frozen=True)
class SceneSpec:
    seed: int
    room_size: float
    wall_thickness: float
    num_primitives: int
    sdf_resolution: int
    atlas_resolution: int
    sdf_format: int = N.STORAGE_FP32
    cascades: int = 1
    sphere_radius: tuple = (0.3, 1.5)
    box_half_extent: tuple = (0.2, 1.2)
    albedo_range: tuple = (0.1, 0.9)
    sun_direction: tuple = (0.0, 0.0, 0.0)     # zeros = seeded on the upper hemisphere
    sun_color: tuple = (2.0, 1.9, 1.7)
    tile_resolution: int = 0


@dataclass(frozen=True)
class VolumeSpec:
    probe_counts: tuple
    spacing: float
    rays_per_probe: int
    irradiance_side: int = 6
    depth_side: int = 14
    hysteresis: float = 0.98
    normal_bias: float = 0.1
    sharpness: float = 50.0
    ddgi_gamma: float = 5.0
    max_steps: int = 128
    storage: int = N.STORAGE_FP32
    light_mode: int = N.LIGHT_PER_HIT
    blend: int = N.BLEND_FP32
    infinite_bounce: bool = True
    intensity: float = 1.0
    sky: tuple = (0.5, 0.6, 0.8)
    march_variant: int = 0
    shade_variant: int = 0
    ray_order: int = 0
    march_budget: int = 0
    shade_order: int = 0
    shade_split: int = 0

    @property
    def probes(self) -> int:
        x, y, z = self.probe_counts
        return x * y * z

    def uniform(self, derive=None) -> N.DDGIUniform:
        """DDGIUniform of a grid centred on the origin, maxDistance = 1.5 x
        spacing (DDGIRenderer.cpp:665-683).  The atlas sizes come from
        luxgi_ddgi_derive_uniform, or from `derive(u)` when given (a
        CPU-only caller that must not load the CUDA library)."""
        u = N.DDGIUniform()
        for k in range(3):
            u.start_position[k] = -0.5 * (self.probe_counts[k] - 1) * self.spacing
            u.step[k] = self.spacing
            u.probe_counts[k] = self.probe_counts[k]
        u.max_distance = 1.5 * self.spacing
        u.sharpness = self.sharpness
        u.hysteresis = self.hysteresis
        u.normal_bias = self.normal_bias
        u.ddgi_gamma = self.ddgi_gamma
        u.irradiance_probe_side = self.irradiance_side
        u.depth_probe_side = self.depth_side
        u.rays_per_probe = self.rays_per_probe
        if derive is not None:
            derive(u)
        else:
            N.check(N.ddgi().luxgi_ddgi_derive_uniform(ctypes.byref(u)), "derive_uniform")
        return u

    def desc(self, derive=None) -> N.VolumeDesc:
        d = N.VolumeDesc()
        d.uniform = self.uniform(derive)
        d.storage = self.storage
        d.light_mode = self.light_mode
        d.blend = self.blend
        d.max_steps = self.max_steps
        d.infinite_bounce = 1 if self.infinite_bounce else 0
        d.intensity = self.intensity
        for k in range(3):
            d.sky_radiance[k] = self.sky[k]
        d.march_variant = self.march_variant
        d.shade_variant = self.shade_variant
        d.ray_order = self.ray_order
        d.march_budget = self.march_budget
        d.shade_order = self.shade_order
        d.shade_split = self.shade_split
        return d


@dataclass(frozen=True)
class Workload:
    name: str
    volume: VolumeSpec
    scene: SceneSpec
    frames: int


SEED0 = 0xC0FFEE

# Plain method, small: 8x4x8 probes at 1 m, 128 rays, 64^3 FP32 SDF over a
# 16 m room with 12 primitives, 512^2 atlases, 64 steps, h = 0.97, 8 frames.
PLAIN_SMALL = Workload(
    "plain_small_8x4x8_r128_sdf64",
    VolumeSpec((8, 4, 8), 1.0, 128, hysteresis=0.97, max_steps=64, light_mode=N.LIGHT_PER_HIT),
    SceneSpec(SEED0 + 1, 16.0, 0.5, 12, 64, 512),
    8,
)
# The same scene driven like the reference: 8/16 octahedral sides, the
# 250-step cap, FP16 storage and the light-cache bounce.
PLAIN_SMALL_REF = replace(
    PLAIN_SMALL, name="plain_small_refparity_8x4x8_r128_oct8_16",
    volume=replace(PLAIN_SMALL.volume, irradiance_side=8, depth_side=16, max_steps=250,
                   storage=N.STORAGE_FP16, light_mode=N.LIGHT_CACHE))
# Plain FP32 at production size: 32x16x32 probes, 256 rays (4.19M rays per
# frame), 256^3 FP32 SDF with 96 primitives in a 64 m scene, 2048^2 atlases,
# 128 steps, infinite bounce, 16 frames, one seeded sun.
PRODUCTION = Workload(
    "production_32x16x32_r256_sdf256",
    VolumeSpec((32, 16, 32), 1.9, 256, max_steps=128, light_mode=N.LIGHT_PER_HIT),
    SceneSpec(SEED0 + 2, 64.0, 1.0, 96, 256, 2048),
    16,
)
# Precision form: 64x32x64 probes, 256 rays (33.5M rays per frame), FP16 SDF
# marched in FP32, tensor-core blend.
PRECISION = Workload(
    "precision_64x32x64_r256_sdf256h",
    VolumeSpec((64, 32, 64), 0.95, 256, max_steps=128, light_mode=N.LIGHT_PER_HIT, blend=N.BLEND_TENSOR),
    SceneSpec(SEED0 + 3, 64.0, 1.0, 96, 256, 2048, sdf_format=N.STORAGE_FP16),
    16,
)

WORKLOADS = {w.name: w for w in (PLAIN_SMALL, PLAIN_SMALL_REF, PRODUCTION, PRECISION)}


def scaled(w: Workload, probe_counts=None, rays=None, sdf_resolution=None, atlas=None, num_primitives=None,
           name=None) -> Workload:
    """A smaller (or larger) variant of a workload with the same scene kind."""
    v = w.volume
    s = w.scene
    if probe_counts is not None:
        span = [(c - 1) * v.spacing for c in v.probe_counts]
        sp = min(span[k] / max(probe_counts[k] - 1, 1) for k in range(3)) if max(probe_counts) > 1 else v.spacing
        v = replace(v, probe_counts=tuple(probe_counts), spacing=max(sp, 1e-3))
    if rays is not None:
        v = replace(v, rays_per_probe=rays)
    if sdf_resolution is not None:
        s = replace(s, sdf_resolution=sdf_resolution)
    if atlas is not None:
        s = replace(s, atlas_resolution=atlas)
    if num_primitives is not None:
        s = replace(s, num_primitives=num_primitives)
    return replace(w, name=name or w.name + "_scaled", volume=v, scene=s)


# The production scene with an eighth of the probes (16x8x16 at 3.8 m):
# the case ncu captures are taken on (a few hundred MB on the device).
PRODUCTION_PROFILE = scaled(PRODUCTION, probe_counts=(16, 8, 16), name="production_16x8x16_r256_sdf256")
WORKLOADS[PRODUCTION_PROFILE.name] = PRODUCTION_PROFILE
# The precision scene at 32x16x32 probes: the case tensor-core blend
# captures are taken on.
PRECISION_PROFILE = scaled(PRECISION, probe_counts=(32, 16, 32), name="precision_32x16x32_r256_sdf256h")
WORKLOADS[PRECISION_PROFILE.name] = PRECISION_PROFILE


# Batching form: many volumes of uneven size, each with its own scene.  Grid
# dims log-uniform per axis from 4x4x4 to 32x16x32, rays per probe from
# {64, 128, 192, 256, 288}, FP16 SDF of 64^3-256^3 (multiples of 32; the room
# grows with it at a 0.25 m voxel), surface-cache atlas of 512^2-2048^2,
# tensor-core blend.
BATCH_RAYS = (64, 128, 192, 256, 288)


def batch_workloads(count: int = 48, seed: int = SEED0 + 4, max_counts=(32, 16, 32), min_counts=(4, 4, 4),
                    sdf_range=(64, 256), atlas_range=(512, 2048), blend: int = N.BLEND_TENSOR,
                    storage: int = N.STORAGE_FP32, max_steps: int = 128) -> list[Workload]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        counts = tuple(int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
                       for lo, hi in zip(min_counts, max_counts))
        rays = int(rng.choice(BATCH_RAYS))
        res = int(round(math.exp(rng.uniform(math.log(sdf_range[0]), math.log(sdf_range[1]))) / 32.0)) * 32
        res = min(max(res, sdf_range[0]), sdf_range[1])
        atlas = int(2 ** round(rng.uniform(math.log2(atlas_range[0]), math.log2(atlas_range[1]))))
        room = 0.25 * res
        prims = max(4, int(round(12 * (res / 64.0) ** 1.5)))
        spacing = 0.8 * room / max(counts)
        v = VolumeSpec(counts, spacing, rays, max_steps=max_steps, light_mode=N.LIGHT_PER_HIT, blend=blend,
                       storage=storage)
        sc = SceneSpec(seed * 1000 + i, room, 0.25 * room / 16.0, prims, res, atlas, sdf_format=N.STORAGE_FP16)
        out.append(Workload(f"batch{count}_v{i:02d}", v, sc, 16))
    return out


# --------------------------------------------------------------- host scene
class HostScene:
    """Scene arrays on the host (numpy), copied out of libluxgi_scene."""

    def __init__(self, spec: SceneSpec):
        lib = N.scene_lib()
        cfg = N.SceneConfig()
        cfg.seed = spec.seed
        cfg.room_size = spec.room_size
        cfg.wall_thickness = spec.wall_thickness
        cfg.num_primitives = spec.num_primitives
        cfg.sphere_radius[:] = list(spec.sphere_radius)
        cfg.box_half_extent[:] = list(spec.box_half_extent)
        cfg.sdf_resolution = spec.sdf_resolution
        cfg.cascades = spec.cascades
        cfg.sdf_format = spec.sdf_format
        cfg.atlas_resolution = spec.atlas_resolution
        cfg.albedo_range[:] = list(spec.albedo_range)
        cfg.sun_direction[:] = list(spec.sun_direction)
        cfg.sun_color[:] = list(spec.sun_color)
        cfg.tile_resolution = spec.tile_resolution
        h = ctypes.c_void_p()
        N.check(lib.luxgi_scene_build(ctypes.byref(cfg), ctypes.byref(h)), "scene_build")
        self._h = h
        v = N.SceneView()
        N.check(lib.luxgi_scene_view_get(h, ctypes.byref(v)), "scene_view")
        self.spec = spec
        self.sdf_data = N.SdfData.from_buffer_copy(v.sdf_data)
        self.sdf_format = v.sdf_format
        self.res = v.sdf_resolution
        self.mres = v.mip_resolution
        self.cascades = v.cascades
        n_sdf = self.res * self.cascades * self.res * self.res
        dt = np.uint16 if self.sdf_format == N.STORAGE_FP16 else np.float32
        self.sdf = np.ctypeslib.as_array(ctypes.cast(v.sdf, ctypes.POINTER(
            ctypes.c_uint16 if dt is np.uint16 else ctypes.c_float)), shape=(n_sdf,)).copy()
        self.surface_data = N.SurfaceData.from_buffer_copy(v.surface_data)
        self.num_objects = v.num_objects
        self.num_tiles = v.num_tiles
        self.objects = np.frombuffer(ctypes.string_at(v.objects, 128 * v.num_objects), dtype=np.uint8).copy()
        self.tiles = np.frombuffer(ctypes.string_at(v.tiles, 96 * v.num_tiles), dtype=np.uint8).copy()
        A = v.atlas_resolution
        self.atlas = A
        self.direct = np.frombuffer(ctypes.string_at(v.direct_light, A * A * 8), dtype=np.uint16).copy()
        self.depth = np.frombuffer(ctypes.string_at(v.depth, A * A * 4), dtype=np.float32).copy()
        self.albedo = np.frombuffer(ctypes.string_at(v.albedo, A * A * 4), dtype=np.uint8).copy()
        self.gbuffer0 = np.frombuffer(ctypes.string_at(v.gbuffer0, A * A * 16), dtype=np.float32).copy()
        self.gbuffer1 = np.frombuffer(ctypes.string_at(v.gbuffer1, A * A * 16), dtype=np.float32).copy()
        self.pbr = np.frombuffer(ctypes.string_at(v.pbr, A * A * 4), dtype=np.uint8).copy()
        self.emissive = np.frombuffer(ctypes.string_at(v.emissive, A * A * 8), dtype=np.uint16).copy()
        prims = (N.ScenePrimitive * v.num_primitives).from_address(v.primitives)
        self.primitives = [(p.kind, tuple(p.center), tuple(p.half_extent), tuple(p.albedo)) for p in prims]
        self.sun_direction = tuple(v.sun_direction)

    def distance(self, p) -> float:
        return float(N.scene_lib().luxgi_scene_distance(self._h, N.floats(p)))

    def sdf_float(self) -> np.ndarray:
        if self.sdf_format == N.STORAGE_FP16:
            return self.sdf.view(np.float16).astype(np.float32)
        return self.sdf

    def cull_capacity(self) -> int:
        return 1 + 40 * 40 * 40 * (self.num_objects + 1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.scene_lib().luxgi_scene_destroy(h)
            self._h = None


# ------------------------------------------------------------- device scene
class DeviceScene:
    """The scene resident in HBM, with the SDF mip and culling built on the
    GPU through the C ABI."""

    def __init__(self, host: HostScene, light_mode: int, device: str = "cuda"):
        import torch

        self.host = host
        self.light_mode = light_mode
        dev = torch.device(device)
        self.device = dev
        lib = N.ddgi()
        sdf_t = torch.from_numpy(host.sdf.view(np.int16) if host.sdf_format == N.STORAGE_FP16 else host.sdf)
        self.sdf = sdf_t.to(dev)
        elem = torch.int16 if host.sdf_format == N.STORAGE_FP16 else torch.float32
        C, m = host.cascades, host.mres
        self.mip = torch.zeros(m * C * m * m, dtype=elem, device=dev)
        self.mip_tmp = torch.zeros(m * m * m, dtype=elem, device=dev)
        self.sdf_desc = N.SdfDesc()
        self.sdf_desc.data = host.sdf_data
        self.sdf_desc.format = host.sdf_format
        self.sdf_desc.resolution = host.res
        self.sdf_desc.mip_resolution = host.mres
        self.sdf_desc.sdf = self.sdf.data_ptr()
        self.sdf_desc.mip = self.mip.data_ptr()
        stream = torch.cuda.current_stream(dev).cuda_stream
        N.check(lib.luxgi_sdf_build_mip(ctypes.byref(self.sdf_desc), self.mip.data_ptr(), self.mip_tmp.data_ptr(),
                                        stream), "sdf_build_mip")
        self.objects = torch.from_numpy(host.objects).to(dev)
        self.tiles = torch.from_numpy(host.tiles).to(dev)
        self.depth = torch.from_numpy(host.depth).to(dev)
        self.direct = torch.from_numpy(host.direct.view(np.int16)).to(dev)
        self.light_cache = self.direct.clone()
        self.albedo = torch.from_numpy(host.albedo).to(dev)
        self.gbuffer0 = torch.from_numpy(host.gbuffer0).to(dev)
        self.gbuffer1 = torch.from_numpy(host.gbuffer1).to(dev)
        self.pbr = torch.from_numpy(host.pbr).to(dev)
        self.emissive = torch.from_numpy(host.emissive.view(np.int16)).to(dev)
        cap = host.cull_capacity()
        self.capacity = cap
        self.chunks = torch.zeros(40 * 40 * 40, dtype=torch.int32, device=dev)
        self.culled = torch.zeros(cap, dtype=torch.int32, device=dev)
        sd = N.SurfaceData.from_buffer_copy(host.surface_data)
        sd.culled_objects_capacity = cap
        self.surface_desc = N.SurfaceDesc()
        self.surface_desc.data = sd
        self.surface_desc.num_objects = host.num_objects
        self.surface_desc.num_tiles = host.num_tiles
        self.surface_desc.objects = self.objects.data_ptr()
        self.surface_desc.tiles = self.tiles.data_ptr()
        self.surface_desc.chunks = self.chunks.data_ptr()
        self.surface_desc.culled_objects = self.culled.data_ptr()
        self.surface_desc.light_cache = self.light_cache.data_ptr()
        self.surface_desc.depth = self.depth.data_ptr()
        self.surface_desc.direct_light = self.direct.data_ptr()
        self.surface_desc.albedo = self.albedo.data_ptr()
        self.surface_desc.gbuffer0 = self.gbuffer0.data_ptr()
        self.surface_desc.gbuffer1 = self.gbuffer1.data_ptr()
        self.surface_desc.pbr = self.pbr.data_ptr()
        self.surface_desc.emissive = self.emissive.data_ptr()
        N.check(lib.luxgi_surface_cull(ctypes.byref(self.surface_desc), self.chunks.data_ptr(),
                                       self.culled.data_ptr(), cap, stream), "surface_cull")

    def set_surface_formats(self, light_format: int, gbuffer_format: int, direct, emissive, gbuffer0,
                            gbuffer1) -> None:
        """Re-binds the surface cache in other texture formats: the colour
        textures (direct light; the light cache, a copy of it; emissive) in
        `light_format` (luxgi_color_format: uint32 a texel for R11G11B10F,
        4 x uint16 for RGBA16F) and the G-buffers in `gbuffer_format` (4 x
        float32 or 4 x uint16 a texel), from host arrays already in those
        formats -- the engine's own surface textures are R11G11B10F and
        RGBA16F."""
        import torch

        def up(a):
            a = np.ascontiguousarray(a)
            view = {np.dtype(np.uint32): np.int32, np.dtype(np.uint16): np.int16}.get(a.dtype, a.dtype)
            return torch.from_numpy(a.view(view)).to(self.device)

        self.direct = up(direct)
        self.light_cache = self.direct.clone()
        self.emissive = up(emissive)
        self.gbuffer0 = up(gbuffer0)
        self.gbuffer1 = up(gbuffer1)
        d = self.surface_desc
        d.direct_light = self.direct.data_ptr()
        d.light_cache = self.light_cache.data_ptr()
        d.emissive = self.emissive.data_ptr()
        d.gbuffer0 = self.gbuffer0.data_ptr()
        d.gbuffer1 = self.gbuffer1.data_ptr()
        d.light_format = int(light_format)
        d.gbuffer_format = int(gbuffer_format)

    def nbytes(self) -> int:
        ts = [self.sdf, self.mip, self.mip_tmp, self.objects, self.tiles, self.depth, self.direct, self.light_cache,
              self.albedo, self.gbuffer0, self.gbuffer1, self.pbr, self.emissive, self.chunks, self.culled]
        return sum(t.numel() * t.element_size() for t in ts)
