"""Surface-cache lighting above the C ABI.

Mirrors the reference's deferred-lighting system of the global surface
atlas (Engine/DDGI/GlobalSurfaceAtlas.cpp:789-996):

* `make_light` builds a `luxgi_light` (Common/Light.glsl:19-28);
* `LightingSchedule` decides which camera-culled objects are redrawn this
  frame (:826-870: every object when a directional light is due or every
  GI_FRAMES frames, else the objects near point and spot lights that are
  due);
* `select_tiles` turns the redrawn objects into the tile list and per-tile
  light masks of one `luxgi_surface_light` call (:873-944: every tile of a
  redrawn object gets the emissive copy; a light draws the tiles of objects
  within its radius, a directional light only tiles whose view direction
  has a positive dot product with its direction);
* `SurfaceLighting` runs that pass on the GPU for a `DeviceScene`, writing
  the scene's direct-light atlas that light-cache injection then reads.

One deliberate difference: the reference appends an object to its redraw
list once per due point or spot light that reaches it, so an object near two
such lights is drawn twice by every light that frame (its light cache gets
twice the direct light).  `LightingSchedule` lists each object once.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

REDRAW_FRAMES = 120     # REDRWA_FRAMES (STATIC_REDRWA_FRAMES), GlobalSurfaceAtlas.cpp:48-49
GI_FRAMES = 15          # GI_FRAMES, :50
SHADOW_BIAS = 1.0       # GlobalSurface::shadowBias default, :99
SHADOW_MAX_STEPS = 250  # tracyGlobalSDF step cap, SDFCommon.glsl:143


def make_light(kind: int, color=(1.0, 1.0, 1.0), intensity: float = 1.0, position=(0.0, 0.0, 0.0),
               direction=(0.0, -1.0, 0.0), radius: float = 1.0, angle: float = 0.0) -> N.Light:
    """A luxgi_light; `direction` is normalised (directional and spot)."""
    if kind not in (N.LIGHT_DIRECTIONAL, N.LIGHT_SPOT, N.LIGHT_POINT):
        raise ValueError(f"light type {kind}")
    d = np.asarray(direction, dtype=np.float64)
    n = float(np.linalg.norm(d))
    if n > 0.0:
        d = d / n
    L = N.Light()
    L.color[:] = [float(color[0]), float(color[1]), float(color[2]), 1.0]
    L.position[:] = [float(position[0]), float(position[1]), float(position[2]), 1.0]
    L.direction[:] = [float(d[0]), float(d[1]), float(d[2]), 0.0]
    L.intensity = float(intensity)
    L.radius = float(radius)
    L.type = float(kind)
    L.angle = float(angle)
    return L


def light_array(lights) -> ctypes.Array:
    if len(lights) > N.MAX_LIGHTS:
        raise ValueError(f"at most {N.MAX_LIGHTS} lights per pass")
    arr = (N.Light * max(1, len(lights)))()
    for i, L in enumerate(lights):
        arr[i] = L
    return arr


def scene_lights(host, count: int = 3, seed: int = 0) -> list:
    """The scene's sun as a directional light plus `count - 1` seeded point
    and spot lights inside the room."""
    sun = np.asarray(host.sun_direction, dtype=np.float64)
    out = [make_light(N.LIGHT_DIRECTIONAL, (1.0, 0.96, 0.9), 2.0, direction=-sun)]
    rng = np.random.default_rng(seed)
    half = 0.5 * float(host.spec.room_size) - float(host.spec.wall_thickness)
    for i in range(1, count):
        pos = rng.uniform(-0.8 * half, 0.8 * half, size=3)
        col = rng.uniform(0.3, 1.0, size=3)
        if i % 2:
            out.append(make_light(N.LIGHT_POINT, col, float(rng.uniform(1.0, 4.0)), position=pos,
                                  radius=float(rng.uniform(0.5, 1.0) * half)))
        else:
            out.append(make_light(N.LIGHT_SPOT, col, float(rng.uniform(1.0, 4.0)), position=pos,
                                  direction=rng.normal(size=3), radius=float(rng.uniform(0.5, 1.0) * half),
                                  angle=float(rng.uniform(0.1, 0.5))))
    return out


def _objects(objects_bytes: np.ndarray, n: int) -> ctypes.Array:
    return (N.SurfaceObject * n).from_buffer_copy(np.ascontiguousarray(objects_bytes).tobytes())


def _tiles(tiles_bytes: np.ndarray, n: int) -> ctypes.Array:
    return (N.SurfaceTile * n).from_buffer_copy(np.ascontiguousarray(tiles_bytes).tobytes())


def tile_view_directions(tiles_bytes: np.ndarray, n: int) -> np.ndarray:
    """SurfaceAtlasTile::viewDirection of every tile slot (float32 [n, 3]).
    The tile transform is the lookAt view matrix with the translation zeroed
    (GlobalSurfaceAtlas.cpp:263-278), whose third row is -viewDirection."""
    t = _tiles(tiles_bytes, n)
    out = np.zeros((n, 3), dtype=np.float32)
    for i in range(n):
        m = t[i].transform
        out[i] = (-m[2], -m[6], -m[10])
    return out


def select_tiles(host, updated, lights) -> tuple[np.ndarray, np.ndarray]:
    """The tile list and per-tile light masks (bit l = light l draws the
    tile) of one pass over the redrawn objects `updated` (object indices):
    GlobalSurfaceAtlas.cpp:873-883 (emissive copy of every tile) and
    :912-944 (per-light object and tile selection)."""
    objs = _objects(host.objects, host.num_objects)
    view = tile_view_directions(host.tiles, host.num_tiles)
    order: list[int] = []
    mask: dict[int, int] = {}
    for o in updated:
        for i in range(6):
            t = int(objs[o].tile_offset[i])
            if t and t not in mask:
                mask[t] = 0
                order.append(t)
    for li, L in enumerate(lights):
        lpos = np.array(L.position[:3], dtype=np.float32)
        ldir = np.array(L.direction[:3], dtype=np.float32)
        for o in updated:
            ob = objs[o]
            if L.type in (float(N.LIGHT_POINT), float(N.LIGHT_SPOT)):
                center = np.array(ob.object_bounds[:3], dtype=np.float32)
                if float(np.linalg.norm(center - lpos)) > float(np.float32(ob.object_bounds[3]) + np.float32(L.radius)):
                    continue
            for i in range(6):
                t = int(ob.tile_offset[i])
                if not t:
                    continue
                if L.type == float(N.LIGHT_DIRECTIONAL) and float(np.dot(view[t], ldir)) < 1e-6:
                    continue
                mask[t] |= 1 << li
    tiles = np.array(order, dtype=np.uint32)
    masks = np.array([mask[t] for t in order], dtype=np.uint32)
    return tiles, masks


class LightingSchedule:
    """Which camera-culled objects get their surface lighting redrawn in a
    frame (GlobalSurfaceAtlas.cpp:826-870).  Per light it keeps the frame it
    was last used and last updated (component::LightFrameData, :80-84)."""

    def __init__(self):
        self.last_gi_updated = 0
        self.last_used: dict[int, int] = {}
        self.last_updated: dict[int, int] = {}

    def updated_objects(self, host, frame: int, culled, lights) -> list[int]:
        culled = list(culled)
        if not culled:
            return []
        updated: list[int] = []
        all_dirty = False
        for li, L in enumerate(lights):
            self.last_used[li] = frame
            if frame - self.last_updated.get(li, 0) < REDRAW_FRAMES:
                continue
            if L.type == float(N.LIGHT_DIRECTIONAL):
                all_dirty = True
                updated = list(culled)
                break
        if frame - self.last_gi_updated > GI_FRAMES:
            self.last_gi_updated = frame
            all_dirty = True
            updated = list(culled)
        if not all_dirty:
            objs = _objects(host.objects, host.num_objects)
            seen = set()
            for li, L in enumerate(lights):
                self.last_used[li] = frame
                if frame - self.last_updated.get(li, 0) < REDRAW_FRAMES:
                    continue
                if L.type in (float(N.LIGHT_POINT), float(N.LIGHT_SPOT)):
                    self.last_updated[li] = frame
                    lpos = np.array(L.position[:3], dtype=np.float32)
                    for o in culled:
                        ob = objs[o]
                        center = np.array(ob.object_bounds[:3], dtype=np.float32)
                        if float(np.linalg.norm(center - lpos)) < float(np.float32(ob.object_bounds[3]) +
                                                                        np.float32(L.radius)):
                            if o not in seen:
                                seen.add(o)
                                updated.append(o)
        return updated


class SurfaceLighting:
    """The GPU surface-lighting pass (luxgi_surface_light) on a DeviceScene.
    `run` writes the scene's direct-light atlas unless `out` (a device
    tensor of the atlas size in the surface's light format: int16 or
    float16 x 4 for RGBA16F, int32 for R11G11B10F) is given."""

    def __init__(self, scene, shadow_bias: float = SHADOW_BIAS, max_steps: int = SHADOW_MAX_STEPS):
        self.scene = scene
        self.shadow_bias = float(shadow_bias)
        self.max_steps = int(max_steps)
        self._keep = None

    def run(self, lights, tiles, masks=None, camera=None, copy_emissive: bool = True, out=None, stream=None) -> None:
        import torch

        from .ddgi import _stream

        dev = self.scene.device
        t = torch.as_tensor(np.ascontiguousarray(tiles, dtype=np.uint32).view(np.int32)).to(dev)
        m = None if masks is None else torch.as_tensor(
            np.ascontiguousarray(masks, dtype=np.uint32).view(np.int32)).to(dev)
        arr = light_array(lights)
        d = N.SurfaceLighting()
        d.lights = ctypes.cast(arr, ctypes.c_void_p)
        d.num_lights = len(lights)
        d.num_tiles = int(t.numel())
        d.tiles = t.data_ptr()
        d.light_masks = None if m is None else m.data_ptr()
        cam = self.scene.host.surface_data.camera_pos if camera is None else camera
        d.camera_pos[:] = [float(cam[0]), float(cam[1]), float(cam[2])]
        d.shadow_bias = self.shadow_bias
        d.copy_emissive = int(bool(copy_emissive))
        d.max_steps = self.max_steps
        target = self.scene.direct if out is None else out
        N.check(N.ddgi().luxgi_surface_light(ctypes.byref(self.scene.sdf_desc), ctypes.byref(self.scene.surface_desc),
                                             ctypes.byref(d), target.data_ptr(), _stream(stream)), "surface_light")
        if isinstance(stream, torch.cuda.Stream):
            t.record_stream(stream)
            if m is not None:
                m.record_stream(stream)
        self._keep = (t, m, arr)
