"""Serving loop over many DDGI volumes (libluxgi_ddgi's luxgi_server_*).

Sessions are volumes with their own scenes; requests are single frames.
The server (a native scheduler thread) admits sessions to the device by a
memory budget, keeps them resident, evicts the least recently used idle
session when short of memory (saving its atlases), and runs pending
requests of many sessions as batched launch groups that overlap on the
device.  executor="sim" runs the same scheduling policy with modelled
timings and no device work (host-only tests).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .scene import HostScene, VolumeSpec


def session_scene(host: HostScene) -> N.SessionScene:
    """Host-memory scene description of a HostScene (arrays stay owned by it)."""
    sc = N.SessionScene()
    sc.sdf.data = host.sdf_data
    sc.sdf.format = host.sdf_format
    sc.sdf.resolution = host.res
    sc.sdf.mip_resolution = host.mres
    sc.sdf.sdf = host.sdf.ctypes.data
    sc.sdf.mip = None
    sd = N.SurfaceData.from_buffer_copy(host.surface_data)
    sd.culled_objects_capacity = host.cull_capacity()
    sc.surface.data = sd
    sc.surface.num_objects = host.num_objects
    sc.surface.num_tiles = host.num_tiles
    sc.surface.objects = host.objects.ctypes.data
    sc.surface.tiles = host.tiles.ctypes.data
    sc.surface.depth = host.depth.ctypes.data
    sc.surface.direct_light = host.direct.ctypes.data
    sc.surface.albedo = host.albedo.ctypes.data
    sc.surface.light_cache = None
    sc.atlas_resolution = host.atlas
    return sc


class Server:
    def __init__(self, memory_budget: int, executor: str = "cuda", max_group: int = 64, max_inflight: int = 3,
                 tuning: dict | None = None, sim_rate: float = 1e9, sim_admit_s: float = 0.0,
                 sim_evict_s: float = 0.0):
        d = N.ServerDesc()
        d.memory_budget = int(memory_budget)
        d.executor = N.SERVE_EXEC_SIM if executor == "sim" else N.SERVE_EXEC_CUDA
        d.max_group = max_group
        d.max_inflight = max_inflight
        for k, v in (tuning or {}).items():
            setattr(d.tuning, k, v)
        d.sim_rate = sim_rate
        d.sim_admit_s = sim_admit_s
        d.sim_evict_s = sim_evict_s
        h = ctypes.c_void_p()
        N.check(N.ddgi().luxgi_server_create(ctypes.byref(d), ctypes.byref(h)), "server_create")
        self._h = h
        self._keep = []          # host scenes referenced by the sessions
        self.sim = executor == "sim"

    def add_session(self, spec: VolumeSpec, host: HostScene) -> int:
        desc = spec.desc()
        sc = session_scene(host)
        sid = ctypes.c_int32()
        N.check(N.ddgi().luxgi_server_add_session(self._h, ctypes.byref(desc), ctypes.byref(sc), ctypes.byref(sid)),
                "server_add_session")
        self._keep.append(host)
        return sid.value

    def session_bytes(self, sid: int) -> int:
        b = ctypes.c_uint64()
        N.check(N.ddgi().luxgi_server_session_bytes(self._h, sid, ctypes.byref(b)), "server_session_bytes")
        return b.value

    def submit(self, sid: int, rot) -> int:
        r = N.floats(np.asarray(rot, dtype=np.float32).ravel())
        t = ctypes.c_uint64()
        N.check(N.ddgi().luxgi_server_submit(self._h, sid, r, ctypes.byref(t)), "server_submit")
        return t.value

    def drain(self, timeout: float = 0.0) -> None:
        N.check(N.ddgi().luxgi_server_drain(self._h, timeout), "server_drain")

    def run_poisson(self, ids, rate: float, seconds: float, seed: int = 1) -> None:
        arr = (ctypes.c_int32 * len(ids))(*ids)
        N.check(N.ddgi().luxgi_server_run_poisson(self._h, arr, len(ids), rate, seconds, seed), "server_run_poisson")

    def stats(self, reset: bool = False) -> dict:
        s = N.ServerStats()
        N.check(N.ddgi().luxgi_server_stats_get(self._h, ctypes.byref(s), 1 if reset else 0), "server_stats")
        return {name: getattr(s, name) for name, _ in N.ServerStats._fields_}

    def touch(self, sid: int) -> None:
        N.check(N.ddgi().luxgi_server_touch(self._h, sid), "server_touch")

    def state(self, sid: int) -> tuple[bool, int]:
        r, f = ctypes.c_int32(), ctypes.c_int32()
        N.check(N.ddgi().luxgi_server_session_state(self._h, sid, ctypes.byref(r), ctypes.byref(f)), "server_state")
        return bool(r.value), f.value

    def atlases(self, sid: int):
        """(irradiance [H, W, 4], distance [H, W, 2]) torch views of an idle resident session."""
        from .ddgi import _view

        a = N.Atlases()
        N.check(N.ddgi().luxgi_server_session_atlases(self._h, sid, ctypes.byref(a)), "server_atlases")
        ts = "<f2" if a.storage == N.STORAGE_FP16 else "<f4"
        return (_view(a.irradiance, (a.irradiance_height, a.irradiance_width, 4), ts, self),
                _view(a.distance, (a.depth_height, a.depth_width, 2), ts, self))

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.ddgi().luxgi_server_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
