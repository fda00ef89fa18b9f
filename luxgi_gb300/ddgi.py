"""Host-side mirror of the reference's DDGI volume interface.

LuxGI drives the probe update through ECS systems over the components
IrradianceVolume / DDGIUniform / DDGIPipelineInternal
(Engine/DDGI/DDGIRenderer.h:22-66, DDGIRenderer.cpp:85-97, 217-464).  The
same steps are methods here, each one C ABI call into libluxgi_ddgi:

    trace()          trace_rays::system    (DDGIRenderer.cpp:217-330)
    probe_update()   probe_update::system  (:347-413), border copy fused
    border_update()  border_update::system (:418-464)
    end_frame()      end_frame::system     (:335-342)
    update()         all of the above for one frame

Device buffers are owned by the library; atlases()/rays() return zero-copy
torch views of them.  Errors raise LuxgiError with the C status.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .scene import DeviceScene, VolumeSpec


class _CudaArray:
    """Minimal __cuda_array_interface__ exporter for library-owned memory."""

    def __init__(self, ptr: int, shape, typestr: str, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}
        self._owner = owner


def _view(ptr: int, shape, typestr: str, owner):
    import torch

    return torch.as_tensor(_CudaArray(ptr, shape, typestr, owner), device="cuda")


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


STATE_FORMAT = 1   # probe-state checkpoint files (DDGIVolume.save_state)


def frame_rotation(seed: int, frame: int) -> np.ndarray:
    """Seeded stand-in for the reference's std::random_device rotation
    (DDGIRenderer.cpp:267-272): column-major 3x3."""
    out = (ctypes.c_float * 9)()
    N.check(N.ddgi().luxgi_ddgi_frame_rotation(seed, frame, out), "frame_rotation")
    return np.array(out[:], dtype=np.float32)


def rotation(axis, angle: float) -> np.ndarray:
    out = (ctypes.c_float * 9)()
    N.check(N.ddgi().luxgi_ddgi_rotation(N.floats(axis), angle, out), "rotation")
    return np.array(out[:], dtype=np.float32)


class DDGIVolume:
    def __init__(self, spec: VolumeSpec):
        self.spec = spec
        self.desc = spec.desc()
        self.uniform = self.desc.uniform
        h = ctypes.c_void_p()
        N.check(N.ddgi().luxgi_ddgi_create(ctypes.byref(self.desc), ctypes.byref(h)), "ddgi_create")
        self._h = h
        self.scene = None

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def bind_scene(self, scene: DeviceScene) -> None:
        N.check(N.ddgi().luxgi_ddgi_bind_scene(self._h, ctypes.byref(scene.sdf_desc), ctypes.byref(scene.surface_desc)),
                "bind_scene")
        self.scene = scene

    def check_status(self, stream=None) -> None:
        """Raises LuxgiError(LUXGI_ETIMEOUT) if a bounded device wait gave up."""
        N.check(N.ddgi().luxgi_ddgi_check_status(self._h, _stream(stream)), "check_status")

    def set_debug_rays(self, on: bool = True) -> None:
        N.check(N.ddgi().luxgi_ddgi_set_debug_rays(self._h, 1 if on else 0), "set_debug_rays")

    def set_stage_timing(self, on: bool = True) -> None:
        N.check(N.ddgi().luxgi_ddgi_set_stage_timing(self._h, 1 if on else 0), "set_stage_timing")

    def stage_times(self) -> dict:
        """Milliseconds of the last frame's stages (waits for them)."""
        out = (ctypes.c_float * 4)()
        N.check(N.ddgi().luxgi_ddgi_stage_times(self._h, out), "stage_times")
        return {"setup": out[0], "march": out[1], "shade": out[2], "blend": out[3]}

    def trace(self, rot, stream=None) -> None:
        r = N.floats(np.asarray(rot, dtype=np.float32).ravel())
        N.check(N.ddgi().luxgi_ddgi_trace(self._h, r, _stream(stream)), "trace")

    def probe_update(self, stream=None) -> None:
        N.check(N.ddgi().luxgi_ddgi_probe_update(self._h, _stream(stream)), "probe_update")

    def border_update(self, stream=None) -> None:
        N.check(N.ddgi().luxgi_ddgi_border_update(self._h, _stream(stream)), "border_update")

    def end_frame(self) -> None:
        N.check(N.ddgi().luxgi_ddgi_end_frame(self._h), "end_frame")

    def update(self, rot, stream=None) -> None:
        r = N.floats(np.asarray(rot, dtype=np.float32).ravel())
        N.check(N.ddgi().luxgi_ddgi_update(self._h, r, _stream(stream)), "update")

    def inject_indirect(self, stream=None) -> None:
        N.check(N.ddgi().luxgi_ddgi_inject_indirect(self._h, _stream(stream)), "inject_indirect")

    def atlas_info(self) -> N.Atlases:
        a = N.Atlases()
        N.check(N.ddgi().luxgi_ddgi_get_atlases(self._h, ctypes.byref(a)), "get_atlases")
        return a

    def atlases(self, which: str = "current"):
        """(irradiance [H, W, 4], distance [H, W, 2]) torch views."""
        a = self.atlas_info()
        ts = "<f2" if a.storage == N.STORAGE_FP16 else "<f4"
        irr = a.irradiance if which == "current" else a.prev_irradiance
        dist = a.distance if which == "current" else a.prev_distance
        return (_view(irr, (a.irradiance_height, a.irradiance_width, 4), ts, self),
                _view(dist, (a.depth_height, a.depth_width, 2), ts, self))

    def rays(self):
        """(directions [R, 4] f32, radiance [P, R, 4], hit_info [P, R, 4] or None)."""
        r = N.Rays()
        N.check(N.ddgi().luxgi_ddgi_get_rays(self._h, ctypes.byref(r)), "get_rays")
        ts = "<f2" if r.storage == N.STORAGE_FP16 else "<f4"
        dirs = _view(r.directions, (r.rays, 4), "<f4", self)
        rad = _view(r.radiance, (r.probes, r.rays, 4), ts, self)
        info = _view(r.hit_info, (r.probes, r.rays, 4), "<i4", self) if r.hit_info else None
        return dirs, rad, info

    def load_atlases(self, irradiance: np.ndarray, distance: np.ndarray, frames: int, stream=None) -> None:
        irr = np.ascontiguousarray(irradiance)
        dist = np.ascontiguousarray(distance)
        N.check(N.ddgi().luxgi_ddgi_load_atlases(self._h, irr.ctypes.data, dist.ctypes.data, frames, _stream(stream)),
                "load_atlases")

    def sample_probe_image(self, depth, normal, camera_pos, view_proj_inv, out=None, stream=None):
        """SampleProbe.comp over a screen G-buffer: depth (H, W) float32 and
        normal (H, W, C) float32 device tensors, C >= 2 with the octahedral
        normal first; returns the (H, W, 4) float16 indirect-lighting image."""
        import torch

        H, W = depth.shape
        nch = normal.shape[-1]
        if out is None:
            out = torch.empty((H, W, 4), dtype=torch.float16, device=depth.device)
        cam = (ctypes.c_float * 3)(*[float(c) for c in camera_pos])
        vpi = (ctypes.c_float * 16)(*[float(c) for c in np.asarray(view_proj_inv, np.float32).reshape(-1)])
        N.check(N.ddgi().luxgi_ddgi_sample_probe_image(self._h, depth.data_ptr(), normal.data_ptr(), nch, W, H, cam,
                                                       vpi, out.data_ptr(), _stream(stream)), "sample_probe_image")
        return out

    def save_atlases(self, stream=None):
        """(irradiance, distance, frames): host copies of the current atlases."""
        a = self.atlas_info()
        dt = np.float16 if a.storage == N.STORAGE_FP16 else np.float32
        irr = np.empty((a.irradiance_height, a.irradiance_width, 4), dtype=dt)
        dist = np.empty((a.depth_height, a.depth_width, 2), dtype=dt)
        frames = ctypes.c_int32()
        N.check(N.ddgi().luxgi_ddgi_save_atlases(self._h, irr.ctypes.data, dist.ctypes.data, ctypes.byref(frames),
                                                 _stream(stream)), "save_atlases")
        return irr, dist, int(frames.value)

    def save_state(self, path, stream=None) -> None:
        """A checkpoint file of the volume's probe state: the DDGIUniform,
        storage and frame counter with both atlases (numpy .npz)."""
        irr, dist, frames = self.save_atlases(stream)
        np.savez(path, format=np.array([STATE_FORMAT], np.int32), uniform=np.frombuffer(bytes(self.uniform), np.uint8),
                 storage=np.array([self.desc.storage], np.int32), frames=np.array([frames], np.int32),
                 irradiance=irr, distance=dist)

    def load_state(self, path, stream=None) -> None:
        """Restores a checkpoint written by save_state for a volume of the
        same layout (DDGIUniform and storage); raises ValueError otherwise."""
        with np.load(path) as z:
            if int(z["format"][0]) != STATE_FORMAT:
                raise ValueError("not a probe-state checkpoint of this format")
            if bytes(z["uniform"]) != bytes(self.uniform) or int(z["storage"][0]) != self.desc.storage:
                raise ValueError("checkpoint of a volume with another layout")
            self.load_atlases(z["irradiance"], z["distance"], int(z["frames"][0]), stream)

    def sample_irradiance(self, pos, nrm, wo, out, stream=None) -> None:
        n = pos.shape[0]
        N.check(N.ddgi().luxgi_ddgi_sample_irradiance(self._h, pos.data_ptr(), nrm.data_ptr(), wo.data_ptr(),
                                                      out.data_ptr(), n, _stream(stream)), "sample_irradiance")

    @property
    def frames(self) -> int:
        return self.atlas_info().frames

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.ddgi().luxgi_ddgi_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def update_batch(volumes, rots, stream=None) -> None:
    """luxgi_ddgi_update_batch over several volumes (one frame each)."""
    n = len(volumes)
    hs = (ctypes.c_void_p * n)(*[v.handle.value for v in volumes])
    r = np.ascontiguousarray(np.asarray(rots, dtype=np.float32).reshape(n, 9))
    N.check(N.ddgi().luxgi_ddgi_update_batch(hs, n, r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _stream(stream)),
            "update_batch")


class DDGIBatch:
    """A fixed set of volumes updated together frame after frame
    (luxgi_ddgi_batch_*): one launch per stage over all volumes, replayed
    as a CUDA graph.  The volumes must stay alive while the batch exists."""

    def __init__(self, volumes, tuning: dict | None = None):
        self.volumes = list(volumes)
        n = len(self.volumes)
        hs = (ctypes.c_void_p * n)(*[v.handle.value for v in self.volumes])
        t = None
        if tuning is not None:
            t = N.BatchTuning()
            for k, v in {**self.default_tuning(), **tuning}.items():
                setattr(t, k, v)
        h = ctypes.c_void_p()
        N.check(N.ddgi().luxgi_ddgi_batch_create(hs, n, ctypes.byref(t) if t is not None else None, ctypes.byref(h)),
                "batch_create")
        self._h = h

    @staticmethod
    def default_tuning() -> dict:
        return {"march_variant": 4, "march_threads": 256, "shade_variant": 1, "blend_probes": 2, "use_graph": 1,
                "march_budget": 0, "shade_order": 0}

    def update(self, rots, stream=None) -> None:
        r = np.ascontiguousarray(np.asarray(rots, dtype=np.float32).reshape(len(self.volumes), 9))
        N.check(N.ddgi().luxgi_ddgi_batch_update(self._h, r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                 _stream(stream)), "batch_update")

    def autotune(self, frames: int = 3, stream=None) -> dict:
        t = N.BatchTuning()
        N.check(N.ddgi().luxgi_ddgi_batch_autotune(self._h, frames, _stream(stream), ctypes.byref(t)),
                "batch_autotune")
        return self._as_dict(t)

    @property
    def tuning(self) -> dict:
        t = N.BatchTuning()
        N.check(N.ddgi().luxgi_ddgi_batch_get_tuning(self._h, ctypes.byref(t)), "batch_get_tuning")
        return self._as_dict(t)

    @tuning.setter
    def tuning(self, values: dict) -> None:
        t = N.BatchTuning()
        for k, v in {**self.tuning, **values}.items():
            setattr(t, k, v)
        N.check(N.ddgi().luxgi_ddgi_batch_set_tuning(self._h, ctypes.byref(t)), "batch_set_tuning")

    @staticmethod
    def _as_dict(t) -> dict:
        return {"march_variant": t.march_variant, "march_threads": t.march_threads, "shade_variant": t.shade_variant,
                "blend_probes": t.blend_probes, "use_graph": t.use_graph, "march_budget": t.march_budget,
                "shade_order": t.shade_order, "frame_ms": t.frame_ms}

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.ddgi().luxgi_ddgi_batch_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
