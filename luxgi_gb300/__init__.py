"""GB300-native (sm_103a) DDGI probe-update path of LuxGI.

libluxgi_ddgi.so (CUDA kernels behind the C ABI in include/luxgi_ddgi.h) does
the work; this package is the host-side mirror of the reference's DDGI volume
interface plus the seeded synthetic scene inputs.
"""
from . import _native
from .ddgi import DDGIBatch, DDGIVolume, frame_rotation, rotation, update_batch
from .serve import Server
from .surface import LightingSchedule, SurfaceLighting, make_light, scene_lights, select_tiles
from .scene import (PLAIN_SMALL, PLAIN_SMALL_REF, PRECISION, PRODUCTION, WORKLOADS, DeviceScene, HostScene,
                    SceneSpec, VolumeSpec, Workload, scaled)

__all__ = ["DDGIBatch", "DDGIVolume", "DeviceScene", "HostScene", "SceneSpec", "VolumeSpec", "Workload", "WORKLOADS",
           "PLAIN_SMALL", "PLAIN_SMALL_REF", "PRODUCTION", "PRECISION", "frame_rotation", "rotation",
           "update_batch", "scaled", "Server", "SurfaceLighting", "LightingSchedule", "make_light", "scene_lights",
           "select_tiles", "_native"]
