"""Shared helpers of the test suite (workload set-up, comparisons)."""
from __future__ import annotations

import numpy as np

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.scene import HostScene, SceneSpec, VolumeSpec, Workload


def tiny_workload(probe_counts=(3, 2, 3), spacing=1.5, rays=48, irr=6, dist=14, sdf=32, room=10.0, prims=6,
                  atlas=256, storage=N.STORAGE_FP32, light=N.LIGHT_PER_HIT, steps=64, cascades=1, seed=7,
                  sdf_format=N.STORAGE_FP32, blend=N.BLEND_FP32, hysteresis=0.95, frames=3) -> Workload:
    v = VolumeSpec(tuple(probe_counts), spacing, rays, irradiance_side=irr, depth_side=dist, hysteresis=hysteresis,
                   max_steps=steps, storage=storage, light_mode=light, blend=blend)
    s = SceneSpec(seed, room, 0.5, prims, sdf, atlas, sdf_format=sdf_format, cascades=cascades,
                  sphere_radius=(0.3, 1.2), box_half_extent=(0.2, 1.0))
    return Workload("tiny", v, s, frames)


def analytic_sdf(host: HostScene, fn) -> np.ndarray:
    """Replaces the host scene's SDF by fn(points) (world units) sampled at
    the voxel centres of every cascade, normalised like the generator."""
    d = host.sdf_data
    res, C = host.res, host.cascades
    out = np.zeros((res, res, res * C), dtype=np.float32)
    for k in range(C):
        half = d.cascade_pos_distance[k][3]
        voxel = d.cascade_voxel_size[k]
        c = np.arange(res, dtype=np.float32)
        p = -half + (c + 0.5) * voxel
        Z, Y, X = np.meshgrid(p, p, p, indexing="ij")
        val = fn(X, Y, Z) / (2.0 * half)
        out[:, :, k * res:(k + 1) * res] = np.clip(val, -1.0, 1.0)
    flat = out.reshape(-1)
    if host.sdf_format == N.STORAGE_FP16:
        host.sdf = flat.astype(np.float16).view(np.uint16)
    else:
        host.sdf = flat.astype(np.float32)
    return host.sdf


def rel_err(a: np.ndarray, b: np.ndarray, floor: float = 1e-3) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def interior_mask(uniform, depth: bool) -> np.ndarray:
    """Texels that belong to a probe cell (interior + border) of the atlas."""
    n = uniform.depth_probe_side if depth else uniform.irradiance_probe_side
    W = uniform.depth_width if depth else uniform.irradiance_width
    H = uniform.depth_height if depth else uniform.irradiance_height
    m = np.zeros((H, W), dtype=bool)
    m[1:H - 1, 1:W - 1] = True
    return m
