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


def probe_ranges(probes: int, count: int, length: int, seed: int) -> list[tuple[int, int]]:
    """`count` disjoint seeded ranges [p0, p0 + length) of probe indices,
    sorted (each range spans whole rows of the probe grid when `length` is a
    multiple of the grid's x count)."""
    slots = probes // length
    rng = np.random.default_rng(seed)
    picks = sorted(rng.choice(slots, size=min(count, slots), replace=False))
    return [(int(s) * length, int(s) * length + length) for s in picks]


def cell_errors(got: np.ndarray, ref: np.ndarray, uniform, probes, depth: bool, floor: float = 1e-3) -> np.ndarray:
    """Relative errors (|got - ref| / max(|ref|, floor)) over the atlas cells
    (interior and border texels, every channel) of the given probes; cell
    of probe p at (p mod XY, p div XY), (n + 2)^2 texels from texel 1
    (DDGICommon.glsl:94-99)."""
    n = uniform.depth_probe_side if depth else uniform.irradiance_probe_side
    XY = uniform.probe_counts[0] * uniform.probe_counts[1]
    out = []
    for p in probes:
        cx, cy = p % XY, p // XY
        ys = slice(1 + cy * (n + 2), 1 + (cy + 1) * (n + 2))
        xs = slice(1 + cx * (n + 2), 1 + (cx + 1) * (n + 2))
        a = got[ys, xs].astype(np.float64)
        b = ref[ys, xs].astype(np.float64)
        out.append((np.abs(a - b) / np.maximum(np.abs(b), floor)).ravel())
    return np.concatenate(out) if out else np.zeros(0)


def interior_mask(uniform, depth: bool) -> np.ndarray:
    """Texels that belong to a probe cell (interior + border) of the atlas."""
    n = uniform.depth_probe_side if depth else uniform.irradiance_probe_side
    W = uniform.depth_width if depth else uniform.irradiance_width
    H = uniform.depth_height if depth else uniform.irradiance_height
    m = np.zeros((H, W), dtype=bool)
    m[1:H - 1, 1:W - 1] = True
    return m


def synthetic_gbuffer(width, height, seed=0, camera=(0.0, 0.5, -3.0), target=(0.0, 0.0, 2.0), fov=1.0,
                      near=0.1, far=100.0, dist_range=(1.0, 8.0), background=0.1, channels=4):
    """A screen G-buffer for SampleProbe.comp: a perspective camera (depth
    0..1), per-pixel view distances in dist_range, a fraction of background
    pixels (depth 1), random octahedral normals.  Returns (depth (H, W)
    float32, normal (H, W, channels) float32, camera float32[3],
    inverse(proj * view) float32[16] column-major)."""
    rng = np.random.default_rng(seed)
    cam = np.asarray(camera, np.float64)
    f = np.asarray(target, np.float64) - cam
    f /= np.linalg.norm(f)
    up = np.array([0.0, 1.0, 0.0])
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ cam
    aspect = width / height
    t = 1.0 / np.tan(fov / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / aspect, t
    proj[2, 2], proj[2, 3] = far / (near - far), near * far / (near - far)
    proj[3, 2] = -1.0
    pv = proj @ view
    ys, xs = np.mgrid[0:height, 0:width]
    sx = (xs + 0.5) / width * 2 - 1
    sy = (ys + 0.5) / height * 2 - 1
    dist = rng.uniform(dist_range[0], dist_range[1], size=(height, width))
    # view-space point at distance `dist` along the pixel's ray
    dv = np.stack([sx * aspect / t, sy / t, -np.ones_like(sx)], axis=-1)
    dv /= np.linalg.norm(dv, axis=-1, keepdims=True)
    pv_pts = dv * dist[..., None]
    clip = pv_pts @ proj[:3, :3].T + proj[:3, 3]
    w = pv_pts @ proj[3, :3] + proj[3, 3]
    depth = (clip[..., 2] / w).astype(np.float32)
    depth[rng.uniform(size=depth.shape) < background] = 1.0
    n = rng.normal(size=(height, width, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    l1 = np.abs(n).sum(-1, keepdims=True)
    o = n[..., :2] / l1
    neg = n[..., 2] < 0
    fx = (1 - np.abs(o[..., 1])) * np.where(o[..., 0] >= 0, 1.0, -1.0)
    fy = (1 - np.abs(o[..., 0])) * np.where(o[..., 1] >= 0, 1.0, -1.0)
    o[neg, 0], o[neg, 1] = fx[neg], fy[neg]
    normal = np.zeros((height, width, channels), np.float32)
    normal[..., :2] = o
    vpi = np.linalg.inv(pv).T.astype(np.float32).reshape(-1)       # column-major
    return depth, normal, cam.astype(np.float32), vpi
