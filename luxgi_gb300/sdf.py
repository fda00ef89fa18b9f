"""Global SDF from placed mesh SDFs, above the C ABI.

Mirrors the reference's mesh-SDF assets and the global-SDF merge system:

* `MeshSDF` is a baked mesh SDF -- the MeshDistanceField component
  (Engine/DDGI/MeshDistanceField.h:15-26) plus its FP16 volume and mips --
  read from a baked `.sdf` file (`MeshSDF.load`, the cereal layout of
  SDFBaker.cpp:158-205, parsed by `luxgi_mesh_sdf_parse`) or baked here from
  an analytic shape (`MeshSDF.bake`, SDFBaker.cpp's grid, padding, encoding
  and mip rule, with the exact distance of the shape instead of a BVH query);
* `GlobalSDF` places objects (a world matrix and a mesh each) and builds the
  cascaded global SDF and its mip on the GPU (`luxgi_sdf_build`, the first
  build of merge_sdf::system, GlobalDistanceField.cpp:576-842), producing the
  `luxgi_sdf_desc` the probe update traces.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

GI_DISTANCE = 4000.0       # GlobalDistanceFieldPublic::giDistance (GlobalDistanceField.h:39)
GLOBAL_SCALE = 0.1         # ::gloalScale (:35)
MIN_OBJECT_RADIUS = 10.0   # ::minObjectRadius (:34)


def _half(x) -> np.ndarray:
    """float32 -> binary16 bits the way glm::packHalf converts
    (glm/detail/type_half.inl, toFloat16): round to nearest with ties away
    from zero, subnormals from the truncated significand rounded on its
    13th bit, overflow to infinity."""
    i = np.asarray(x, dtype=np.float32).view(np.int32).astype(np.int64)
    s = (i >> 16) & 0x8000
    e = ((i >> 23) & 0xFF) - (127 - 15)
    m = i & 0x7FFFFF
    sub = e <= 0
    ms = (m | 0x800000) >> np.clip(1 - e, 0, 31)
    ms = np.where(ms & 0x1000, ms + 0x2000, ms)
    out = np.where(e < -10, s, s | (ms >> 13))
    special = e == 0xFF - (127 - 15)
    mn = m >> 13
    out = np.where(special, np.where(m == 0, s | 0x7C00, s | 0x7C00 | mn | (mn == 0)), out)
    mr = np.where(m & 0x1000, m + 0x2000, m)
    e2 = np.where(mr & 0x800000, e + 1, e)
    mr = np.where(mr & 0x800000, 0, mr)
    norm = np.where(e2 > 30, s | 0x7C00, s | (e2 << 10) | (mr >> 13))
    out = np.where(~sub & ~special, norm, out)
    return out.astype(np.uint16)


def _mip_down(level: np.ndarray) -> np.ndarray:
    """SDFBaker.cpp:166-204: the mean of each 2x2x2 block of the previous
    level (half values summed in FP32, times 1/8, rounded to half); odd
    dimensions drop their last texel.  level: uint16 [d, h, w]."""
    d, h, w = level.shape
    nd, nh, nw = max(d // 2, 1), max(h // 2, 1), max(w // 2, 1)
    f = level.view(np.float16).astype(np.float32)
    acc = np.zeros((nd, nh, nw), dtype=np.float32)
    for dz in range(2):
        for dy in range(2):
            for dx in range(2):
                zs = np.minimum(np.arange(nd) * 2 + dz, d - 1)
                ys = np.minimum(np.arange(nh) * 2 + dy, h - 1)
                xs = np.minimum(np.arange(nw) * 2 + dx, w - 1)
                acc += f[np.ix_(zs, ys, xs)]
    return _half(acc * np.float32(1.0 / 8.0))


@dataclass
class MeshSDF:
    aabb_min: tuple
    aabb_max: tuple
    size: tuple                       # (x, y, z) texels of mip 0
    mips: list = field(default_factory=list)   # uint16 arrays [d, h, w]

    @property
    def extent(self) -> np.ndarray:
        return np.asarray(self.aabb_max, np.float32) - np.asarray(self.aabb_min, np.float32)

    @property
    def max_distance(self) -> float:
        return float(np.max(self.extent))

    def desc(self, pointers=None) -> N.MeshSdf:
        """The luxgi_mesh_sdf record; `pointers` = the mip volumes' addresses
        (device for luxgi_sdf_build, host for the oracle)."""
        m = N.MeshSdf()
        mn = np.asarray(self.aabb_min, np.float32)
        size = self.extent
        m.aabb_min[:] = [float(v) for v in mn]
        m.aabb_max[:] = [float(v) for v in np.asarray(self.aabb_max, np.float32)]
        mul = (np.float32(1.0) / size).astype(np.float32)            # SDFBaker.cpp:75-77
        add = (-mn / size).astype(np.float32)
        m.local_to_uvw_mul[:] = [float(v) for v in mul]
        m.local_to_uvw_add[:] = [float(v) for v in add]
        m.max_distance = self.max_distance
        m.size[:] = list(self.size)
        m.mip_count = len(self.mips)
        if pointers is not None:
            for i, p in enumerate(pointers):
                m.mips[i] = p
        return m

    @staticmethod
    def padded_box(bmin, bmax):
        """paddingSDFBox (SDFBaker.h:39-45): 5 % of the size, at least 0.1."""
        bmin = np.asarray(bmin, np.float32)
        bmax = np.asarray(bmax, np.float32)
        pad = np.maximum(np.float32(0.05) * (bmax - bmin), np.float32(0.1))
        return bmin - pad, bmax + pad

    @classmethod
    def bake(cls, distance_fn, bmin, bmax, size, mip_count: int = 3) -> "MeshSDF":
        """Bake a shape with exact distance `distance_fn(x, y, z)` (arrays,
        local units, negative inside) over its bounds [bmin, bmax] on the
        baker's grid: texel (x, y, z) at (x, y, z) * padded_size / (size - 1)
        + padded_min, stored as (d / max_distance + 1) / 2 in half
        (SDFBaker.cpp:96-156)."""
        pmin, pmax = cls.padded_box(bmin, bmax)
        sz = np.asarray(size, np.int64)
        grid = (pmax - pmin) / (sz - 1).astype(np.float32)
        xs = np.arange(sz[0], dtype=np.float32) * grid[0] + pmin[0]
        ys = np.arange(sz[1], dtype=np.float32) * grid[1] + pmin[1]
        zs = np.arange(sz[2], dtype=np.float32) * grid[2] + pmin[2]
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        d = np.asarray(distance_fn(X, Y, Z), dtype=np.float32)
        maxd = np.float32(np.max(pmax - pmin))
        mip0 = _half((d / maxd + np.float32(1.0)) / np.float32(2.0))
        mips = [mip0]
        for _ in range(1, max(1, min(mip_count, 3))):
            mips.append(_mip_down(mips[-1]))
        return cls(tuple(float(v) for v in pmin), tuple(float(v) for v in pmax), tuple(int(v) for v in sz), mips)

    @classmethod
    def load(cls, data: bytes, aabb_min, aabb_max) -> "MeshSDF":
        """A baked .sdf file's texels with the component's padded bounds
        (the scene stores them beside the file's path)."""
        buf = (ctypes.c_ubyte * len(data)).from_buffer_copy(data)
        info = N.MeshSdfFile()
        N.check(N.ddgi().luxgi_mesh_sdf_parse(ctypes.cast(buf, ctypes.c_void_p), len(data), ctypes.byref(info)),
                "mesh_sdf_parse")
        w, h, d = info.size[0], info.size[1], info.size[2]
        mips = []
        for m in range(info.mip_count):
            lw, lh, ld = max(w >> m, 1), max(h >> m, 1), max(d >> m, 1)
            off, n = int(info.mip_offset[m]), int(info.mip_bytes[m])
            mips.append(np.frombuffer(data[off:off + n], dtype=np.uint16).reshape(ld, lh, lw).copy())
        return cls(tuple(aabb_min), tuple(aabb_max), (w, h, d), mips)


def box_distance(half):
    """Exact distance to a box of half extents `half` centred at 0."""
    hx, hy, hz = (np.float32(v) for v in half)

    def fn(x, y, z):
        qx, qy, qz = np.abs(x) - hx, np.abs(y) - hy, np.abs(z) - hz
        out = np.sqrt(np.maximum(qx, 0) ** 2 + np.maximum(qy, 0) ** 2 + np.maximum(qz, 0) ** 2)
        return out + np.minimum(np.maximum(qx, np.maximum(qy, qz)), 0)
    return fn


def sphere_distance(radius):
    r = np.float32(radius)
    return lambda x, y, z: np.sqrt(x * x + y * y + z * z) - r


def trs(translation=(0.0, 0.0, 0.0), axis=(0.0, 1.0, 0.0), angle: float = 0.0, scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """A column-major world matrix T * R * S (float32 [16])."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    c, s = np.cos(angle), np.sin(angle)
    x, y, z = a
    R = np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                  [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                  [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(scale, np.float64)[None, :]
    M[:3, 3] = translation
    return M.T.astype(np.float32).reshape(-1)          # column-major


def build_desc(resolution: int = 192, cascades: int = 2, storage: int = N.STORAGE_FP16, gi_distance: float = GI_DISTANCE,
               global_scale: float = GLOBAL_SCALE, min_object_radius: float = MIN_OBJECT_RADIUS) -> N.SdfBuildDesc:
    d = N.SdfBuildDesc()
    d.gi_distance = gi_distance
    d.global_scale = global_scale
    d.min_object_radius = min_object_radius
    d.resolution = resolution
    d.cascades = cascades
    d.format = storage
    d.near_plane = 0.1
    d.far_plane = 1000.0
    return d


def objects_array(objects) -> ctypes.Array:
    """objects: sequence of (world float32[16] column-major, mesh index)."""
    arr = (N.SdfObject * max(1, len(objects)))()
    for i, (world, mesh) in enumerate(objects):
        arr[i].world[:] = [float(v) for v in np.asarray(world, np.float32).reshape(-1)]
        arr[i].mesh = int(mesh)
    return arr


def plan(desc: N.SdfBuildDesc, meshes, objects, cascade: int):
    """luxgi_sdf_build_plan: (raster records, their mesh indices, chunks)."""
    lib = N.ddgi()
    md = (N.MeshSdf * max(1, len(meshes)))(*[m.desc() for m in meshes])
    ob = objects_array(objects)
    nr, nc = ctypes.c_int(), ctypes.c_int()
    N.check(lib.luxgi_sdf_build_plan(ctypes.byref(desc), md, len(meshes), ob, len(objects), cascade, None, 0,
                                     ctypes.byref(nr), None, None, 0, ctypes.byref(nc)), "sdf_build_plan")
    recs = (N.SdfRasterObject * max(1, nr.value))()
    mesh = (ctypes.c_int32 * max(1, nr.value))()
    chunks = (N.SdfChunk * max(1, nc.value))()
    N.check(lib.luxgi_sdf_build_plan(ctypes.byref(desc), md, len(meshes), ob, len(objects), cascade, recs, nr.value,
                                     ctypes.byref(nr), mesh, chunks, nc.value, ctypes.byref(nc)), "sdf_build_plan")
    return recs[:nr.value], list(mesh[:nr.value]), chunks[:nc.value]


class GlobalSDF:
    """A cascaded global SDF built on the GPU from placed mesh SDFs.  After
    `build`, `sdf_desc` (a luxgi_sdf_desc) binds it to a DDGI volume."""

    def __init__(self, desc: N.SdfBuildDesc, device: str = "cuda"):
        import torch

        self.desc = desc
        self.device = torch.device(device)
        res, C = desc.resolution, desc.cascades
        elem = torch.int16 if desc.format == N.STORAGE_FP16 else torch.float32
        m = res // 4
        self.sdf = torch.empty(res * C * res * res, dtype=elem, device=self.device)
        self.mip = torch.empty(m * C * m * m, dtype=elem, device=self.device)
        self.tmp = torch.empty(m * m * m, dtype=elem, device=self.device)
        self.data = N.SdfData()
        self._meshes = []

    def upload(self, meshes) -> list:
        """Device copies of the meshes' volumes; returns luxgi_mesh_sdf records."""
        import torch

        self._meshes = []
        descs = []
        for m in meshes:
            vols = [torch.from_numpy(np.ascontiguousarray(v).view(np.int16).reshape(-1)).to(self.device)
                    for v in m.mips]
            self._meshes.append(vols)
            descs.append(m.desc([v.data_ptr() for v in vols]))
        return descs

    def build(self, meshes, objects, stream=None) -> None:
        from .ddgi import _stream

        descs = self.upload(meshes)
        md = (N.MeshSdf * max(1, len(descs)))(*descs)
        ob = objects_array(objects)
        N.check(N.ddgi().luxgi_sdf_build(ctypes.byref(self.desc), md, len(descs), ob, len(objects),
                                         self.sdf.data_ptr(), self.mip.data_ptr(), self.tmp.data_ptr(),
                                         ctypes.byref(self.data), _stream(stream)), "sdf_build")

    @property
    def sdf_desc(self) -> N.SdfDesc:
        s = N.SdfDesc()
        s.data = self.data
        s.format = self.desc.format
        s.resolution = self.desc.resolution
        s.mip_resolution = self.desc.resolution // 4
        s.sdf = self.sdf.data_ptr()
        s.mip = self.mip.data_ptr()
        return s
