"""ORACLE -- test infrastructure only; never part of the product path.

ctypes wrapper of oracle/oracle.cpp, the CPU restatement (FP32 and FP64,
OpenMP over probes) of LuxGI's non-raytracing DDGI probe update.  Only the
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg import it.

Parity pins: the reference ships no tests, fixtures or golden data for
this path.  The oracle is pinned three ways:
  - against the reference's own code: its GLSL function libraries
    (DDGICommon.glsl, SDFCommon.glsl, AtlasCommon.glsl, Math.glsl,
    Random.glsl) compiled as C++ into oracle/_ref/libref.so by
    oracle/build_ref.py (tests/test_reference_pin.py);
  - by the border offset tables read out of the reference source
    (tests/golden/border_tables.json);
  - by analytic known-answer tests (empty scene / constant sky, hysteresis
    closed form, octahedral round trips, Fibonacci, probe inside a sphere).
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_float, c_int, c_int32, c_uint16, c_uint32, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.cpp"
LIB = HERE / "liboracle.so"
INCLUDE = HERE.parent / "include"


def build() -> Path:
    deps = [SRC, HERE / "packed_color.h"] + sorted(INCLUDE.glob("*.h"))
    if not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        vp = c_void_p
        sig = {
            "oracle_num_threads": (c_int, []),
            "oracle_set_threads": (None, [c_int]),
            "oracle_ray_dirs": (c_int, [vp, c_int, c_int, c_int, vp]),
            "oracle_rotation": (c_int, [vp, c_float, vp]),
            "oracle_frame_rotation": (c_int, [ctypes.c_uint64, c_uint32, vp]),
            "oracle_derive_uniform": (c_int, [vp]),
            "oracle_pack_colors": (c_int, [vp, ctypes.c_int64, c_int, vp]),
            "oracle_march_trails": (c_int, [vp, vp, vp, vp, vp, c_int, c_int, vp]),
            "oracle_unpack_colors": (c_int, [vp, ctypes.c_int64, c_int, vp]),
            "oracle_trace": (c_int, [vp, vp, vp, vp, vp, c_int, vp, c_int, c_int, c_int, vp, vp]),
            "oracle_blend": (c_int, [vp, vp, vp, vp, vp, vp, vp, c_int, c_int, c_int, c_int, c_int]),
            "oracle_border": (c_int, [vp, vp, vp]),
            "oracle_border_pairs": (c_int, [c_int, vp]),
            "oracle_build_mip": (c_int, [vp, vp, vp]),
            "oracle_cull": (c_int, [vp, vp, vp, c_uint32]),
            "oracle_inject": (c_int, [vp, vp, vp, vp, c_int, c_int, vp]),
            "oracle_sample_irradiance": (c_int, [vp, vp, vp, vp, vp, vp, vp, c_int, c_int]),
            "oracle_surface_light": (c_int, [vp, vp, vp, c_int, vp, vp, c_int, vp, c_float, c_int, c_int, c_int,
                                             vp, vp]),
            "oracle_sdf_build": (c_int, [vp, vp, c_int, vp, c_int, vp, vp, vp]),
            "oracle_sample_probe_image": (c_int, [vp, vp, vp, vp, vp, c_int, c_int, c_int, vp, vp, vp]),
            "oracle_sdf_plan": (c_int, [vp, vp, c_int, vp, c_int, c_int, vp, c_int, vp, vp, vp, c_int, vp]),
            "oracle_texel_dirs": (c_int, [c_int, c_int, vp]),
            "oracle_oct_encode": (c_int, [vp, c_int, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def ray_dirs(rot, nrays: int, precision: int = 0, fp16_round: bool = False) -> np.ndarray:
    rot = np.ascontiguousarray(rot, dtype=np.float32)
    out = np.zeros((nrays, 4), dtype=np.float32)
    lib().oracle_ray_dirs(_p(rot), nrays, precision, 1 if fp16_round else 0, _p(out))
    return out


def rotation(axis, angle: float) -> np.ndarray:
    a = np.ascontiguousarray(axis, dtype=np.float32)
    out = np.zeros(9, dtype=np.float32)
    lib().oracle_rotation(_p(a), angle, _p(out))
    return out


def frame_rotation(seed: int, frame: int) -> np.ndarray:
    """The synthetic workloads' seeded rotation of `frame` (column-major 3x3)."""
    out = np.zeros(9, dtype=np.float32)
    lib().oracle_frame_rotation(seed & (2 ** 64 - 1), frame, _p(out))
    return out


def pack_colors(rgba: np.ndarray, fmt: int) -> np.ndarray:
    """Float rgba texels ([..., 4]) in a surface colour format: uint16 x 4
    (RGBA16F) or uint32 (R11G11B10F) a texel, rounded like a render target."""
    from luxgi_gb300 import _native as N

    a = np.ascontiguousarray(rgba, dtype=np.float32).reshape(-1, 4)
    out = np.zeros(a.shape[0] if fmt == N.COLOR_R11G11B10F else a.shape[0] * 4,
                   dtype=np.uint32 if fmt == N.COLOR_R11G11B10F else np.uint16)
    lib().oracle_pack_colors(_p(a), a.shape[0], fmt, _p(out))
    return out


def unpack_colors(texels: np.ndarray, fmt: int) -> np.ndarray:
    """A surface colour texture's texels as float rgba [n, 4]."""
    from luxgi_gb300 import _native as N

    t = np.ascontiguousarray(texels)
    n = t.size if fmt == N.COLOR_R11G11B10F else t.size // 4
    out = np.zeros((n, 4), dtype=np.float32)
    lib().oracle_unpack_colors(_p(t), n, fmt, _p(out))
    return out


def march_trails(vdesc, inputs: HostInputs, rot, probes, rays, cap: int = 128) -> np.ndarray:
    """The FP32 march's sample points of rays (probes[i], rays[i]): [n, cap,
    4] = (u, v, w, full-resolution sampled) per step, -1 past the end."""
    pr = np.ascontiguousarray(probes, dtype=np.int32)
    ry = np.ascontiguousarray(rays, dtype=np.int32)
    out = np.zeros((pr.size, cap, 4), dtype=np.float32)
    r = np.ascontiguousarray(rot, dtype=np.float32)
    lib().oracle_march_trails(ctypes.byref(vdesc), ctypes.byref(inputs.sdf_desc), _p(r), _p(pr), _p(ry), pr.size,
                              cap, _p(out))
    return out


def derive_uniform(u) -> None:
    """Fills the atlas width/height fields of a DDGIUniform in place."""
    lib().oracle_derive_uniform(ctypes.byref(u))


def texel_dirs(n: int, precision: int = 0) -> np.ndarray:
    out = np.zeros((n * n, 3), dtype=np.float32)
    lib().oracle_texel_dirs(n, precision, _p(out))
    return out


def oct_encode(dirs: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.zeros((d.shape[0], 2), dtype=np.float32)
    lib().oracle_oct_encode(_p(d), d.shape[0], _p(out))
    return out


def border_pairs(n: int) -> np.ndarray:
    out = np.zeros((4 * n + 4, 4), dtype=np.int32)
    k = lib().oracle_border_pairs(n, _p(out))
    return out[:k]


class HostInputs:
    """Host-side descriptors of a scene for the oracle (numpy-backed)."""

    def __init__(self, host, light_mode: int, mip: np.ndarray | None = None, chunks: np.ndarray | None = None,
                 culled: np.ndarray | None = None, light_cache: np.ndarray | None = None,
                 light_format: int = 0, gbuffer_format: int = 0):
        """light_format / gbuffer_format: the surface textures' formats; the
        host scene's RGBA16F colours and FP32 G-buffers are converted to
        them (see colour_textures)."""
        from luxgi_gb300 import _native as N

        self.host = host
        self.sdf = host.sdf
        self.sdf_desc = N.SdfDesc()
        self.sdf_desc.data = host.sdf_data
        self.sdf_desc.format = host.sdf_format
        self.sdf_desc.resolution = host.res
        self.sdf_desc.mip_resolution = host.mres
        self.sdf_desc.sdf = self.sdf.ctypes.data
        if mip is None:
            mipf = build_mip(self.sdf_desc, host.sdf_float())
            mip = mipf.astype(np.float16).view(np.uint16) if host.sdf_format == N.STORAGE_FP16 else mipf
        self.mip = np.ascontiguousarray(mip)
        self.sdf_desc.mip = self.mip.ctypes.data
        self.surface_desc = N.SurfaceDesc()
        sd = N.SurfaceData.from_buffer_copy(host.surface_data)
        sd.culled_objects_capacity = host.cull_capacity()
        self.surface_desc.data = sd
        self.surface_desc.num_objects = host.num_objects
        self.surface_desc.num_tiles = host.num_tiles
        self.objects = host.objects
        self.tiles = host.tiles
        self.surface_desc.objects = self.objects.ctypes.data
        self.surface_desc.tiles = self.tiles.ctypes.data
        if chunks is None or culled is None:
            chunks, culled, _ = cull(self.surface_desc, host.cull_capacity())
        self.chunks = np.ascontiguousarray(chunks, dtype=np.uint32)
        self.culled = np.ascontiguousarray(culled, dtype=np.uint32)
        self.surface_desc.chunks = self.chunks.ctypes.data
        self.surface_desc.culled_objects = self.culled.ctypes.data
        tex = colour_textures(host, light_format, gbuffer_format)
        self.direct, self.emissive, self.gbuffer0, self.gbuffer1 = tex
        self.light_cache = np.ascontiguousarray(self.direct.copy() if light_cache is None else light_cache)
        self.surface_desc.light_cache = self.light_cache.ctypes.data
        self.surface_desc.depth = host.depth.ctypes.data
        self.surface_desc.direct_light = self.direct.ctypes.data
        self.surface_desc.albedo = host.albedo.ctypes.data
        self.surface_desc.gbuffer0 = self.gbuffer0.ctypes.data
        self.surface_desc.gbuffer1 = self.gbuffer1.ctypes.data
        self.surface_desc.pbr = host.pbr.ctypes.data
        self.surface_desc.emissive = self.emissive.ctypes.data
        self.surface_desc.light_format = light_format
        self.surface_desc.gbuffer_format = gbuffer_format


def colour_textures(host, light_format: int = 0, gbuffer_format: int = 0):
    """(direct light, emissive, gbuffer0, gbuffer1) of a host scene in the
    given formats: the scene's RGBA16F colours re-encoded as R11G11B10F
    (rounded to nearest even) or kept, its FP32 G-buffers rounded to
    RGBA16F or kept."""
    from luxgi_gb300 import _native as N

    direct, emissive = host.direct, host.emissive
    if light_format == N.COLOR_R11G11B10F:
        direct = pack_colors(unpack_colors(direct, N.COLOR_RGBA16F), light_format)
        emissive = pack_colors(unpack_colors(emissive, N.COLOR_RGBA16F), light_format)
    g0, g1 = host.gbuffer0, host.gbuffer1
    if gbuffer_format == N.GBUFFER_RGBA16F:
        g0 = g0.astype(np.float16).view(np.uint16)
        g1 = g1.astype(np.float16).view(np.uint16)
    return (np.ascontiguousarray(direct), np.ascontiguousarray(emissive), np.ascontiguousarray(g0),
            np.ascontiguousarray(g1))


def build_mip(sdf_desc, sdf_float: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(sdf_float, dtype=np.float32)
    m, C = sdf_desc.mip_resolution, sdf_desc.data.cascades_count
    out = np.zeros(m * C * m * m, dtype=np.float32)
    lib().oracle_build_mip(ctypes.byref(sdf_desc), _p(s), _p(out))
    return out


def cull(surface_desc, capacity: int):
    chunks = np.zeros(40 ** 3, dtype=np.uint32)
    culled = np.zeros(capacity, dtype=np.uint32)
    st = lib().oracle_cull(ctypes.byref(surface_desc), _p(chunks), _p(culled), capacity)
    return chunks, culled, st


def trace(vdesc, inputs: HostInputs, rot, frames: int = 0, prev_irr=None, prev_dist=None, precision: int = 0,
          probes: tuple | None = None, want_info: bool = True):
    """GISDFRays.comp for probes [p0, p1): (rays [n, R, 4], info [n, R, 4]:
    steps, hit cascade or -1, full-resolution samples, 0)."""
    u = vdesc.uniform
    P = u.probe_counts[0] * u.probe_counts[1] * u.probe_counts[2]
    p0, p1 = probes if probes is not None else (0, P)
    R = u.rays_per_probe
    out = np.zeros((p1 - p0, R, 4), dtype=np.float32)
    info = np.zeros((p1 - p0, R, 4), dtype=np.int32) if want_info else None
    rot = np.ascontiguousarray(rot, dtype=np.float32)
    pi = None if prev_irr is None else np.ascontiguousarray(prev_irr, dtype=np.float32)
    pd = None if prev_dist is None else np.ascontiguousarray(prev_dist, dtype=np.float32)
    lib().oracle_trace(ctypes.byref(vdesc), ctypes.byref(inputs.sdf_desc), ctypes.byref(inputs.surface_desc), _p(pi),
                       _p(pd), frames, _p(rot), precision, p0, p1, _p(out), _p(info))
    return out, info


def blend(vdesc, dirs: np.ndarray, rays: np.ndarray, prev_irr=None, prev_dist=None, first: bool = True,
          precision: int = 0, border: bool = True, probes: tuple | None = None):
    """ProbeUpdate.glsl (+ BorderUpdate.glsl): float atlases (irr [H,W,4],
    dist [H,W,2]); `rays` holds probes [p0, p1) when `probes` is given."""
    p0, p1 = probes if probes is not None else (0, 0)
    u = vdesc.uniform
    irr = np.zeros((u.irradiance_height, u.irradiance_width, 4), dtype=np.float32)
    dist = np.zeros((u.depth_height, u.depth_width, 2), dtype=np.float32)
    if prev_irr is not None:
        irr[...] = prev_irr
    if prev_dist is not None:
        dist[...] = prev_dist
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    r = np.ascontiguousarray(rays, dtype=np.float32)
    pi = None if prev_irr is None else np.ascontiguousarray(prev_irr, dtype=np.float32)
    pd = None if prev_dist is None else np.ascontiguousarray(prev_dist, dtype=np.float32)
    lib().oracle_blend(ctypes.byref(vdesc), _p(d), _p(r), _p(pi), _p(pd), _p(irr), _p(dist), 1 if first else 0,
                       precision, 1 if border else 0, p0, p1)
    return irr, dist


def border(uniform, irr: np.ndarray | None, dist: np.ndarray | None) -> None:
    lib().oracle_border(ctypes.byref(uniform), _p(irr), _p(dist))


def inject(vdesc, inputs: HostInputs, irr, dist, frames: int, precision: int = 0, base=None) -> np.ndarray:
    """SDFAtlasIndirectLight over every tile footprint; texels outside the
    footprints keep `base` (default: the inputs' current light cache)."""
    out = np.array(inputs.light_cache if base is None else base, copy=True)
    i = np.ascontiguousarray(irr, dtype=np.float32)
    d = np.ascontiguousarray(dist, dtype=np.float32)
    lib().oracle_inject(ctypes.byref(vdesc), ctypes.byref(inputs.surface_desc), _p(i), _p(d), frames, precision,
                        _p(out))
    return out


def surface_light(inputs: HostInputs, lights, tiles, masks=None, camera=(0.0, 0.0, 0.0), shadow_bias: float = 1.0,
                  copy_emissive: bool = True, max_steps: int = 250, precision: int = 0, out=None,
                  want_shadow: bool = False):
    """CopyEmissive + SDFDeferredLight per light over `tiles` (tile
    addresses).  lights: sequence of luxgi_light; masks: u32 per tile
    (None = every light).  Returns the RGBA16F atlas (u16 bits) and, with
    want_shadow, a u32 per texel with bit l set where light l was blocked."""
    from luxgi_gb300 import _native as N

    res = inputs.surface_desc.data.resolution
    o = np.array(inputs.direct if out is None else out, copy=True)
    t = np.ascontiguousarray(tiles, dtype=np.uint32)
    m = None if masks is None else np.ascontiguousarray(masks, dtype=np.uint32)
    sh = np.zeros(res * res, dtype=np.uint32) if want_shadow else None
    cam = (c_float * 3)(*camera)
    arr = (N.Light * max(1, len(lights)))(*lights)
    st = lib().oracle_surface_light(ctypes.byref(inputs.sdf_desc), ctypes.byref(inputs.surface_desc),
                                    ctypes.cast(arr, c_void_p), len(lights), _p(t), _p(m), t.size, cam,
                                    float(shadow_bias), int(copy_emissive), int(max_steps), precision, _p(o), _p(sh))
    if st != 0:
        raise RuntimeError(f"oracle_surface_light status {st}")
    return (o, sh) if want_shadow else o


def _mesh_descs(meshes):
    """luxgi_mesh_sdf records pointing at the meshes' host volumes."""
    from luxgi_gb300 import _native as N

    keep = [[np.ascontiguousarray(v, dtype=np.uint16) for v in m.mips] for m in meshes]
    descs = [m.desc([v.ctypes.data for v in vols]) for m, vols in zip(meshes, keep)]
    return (N.MeshSdf * max(1, len(descs)))(*descs), keep


def sdf_build(desc, meshes, objects):
    """The global SDF from objects on the CPU: (sdf float [(res*C)*res*res],
    mip float, luxgi_sdf_data).  meshes: luxgi_gb300.sdf.MeshSDF; objects:
    (world[16], mesh) pairs."""
    from luxgi_gb300 import _native as N
    from luxgi_gb300.sdf import objects_array

    res, C = desc.resolution, desc.cascades
    m = res // 4
    sdf = np.zeros(res * C * res * res, dtype=np.float32)
    mip = np.zeros(m * C * m * m, dtype=np.float32)
    md, keep = _mesh_descs(meshes)
    ob = objects_array(objects)
    data = N.SdfData()
    st = lib().oracle_sdf_build(ctypes.byref(desc), md, len(meshes), ob, len(objects), _p(sdf), _p(mip),
                                ctypes.byref(data))
    if st != 0:
        raise RuntimeError(f"oracle_sdf_build status {st}")
    return sdf, mip, data


def sdf_plan(desc, meshes, objects, cascade: int):
    """(raster records, their meshes, chunks) of one cascade on the CPU."""
    from luxgi_gb300 import _native as N
    from luxgi_gb300.sdf import objects_array

    md, keep = _mesh_descs(meshes)
    ob = objects_array(objects)
    cap = 4096 + 64 * len(objects)
    recs = (N.SdfRasterObject * max(1, len(objects)))()
    mesh = (ctypes.c_int32 * max(1, len(objects)))()
    chunks = (N.SdfChunk * cap)()
    nr, nc = ctypes.c_int(), ctypes.c_int()
    st = lib().oracle_sdf_plan(ctypes.byref(desc), md, len(meshes), ob, len(objects), cascade, recs, len(objects),
                               ctypes.byref(nr), mesh, chunks, cap, ctypes.byref(nc))
    if st != 0:
        raise RuntimeError(f"oracle_sdf_plan status {st}")
    return recs[:nr.value], list(mesh[:nr.value]), chunks[:nc.value]


def sample_probe_image(uniform, irr, dist, depth, normal, camera, view_proj_inv) -> np.ndarray:
    """SampleProbe.comp over a G-buffer: depth (H, W) float32, normal (H, W, C)
    float32; returns the (H, W, 4) RGBA16F image as uint16 bits."""
    H, W = depth.shape
    nch = normal.shape[-1]
    out = np.zeros((H, W, 4), dtype=np.uint16)
    i = np.ascontiguousarray(irr, dtype=np.float32)
    d = np.ascontiguousarray(dist, dtype=np.float32)
    dp = np.ascontiguousarray(depth, dtype=np.float32)
    nm = np.ascontiguousarray(normal, dtype=np.float32)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    vpi = np.ascontiguousarray(view_proj_inv, dtype=np.float32).reshape(-1)
    lib().oracle_sample_probe_image(ctypes.byref(uniform), _p(i), _p(d), _p(dp), _p(nm), nch, W, H, _p(cam), _p(vpi),
                                    _p(out))
    return out


def sample_irradiance(uniform, irr, dist, pos, nrm, wo, precision: int = 0) -> np.ndarray:
    i = np.ascontiguousarray(irr, dtype=np.float32)
    d = np.ascontiguousarray(dist, dtype=np.float32)
    p = np.ascontiguousarray(pos, dtype=np.float32)
    n = np.ascontiguousarray(nrm, dtype=np.float32)
    w = np.ascontiguousarray(wo, dtype=np.float32)
    out = np.zeros_like(p)
    lib().oracle_sample_irradiance(ctypes.byref(uniform), _p(i), _p(d), _p(p), _p(n), _p(w), _p(out), p.shape[0],
                                   precision)
    return out


def run_frames(vdesc, inputs: HostInputs, rots, precision: int = 0, inject_every: int = 0,
               state: tuple | None = None):
    """Whole frames (trace, blend + border, ping-pong) on the CPU.

    Returns (irr, dist, frames_done, last_rays).  Mode-A volumes refresh the
    light cache with inject() every `inject_every` frames (0 = never),
    before that frame's trace."""
    from luxgi_gb300 import _native as N

    u = vdesc.uniform
    fp16 = vdesc.storage == N.STORAGE_FP16
    irr, dist, frames = (None, None, 0) if state is None else state
    rays = None
    for rot in rots:
        if inject_every and vdesc.light_mode == N.LIGHT_CACHE and frames % inject_every == 0 and frames > 0:
            inputs.light_cache[...] = inject(vdesc, inputs, irr, dist, frames, precision)
        rays, _ = trace(vdesc, inputs, rot, frames, irr, dist, precision, want_info=False)
        dirs = ray_dirs(rot, u.rays_per_probe, precision, fp16)
        irr, dist = blend(vdesc, dirs, rays, irr, dist, first=(frames == 0), precision=precision)
        frames += 1
    return irr, dist, frames, rays


# ------------------------------------------------------------------ reference
# oracle/_ref/libref.so: the reference's own GLSL function libraries compiled
# as C++ (oracle/build_ref.py); present only where the reference checkout is.
_ref = None


def ref_lib():
    """The compiled reference library, or None when it cannot be built here."""
    global _ref
    if _ref is None:
        from . import build_ref

        path = build_ref.build()
        if path is None or not Path(path).exists():
            return None
        L = ctypes.CDLL(str(path))
        vp = c_void_p
        sig = {
            "ref_trace": (c_int, [vp, vp, vp, vp, vp, c_int, vp, c_int, c_int, vp, vp, vp]),
            "ref_blend": (c_int, [vp, vp, vp, vp, vp, vp, vp, c_int]),
            "ref_mip": (c_int, [vp, vp, vp]),
            "ref_cull": (c_int, [vp, vp, vp, c_uint32]),
            "ref_sample_irradiance": (c_int, [vp, vp, vp, vp, vp, vp, vp, c_int]),
            "ref_ray_dirs": (c_int, [vp, c_int, vp]),
            "ref_surface_light": (c_int, [vp, vp, vp, c_int, vp, vp, c_int, vp, c_float, c_int, vp]),
            "ref_inject": (c_int, [vp, vp, vp, vp, vp]),
            "ref_sdf_raster": (c_int, [vp, vp, c_int, vp, vp, vp, c_int, vp, vp]),
            "ref_sample_probe_image": (c_int, [vp, vp, vp, vp, vp, c_int, c_int, c_int, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _ref = L
    return _ref


def ref_ray_dirs(rot, nrays: int) -> np.ndarray:
    rot = np.ascontiguousarray(rot, dtype=np.float32)
    out = np.zeros((nrays, 4), dtype=np.float32)
    ref_lib().ref_ray_dirs(_p(rot), nrays, _p(out))
    return out


def ref_trace(vdesc, inputs: HostInputs, rot, frames: int = 0, prev_irr=None, prev_dist=None,
              probes: tuple | None = None, dirs: np.ndarray | None = None):
    """GISDFRays.comp through the reference's compiled functions; `dirs`
    (float4 [R]) overrides the ray directions."""
    u = vdesc.uniform
    dd = None if dirs is None else np.ascontiguousarray(dirs, dtype=np.float32)
    P = u.probe_counts[0] * u.probe_counts[1] * u.probe_counts[2]
    p0, p1 = probes if probes is not None else (0, P)
    R = u.rays_per_probe
    out = np.zeros((p1 - p0, R, 4), dtype=np.float32)
    info = np.zeros((p1 - p0, R, 2), dtype=np.int32)
    rot = np.ascontiguousarray(rot, dtype=np.float32)
    pi = None if prev_irr is None else np.ascontiguousarray(prev_irr, dtype=np.float32)
    pd = None if prev_dist is None else np.ascontiguousarray(prev_dist, dtype=np.float32)
    ref_lib().ref_trace(ctypes.byref(vdesc), ctypes.byref(inputs.sdf_desc), ctypes.byref(inputs.surface_desc), _p(pi),
                        _p(pd), frames, _p(rot), p0, p1, _p(out), _p(info), _p(dd))
    return out, info


def ref_blend(vdesc, dirs, rays, prev_irr=None, prev_dist=None, first: bool = True):
    u = vdesc.uniform
    irr = np.zeros((u.irradiance_height, u.irradiance_width, 4), dtype=np.float32)
    dist = np.zeros((u.depth_height, u.depth_width, 2), dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    r = np.ascontiguousarray(rays, dtype=np.float32)
    pi = None if prev_irr is None else np.ascontiguousarray(prev_irr, dtype=np.float32)
    pd = None if prev_dist is None else np.ascontiguousarray(prev_dist, dtype=np.float32)
    ref_lib().ref_blend(ctypes.byref(vdesc), _p(d), _p(r), _p(pi), _p(pd), _p(irr), _p(dist), 1 if first else 0)
    return irr, dist


def ref_mip(sdf_desc, sdf_float: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(sdf_float, dtype=np.float32)
    m, C = sdf_desc.mip_resolution, sdf_desc.data.cascades_count
    out = np.zeros(m * C * m * m, dtype=np.float32)
    ref_lib().ref_mip(ctypes.byref(sdf_desc), _p(s), _p(out))
    return out


def ref_surface_light(inputs: HostInputs, lights, tiles, masks=None, camera=(0.0, 0.0, 0.0),
                      shadow_bias: float = 1.0, copy_emissive: bool = True, out=None) -> np.ndarray:
    """CopyEmissive + SDFDeferredLight through the reference's compiled
    functions (250-step shadow march), RGBA16F bits."""
    o = np.array(inputs.direct if out is None else out, copy=True)
    from luxgi_gb300 import _native as N

    t = np.ascontiguousarray(tiles, dtype=np.uint32)
    m = None if masks is None else np.ascontiguousarray(masks, dtype=np.uint32)
    cam = (c_float * 3)(*camera)
    arr = (N.Light * max(1, len(lights)))(*lights)
    ref_lib().ref_surface_light(ctypes.byref(inputs.sdf_desc), ctypes.byref(inputs.surface_desc),
                                ctypes.cast(arr, c_void_p), len(lights), _p(t), _p(m), t.size, cam,
                                float(shadow_bias), int(copy_emissive), _p(o))
    return o


def ref_inject(vdesc, inputs: HostInputs, irr, dist, base=None) -> np.ndarray:
    """SDFAtlasIndirectLight through the reference's compiled functions."""
    o = np.array(inputs.light_cache if base is None else base, copy=True)
    i = np.ascontiguousarray(irr, dtype=np.float32)
    d = np.ascontiguousarray(dist, dtype=np.float32)
    ref_lib().ref_inject(ctypes.byref(vdesc), ctypes.byref(inputs.surface_desc), _p(i), _p(d), _p(o))
    return o


def ref_sdf_raster(desc, data, cascade: int, meshes, recs, rec_mesh, chunks, sdf: np.ndarray) -> np.ndarray:
    """SDFRasterizeModel.glsl over a cascade's chunks through the reference's
    compiled distanceToModelSDF; writes into a copy of `sdf` (float)."""
    from luxgi_gb300 import _native as N

    out = np.array(sdf, dtype=np.float32, copy=True)
    md, keep = _mesh_descs(meshes)
    R = (N.SdfRasterObject * max(1, len(recs)))(*recs)
    M = (ctypes.c_int32 * max(1, len(rec_mesh)))(*rec_mesh)
    Ch = (N.SdfChunk * max(1, len(chunks)))(*chunks)
    ref_lib().ref_sdf_raster(ctypes.byref(desc), ctypes.byref(data), cascade, R, M, Ch, len(chunks), md, _p(out))
    return out


def ref_sample_probe_image(uniform, irr, dist, depth, normal, camera, view_proj_inv) -> np.ndarray:
    """SampleProbe.comp through the reference's compiled functions: (H, W, 4) float."""
    H, W = depth.shape
    nch = normal.shape[-1]
    out = np.zeros((H, W, 4), dtype=np.float32)
    args = [np.ascontiguousarray(a, dtype=np.float32) for a in (irr, dist, depth, normal, camera, view_proj_inv)]
    ref_lib().ref_sample_probe_image(ctypes.byref(uniform), _p(args[0]), _p(args[1]), _p(args[2]), _p(args[3]), nch,
                                     W, H, _p(args[4]), _p(args[5].reshape(-1)), _p(out))
    return out


def ref_cull(surface_desc, capacity: int):
    chunks = np.zeros(40 ** 3, dtype=np.uint32)
    culled = np.zeros(capacity, dtype=np.uint32)
    st = ref_lib().ref_cull(ctypes.byref(surface_desc), _p(chunks), _p(culled), capacity)
    return chunks, culled, st


def ref_sample_irradiance(uniform, irr, dist, pos, nrm, wo) -> np.ndarray:
    i = np.ascontiguousarray(irr, dtype=np.float32)
    d = np.ascontiguousarray(dist, dtype=np.float32)
    p = np.ascontiguousarray(pos, dtype=np.float32)
    n = np.ascontiguousarray(nrm, dtype=np.float32)
    w = np.ascontiguousarray(wo, dtype=np.float32)
    out = np.zeros_like(p)
    ref_lib().ref_sample_irradiance(ctypes.byref(uniform), _p(i), _p(d), _p(p), _p(n), _p(w), _p(out), p.shape[0])
    return out
