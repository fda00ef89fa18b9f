"""Pins the CPU oracle to the reference's own code: the GLSL function
libraries of the reference (DDGICommon.glsl, SDFCommon.glsl,
AtlasCommon.glsl, Math.glsl, Random.glsl) compiled as C++ by
oracle/build_ref.py, driven the way the shader entry points drive them
(oracle/ref_harness.cpp).  Runs on the host; skipped where the reference
checkout is absent (the compiled library cannot be rebuilt there).

Tolerances: mip and culling bit-exact; with identical ray directions the
march takes the same steps and hits within 1e-3 voxel, radiance within
1e-3 relative (p99 1e-5); blend 1e-5 relative; sampleIrradiance 1e-4.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import frame_rotation
from luxgi_gb300.scene import PLAIN_SMALL, HostScene
from tests._helpers import rel_err, tiny_workload


@pytest.fixture(scope="module")
def ref():
    lib = oracle.ref_lib()
    if lib is None:
        pytest.skip("reference checkout not available: compiled reference library absent")
    return lib


@pytest.mark.parametrize("fmt,cascades", [(N.STORAGE_FP32, 1), (N.STORAGE_FP16, 1), (N.STORAGE_FP32, 2)])
def test_mip_equals_reference(ref, fmt, cascades):
    w = tiny_workload(sdf=64, sdf_format=fmt, cascades=cascades)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    a = oracle.ref_mip(inp.sdf_desc, host.sdf_float())
    b = oracle.build_mip(inp.sdf_desc, host.sdf_float())
    assert np.array_equal(a, b)


def test_cull_equals_reference(ref):
    host = HostScene(PLAIN_SMALL.scene)
    inp = oracle.HostInputs(host, PLAIN_SMALL.volume.light_mode)
    ch, cu, st = oracle.ref_cull(inp.surface_desc, host.cull_capacity())
    assert st == 0
    assert np.array_equal(ch, inp.chunks) and np.array_equal(cu, inp.culled)


def test_ray_directions_vs_reference(ref):
    for f in range(3):
        rot = frame_rotation(40, f)
        r = oracle.ref_ray_dirs(rot, 256)          # the reference formula in plain FP32
        d64 = oracle.ray_dirs(rot, 256, precision=1)
        d32 = oracle.ray_dirs(rot, 256, precision=0)
        assert np.max(np.abs(r - d64)) < 5e-5       # plain FP32 madfrac loses ~2^-24 * i turns
        assert np.max(np.abs(d32 - d64)) < 2e-6     # the compensated evaluation does not


def _trace_pair(w, frames=0, prev=None, seed=41):
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    vd = w.volume.desc()
    rot = frame_rotation(seed, frames)
    dirs = oracle.ray_dirs(rot, vd.uniform.rays_per_probe, 0)
    pi, pd = (None, None) if prev is None else prev
    a, ia = oracle.ref_trace(vd, inp, rot, frames, pi, pd, dirs=dirs)
    b, ib = oracle.trace(vd, inp, rot, frames, pi, pd, precision=0)
    return host, a, ia, b, ib


@pytest.mark.parametrize("light", [N.LIGHT_PER_HIT, N.LIGHT_CACHE])
def test_trace_matches_reference_functions(ref, light):
    w = replace(PLAIN_SMALL, volume=replace(PLAIN_SMALL.volume, light_mode=light))
    host, a, ia, b, ib = _trace_pair(w)
    voxel = host.sdf_data.cascade_voxel_size[0]
    assert np.array_equal(ia[..., 0], ib[..., 0])            # march steps
    assert np.array_equal(ia[..., 1], ib[..., 1])            # hit cascade / miss
    assert np.all(np.abs(a[..., 3] - b[..., 3]) <= 1e-3 * voxel)
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-3 and np.quantile(rel, 0.99) < 1e-5


def test_trace_two_cascades_matches_reference(ref):
    w = tiny_workload(probe_counts=(4, 3, 4), rays=96, sdf=64, cascades=2, room=24.0, prims=10, steps=250)
    host, a, ia, b, ib = _trace_pair(w)
    assert (ia[..., 1] >= 0).any() and (ia[..., 1] == 1).any()   # both cascades used
    same = (ia[..., 0] == ib[..., 0]) & (ia[..., 1] == ib[..., 1])
    assert same.mean() > 0.999
    voxel = host.sdf_data.cascade_voxel_size[1]
    assert (np.abs(a[..., 3] - b[..., 3]) <= 1e-3 * voxel)[same].all()


def test_trace_bounce_matches_reference(ref):
    """Per-hit bounce (frame > 0) through the reference's sampleIrradiance."""
    w = PLAIN_SMALL
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    rots = [frame_rotation(42, f) for f in range(2)]
    irr, dist, frames, _ = oracle.run_frames(w.volume.desc(), inp, rots, precision=0)
    host2, a, ia, b, ib = _trace_pair(w, frames=frames, prev=(irr, dist), seed=42)
    assert np.array_equal(ia, ib[..., :2])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 2e-3 and np.quantile(rel, 0.99) < 1e-5


@pytest.mark.parametrize("sides", [(6, 14), (8, 16)])
def test_blend_matches_reference(ref, sides):
    w = tiny_workload(probe_counts=(5, 2, 3), rays=128, irr=sides[0], dist=sides[1])
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    vd = w.volume.desc()
    prev = None
    for f in range(3):
        rot = frame_rotation(43, f)
        rays, _ = oracle.trace(vd, inp, rot, f, *(prev or (None, None)), precision=0, want_info=False)
        dirs = oracle.ray_dirs(rot, vd.uniform.rays_per_probe, 0)
        pi, pd = prev or (None, None)
        a = oracle.ref_blend(vd, dirs, rays, pi, pd, first=(f == 0))
        b = oracle.blend(vd, dirs, rays, pi, pd, first=(f == 0), precision=0, border=False)
        u = vd.uniform
        for k, n in ((0, u.irradiance_probe_side), (1, u.depth_probe_side)):
            # interiors only: the reference writes borders in a separate pass
            H, W = a[k].shape[:2]
            m = np.zeros((H, W), dtype=bool)
            for cy in range(u.probe_counts[2]):
                for cx in range(u.probe_counts[0] * u.probe_counts[1]):
                    m[cy * (n + 2) + 2: cy * (n + 2) + 2 + n, cx * (n + 2) + 2: cx * (n + 2) + 2 + n] = True
            assert rel_err(a[k][m], b[k][m]) < 1e-5
        prev = oracle.blend(vd, dirs, rays, pi, pd, first=(f == 0), precision=0, border=True)


def test_sample_irradiance_matches_reference(ref):
    w = PLAIN_SMALL
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    rots = [frame_rotation(44, f) for f in range(3)]
    irr, dist, _, _ = oracle.run_frames(w.volume.desc(), inp, rots, precision=0)
    rng = np.random.default_rng(8)
    n = 2000
    pos = rng.uniform(-4, 4, size=(n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    u = w.volume.uniform()
    a = oracle.ref_sample_irradiance(u, irr, dist, pos, nrm, wo)
    b = oracle.sample_irradiance(u, irr, dist, pos, nrm, wo, precision=0)
    assert rel_err(a, b, floor=1e-2) < 1e-4


def _f16(bits) -> np.ndarray:
    return np.asarray(bits, dtype=np.uint16).view(np.float16).astype(np.float32)


def _test_lights():
    from luxgi_gb300.surface import make_light

    L = [None] * 3
    L[0] = make_light(N.LIGHT_DIRECTIONAL, (1.0, 0.95, 0.9), 2.0, direction=(0.3, -0.8, 0.5))
    L[1] = make_light(N.LIGHT_POINT, (0.4, 0.6, 1.0), 3.0, position=(1.0, 2.0, -0.5), radius=6.0)
    L[2] = make_light(N.LIGHT_SPOT, (1.0, 0.5, 0.2), 4.0, position=(-2.0, 3.0, 1.0), direction=(0.5, -1.0, -0.2),
                      radius=8.0, angle=0.3)
    return L


@pytest.mark.parametrize("fmt,copy_emissive", [(N.STORAGE_FP32, True), (N.STORAGE_FP16, False)])
def test_surface_light_matches_reference(ref, fmt, copy_emissive):
    """CopyEmissive + SDFDeferredLight (three lights, random per-tile light
    masks) against the reference's compiled BRDF, Light and tracyGlobalSDF:
    each light's draw rounds the FP16 target once, so the two agree within
    one rounding step per light (1e-3 relative), and no fragment's shadow
    test differs (a flip would change its value by far more)."""
    w = tiny_workload(sdf=32, prims=8, atlas=256, sdf_format=fmt)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    L = _test_lights()
    tiles = np.arange(1, host.num_tiles, dtype=np.uint32)
    masks = np.random.default_rng(3).integers(0, 8, size=tiles.size).astype(np.uint32)
    cam = (0.3, 0.5, -2.0)
    a, shadow = oracle.surface_light(inp, L, tiles, masks, cam, 1.0, copy_emissive, 250, 0, want_shadow=True)
    b = oracle.ref_surface_light(inp, L, tiles, masks, cam, 1.0, copy_emissive)
    assert np.count_nonzero(shadow) > 1000                  # shadows are exercised
    assert np.count_nonzero(a != host.direct) > 10000       # and the pass wrote the footprints
    assert np.isfinite(_f16(a)).all()
    assert rel_err(_f16(a), _f16(b)) < 3e-3
    assert np.mean(np.abs(_f16(a) - _f16(b)) > 1e-3 * np.maximum(np.abs(_f16(b)), 1e-3)) < 1e-4


def test_inject_matches_reference(ref):
    """SDFAtlasIndirectLight over the tile quads against the reference's
    compiled sampleIrradiance (metallic from the PBR atlas)."""
    w = tiny_workload(light=N.LIGHT_CACHE, prims=8)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    vd = w.volume.desc()
    rots = [frame_rotation(45, f) for f in range(2)]
    irr, dist, frames, _ = oracle.run_frames(vd, inp, rots, precision=0)
    a = oracle.inject(vd, inp, irr, dist, frames, precision=0)
    b = oracle.ref_inject(vd, inp, irr, dist)
    assert np.count_nonzero(a != host.direct) > 10000
    assert rel_err(_f16(a), _f16(b)) < 2e-3


@pytest.mark.parametrize("cascades,res", [(2, 64), (3, 32)])
def test_sdf_raster_matches_reference(ref, cascades, res):
    """The global SDF from placed mesh SDFs: the oracle's voxels against
    SDFRasterizeModel.glsl's main around the reference's compiled
    distanceToModelSDF / combineDistanceToSDF, cascade after cascade on the
    same plan (objects scattered beyond cascade 0, so chunks reach past
    it): within 2 ulps."""
    from luxgi_gb300.sdf import MeshSDF, box_distance, build_desc, sphere_distance, trs

    meshes = [MeshSDF.bake(box_distance((2.0, 1.0, 1.5)), (-2, -1, -1.5), (2, 1, 1.5), (24, 16, 20)),
              MeshSDF.bake(sphere_distance(1.2), (-1.2,) * 3, (1.2,) * 3, (16, 16, 16), mip_count=2)]
    rng = np.random.default_rng(cascades)
    objs = [(trs(rng.uniform(-90, 90, 3), rng.normal(size=3), rng.uniform(0, 6),
                 (1, 1, 1) if i % 2 else rng.uniform(0.5, 3, 3)), i % 2) for i in range(40)]
    d = build_desc(resolution=res, cascades=cascades, storage=N.STORAGE_FP32, global_scale=0.05)
    sdf, _, data = oracle.sdf_build(d, meshes, objs)
    b = np.ones_like(sdf)
    for c in range(cascades):
        recs, mesh, chunks = oracle.sdf_plan(d, meshes, objs, c)
        b = oracle.ref_sdf_raster(d, data, c, meshes, recs, mesh, chunks, b)
    assert (sdf < 1.0).mean() > 0.5
    assert np.max(np.abs(sdf - b)) <= 2.4e-7


def test_sample_probe_image_matches_reference(ref):
    """SampleProbe.comp (worldPositionFromDepth + octohedralToDirection +
    sampleIrradiance) over a synthetic G-buffer: the oracle's RGBA16F image
    against the reference's compiled functions, within one half-float
    rounding; background pixels 0."""
    from tests._helpers import synthetic_gbuffer

    w = tiny_workload(probe_counts=(4, 3, 4), rays=64)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode)
    rots = [frame_rotation(46, f) for f in range(3)]
    irr, dist, _, _ = oracle.run_frames(w.volume.desc(), inp, rots, precision=0)
    depth, normal, cam, vpi = synthetic_gbuffer(96, 64, seed=2)
    u = w.volume.uniform()
    a = oracle.sample_probe_image(u, irr, dist, depth, normal, cam, vpi).view(np.float16).astype(np.float32)
    b = oracle.ref_sample_probe_image(u, irr, dist, depth, normal, cam, vpi)
    bg = depth == 1.0
    assert bg.any() and (~bg).any()
    assert (a[bg] == 0).all() and (b[bg] == 0).all()
    assert np.isfinite(a).all() and (a[~bg][:, 3] == 1).all()
    assert rel_err(a[~bg], b[~bg], floor=1e-2) < 1.5e-3


def _r11(texels) -> np.ndarray:
    return oracle.unpack_colors(texels, N.COLOR_R11G11B10F)


def _engine_formats_close(a, b, draws):
    """Two R11G11B10F atlases written through `draws` rounding steps each:
    most codes identical, the rest within one code step (2^-6 relative for R
    and G, 2^-5 for B) per draw."""
    x, y = _r11(a)[:, :3], _r11(b)[:, :3]
    assert np.isfinite(x).all() and np.isfinite(y).all()
    assert np.mean(a != b) < 2e-3
    assert rel_err(x, y) <= draws * 2.0 ** -5


@pytest.mark.parametrize("copy_emissive", [True, False])
def test_surface_light_engine_formats_match_reference(ref, copy_emissive):
    """The lighting pass on the engine's texture formats -- R11G11B10F
    emissive and lit atlas, RGBA16F G-buffers (GlobalSurfaceAtlas.cpp:
    407-411) -- against the reference's compiled functions, each draw's
    result rounded to the 11/11/10-bit target by both."""
    w = tiny_workload(sdf=32, prims=8, atlas=256)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode, light_format=N.COLOR_R11G11B10F,
                            gbuffer_format=N.GBUFFER_RGBA16F)
    assert inp.direct.dtype == np.uint32 and inp.gbuffer0.dtype == np.uint16
    L = _test_lights()
    tiles = np.arange(1, host.num_tiles, dtype=np.uint32)
    masks = np.random.default_rng(4).integers(0, 8, size=tiles.size).astype(np.uint32)
    cam = (0.3, 0.5, -2.0)
    a = oracle.surface_light(inp, L, tiles, masks, cam, 1.0, copy_emissive, 250, 0)
    b = oracle.ref_surface_light(inp, L, tiles, masks, cam, 1.0, copy_emissive)
    assert a.dtype == np.uint32 and np.count_nonzero(a != inp.direct) > 10000
    _engine_formats_close(a, b, 1 + len(L))


def test_inject_and_trace_engine_formats_match_reference(ref):
    """Injection into an R11G11B10F light cache from RGBA16F G-buffers, and
    the light-cache trace sampling it, against the reference's compiled
    sampleIrradiance and sampleGlobalSurfaceAtlas."""
    w = tiny_workload(light=N.LIGHT_CACHE, prims=8)
    host = HostScene(w.scene)
    inp = oracle.HostInputs(host, w.volume.light_mode, light_format=N.COLOR_R11G11B10F,
                            gbuffer_format=N.GBUFFER_RGBA16F)
    vd = w.volume.desc()
    rots = [frame_rotation(47, f) for f in range(2)]
    irr, dist, frames, _ = oracle.run_frames(vd, inp, rots, precision=0)
    a = oracle.inject(vd, inp, irr, dist, frames, precision=0)
    b = oracle.ref_inject(vd, inp, irr, dist)
    assert np.count_nonzero(a != inp.direct) > 10000
    _engine_formats_close(a, b, 1)
    inp.light_cache[:] = a
    rot = frame_rotation(47, 2)
    rays, info = oracle.trace(vd, inp, rot, frames, irr, dist, precision=0)
    rr, rinfo = oracle.ref_trace(vd, inp, rot, frames, irr, dist, dirs=oracle.ray_dirs(rot, vd.uniform.rays_per_probe))
    assert np.array_equal(info[..., :2], rinfo)
    assert rel_err(rays[..., :3], rr[..., :3], floor=1e-2) < 1e-5
