"""GPU parity of the global SDF built from placed mesh SDFs
(luxgi_sdf_build) against the oracle, and of a probe update traced through
it.

Tolerances: the rasterisation and the mip are FP32 without FMA contraction
on both sides with the same association, so the SDF and its mip are
bit-identical (FP16 and FP32 storage); the probe update over the built SDF
is held to the bars of the probe-update parity tests (march records
bit-exact, atlases 1e-3 relative with FP16 storage).
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import DeviceScene, HostScene
from luxgi_gb300.sdf import GlobalSDF, MeshSDF, box_distance, build_desc, sphere_distance, trs
from tests._helpers import rel_err, tiny_workload

pytestmark = pytest.mark.gpu


def _meshes():
    return [MeshSDF.bake(box_distance((2.0, 1.0, 1.5)), (-2, -1, -1.5), (2, 1, 1.5), (24, 16, 20)),
            MeshSDF.bake(sphere_distance(1.2), (-1.2,) * 3, (1.2,) * 3, (16, 16, 16), mip_count=2),
            MeshSDF.bake(box_distance((0.3, 3.0, 0.3)), (-0.3, -3, -0.3), (0.3, 3, 0.3), (8, 40, 8), mip_count=1)]


def _objects(n, seed, spread):
    rng = np.random.default_rng(seed)
    return [(trs(rng.uniform(-spread, spread, 3), rng.normal(size=3), rng.uniform(0, 6),
                 (1, 1, 1) if i % 3 else rng.uniform(0.5, 3, 3)), i % 3) for i in range(n)]


def _host(t, fmt):
    a = t.cpu().numpy()
    return a.view(np.float16).astype(np.float32) if fmt == N.STORAGE_FP16 else a


@pytest.mark.parametrize("fmt", [N.STORAGE_FP16, N.STORAGE_FP32])
@pytest.mark.parametrize("cascades,res,spread", [(1, 64, 40.0), (2, 64, 90.0), (4, 32, 300.0)])
def test_sdf_build_bit_exact(cuda, fmt, cascades, res, spread):
    import torch

    meshes = _meshes()
    objs = _objects(48, seed=cascades * 7 + res, spread=spread)
    d = build_desc(resolution=res, cascades=cascades, storage=fmt, global_scale=0.05)
    g = GlobalSDF(d)
    g.build(meshes, objs)
    torch.cuda.synchronize()
    sdf, mip, data = oracle.sdf_build(d, meshes, objs)
    assert bytes(g.data) == bytes(data)
    gs, gm = _host(g.sdf, fmt), _host(g.mip, fmt)
    assert (sdf < 1.0).mean() > 0.3
    np.testing.assert_array_equal(gs, sdf)
    np.testing.assert_array_equal(gm, mip)


def test_sdf_build_empty_and_crowded(cuda):
    """No objects (every voxel 1, no flood passes) and 40 objects in one
    chunk (the chunk table keeps the last 12)."""
    import torch

    meshes = _meshes()
    d = build_desc(resolution=32, cascades=2, storage=N.STORAGE_FP16, global_scale=0.05)
    g = GlobalSDF(d)
    g.build(meshes, [])
    torch.cuda.synchronize()
    sdf, mip, _ = oracle.sdf_build(d, meshes, [])
    assert (sdf == 1.0).all()
    np.testing.assert_array_equal(_host(g.sdf, d.format), sdf)
    np.testing.assert_array_equal(_host(g.mip, d.format), mip)
    objs = [(trs((3.0 + 0.3 * i, 2.0, 1.0)), i % 2) for i in range(40)]
    g.build(meshes, objs)
    torch.cuda.synchronize()
    sdf, mip, _ = oracle.sdf_build(d, meshes, objs)
    np.testing.assert_array_equal(_host(g.sdf, d.format), sdf)
    np.testing.assert_array_equal(_host(g.mip, d.format), mip)


def test_probe_update_over_built_sdf(cuda):
    """The built SDF feeds the path: a probe volume traced and blended over
    the GPU-built global SDF equals the oracle's frames over the oracle-built
    one (march records bit-exact, atlases within 1e-3)."""
    import torch

    meshes = _meshes()
    objs = _objects(60, seed=3, spread=14.0)
    d = build_desc(resolution=64, cascades=2, storage=N.STORAGE_FP16, gi_distance=400.0, global_scale=0.1)
    g = GlobalSDF(d)
    g.build(meshes, objs)
    w = tiny_workload(light=N.LIGHT_CACHE, prims=6, steps=128, storage=N.STORAGE_FP16)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    vol = DDGIVolume(w.volume)
    vol.bind_scene(SimpleNamespace(sdf_desc=g.sdf_desc, surface_desc=dev.surface_desc, keep=(g, dev)))
    vol.set_debug_rays(True)
    rots = [frame_rotation(81, f) for f in range(3)]
    for r in rots:
        vol.update(r)
    torch.cuda.synchronize()
    sdf, mip, data = oracle.sdf_build(d, meshes, objs)
    inp = oracle.HostInputs(host, w.volume.light_mode, chunks=dev.chunks.cpu().numpy().view(np.uint32),
                            culled=dev.culled.cpu().numpy().view(np.uint32))
    s16 = sdf.astype(np.float16).view(np.uint16)
    m16 = mip.astype(np.float16).view(np.uint16)
    inp.sdf_desc.data = data
    inp.sdf_desc.format = N.STORAGE_FP16
    inp.sdf_desc.resolution = d.resolution
    inp.sdf_desc.mip_resolution = d.resolution // 4
    inp.sdf_desc.sdf = s16.ctypes.data
    inp.sdf_desc.mip = m16.ctypes.data
    oi, od, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=0)
    irr, dist = vol.atlases()
    gi = irr.detach().cpu().float().numpy()
    gd = dist.detach().cpu().float().numpy()
    assert rel_err(gi, oi) < 1e-3
    assert rel_err(gd, od) < 1e-3
    # the rays hit the placed objects
    info = vol.rays()[2].cpu().numpy().reshape(-1, 4)
    assert (info[:, 1] >= 0).mean() > 0.1
