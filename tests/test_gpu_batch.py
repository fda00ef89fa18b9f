"""Batched updates of many volumes (luxgi_ddgi_update_batch and the
luxgi_ddgi_batch_* objects) against the same volumes updated alone.

The batched kernels run the per-ray and per-texel code of the single-volume
kernels from the same translation units; the compiler's FMA contraction in
the shading and blend units may still round a few values one ulp apart, so
atlases must agree within 1e-6 relative (FP32 storage) or one FP16 rounding
step (1e-3, FP16 storage), and the march (no contraction) exactly.  Where
the autotuner picks a different shade variant the shading differs by its
approximate division (1e-4 relative, as in test_gpu_parity).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIBatch, DDGIVolume, frame_rotation, update_batch
from luxgi_gb300.scene import DeviceScene, HostScene, batch_workloads
from tests._helpers import rel_err, tiny_workload

pytestmark = pytest.mark.gpu


def _np(t):
    import torch

    t = t.detach().cpu()
    if t.dtype == torch.float16:
        t = t.float()
    return t.numpy()


def _pairs(blend, storage=N.STORAGE_FP32, n=5, seed=11):
    """n uneven small volumes, each with its own scene, twice: (alone, batched)."""
    ws = batch_workloads(count=n, seed=seed, max_counts=(7, 4, 6), min_counts=(2, 2, 2), sdf_range=(32, 64),
                         atlas_range=(256, 512), blend=blend, storage=storage, max_steps=48)
    scenes, alone, batched = [], [], []
    for w in ws:
        host = HostScene(w.scene)
        dev = DeviceScene(host, w.volume.light_mode)
        a, b = DDGIVolume(w.volume), DDGIVolume(w.volume)
        a.bind_scene(dev)
        b.bind_scene(dev)
        a.set_debug_rays(True)
        b.set_debug_rays(True)
        scenes.append((host, dev))
        alone.append(a)
        batched.append(b)
    return scenes, alone, batched


def _rots(n, frame):
    return np.stack([frame_rotation(0xBA7C + i, frame) for i in range(n)])


def _assert_same(alone, batched, exact=True):
    import torch

    torch.cuda.synchronize()
    for a, b in zip(alone, batched):
        assert a.frames == b.frames
        tol = (1e-3 if a.spec.storage == N.STORAGE_FP16 else 1e-6) if exact else 1e-4
        for x, y in zip(a.atlases(), b.atlases()):
            x, y = _np(x), _np(y)
            assert x.shape == y.shape
            assert rel_err(y, x) <= tol
        # march records (no FMA contraction): identical
        ia, ib = a.rays()[2], b.rays()[2]
        if ia is not None and ib is not None:
            np.testing.assert_array_equal(_np(ia), _np(ib))


@pytest.mark.parametrize("blend", [N.BLEND_FP32, N.BLEND_TENSOR])
@pytest.mark.parametrize("use_graph,shade_order,march_budget", [(1, 0, 0), (0, 0, 0), (1, -1, -1), (0, 1, 3)])
def test_batch_equals_single(cuda, blend, use_graph, shade_order, march_budget):
    _, alone, batched = _pairs(blend)
    batch = DDGIBatch(batched, {"use_graph": use_graph, "shade_order": shade_order, "march_budget": march_budget})
    n = len(alone)
    for f in range(3):
        rots = _rots(n, f)
        for v, r in zip(alone, rots):
            v.update(r)
        batch.update(rots)
        _assert_same(alone, batched)


def test_tensor_blend_jobs_spanning_ctas(cuda):
    """Three volumes of 2,048 probes with 64, 192 and 128 rays: the batch's
    one tensor-core launch holds 288 tiles for at most one CTA per SM, so
    CTAs' tile ranges cross from one job into the next and reload the
    weights (of another ray count, a smaller B than the widest job's) after
    the last multiply of the previous job.  Every batched frame's atlases
    are within the tensor-core bound (2e-3) of the FP64 blend of the
    volume's own rays, and within 1e-3 of the volume updated alone (one
    launch of its two jobs, one tile a CTA; the batched and single-volume
    shading kernels may round a radiance one ulp apart, which an FP16
    operand can turn into a few 1e-6).  Weights of the wrong job or a stale
    B would be off by far more."""
    import torch

    ws = [tiny_workload(probe_counts=(16, 8, 16), spacing=0.6, rays=r, blend=N.BLEND_TENSOR, seed=40 + i, steps=32)
          for i, r in enumerate((64, 192, 128))]
    scenes, alone, batched = [], [], []
    for w in ws:
        host = HostScene(w.scene)
        dev = DeviceScene(host, w.volume.light_mode)
        a, b = DDGIVolume(w.volume), DDGIVolume(w.volume)
        a.bind_scene(dev)
        b.bind_scene(dev)
        scenes.append((host, dev))
        alone.append(a)
        batched.append(b)
    batch = DDGIBatch(batched)
    prev = [(None, None)] * len(ws)
    for f in range(3):
        rots = _rots(len(ws), f)
        batch.update(rots)
        for v, r in zip(alone, rots):
            v.update(r)
        torch.cuda.synchronize()
        for i, (a, b) in enumerate(zip(alone, batched)):
            a.check_status()
            b.check_status()
            assert a.frames == b.frames == f + 1
            gi, gd = (_np(t) for t in b.atlases())
            rad = _np(b.rays()[1])
            ref = oracle.blend(b.desc, oracle.ray_dirs(rots[i], b.uniform.rays_per_probe, 1), rad, prev[i][0],
                               prev[i][1], first=(f == 0), precision=1)
            assert rel_err(gi, ref[0]) < 2e-3 and rel_err(gd, ref[1]) < 2e-3, (f, i)
            for x, y in zip(a.atlases(), (gi, gd)):
                assert rel_err(y, _np(x)) < 1e-3, (f, i)
            prev[i] = (gi, gd)


def test_batch_fp16_storage_and_tuning_knobs(cuda):
    _, alone, batched = _pairs(N.BLEND_FP32, storage=N.STORAGE_FP16, n=4, seed=12)
    batch = DDGIBatch(batched, {"march_variant": 5, "march_threads": 128, "blend_probes": 4})
    n = len(alone)
    for f in range(2):
        rots = _rots(n, f)
        for v, r in zip(alone, rots):
            v.update(r)
        batch.update(rots)
    # march variants are bit-identical and the shade variant is the same
    _assert_same(alone, batched)


@pytest.mark.parametrize("tpb,mv", [(128, 10), (256, 10), (128, 11), (256, 11)])
def test_batch_gather_texture_march(cuda, tpb, mv):
    """The batched march over the gather textures (variant 10; variant 11 the
    quad-packed mip with the full-resolution gathers): every volume equals
    its own update (march records exact)."""
    _, alone, batched = _pairs(N.BLEND_FP32, n=4, seed=15)
    batch = DDGIBatch(batched, {"march_variant": mv, "march_threads": tpb})
    assert batch.tuning["march_variant"] == mv
    for f in range(2):
        rots = _rots(len(alone), f)
        for v, r in zip(alone, rots):
            v.update(r)
        batch.update(rots)
    _assert_same(alone, batched)


def test_update_batch_groups_and_falls_back(cuda):
    _, alone, batched = _pairs(N.BLEND_FP32, n=4, seed=13)
    _, alone16, batched16 = _pairs(N.BLEND_FP32, storage=N.STORAGE_FP16, n=2, seed=14)
    vols_a = alone + alone16
    vols_b = batched + batched16
    n = len(vols_a)
    for f in range(3):
        rots = _rots(n, f)
        for v, r in zip(vols_a, rots):
            v.update(r)
        update_batch(vols_b, rots)
        _assert_same(vols_a, vols_b)


def test_batch_autotune_keeps_state(cuda):
    import torch

    _, alone, batched = _pairs(N.BLEND_FP32, n=4, seed=15)
    batch = DDGIBatch(batched)
    n = len(alone)
    for f in range(2):
        rots = _rots(n, f)
        for v, r in zip(alone, rots):
            v.update(r)
        batch.update(rots)
    torch.cuda.synchronize()
    before = [[_np(t).copy() for t in v.atlases("current") + v.atlases("prev")] for v in batched]
    frames = [v.frames for v in batched]
    best = batch.autotune(frames=1)
    assert best["frame_ms"] > 0.0
    assert best == batch.tuning
    torch.cuda.synchronize()
    after = [[_np(t) for t in v.atlases("current") + v.atlases("prev")] for v in batched]
    assert [v.frames for v in batched] == frames
    for x, y in zip(before, after):
        for p, q in zip(x, y):
            np.testing.assert_array_equal(p, q)
    rots = _rots(n, 2)
    for v, r in zip(alone, rots):
        v.update(r)
    batch.update(rots)
    _assert_same(alone, batched, exact=best["shade_variant"] == 1)


def test_batch_rejects_incompatible(cuda):
    _, _, b32 = _pairs(N.BLEND_FP32, n=2, seed=16)
    _, _, b16 = _pairs(N.BLEND_FP32, storage=N.STORAGE_FP16, n=1, seed=17)
    with pytest.raises(N.LuxgiError) as e:
        DDGIBatch(b32 + b16)
    assert e.value.status == N.LUXGI_EINVAL
    with pytest.raises(N.LuxgiError) as e:
        DDGIBatch([b32[0], b32[0]])
    assert e.value.status == N.LUXGI_EINVAL
    with pytest.raises(N.LuxgiError) as e:
        DDGIBatch(b32, {"march_variant": 7})
    assert e.value.status == N.LUXGI_EINVAL
    ws = batch_workloads(count=1, seed=18, max_counts=(3, 3, 3), min_counts=(2, 2, 2), sdf_range=(32, 32),
                         atlas_range=(256, 256), blend=N.BLEND_FP32)
    unbound = DDGIVolume(ws[0].volume)
    with pytest.raises(N.LuxgiError) as e:
        DDGIBatch([b32[0], unbound])
    assert e.value.status == N.LUXGI_ENOTBOUND
    with pytest.raises(N.LuxgiError) as e:
        update_batch([b32[0], b32[0]], _rots(2, 0))
    assert e.value.status == N.LUXGI_EINVAL


@pytest.mark.parametrize("blend", [N.BLEND_FP32, N.BLEND_TENSOR])
def test_batch_launch_count(cuda, blend):
    import torch

    _, _, batched = _pairs(blend, n=3, seed=19)
    batch = DDGIBatch(batched)
    lib = N.ddgi()
    batch.update(_rots(3, 0))          # captures the graph of argument block 0
    batch.update(_rots(3, 1))          # and of block 1
    torch.cuda.synchronize()
    c0 = lib.luxgi_launch_count()
    batch.update(_rots(3, 2))
    torch.cuda.synchronize()
    per_frame = lib.luxgi_launch_count() - c0
    # raygen, weights, march (one pass: small batches do not compact by
    # default), shade (march order) + blend: 2 FP32 launches, or the
    # operand pack and one tensor-core launch for every volume's two kinds
    assert per_frame == 4 + (2 if blend == N.BLEND_FP32 else 1 + 1)
