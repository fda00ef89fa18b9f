"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle
on the same seeded inputs.

Tolerances (stated per test):
  - SDF mip, chunk culling, march steps / hit cascade / hit distance:
    bit-exact against the FP32 oracle (the march is FP32 without FMA
    contraction in both);
  - FP32 blend: 1e-5 relative to the FP32 oracle, 1e-4 to the FP64 oracle;
  - FP16 storage: 2 half-ulps (1e-3 relative);
  - hit distance vs FP64: 1e-3 voxel except branch-flipped rays (< 1%).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import PLAIN_SMALL, PLAIN_SMALL_REF, DeviceScene, HostScene
from tests._helpers import rel_err, tiny_workload

pytestmark = pytest.mark.gpu


def _np(t):
    import torch

    t = t.detach().cpu()
    if t.dtype == torch.float16:
        t = t.float()
    return t.numpy()


def setup(w, debug=True):
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    vol = DDGIVolume(w.volume)
    vol.bind_scene(dev)
    if debug:
        vol.set_debug_rays(True)
    mip = dev.mip.cpu().numpy()
    if host.sdf_format == N.STORAGE_FP16:
        mip = mip.view(np.uint16)
    inp = oracle.HostInputs(host, w.volume.light_mode, mip=mip, chunks=dev.chunks.cpu().numpy().view(np.uint32),
                            culled=dev.culled.cpu().numpy().view(np.uint32))
    return host, dev, vol, inp


def sync():
    import torch

    torch.cuda.synchronize()


@pytest.mark.parametrize("fmt,cascades", [(N.STORAGE_FP32, 1), (N.STORAGE_FP16, 1), (N.STORAGE_FP32, 2)])
def test_sdf_mip_bit_exact(cuda, fmt, cascades):
    w = tiny_workload(sdf=64, sdf_format=fmt, cascades=cascades)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    sync()
    ref = oracle.build_mip(oracle.HostInputs(host, w.volume.light_mode).sdf_desc, host.sdf_float())
    got = dev.mip.cpu().numpy()
    if fmt == N.STORAGE_FP16:
        got = got.view(np.float16).astype(np.float32)
    assert np.array_equal(got, ref)


def test_surface_cull_bit_exact(cuda):
    w = PLAIN_SMALL
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    sync()
    inp = oracle.HostInputs(host, w.volume.light_mode)
    chunks = dev.chunks.cpu().numpy().view(np.uint32)
    culled = dev.culled.cpu().numpy().view(np.uint32)
    assert np.array_equal(chunks, inp.chunks)
    used = int(inp.culled[0])
    assert culled[0] == used
    assert np.array_equal(culled[:used], inp.culled[:used])


def test_surface_cull_capacity_overflow(cuda):
    import ctypes
    import torch

    w = tiny_workload(prims=10)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    need = int(dev.culled[0].item())
    small = torch.zeros(need // 2, dtype=torch.int32, device="cuda")
    chunks = torch.zeros(40 ** 3, dtype=torch.int32, device="cuda")
    st = N.ddgi().luxgi_surface_cull(ctypes.byref(dev.surface_desc), chunks.data_ptr(), small.data_ptr(), need // 2,
                                     torch.cuda.current_stream().cuda_stream)
    assert st == N.LUXGI_ENOMEM
    inp = oracle.HostInputs(host, w.volume.light_mode)
    ch, cu, ost = oracle.cull(inp.surface_desc, need // 2)
    assert ost == N.LUXGI_ENOMEM
    assert np.array_equal(chunks.cpu().numpy().view(np.uint32), ch)


def _check_trace(vol, inp, vd, rot, frames=0, prev=None):
    dirs, rad, info = vol.rays()
    sync()
    rad, info = _np(rad), info.cpu().numpy()
    pi, pd = (None, None) if prev is None else prev
    ref, rinfo = oracle.trace(vd, inp, rot, frames, pi, pd, precision=0)
    assert np.array_equal(info, rinfo), np.argwhere(info != rinfo)[:5]
    assert np.array_equal(rad[..., 3], ref[..., 3])
    # shading runs with approximate division / square root: 1e-4 relative
    # (FP32 storage), one half-ulp when the radiance is stored as FP16
    if vd.storage == N.STORAGE_FP16:
        np.testing.assert_allclose(rad[..., :3], ref[..., :3], rtol=1e-3, atol=1e-4)
    else:
        np.testing.assert_allclose(rad[..., :3], ref[..., :3], rtol=1e-4, atol=2e-6)
    np.testing.assert_array_equal(_np(dirs), oracle.ray_dirs(rot, vd.uniform.rays_per_probe, 0))
    return rad, ref


@pytest.mark.parametrize("light", [N.LIGHT_PER_HIT, N.LIGHT_CACHE])
def test_trace_bit_exact_plain_small(cuda, light):
    from dataclasses import replace

    w = replace(PLAIN_SMALL, volume=replace(PLAIN_SMALL.volume, light_mode=light))
    host, dev, vol, inp = setup(w)
    rot = frame_rotation(21, 0)
    vol.trace(rot)
    _check_trace(vol, inp, vol.desc, rot)


def test_trace_hit_distance_vs_fp64(cuda):
    w = PLAIN_SMALL
    host, dev, vol, inp = setup(w)
    rot = frame_rotation(22, 0)
    vol.trace(rot)
    _, rad, info = vol.rays()
    sync()
    rad = _np(rad)
    ref, _ = oracle.trace(vol.desc, inp, rot, precision=1)
    voxel = host.sdf_data.cascade_voxel_size[0]
    ok = np.abs(rad[..., 3] - ref[..., 3]) <= 1e-3 * voxel
    assert ok.mean() > 0.99, f"flip fraction {1 - ok.mean():.4f}"


def test_blend_matches_oracle_fp32_and_fp64(cuda):
    w = PLAIN_SMALL
    host, dev, vol, inp = setup(w, debug=False)
    u = vol.uniform
    rot = frame_rotation(23, 0)
    vol.trace(rot)
    vol.probe_update()
    vol.end_frame()
    irr, dist = vol.atlases()
    _, rad, _ = vol.rays()
    sync()
    rays = _np(rad)
    dirs = oracle.ray_dirs(rot, u.rays_per_probe, 0)
    r32 = oracle.blend(vol.desc, dirs, rays, first=True, precision=0)
    r64 = oracle.blend(vol.desc, oracle.ray_dirs(rot, u.rays_per_probe, 1), rays, first=True, precision=1)
    gi, gd = _np(irr), _np(dist)
    assert rel_err(gi, r32[0]) < 1e-5
    assert rel_err(gd, r32[1]) < 1e-5
    assert rel_err(gi, r64[0]) < 1e-4
    assert rel_err(gd, r64[1]) < 1e-4


def test_border_standalone_equals_fused(cuda):
    w = PLAIN_SMALL
    host, dev, vol, inp = setup(w, debug=False)
    rot = frame_rotation(24, 0)
    vol.trace(rot)
    vol.probe_update()
    vol.end_frame()
    irr, dist = vol.atlases()
    a, b = irr.clone(), dist.clone()
    # zero the border of the last written copy, then rebuild it in place
    u = vol.uniform
    for t, n in ((irr, u.irradiance_probe_side), (dist, u.depth_probe_side)):
        H, W = t.shape[:2]
        for y in range(1, H - 1, n + 2):
            t[y, :] = 0
            t[y + n + 1, :] = 0
        for x in range(1, W - 1, n + 2):
            t[:, x] = 0
            t[:, x + n + 1] = 0
    # border_update works on the write copy (1 - pingPong): step back a frame
    N.ddgi().luxgi_ddgi_end_frame(vol.handle)
    vol.border_update()
    sync()
    irr2, dist2 = vol.atlases("prev")
    assert np.array_equal(_np(irr2), _np(a))
    assert np.array_equal(_np(dist2), _np(b))


def test_multi_frame_per_hit_bounce(cuda):
    """Eight frames with infinite bounce from the previous frame's atlases."""
    w = PLAIN_SMALL
    host, dev, vol, inp = setup(w, debug=False)
    rots = [frame_rotation(25, f) for f in range(w.frames)]
    for r in rots:
        vol.update(r)
    irr, dist = vol.atlases()
    sync()
    oi, od, frames, _ = oracle.run_frames(vol.desc, inp, rots, precision=0)
    assert frames == w.frames == vol.frames
    assert rel_err(_np(irr), oi) < 1e-4
    assert rel_err(_np(dist), od) < 1e-4
    oi64, od64, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=1)
    assert rel_err(_np(irr), oi64) < 1e-4
    assert rel_err(_np(dist), od64) < 1e-4


def test_reference_parity_mode_fp16_light_cache(cuda):
    """8/16 sides, 250 steps, FP16 storage, light-cache bounce injected
    every 2 frames (the reference's own configuration of the path)."""
    w = PLAIN_SMALL_REF
    host, dev, vol, inp = setup(w, debug=False)
    rots = [frame_rotation(26, f) for f in range(5)]
    for f, r in enumerate(rots):
        if f > 0 and f % 2 == 0:
            vol.inject_indirect()
        vol.update(r)
    irr, dist = vol.atlases()
    light = dev.light_cache.cpu().numpy().view(np.uint16)
    sync()
    oi, od, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=0, inject_every=2)
    assert rel_err(_np(irr), oi) < 2e-3
    assert rel_err(_np(dist), od) < 2e-3
    lo = inp.light_cache.view(np.float16).astype(np.float32)
    lg = light.view(np.float16).astype(np.float32)
    assert rel_err(lg, lo, floor=1e-2) < 2e-3


def test_sample_irradiance_matches_oracle(cuda):
    import torch

    w = PLAIN_SMALL
    host, dev, vol, inp = setup(w, debug=False)
    for f in range(3):
        vol.update(frame_rotation(27, f))
    irr, dist = vol.atlases()
    rng = np.random.default_rng(5)
    n = 4096
    pos = rng.uniform(-4, 4, size=(n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    out = torch.zeros(n, 3, device="cuda")
    vol.sample_irradiance(torch.from_numpy(pos).cuda(), torch.from_numpy(nrm).cuda(), torch.from_numpy(wo).cuda(), out)
    sync()
    ref = oracle.sample_irradiance(vol.uniform, _np(irr), _np(dist), pos, nrm, wo, precision=1)
    assert rel_err(out.cpu().numpy(), ref, floor=1e-2) < 1e-4


@pytest.mark.parametrize("storage,channels", [(N.STORAGE_FP32, 4), (N.STORAGE_FP16, 2)])
def test_sample_probe_image_matches_oracle(cuda, storage, channels):
    """SampleProbe.comp over a synthetic screen G-buffer (luxgi_ddgi_sample_probe_image)
    against the oracle: the same RGBA16F image within one half-float
    rounding; background pixels exactly 0."""
    import torch

    from tests._helpers import synthetic_gbuffer

    w = tiny_workload(probe_counts=(4, 3, 4), rays=64, storage=storage)
    host, dev, vol, inp = setup(w, debug=False)
    for f in range(3):
        vol.update(frame_rotation(28, f))
    irr, dist = vol.atlases()
    depth, normal, cam, vpi = synthetic_gbuffer(160, 96, seed=3, channels=channels)
    out = vol.sample_probe_image(torch.from_numpy(depth).cuda(), torch.from_numpy(normal).cuda(), cam, vpi)
    sync()
    g = out.cpu().float().numpy()
    o = oracle.sample_probe_image(vol.uniform, _np(irr), _np(dist), depth, normal, cam, vpi)
    o = o.view(np.float16).astype(np.float32)
    bg = depth == 1.0
    assert (g[bg] == 0).all()
    assert rel_err(g[~bg], o[~bg], floor=1e-2) < 1.5e-3
    assert np.mean(g[~bg] != o[~bg]) < 0.01


@pytest.mark.parametrize("kw", [
    dict(probe_counts=(1, 1, 1), rays=1),
    dict(probe_counts=(1, 1, 1), rays=33, irr=1, dist=2),
    dict(probe_counts=(5, 1, 3), rays=17, irr=2, dist=3),
    dict(probe_counts=(2, 3, 2), rays=64, cascades=2, sdf=32),
    dict(probe_counts=(4, 2, 2), rays=40, sdf_format=N.STORAGE_FP16, storage=N.STORAGE_FP16),
    dict(probe_counts=(3, 3, 3), rays=32, spacing=9.0),       # probes outside the room: misses
])
@pytest.mark.parametrize("mv", [0, 4, 10, 11])
def test_edge_shapes(cuda, kw, mv):
    """Degenerate and small shapes, with the default march variant and
    with the quad-packed (4), gather-texture (10) and mixed (11: quad mip,
    gather full resolution) samplers, whose hit normals sample one texel
    past the cascade's edges."""
    from dataclasses import replace

    w = tiny_workload(**kw)
    w = replace(w, volume=replace(w.volume, march_variant=mv))
    host, dev, vol, inp = setup(w)
    rots = [frame_rotation(28, f) for f in range(3)]
    prev = None
    for f, r in enumerate(rots):
        vol.trace(r)
        _check_trace(vol, inp, vol.desc, r, f, prev)
        vol.probe_update()
        vol.end_frame()
        irr, dist = vol.atlases()
        sync()
        prev = (_np(irr), _np(dist))
    oi, od, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=0)
    tol = 2e-3 if w.volume.storage == N.STORAGE_FP16 else 1e-4
    assert rel_err(prev[0], oi) < tol
    assert rel_err(prev[1], od) < tol


def test_runs_are_deterministic(cuda):
    w = tiny_workload(probe_counts=(6, 3, 6), rays=96)
    outs = []
    for _ in range(2):
        host, dev, vol, inp = setup(w, debug=False)
        for f in range(3):
            vol.update(frame_rotation(29, f))
        irr, dist = vol.atlases()
        outs.append((_np(irr), _np(dist)))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_unbound_volume_reports(cuda):
    w = tiny_workload()
    vol = DDGIVolume(w.volume)
    with pytest.raises(N.LuxgiError) as e:
        vol.trace(frame_rotation(1, 0))
    assert e.value.status == N.LUXGI_ENOTBOUND


# ------------------------------------------------------------ tensor-core blend
# Tolerance: 2e-3 relative to the FP64 oracle (FP16 operands, FP32
# accumulation; the distance data split hi + lo).
@pytest.mark.parametrize("sides,rays", [((6, 14), 256), ((8, 16), 128), ((6, 14), 288), ((8, 16), 64)])
def test_tensor_blend_vs_fp64(cuda, sides, rays):
    from dataclasses import replace

    w = tiny_workload(probe_counts=(7, 3, 5), rays=rays, irr=sides[0], dist=sides[1], blend=N.BLEND_TENSOR)
    host, dev, vol, inp = setup(w, debug=False)
    u = vol.uniform
    rots = [frame_rotation(31, f) for f in range(3)]
    prev = None
    for f, r in enumerate(rots):
        vol.trace(r)
        _, rad, _ = vol.rays()
        sync()
        rays_np = _np(rad)
        vol.probe_update()
        vol.end_frame()
        vol.check_status()
        irr, dist = vol.atlases()
        sync()
        pi, pd = (None, None) if prev is None else prev
        ref = oracle.blend(vol.desc, oracle.ray_dirs(r, u.rays_per_probe, 1), rays_np, pi, pd, first=(f == 0),
                           precision=1)
        gi, gd = _np(irr), _np(dist)
        assert rel_err(gi, ref[0]) < 2e-3
        assert rel_err(gd, ref[1]) < 2e-3
        prev = (gi, gd)


def test_tensor_blend_fp16_storage_vs_fp64(cuda):
    """The tensor-core blend writing FP16 atlases (its half-precision
    history loads and stores): within the tensor-core bound plus one FP16
    rounding step (2^-10) of the FP64 blend, which rounds its stored values
    to FP16 the same way and weights the rays by their FP16-stored
    directions (the reference's RGBA16F direction-distance texture)."""
    w = tiny_workload(probe_counts=(7, 3, 5), rays=128, irr=6, dist=14, blend=N.BLEND_TENSOR,
                      storage=N.STORAGE_FP16)
    host, dev, vol, inp = setup(w, debug=False)
    u = vol.uniform
    prev = None
    for f in range(3):
        r = frame_rotation(33, f)
        vol.trace(r)
        _, rad, _ = vol.rays()
        sync()
        rays_np = _np(rad)
        vol.probe_update()
        vol.end_frame()
        vol.check_status()
        irr, dist = vol.atlases()
        sync()
        pi, pd = (None, None) if prev is None else prev
        ref = oracle.blend(vol.desc, oracle.ray_dirs(r, u.rays_per_probe, 1, True), rays_np, pi, pd, first=(f == 0),
                           precision=1)
        gi, gd = _np(irr), _np(dist)
        assert rel_err(gi, ref[0]) < 2e-3 + 2.0 ** -10, (f, rel_err(gi, ref[0]))
        assert rel_err(gd, ref[1]) < 2e-3 + 2.0 ** -10, (f, rel_err(gd, ref[1]))
        prev = (gi, gd)


def test_tensor_blend_matches_fp32_blend_on_plain_small(cuda):
    from dataclasses import replace

    outs = {}
    for blend in (N.BLEND_FP32, N.BLEND_TENSOR):
        w = replace(PLAIN_SMALL, volume=replace(PLAIN_SMALL.volume, blend=blend))
        host, dev, vol, inp = setup(w, debug=False)
        for f in range(4):
            vol.update(frame_rotation(32, f))
        vol.check_status()
        irr, dist = vol.atlases()
        outs[blend] = (_np(irr), _np(dist))
    assert rel_err(outs[N.BLEND_TENSOR][0], outs[N.BLEND_FP32][0]) < 2e-3
    assert rel_err(outs[N.BLEND_TENSOR][1], outs[N.BLEND_FP32][1]) < 2e-3


@pytest.mark.parametrize("fmt", [N.STORAGE_FP32, N.STORAGE_FP16])
def test_march_variants_bit_identical(cuda, fmt):
    """Every march variant (register bound, quad-packed mip / volume, gather
    textures) reads the same texel values: per-ray results are identical and
    equal the FP32 oracle."""
    from dataclasses import replace

    base = tiny_workload(probe_counts=(6, 3, 5), rays=64, sdf=64, sdf_format=fmt, cascades=2, room=20.0, prims=10)
    outs = []
    for mv in (1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11):
        w = replace(base, volume=replace(base.volume, march_variant=mv))
        host, dev, vol, inp = setup(w)
        rot = frame_rotation(50, 0)
        vol.trace(rot)
        rad, ref = _check_trace(vol, inp, vol.desc, rot)
        _, _, info = vol.rays()
        outs.append((rad, info.cpu().numpy()))
    for rad, info in outs[1:]:
        assert np.array_equal(rad, outs[0][0]) and np.array_equal(info, outs[0][1])


@pytest.mark.parametrize("fmt", [N.STORAGE_FP32, N.STORAGE_FP16])
def test_march_compaction_and_ray_order_bit_identical(cuda, fmt):
    """Suspending marches after a step budget and resuming them from the
    queues (budgets 1, 2, 8; budget 1 overflows the queues, whose rays then
    finish in place), the tiled ray order, shading in hit-chunk order, and
    that shading split in two (the pass-1 finishers on a second stream while
    the resume passes run, the queued rays after them) give exactly the
    one-pass results, and those equal the FP32 oracle."""
    from dataclasses import replace

    base = tiny_workload(probe_counts=(7, 3, 5), rays=64, sdf=64, sdf_format=fmt, cascades=2, room=20.0, prims=10)
    outs = []
    for mv, budget, order, sorder, split in ((4, -1, 0, -1, 0), (4, 1, 0, 1, 1), (4, 1, 0, 1, -1), (4, 2, 0, -1, 0),
                                             (4, 8, 0, 0, 0), (3, 2, 1, 1, 1), (4, 3, 1, 1, -1), (5, 8, 1, -1, 0),
                                             (1, -1, 1, 0, 0), (10, 2, 0, 1, 1), (10, -1, 1, -1, 0), (11, 2, 0, 1, 1),
                                             (11, 1, 1, 1, -1)):
        w = replace(base, volume=replace(base.volume, march_variant=mv, march_budget=budget, ray_order=order,
                                         shade_order=sorder, shade_split=split))
        host, dev, vol, inp = setup(w)
        rot = frame_rotation(51, 0)
        vol.trace(rot)
        rad, ref = _check_trace(vol, inp, vol.desc, rot)
        _, _, info = vol.rays()
        outs.append((rad, info.cpu().numpy()))
    assert outs[0][1][..., 0].max() > 8          # some rays outlast the budgets
    for rad, info in outs[1:]:
        assert np.array_equal(rad, outs[0][0]) and np.array_equal(info, outs[0][1])


def test_shade_variants_consistent(cuda):
    """Unrolling the cage-probe loop of sampleIrradiance changes scheduling
    (and where FMAs contract): the per-hit bounce radiance of every shade
    variant agrees within 1e-5 relative."""
    from dataclasses import replace

    outs = []
    for sv in (1, 2, 4, 8):
        w = replace(PLAIN_SMALL, volume=replace(PLAIN_SMALL.volume, shade_variant=sv))
        host, dev, vol, inp = setup(w, debug=False)
        for f in range(2):
            vol.update(frame_rotation(51, f))
        vol.trace(frame_rotation(51, 2))                 # frame 2: bounce on
        _, rad, _ = vol.rays()
        outs.append(_np(rad))
    for r in outs[1:]:
        assert np.array_equal(r[..., 3], outs[0][..., 3])
        np.testing.assert_allclose(r[..., :3], outs[0][..., :3], rtol=1e-5, atol=1e-7)
