"""GPU parity of the surface-cache lighting pass (luxgi_surface_light:
CopyEmissive + SDF-shadowed SDFDeferredLight per light) and of the chain
lighting -> light-cache injection -> probe update, against the CPU oracle.

Tolerances: the shadow march is FP32 without FMA contraction on both sides,
so every fragment takes the oracle's blocked / lit decision; the shading
differs only by the device powf against the C library's pow (a few ulps),
which after the FP16 rounding of each light's draw leaves at most one
rounding step per light: 3e-3 relative for three lights, with at most 1e-4
of the texels beyond 1e-3.  Atlases after the chain: 2e-3 relative (FP16
light cache sampled by the hit shading).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import DeviceScene, HostScene
from luxgi_gb300.surface import SurfaceLighting, make_light, scene_lights, select_tiles
from tests._helpers import rel_err, tiny_workload

pytestmark = pytest.mark.gpu


def _f16(bits) -> np.ndarray:
    return np.asarray(bits, dtype=np.uint16).view(np.float16).astype(np.float32)


def _setup(w, camera=None):
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    mip = dev.mip.cpu().numpy()
    if host.sdf_format == N.STORAGE_FP16:
        mip = mip.view(np.uint16)
    inp = oracle.HostInputs(host, w.volume.light_mode, mip=mip, chunks=dev.chunks.cpu().numpy().view(np.uint32),
                            culled=dev.culled.cpu().numpy().view(np.uint32))
    if camera is not None:          # GlobalSurfaceAtlasData.cameraPos, read by the injection
        dev.surface_desc.data.camera_pos[:] = camera
        inp.surface_desc.data.camera_pos[:] = camera
    return host, dev, inp


def _lights():
    return [make_light(N.LIGHT_DIRECTIONAL, (1.0, 0.95, 0.9), 2.0, direction=(0.3, -0.8, 0.5)),
            make_light(N.LIGHT_POINT, (0.4, 0.6, 1.0), 3.0, position=(1.0, 2.0, -0.5), radius=6.0),
            make_light(N.LIGHT_SPOT, (1.0, 0.5, 0.2), 4.0, position=(-2.0, 3.0, 1.0), direction=(0.5, -1.0, -0.2),
                       radius=8.0, angle=0.3)]


def _run_gpu(dev, lights, tiles, masks, cam, copy_emissive, base):
    import torch

    out = torch.from_numpy(base.view(np.int16).copy()).to(dev.device)
    SurfaceLighting(dev).run(lights, tiles, masks, cam, copy_emissive, out=out)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint16)


def _close(g, o, lights=3):
    a, b = _f16(g), _f16(o)
    # empty atlas texels have world position 0; with the camera at the
    # origin the view vector is zero and the shader's normalize gives NaN,
    # which the kernel reproduces texel for texel
    assert np.array_equal(np.isfinite(a), np.isfinite(b))
    keep = np.isfinite(b)
    a, b = a[keep], b[keep]
    assert rel_err(a, b) < 1e-3 * lights
    assert np.mean(np.abs(a - b) > 1e-3 * np.maximum(np.abs(b), 1e-3)) < 1e-4


@pytest.mark.parametrize("fmt,cascades", [(N.STORAGE_FP32, 1), (N.STORAGE_FP16, 1), (N.STORAGE_FP16, 2)])
@pytest.mark.parametrize("copy_emissive,random_masks", [(True, True), (False, False), (True, False)])
def test_surface_light_matches_oracle(cuda, fmt, cascades, copy_emissive, random_masks):
    w = tiny_workload(sdf=32, prims=8, atlas=256, sdf_format=fmt, cascades=cascades,
                      room=10.0 if cascades == 1 else 24.0)
    host, dev, inp = _setup(w)
    lights = _lights()
    tiles = np.arange(1, host.num_tiles, dtype=np.uint32)
    masks = np.random.default_rng(5).integers(0, 8, size=tiles.size).astype(np.uint32) if random_masks else None
    cam = (0.3, 0.5, -2.0)
    o, shadow = oracle.surface_light(inp, lights, tiles, masks, cam, 1.0, copy_emissive, 250, 0, want_shadow=True)
    g = _run_gpu(dev, lights, tiles, masks, cam, copy_emissive, host.direct)
    assert np.count_nonzero(shadow) > 1000
    assert np.count_nonzero(g != host.direct) > 10000
    _close(g, o)


def test_surface_light_selected_tiles_and_edges(cuda):
    """A scheduled subset of tiles (select_tiles), invalid addresses in the
    list (skipped), an empty list, and no lights (emissive copy only)."""
    import torch

    w = tiny_workload(sdf=32, prims=10, atlas=256, seed=9)
    host, dev, inp = _setup(w)
    lights = scene_lights(host, 4, seed=2)
    updated = [o for o in range(host.num_objects) if o % 3 != 1]
    tiles, masks = select_tiles(host, updated, lights)
    assert 0 < tiles.size < host.num_tiles - 1
    assert (masks != 0).any() and (masks != masks[0]).any()
    cam = tuple(host.surface_data.camera_pos)
    o = oracle.surface_light(inp, lights, tiles, masks, cam)
    bad = np.concatenate([tiles, np.array([0, host.num_tiles, 0xFFFFFFFF], np.uint32)])
    g = _run_gpu(dev, lights, bad, np.concatenate([masks, np.full(3, 0xF, np.uint32)]), cam, True, host.direct)
    _close(g, o, lights=len(lights))
    # texels of tiles that were not listed keep their value
    untouched = np.ones(host.atlas * host.atlas, dtype=bool)
    res = host.atlas
    tb = N.SurfaceTile * host.num_tiles
    tl = tb.from_buffer_copy(host.tiles.tobytes())
    for t in tiles:
        e = tl[int(t)].extends
        x0, y0 = round(e[0] * res), round(e[1] * res)
        untouched.reshape(res, res)[y0:y0 + round(e[3] * res) + 1, x0:x0 + round(e[2] * res) + 1] = False
    px = g.reshape(-1, 4)
    assert np.array_equal(px[untouched], host.direct.reshape(-1, 4)[untouched])
    # empty list: nothing written
    g0 = _run_gpu(dev, lights, np.zeros(0, np.uint32), None, cam, True, host.direct)
    assert np.array_equal(g0, host.direct)
    # no lights: the footprints get the sampled emissive
    oe = oracle.surface_light(inp, [], tiles, None, cam)
    ge = _run_gpu(dev, [], tiles, None, cam, True, host.direct)
    assert np.array_equal(ge, oe)
    torch.cuda.synchronize()


def test_lighting_inject_and_update_chain(cuda):
    """Direct lighting written into the direct-light atlas, injected into
    the light cache with the probe irradiance, sampled by the next frames'
    hit shading: the whole surface-lighting chain on the GPU against the
    oracle's."""
    import torch

    w = tiny_workload(light=N.LIGHT_CACHE, prims=8, frames=4, seed=11)
    # a camera away from the origin: with it at the origin the empty atlas
    # texels (world position 0) get NaN light, which the hit shading's
    # bilinear weights carry into the atlases -- on both sides alike, but
    # then nothing is left to compare
    cam = (0.4, 0.7, -1.3)
    host, dev, inp = _setup(w, cam)
    vol = DDGIVolume(w.volume)
    vol.bind_scene(dev)
    lights = scene_lights(host, 3, seed=4)
    tiles, masks = select_tiles(host, range(host.num_objects), lights)
    SurfaceLighting(dev).run(lights, tiles, masks, cam)
    direct = oracle.surface_light(inp, lights, tiles, masks, cam)
    torch.cuda.synchronize()
    gd = dev.direct.cpu().numpy().view(np.uint16)
    _close(gd, direct, lights=len(lights))
    # the oracle continues from the GPU's direct light, so the chain test
    # measures injection and tracing, not the lighting pass twice
    host.direct[:] = gd
    inp.light_cache[:] = gd
    dev.light_cache.copy_(dev.direct)
    rots = [frame_rotation(71, f) for f in range(4)]
    for f, r in enumerate(rots):
        if f > 0 and f % 2 == 0:
            vol.inject_indirect()
        vol.update(r)
    irr, dist = vol.atlases()
    torch.cuda.synchronize()
    oi, od, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=0, inject_every=2)
    gi = irr.detach().cpu().float().numpy()
    gdist = dist.detach().cpu().float().numpy()
    assert rel_err(gi, oi) < 2e-3
    assert rel_err(gdist, od) < 2e-3
    lc = dev.light_cache.cpu().numpy().view(np.uint16)
    assert rel_err(_f16(lc), _f16(inp.light_cache), floor=1e-2) < 2e-3


# ---------------------------------------------------------------- engine formats
# The engine's surface textures: R11G11B10F emissive / lit atlas / light
# cache and RGBA16F G-buffers (GlobalSurfaceAtlas.cpp:407-411).  Every draw
# rounds the 11/11/10-bit target on both sides; the kernels and the oracle
# make every discrete decision alike, so most codes are identical and the
# rest lie within one code step (2^-6 relative for R and G, 2^-5 for B) per
# draw.


def _engine_setup(w, camera=None):
    host, dev, _ = _setup(w, camera)
    mip = dev.mip.cpu().numpy()
    if host.sdf_format == N.STORAGE_FP16:
        mip = mip.view(np.uint16)
    inp = oracle.HostInputs(host, w.volume.light_mode, mip=mip, chunks=dev.chunks.cpu().numpy().view(np.uint32),
                            culled=dev.culled.cpu().numpy().view(np.uint32), light_format=N.COLOR_R11G11B10F,
                            gbuffer_format=N.GBUFFER_RGBA16F)
    if camera is not None:
        inp.surface_desc.data.camera_pos[:] = camera
    dev.set_surface_formats(N.COLOR_R11G11B10F, N.GBUFFER_RGBA16F, inp.direct, inp.emissive, inp.gbuffer0,
                            inp.gbuffer1)
    return host, dev, inp


def _r11_close(g, o, draws):
    x = oracle.unpack_colors(g, N.COLOR_R11G11B10F)[:, :3]
    y = oracle.unpack_colors(o, N.COLOR_R11G11B10F)[:, :3]
    assert np.array_equal(np.isfinite(x), np.isfinite(y))
    keep = np.isfinite(y).all(axis=1)
    assert np.mean(g != o) < 2e-3
    assert rel_err(x[keep], y[keep]) <= draws * 2.0 ** -5


@pytest.mark.parametrize("fmt,copy_emissive", [(N.STORAGE_FP32, True), (N.STORAGE_FP16, False)])
def test_surface_light_engine_formats_match_oracle(cuda, fmt, copy_emissive):
    import torch

    w = tiny_workload(sdf=32, prims=8, atlas=256, sdf_format=fmt)
    host, dev, inp = _engine_setup(w)
    lights = _lights()
    tiles = np.arange(1, host.num_tiles, dtype=np.uint32)
    masks = np.random.default_rng(9).integers(0, 8, size=tiles.size).astype(np.uint32)
    cam = (0.3, 0.5, -2.0)
    out = torch.from_numpy(inp.direct.view(np.int32).copy()).to(dev.device)
    SurfaceLighting(dev).run(lights, tiles, masks, cam, copy_emissive, out=out)
    torch.cuda.synchronize()
    g = out.cpu().numpy().view(np.uint32)
    o = oracle.surface_light(inp, lights, tiles, masks, cam, copy_emissive=copy_emissive)
    assert np.count_nonzero(g != inp.direct) > 10000
    _r11_close(g, o, 1 + len(lights))


@pytest.mark.parametrize("light", [N.LIGHT_CACHE, N.LIGHT_PER_HIT])
def test_engine_formats_chain(cuda, light):
    """Lighting into the R11G11B10F direct-light atlas, (light-cache mode)
    injection into the R11G11B10F light cache from RGBA16F G-buffers, and
    the frames whose hit shading samples it: atlases within 2e-3 of the
    oracle's, which continues from the GPU's lit atlas."""
    import torch

    w = tiny_workload(light=light, prims=8, frames=4, seed=12)
    cam = (0.4, 0.7, -1.3)
    host, dev, inp = _engine_setup(w, cam)
    dev.surface_desc.data.camera_pos[:] = cam
    vol = DDGIVolume(w.volume)
    vol.bind_scene(dev)
    lights = scene_lights(host, 3, seed=5)
    tiles, masks = select_tiles(host, range(host.num_objects), lights)
    SurfaceLighting(dev).run(lights, tiles, masks, cam)
    o = oracle.surface_light(inp, lights, tiles, masks, cam)
    torch.cuda.synchronize()
    gd = dev.direct.cpu().numpy().view(np.uint32)
    _r11_close(gd, o, 1 + len(lights))
    inp.direct[:] = gd
    inp.light_cache[:] = gd
    dev.light_cache.copy_(dev.direct)
    rots = [frame_rotation(72, f) for f in range(4)]
    for f, r in enumerate(rots):
        if light == N.LIGHT_CACHE and f > 0 and f % 2 == 0:
            vol.inject_indirect()
        vol.update(r)
    irr, dist = vol.atlases()
    torch.cuda.synchronize()
    oi, od, _, _ = oracle.run_frames(vol.desc, inp, rots, precision=0, inject_every=2)
    assert rel_err(irr.detach().cpu().float().numpy(), oi) < 2e-3
    assert rel_err(dist.detach().cpu().float().numpy(), od) < 2e-3
    if light == N.LIGHT_CACHE:
        _r11_close(dev.light_cache.cpu().numpy().view(np.uint32), inp.light_cache, 1)
