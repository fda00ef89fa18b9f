"""Host side of the surface-cache lighting pass, without a GPU: the
per-light tile selection and the redraw schedule of the reference's
deferred-lighting system (Engine/DDGI/GlobalSurfaceAtlas.cpp:826-944), the
light records, and argument validation of luxgi_surface_light (every check
returns before anything is launched)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.scene import HostScene
from luxgi_gb300.surface import (GI_FRAMES, REDRAW_FRAMES, LightingSchedule, light_array, make_light, scene_lights,
                                 select_tiles, tile_view_directions)
from tests._helpers import tiny_workload


@pytest.fixture(scope="module")
def host():
    return HostScene(tiny_workload(sdf=32, prims=8, atlas=256).scene)


def _objects(host):
    return (N.SurfaceObject * host.num_objects).from_buffer_copy(host.objects.tobytes())


def test_light_record_layout():
    L = make_light(N.LIGHT_SPOT, (0.5, 0.25, 1.0), 3.0, position=(1, 2, 3), direction=(0, 0, -2), radius=4.0,
                   angle=0.2)
    raw = np.frombuffer(bytes(L), dtype=np.float32)
    assert raw.size == 16                                   # Light.glsl std140: 3 vec4 + 4 floats
    assert np.allclose(raw[8:11], [0, 0, -1])               # direction normalised
    assert raw[14] == N.LIGHT_SPOT and np.isclose(raw[15], 0.2)
    with pytest.raises(ValueError):
        make_light(3)
    with pytest.raises(ValueError):
        light_array([L] * (N.MAX_LIGHTS + 1))


def test_tile_view_directions_are_the_tile_axes(host):
    view = tile_view_directions(host.tiles, host.num_tiles)
    objs = _objects(host)
    for o in range(host.num_objects):
        for i in range(6):
            t = objs[o].tile_offset[i]
            z = np.zeros(3)
            z[i // 2] = 1.0 if i & 1 else -1.0              # GlobalSurfaceAtlas.cpp:249
            assert np.allclose(view[t], z, atol=1e-6), (o, i, view[t])


def test_select_tiles_follows_the_reference_rules(host):
    sun = make_light(N.LIGHT_DIRECTIONAL, direction=(0.0, -1.0, 0.0))
    near = make_light(N.LIGHT_POINT, position=tuple(_objects(host)[0].object_bounds[:3]), radius=0.01)
    far = make_light(N.LIGHT_POINT, position=(1e4, 0, 0), radius=1.0)
    updated = [0, 2, 3]
    tiles, masks = select_tiles(host, updated, [sun, near, far])
    objs = _objects(host)
    expect = [objs[o].tile_offset[i] for o in updated for i in range(6)]
    assert tiles.tolist() == expect                          # every tile of a redrawn object, once
    view = tile_view_directions(host.tiles, host.num_tiles)
    for t, m in zip(tiles, masks):
        lit_by_sun = float(np.dot(view[t], [0.0, -1.0, 0.0])) >= 1e-6
        assert bool(m & 1) == lit_by_sun                     # :934-938
        assert bool(m & 2) == (t in [objs[0].tile_offset[i] for i in range(6)])   # :921-925
        assert not m & 4
    assert select_tiles(host, [], [sun])[0].size == 0


def test_schedule_redraw_rules(host):
    s = LightingSchedule()
    pt = make_light(N.LIGHT_POINT, position=tuple(_objects(host)[1].object_bounds[:3]), radius=0.5)
    culled = list(range(host.num_objects))
    assert s.updated_objects(host, 1, culled, [pt]) == []                         # nothing due yet
    assert s.updated_objects(host, GI_FRAMES + 1, culled, [pt]) == culled         # GI refresh: all
    assert s.updated_objects(host, GI_FRAMES + 2, culled, [pt]) == []
    f = REDRAW_FRAMES + 3
    assert s.updated_objects(host, f, culled, [pt]) == culled                     # GI refresh again
    got = s.updated_objects(host, f + 1, culled, [pt])                            # GI not due, the light is
    assert 1 in got and len(got) < len(culled)
    assert s.last_updated[0] == f + 1
    assert s.updated_objects(host, f + 2, culled, [pt]) == []
    sun = make_light(N.LIGHT_DIRECTIONAL)
    s = LightingSchedule()                                  # lights are tracked by index
    s.last_gi_updated = f + 3
    assert s.updated_objects(host, f + 3, culled, [sun]) == culled                # a due sun redraws all
    assert 0 not in s.last_updated           # and, as in the reference, stays due (its frame is never set)
    assert s.updated_objects(host, f + 4, culled, [sun]) == culled
    assert s.updated_objects(host, f + 5, [], [sun]) == []


def test_scene_lights_are_seeded(host):
    a = scene_lights(host, 5, seed=3)
    b = scene_lights(host, 5, seed=3)
    assert [bytes(x) for x in a] == [bytes(x) for x in b]
    assert [x.type for x in a] == [0.0, 2.0, 1.0, 2.0, 1.0]


def test_scene_materials(host):
    pbr = host.pbr.reshape(-1, 4)
    em = host.emissive.view(np.float16).astype(np.float32).reshape(-1, 4)
    solid = pbr[:, 3] == 255
    assert solid.any() and (pbr[solid, 1] >= 63).all()      # roughness >= 0.25
    assert (em[:, 3] == 1.0).all()                          # unused alpha reads 1
    assert (em[:, :3] > 0).any()                            # some solids emit


def test_surface_light_validation_returns_before_launch(host):
    lib = N.ddgi()
    inp = oracle.HostInputs(host, N.LIGHT_CACHE)
    d = N.SurfaceLighting()
    d.num_lights = 1
    good = light_array([make_light(N.LIGHT_POINT)])
    d.lights = ctypes.cast(good, ctypes.c_void_p)
    d.num_tiles = 0
    d.shadow_bias = 1.0
    d.max_steps = 250
    sd, su = ctypes.byref(inp.sdf_desc), ctypes.byref(inp.surface_desc)
    out = ctypes.c_void_p(1)
    assert lib.luxgi_surface_light(None, su, ctypes.byref(d), out, None) == N.LUXGI_EINVAL
    assert lib.luxgi_surface_light(sd, su, None, out, None) == N.LUXGI_EINVAL
    assert lib.luxgi_surface_light(sd, su, ctypes.byref(d), None, None) == N.LUXGI_EINVAL
    bad = N.SurfaceLighting.from_buffer_copy(d)
    bad.num_lights = N.MAX_LIGHTS + 1
    assert lib.luxgi_surface_light(sd, su, ctypes.byref(bad), out, None) == N.LUXGI_EINVAL
    bad = N.SurfaceLighting.from_buffer_copy(d)
    bad.max_steps = 0
    assert lib.luxgi_surface_light(sd, su, ctypes.byref(bad), out, None) == N.LUXGI_EINVAL
    bad = N.SurfaceLighting.from_buffer_copy(d)
    bad.num_tiles = 4                                       # tiles pointer missing
    assert lib.luxgi_surface_light(sd, su, ctypes.byref(bad), out, None) == N.LUXGI_EINVAL
    env = light_array([make_light(N.LIGHT_POINT)])
    env[0].type = 3.0                                       # LIGHT_ENV: fetchLight leaves it unset
    bad = N.SurfaceLighting.from_buffer_copy(d)
    bad.lights = ctypes.cast(env, ctypes.c_void_p)
    assert lib.luxgi_surface_light(sd, su, ctypes.byref(bad), out, None) == N.LUXGI_EINVAL
