"""The C ABI without a GPU: exports, layouts, host-only entry points and
argument validation (nothing here launches a kernel)."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from luxgi_gb300 import _native as N
from luxgi_gb300.scene import HostScene, PLAIN_SMALL, VolumeSpec
from tests._helpers import tiny_workload

ROOT = Path(__file__).resolve().parent.parent


def _declared(header: Path) -> set[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(luxgi_\w+)\s*\(", text)) - {"luxgi_ddgi_volume", "luxgi_scene"}


@pytest.mark.parametrize("header,lib", [("luxgi_ddgi.h", "libluxgi_ddgi.so"), ("luxgi_serve.h", "libluxgi_ddgi.so"),
                                        ("luxgi_scene.h", "libluxgi_scene.so")])
def test_library_exports_every_declared_symbol(header, lib):
    names = _declared(ROOT / "include" / header)
    assert names
    so = ctypes.CDLL(str(N.LIB_DIR / lib))
    missing = [n for n in sorted(names) if not hasattr(so, n)]
    assert not missing, missing


def test_ctypes_mirror_covers_header():
    names = _declared(ROOT / "include" / "luxgi_ddgi.h")
    assert names == {n for n, _, _ in N.DDGI_API}
    names = _declared(ROOT / "include" / "luxgi_serve.h")
    assert names == {n for n, _, _ in N.SERVE_API}
    names = _declared(ROOT / "include" / "luxgi_scene.h")
    assert names == {n for n, _, _ in N.SCENE_API}


def test_struct_sizes():
    assert ctypes.sizeof(N.DDGIUniform) == 96       # scalar layout of DDGICommon.glsl:11-31
    assert ctypes.sizeof(N.SdfData) == 96
    assert ctypes.sizeof(N.SurfaceData) == 32
    assert ctypes.sizeof(N.SurfaceObject) == 128    # std430 ObjectBuffer
    assert ctypes.sizeof(N.SurfaceTile) == 96
    assert ctypes.sizeof(N.BatchTuning) == 36
    assert ctypes.sizeof(N.ServerDesc) == 8 + 16 + 36 + 4 + 16 + 16


def test_derive_uniform_reference_layout():
    u = N.DDGIUniform()
    u.probe_counts[:] = [8, 4, 8, 0]
    u.step[:] = [1, 1, 1, 0]
    u.ddgi_gamma = 5.0
    u.irradiance_probe_side, u.depth_probe_side, u.rays_per_probe = 8, 16, 128
    assert N.ddgi().luxgi_ddgi_derive_uniform(ctypes.byref(u)) == 0
    # (side + 2) * X * Y + 2, (side + 2) * Z + 2 (DDGIRenderer.cpp:182-185)
    assert (u.irradiance_width, u.irradiance_height) == (10 * 32 + 2, 10 * 8 + 2)
    assert (u.depth_width, u.depth_height) == (18 * 32 + 2, 18 * 8 + 2)
    u.probe_counts[1] = 0
    assert N.ddgi().luxgi_ddgi_derive_uniform(ctypes.byref(u)) == N.LUXGI_EINVAL


def test_create_rejects_bad_descriptors_before_touching_the_device():
    lib = N.ddgi()
    h = ctypes.c_void_p()
    assert lib.luxgi_ddgi_create(None, ctypes.byref(h)) == N.LUXGI_EINVAL
    d = PLAIN_SMALL.volume.desc()
    bad = N.VolumeDesc.from_buffer_copy(d)
    bad.uniform.irradiance_width += 1                  # inconsistent layout
    assert lib.luxgi_ddgi_create(ctypes.byref(bad), ctypes.byref(h)) == N.LUXGI_EINVAL
    bad = N.VolumeDesc.from_buffer_copy(d)
    bad.storage = 7
    assert lib.luxgi_ddgi_create(ctypes.byref(bad), ctypes.byref(h)) == N.LUXGI_EINVAL
    bad = N.VolumeDesc.from_buffer_copy(d)
    bad.max_steps = 0
    assert lib.luxgi_ddgi_create(ctypes.byref(bad), ctypes.byref(h)) == N.LUXGI_EINVAL
    bad = N.VolumeDesc.from_buffer_copy(d)
    bad.uniform.rays_per_probe = 0
    assert lib.luxgi_ddgi_create(ctypes.byref(bad), ctypes.byref(h)) == N.LUXGI_EINVAL
    for field, value in (("march_budget", -2), ("shade_split", 2), ("shade_split", -2), ("ray_order", 2)):
        bad = N.VolumeDesc.from_buffer_copy(d)
        setattr(bad, field, value)
        assert lib.luxgi_ddgi_create(ctypes.byref(bad), ctypes.byref(h)) == N.LUXGI_EINVAL, field
    assert h.value is None


def test_null_handles_are_rejected():
    lib = N.ddgi()
    rot = (ctypes.c_float * 9)()
    assert lib.luxgi_ddgi_trace(None, rot, None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_update(None, rot, None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_probe_update(None, None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_end_frame(None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_destroy(None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_update_batch(None, -1, None, None) == N.LUXGI_EINVAL
    assert lib.luxgi_ddgi_update_batch(None, 0, None, None) == N.LUXGI_OK
    assert lib.luxgi_sdf_build_mip(None, None, None, None) == N.LUXGI_EINVAL
    assert lib.luxgi_surface_cull(None, None, None, 0, None) == N.LUXGI_EINVAL
    assert lib.luxgi_strerror(N.LUXGI_ENOMEM) == b"out of device memory or capacity"


def test_frame_rotation_deterministic_and_orthonormal():
    from luxgi_gb300.ddgi import frame_rotation

    a = frame_rotation(1234, 5)
    b = frame_rotation(1234, 5)
    c = frame_rotation(1234, 6)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    m = a.reshape(3, 3)
    np.testing.assert_allclose(m @ m.T, np.eye(3), atol=3e-6)
    assert abs(np.linalg.det(m) - 1.0) < 3e-6


def test_half_conversion_matches_ieee():
    lib = N.scene_lib()
    rng = np.random.default_rng(1)
    vals = np.concatenate([rng.normal(scale=s, size=2000) for s in (1e-7, 1e-4, 1.0, 100.0, 3e4)]).astype(np.float32)
    vals = np.concatenate([vals, np.array([0.0, -0.0, 65504.0, 65520.0, 1e6, -1e6, 6.1e-5, 5.96e-8], np.float32)])
    ref = vals.astype(np.float16).view(np.uint16)
    got = np.array([lib.luxgi_float_to_half(float(v)) for v in vals], dtype=np.uint16)
    assert np.array_equal(got, ref)
    back = np.array([lib.luxgi_half_to_float(int(h)) for h in ref], dtype=np.float32)
    assert np.array_equal(back, ref.view(np.float16).astype(np.float32))


def test_scene_is_deterministic_and_exact():
    w = tiny_workload(sdf=32, prims=8)
    a = HostScene(w.scene)
    b = HostScene(w.scene)
    assert np.array_equal(a.sdf, b.sdf) and np.array_equal(a.direct, b.direct) and np.array_equal(a.depth, b.depth)
    # voxel values are the normalised exact distance at voxel centres
    half = a.sdf_data.cascade_pos_distance[0][3]
    voxel = a.sdf_data.cascade_voxel_size[0]
    res = a.res
    sdf = a.sdf.reshape(res, res, res)
    rng = np.random.default_rng(4)
    for _ in range(50):
        x, y, z = rng.integers(0, res, size=3)
        p = [-half + (x + 0.5) * voxel, -half + (y + 0.5) * voxel, -half + (z + 0.5) * voxel]
        d = a.distance(p)
        assert abs(sdf[z, y, x] - np.clip(min(d, 2 * half) / (2 * half), -1, 1)) < 1e-6


def test_scene_cards_follow_tile_convention():
    """Tile slot 0 is empty; every object's six tile offsets are >= 1 and the
    tile rotation is orthonormal with bounds = 2 |R e|."""
    a = HostScene(tiny_workload(prims=5).scene)
    objs = np.frombuffer(a.objects.tobytes(), dtype=np.float32).reshape(-1, 32)
    offs = np.frombuffer(a.objects.tobytes(), dtype=np.uint32).reshape(-1, 32)[:, 4:10]
    tiles = np.frombuffer(a.tiles.tobytes(), dtype=np.float32).reshape(-1, 24)
    assert np.all(tiles[0] == 0)
    assert np.all(offs >= 1) and len(np.unique(offs)) == offs.size
    for o in range(objs.shape[0]):
        e = np.maximum(objs[o, 28:31], 0.05)
        for t in offs[o]:
            M = tiles[t, 4:20].reshape(4, 4).T      # row-major
            R = M[:3, :3]
            np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-6)
            np.testing.assert_allclose(tiles[t, 20:23], 2 * np.abs(R @ e), rtol=1e-6)


def test_fastdiv_formula_exact():
    """The multiply-high division the kernels use for probe / ray indices
    (FastDiv in luxgi_common.cuh): (mulhi(n, m) + n) >> l == n // d."""
    rng = np.random.default_rng(5)
    divisors = [1, 2, 3, 5, 7, 8, 12, 255, 256, 1000, 16384, 131072, 65535, 65537, (1 << 26), (1 << 26) - 1,
                (1 << 31) + 1, (1 << 32) - 1]
    ns = np.concatenate([rng.integers(0, 1 << 32, 2000, dtype=np.uint64),
                         np.array([0, 1, (1 << 32) - 1, (1 << 31), (1 << 31) - 1], dtype=np.uint64)])
    for d in divisors:
        l = 0
        while (1 << l) < d:
            l += 1
        m = ((1 << 32) * ((1 << l) - d)) // d + 1
        assert 0 < m < (1 << 32) or (d & (d - 1)) == 0
        for n in ns.tolist() + [d - 1, d, d + 1, 2 * d - 1]:
            n &= (1 << 32) - 1
            q = (((n * m) >> 32) + n) >> l
            assert q == n // d, (d, n)


@pytest.mark.parametrize("header", ["luxgi_ddgi.h", "luxgi_serve.h", "luxgi_scene.h"])
def test_headers_are_plain_c(header, tmp_path):
    """The boundary is a C ABI: each header compiles as C99 on its own, and
    a C translation unit that calls every declared entry point links
    against the library (the binding a C, cgo or FFI caller would make)."""
    src = tmp_path / "use.c"
    names = sorted(_declared(ROOT / "include" / header))
    body = "\n".join(f"    (void)&{n};" for n in names)
    src.write_text(f'#include "{header}"\nint main(void) {{\n{body}\n    return 0;\n}}\n')
    lib = "luxgi_scene" if header == "luxgi_scene.h" else "luxgi_ddgi"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o",
                        str(tmp_path / "use"), "-L", str(N.LIB_DIR), f"-l{lib}", f"-Wl,-rpath,{N.LIB_DIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
