"""The global SDF build's host side without a GPU: the cascade layout, the
per-cascade plan (objects, ObjectRasterizeData records, chunk table) of
luxgi_sdf_build_plan against the oracle's restatement, the baked .sdf
parser and the baker's mip rule, and argument validation."""
from __future__ import annotations

import ctypes
import numpy as np
import pytest

import oracle
from oracle import build_ref
from luxgi_gb300 import _native as N
from luxgi_gb300.sdf import MeshSDF, _mip_down, box_distance, build_desc, plan, sphere_distance, trs

_REF = build_ref.reference_root()
ASSETS = None if _REF is None else _REF / "Assets" / "sdf"


def _meshes():
    return [MeshSDF.bake(box_distance((2.0, 1.0, 1.5)), (-2, -1, -1.5), (2, 1, 1.5), (24, 16, 20)),
            MeshSDF.bake(sphere_distance(1.2), (-1.2,) * 3, (1.2,) * 3, (16, 16, 16), mip_count=2)]


def _objects(n, seed, spread=60.0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        scale = (1, 1, 1) if i % 2 else rng.uniform(0.5, 3, 3)
        out.append((trs(rng.uniform(-spread, spread, 3), rng.normal(size=3), rng.uniform(0, 6), scale), i % 2))
    return out


def test_cascade_layout_reference_defaults():
    """giDistance 4000, gloalScale 0.1, Quality::Test (192^3, 2 cascades):
    extents 160 and 400 (GlobalDistanceField.cpp:592-620), the view point
    0.3 x 160 along +z snapped to each cascade's 32-voxel chunk grid."""
    d = build_desc(resolution=192, cascades=2)
    data = N.SdfData()
    assert N.ddgi().luxgi_sdf_cascade_layout(ctypes.byref(d), ctypes.byref(data)) == N.LUXGI_OK
    assert data.cascades_count == 2 and data.resolution == 192.0
    assert [data.cascade_pos_distance[0][3], data.cascade_pos_distance[1][3]] == [160.0, 400.0]
    assert np.isclose(data.cascade_voxel_size[0], 320.0 / 192) and np.isclose(data.cascade_voxel_size[1], 800.0 / 192)
    # chunk sizes 53.3 and 133.3: 48 along z snaps to 0 in both
    for c in range(2):
        assert list(data.cascade_pos_distance[c])[:3] == [0.0, 0.0, 0.0]
    d = build_desc(resolution=256, cascades=1)
    assert N.ddgi().luxgi_sdf_cascade_layout(ctypes.byref(d), ctypes.byref(data)) == N.LUXGI_OK
    # one cascade of extent 400, chunk 100: 0.3 * 400 = 120 snaps to 100
    assert list(data.cascade_pos_distance[0]) == [0.0, 0.0, 100.0, 400.0]


@pytest.mark.parametrize("cascades,n,spread,res", [(1, 12, 30.0, 64), (2, 40, 60.0, 64), (3, 30, 150.0, 96),
                                                   (4, 60, 250.0, 64)])
def test_plan_matches_oracle(cascades, n, spread, res):
    meshes = _meshes()
    objs = _objects(n, seed=cascades, spread=spread)
    d = build_desc(resolution=res, cascades=cascades, storage=N.STORAGE_FP32, global_scale=0.05)
    for c in range(cascades):
        r1, m1, c1 = plan(d, meshes, objs, c)
        r2, m2, c2 = oracle.sdf_plan(d, meshes, objs, c)
        assert m1 == m2
        assert [bytes(a) for a in r1] == [bytes(b) for b in r2]
        assert [bytes(a) for a in c1] == [bytes(b) for b in c2]


def test_plan_selection_chunk_cap_and_spill():
    """Objects below the minimum radius or outside the cascade are dropped;
    a chunk that collects more than 28 objects restarts with the 29th (the
    reference's chunk table overwrites a full layer-0 entry,
    GlobalDistanceField.cpp:516-523); chunks of objects near the cascade's
    +x face reach past it (their coordinates are not clamped)."""
    meshes = _meshes()
    d = build_desc(resolution=64, cascades=1, storage=N.STORAGE_FP32, global_scale=0.05)
    ext = 200.0                                          # one cascade: distance 200
    objs = [(trs((3.0 + 0.01 * i, 2.0, 1.0)), 1) for i in range(30)]      # 30 spheres in one chunk
    objs.append((trs((0, 0, 0), scale=(0.1, 0.1, 0.1)), 1))              # radius 0.22 < 0.5
    objs.append((trs((ext * 3, 0, 0)), 0))                                 # far outside
    objs.append((trs((ext - 1.0, 0, 60.0)), 0))                            # at the +x face
    recs, mesh, chunks = plan(d, meshes, objs, 0)
    assert len(recs) == 31                                  # 30 spheres + the box at the face
    assert len({tuple(c.coord) for c in chunks}) == len(chunks)
    # the spheres' margin-grown bounds cover the 8 chunks around the centre;
    # each kept only the 29th and 30th sphere (records 28 and 29), then
    # possibly the box at the face (record 30)
    spheres = [c for c in chunks if 29 in list(c.models)[:c.count]]
    assert len(spheres) == 8
    for c in spheres:
        assert list(c.models)[:2] == [28, 29] and c.count <= 3
    assert any(c.coord[0] >= 2 for c in chunks)             # past the cascade (64 voxels = 2 chunks)


def test_parse_rejects_bad_files():
    lib = N.ddgi()
    info = N.MeshSdfFile()
    hdr = np.array([4, 4, 4], np.uint32).tobytes() + np.array([2], np.int32).tobytes()
    mip0 = np.array([128], np.uint64).tobytes() + bytes(128)
    mip1 = np.array([16], np.uint64).tobytes() + bytes(16)

    def parse(b):
        buf = (ctypes.c_ubyte * max(1, len(b))).from_buffer_copy(b if b else b"\0")
        return lib.luxgi_mesh_sdf_parse(ctypes.cast(buf, ctypes.c_void_p), len(b), ctypes.byref(info))

    assert parse(hdr + mip0 + mip1) == N.LUXGI_OK
    assert list(info.size) == [4, 4, 4] and info.mip_count == 2
    assert list(info.mip_offset)[:2] == [24, 24 + 128 + 8] and list(info.mip_bytes)[:2] == [128, 16]
    assert parse(hdr + mip0) == N.LUXGI_EINVAL                       # truncated
    assert parse(hdr + mip0 + mip1[:-1]) == N.LUXGI_EINVAL
    bad = np.array([4, 4, 4], np.uint32).tobytes() + np.array([4], np.int32).tobytes()
    assert parse(bad + mip0 + mip1) == N.LUXGI_EINVAL                # more than 3 mips
    wrong = np.array([100], np.uint64).tobytes() + bytes(100)
    assert parse(hdr + wrong + mip1) == N.LUXGI_EINVAL               # length disagrees with the size
    assert parse(b"") == N.LUXGI_EINVAL


@pytest.mark.skipif(ASSETS is None or not ASSETS.is_dir(), reason="reference assets not available")
def test_reference_assets_parse_and_mips_follow_the_baker():
    """Every baked .sdf of the reference's demo scene parses, and each of its
    mips is the baker's 2x2x2 mean of the level above rounded by glm's
    packHalf (SDFBaker.cpp:166-204), bit for bit."""
    files = sorted(ASSETS.glob("*.sdf"))
    assert len(files) >= 50
    for f in files:
        m = MeshSDF.load(f.read_bytes(), (0, 0, 0), (1, 1, 1))
        assert 1 <= len(m.mips) <= 3
        v = m.mips[0].view(np.float16).astype(np.float32)
        assert np.isfinite(v).all() and v.min() >= -0.01 and v.max() <= 1.01
        for k in range(1, len(m.mips)):
            assert np.array_equal(_mip_down(m.mips[k - 1]), m.mips[k]), (f.name, k)


def test_bake_encodes_like_the_baker():
    m = MeshSDF.bake(sphere_distance(1.0), (-1,) * 3, (1,) * 3, (9, 9, 9), mip_count=1)
    # padded by max(5 %, 0.1): [-1.1, 1.1]^3, max distance 2.2
    assert np.allclose(m.aabb_min, (-1.1,) * 3) and np.isclose(m.max_distance, 2.2)
    centre = m.mips[0].view(np.float16).astype(np.float32)[4, 4, 4]
    assert abs(centre - (-1.0 / 2.2 + 1.0) / 2.0) < 1e-3


def test_build_validation_returns_before_launch():
    lib = N.ddgi()
    meshes = _meshes()
    md = (N.MeshSdf * 2)(*[m.desc() for m in meshes])              # no device volumes
    from luxgi_gb300.sdf import objects_array

    ob = objects_array(_objects(3, seed=5))
    d = build_desc(resolution=64, cascades=2)
    dummy = ctypes.c_void_p(1)
    data = N.SdfData()
    # a mesh without volumes stops the build before anything runs
    assert lib.luxgi_sdf_build(ctypes.byref(d), md, 2, ob, 3, dummy, dummy, dummy, ctypes.byref(data), None) == \
        N.LUXGI_EINVAL
    bad = N.SdfBuildDesc.from_buffer_copy(d)
    bad.cascades = 5
    assert lib.luxgi_sdf_build(ctypes.byref(bad), md, 2, ob, 3, dummy, dummy, dummy, None, None) == N.LUXGI_EINVAL
    bad = N.SdfBuildDesc.from_buffer_copy(d)
    bad.resolution = 30
    assert lib.luxgi_sdf_cascade_layout(ctypes.byref(bad), ctypes.byref(data)) == N.LUXGI_EINVAL
    ob[1].mesh = 7
    nr, nc = ctypes.c_int(), ctypes.c_int()
    assert lib.luxgi_sdf_build_plan(ctypes.byref(d), md, 2, ob, 3, 0, None, 0, ctypes.byref(nr), None, None, 0,
                                    ctypes.byref(nc)) == N.LUXGI_EINVAL
