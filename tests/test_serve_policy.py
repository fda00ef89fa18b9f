"""Serving-loop policy on the host: admission by memory budget, rejection,
LRU eviction, continuous batching and latency accounting, driven through
the C ABI with the host-simulated executor (same scheduler code as the
CUDA executor; no device work, no GPU needed)."""
from __future__ import annotations

import time

import numpy as np
import pytest

from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import frame_rotation
from luxgi_gb300.scene import HostScene
from luxgi_gb300.serve import Server
from tests._helpers import tiny_workload


@pytest.fixture(scope="module")
def scene():
    w = tiny_workload(sdf=32, atlas=128)
    return w, HostScene(w.scene)


def _server(scene, n, budget_sessions, **kw):
    w, host = scene
    probe = Server(1 << 50, executor="sim")
    sid = probe.add_session(w.volume, host)
    per = probe.session_bytes(sid)
    probe.close()
    srv = Server(int(per * budget_sessions) if budget_sessions else 1 << 50, executor="sim", **kw)
    ids = [srv.add_session(w.volume, host) for _ in range(n)]
    return srv, ids, per


def test_session_footprint_counts_scene_and_volume(scene):
    w, host = scene
    srv = Server(1 << 50, executor="sim")
    sid = srv.add_session(w.volume, host)
    b = srv.session_bytes(sid)
    sdf = host.sdf.nbytes
    atlas = host.atlas * host.atlas * (4 + 8 + 4)
    u = w.volume.uniform()
    atl = 2 * (u.irradiance_width * u.irradiance_height * 16 + u.depth_width * u.depth_height * 8)
    assert b > sdf + atlas + atl
    srv.close()


def test_rejects_session_larger_than_budget(scene):
    w, host = scene
    srv, ids, per = _server(scene, 1, 2)
    small = Server(per - 1, executor="sim")
    with pytest.raises(N.LuxgiError) as e:
        small.add_session(w.volume, host)
    assert e.value.status == N.LUXGI_ENOMEM
    assert small.stats()["rejected"] == 1
    small.close()
    srv.close()


def test_lru_eviction_and_readmission(scene):
    srv, (a, b, c), per = _server(scene, 3, 2.5)
    rot = frame_rotation(1, 0)
    for sid in (a, b):
        srv.submit(sid, rot)
        srv.drain(5.0)
    assert srv.state(a)[0] and srv.state(b)[0]
    srv.submit(c, rot)                        # budget holds two: evicts a (least recent)
    srv.drain(5.0)
    assert [srv.state(s)[0] for s in (a, b, c)] == [False, True, True]
    srv.submit(a, rot)                        # back in, evicting b
    srv.drain(5.0)
    assert [srv.state(s)[0] for s in (a, b, c)] == [True, False, True]
    st = srv.stats()
    assert st["admissions"] == 4 and st["evictions"] == 2
    assert st["resident_bytes"] == 2 * per and st["peak_resident_bytes"] <= 2.5 * per
    assert srv.state(a)[1] == 2               # frames survive the eviction
    srv.close()


def test_continuous_batching_overlaps_groups(scene):
    w, _ = scene
    pr = w.volume.probes * w.volume.rays_per_probe
    # each group takes ~20 ms of modelled device time per member
    srv, ids, _ = _server(scene, 12, 0, max_group=4, max_inflight=3, sim_rate=pr / 0.005)
    rot = frame_rotation(2, 0)
    for k in range(3):
        for sid in ids:
            srv.submit(sid, rot)
    srv.drain(30.0)
    st = srv.stats()
    assert st["completed"] == 36 and st["pending"] == 0
    assert st["max_overlap"] >= 2             # groups in flight at once
    assert 1.0 < st["mean_group"] <= 4.0
    assert all(srv.state(s)[1] == 3 for s in ids)   # one request per session in flight, none lost
    assert st["latency_ms_p50"] <= st["latency_ms_p95"] <= st["latency_ms_p99"] <= st["latency_ms_max"]
    srv.close()


def test_admission_waits_for_memory_held_by_busy_sessions(scene):
    w, _ = scene
    pr = w.volume.probes * w.volume.rays_per_probe
    srv, ids, per = _server(scene, 4, 1.5, max_group=8, max_inflight=2, sim_rate=pr / 0.02)
    rot = frame_rotation(3, 0)
    for sid in ids:
        srv.submit(sid, rot)
    srv.drain(30.0)
    st = srv.stats()
    # only one session fits: every group has one member, each later one evicts
    assert st["completed"] == 4 and st["groups"] == 4 and st["evictions"] == 3
    assert st["peak_resident_bytes"] <= 1.5 * per
    srv.close()


def test_poisson_load_and_stats_reset(scene):
    w, _ = scene
    pr = w.volume.probes * w.volume.rays_per_probe
    srv, ids, _ = _server(scene, 8, 0, sim_rate=pr / 0.0005)
    srv.run_poisson(ids, rate=400.0, seconds=0.5, seed=7)
    st = srv.stats(reset=True)
    assert st["completed"] == st["submitted"] > 100
    assert 0.0 < st["latency_ms_p50"] < 50.0
    assert st["probe_rays"] == st["completed"] * pr
    st2 = srv.stats()
    assert st2["completed"] == 0 and st2["submitted"] == 0
    srv.close()


def test_drain_times_out_and_destroy_stops(scene):
    srv, ids, _ = _server(scene, 1, 0, sim_rate=1.0)     # a group would take days
    srv.submit(ids[0], frame_rotation(4, 0))
    with pytest.raises(N.LuxgiError) as e:
        srv.drain(0.05)
    assert e.value.status == N.LUXGI_ETIMEOUT
    t = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t < 5.0


def test_bad_arguments(scene):
    w, host = scene
    srv = Server(1 << 40, executor="sim")
    with pytest.raises(N.LuxgiError):
        srv.submit(3, frame_rotation(0, 0))
    with pytest.raises(N.LuxgiError):
        srv.state(-1)
    with pytest.raises(N.LuxgiError) as e:
        srv.atlases(srv.add_session(w.volume, host))      # no device arrays in the simulated executor
    assert e.value.status == N.LUXGI_ENOTBOUND
    srv.close()
    with pytest.raises(N.LuxgiError):
        Server(1 << 40, executor="sim", max_inflight=99)


def test_submit_while_touch_evicts(scene):
    """A request for the session a touch is evicting (the eviction copy runs
    with the server's lock released) waits for the eviction and then
    re-admits the session; it never runs on the session mid-eviction, and
    the victim is not evicted twice (budget: one session)."""
    import threading

    srv, (a, b), per = _server(scene, 2, 1, sim_evict_s=0.3)
    srv.touch(a)
    assert srv.state(a)[0]
    t = threading.Thread(target=srv.touch, args=(b,))
    t.start()
    time.sleep(0.1)                       # the touch is now evicting a
    srv.submit(a, frame_rotation(1, 0))
    t.join()
    srv.drain(timeout=10.0)
    st = srv.stats()
    assert st["completed"] == 1
    # touch a, touch b (evicting a), then a admitted again (evicting b)
    assert st["admissions"] == 3
    assert st["evictions"] == 2
    assert srv.state(a) == (True, 1)
    assert srv.state(b)[0] is False
    assert st["resident_sessions"] == 1 and st["resident_bytes"] == per
    srv.close()
