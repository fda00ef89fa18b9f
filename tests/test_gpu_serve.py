"""Serving loop on the GPU: each session's results are the same alone and
in a mix of concurrently served sessions, across evictions, and equal to
the single-volume path.

Alone and in the mix the session runs through the same batched kernels
(launch groups of one or of many), and an evicted session's atlases and
frame count are restored exactly, so atlases agree bit for bit; against the
single-volume kernels they agree within 1e-6 relative (FP32 storage; FMA
contraction in the shading and blend units, as in test_gpu_batch).
"""
from __future__ import annotations

import numpy as np
import pytest

from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import DeviceScene, HostScene, batch_workloads
from luxgi_gb300.serve import Server
from tests._helpers import rel_err

pytestmark = pytest.mark.gpu

GB = 1 << 30


def _np(t):
    import torch

    t = t.detach().cpu()
    if t.dtype == torch.float16:
        t = t.float()
    return t.numpy()


@pytest.fixture(scope="module")
def sessions():
    ws = batch_workloads(count=5, seed=21, max_counts=(7, 4, 6), min_counts=(2, 2, 2), sdf_range=(32, 64),
                         atlas_range=(256, 512), max_steps=48)
    return [(w, HostScene(w.scene)) for w in ws]


def _rot(i, k):
    return frame_rotation(0x5E55 + i, k)


def _atlases(srv, sid):
    import torch

    torch.cuda.synchronize()
    return [_np(t).copy() for t in srv.atlases(sid)]


def test_same_alone_and_in_mix(cuda, sessions):
    K = 4
    alone = []
    for i, (w, host) in enumerate(sessions[:2]):
        srv = Server(64 * GB)
        sid = srv.add_session(w.volume, host)
        for k in range(K):
            srv.submit(sid, _rot(i, k))
            srv.drain(60.0)
        alone.append(_atlases(srv, sid))
        srv.close()
    mix = Server(64 * GB, max_group=3, max_inflight=2)
    ids = [mix.add_session(w.volume, host) for w, host in sessions]
    for k in range(K):                      # all sessions' requests in flight together
        for i, sid in enumerate(ids):
            mix.submit(sid, _rot(i, k))
    mix.drain(120.0)
    st = mix.stats()
    assert st["completed"] == K * len(ids)
    assert st["groups"] < st["completed"]   # requests shared launch groups
    for i in range(2):
        got = _atlases(mix, ids[i])
        for a, b in zip(alone[i], got):
            np.testing.assert_array_equal(a, b)
        assert mix.state(ids[i]) == (True, K)
    mix.close()


def test_matches_single_volume_path(cuda, sessions):
    import torch

    w, host = sessions[2]
    dev = DeviceScene(host, w.volume.light_mode)
    vol = DDGIVolume(w.volume)
    vol.bind_scene(dev)
    srv = Server(64 * GB)
    sid = srv.add_session(w.volume, host)
    for k in range(3):
        vol.update(_rot(2, k))
        srv.submit(sid, _rot(2, k))
    srv.drain(60.0)
    torch.cuda.synchronize()
    for a, b in zip(vol.atlases(), srv.atlases(sid)):
        assert rel_err(_np(b), _np(a)) <= 1e-6
    srv.close()


def test_eviction_keeps_results(cuda, sessions):
    three = sessions[:3]
    probe = Server(64 * GB)
    sizes = [probe.session_bytes(probe.add_session(w.volume, host)) for w, host in three]
    probe.close()
    tight = Server(sum(sorted(sizes)[1:]) + 1, max_inflight=1)      # any two fit, never three
    roomy = Server(64 * GB)
    ids_t = [tight.add_session(w.volume, host) for w, host in three]
    ids_r = [roomy.add_session(w.volume, host) for w, host in three]
    for k in range(3):
        for i in range(3):
            tight.submit(ids_t[i], _rot(i, k))
            tight.drain(60.0)
            roomy.submit(ids_r[i], _rot(i, k))
    roomy.drain(60.0)
    assert tight.stats()["evictions"] >= 3
    for i in range(3):
        tight.touch(ids_t[i])
        tight_a = _atlases(tight, ids_t[i])
        for a, b in zip(_atlases(roomy, ids_r[i]), tight_a):
            np.testing.assert_array_equal(a, b)
    tight.close()
    roomy.close()


def test_poisson_serving_smoke(cuda, sessions):
    srv = Server(64 * GB)
    ids = [srv.add_session(w.volume, host) for w, host in sessions]
    for sid in ids:
        srv.touch(sid)
    srv.run_poisson(ids, rate=500.0, seconds=1.0, seed=3)
    st = srv.stats()
    assert st["completed"] == st["submitted"] > 200
    assert 0.0 < st["latency_ms_p50"] <= st["latency_ms_p99"] < 1000.0
    assert st["evictions"] == 0
    srv.close()
