"""Probe-state checkpoints (luxgi_ddgi_save_atlases / load_atlases and the
DDGIVolume.save_state file): a volume restored from a checkpoint runs the
following frames bit for bit like the volume that wrote it."""
from __future__ import annotations

import numpy as np
import pytest

from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import DeviceScene, HostScene
from tests._helpers import tiny_workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage,light", [(N.STORAGE_FP32, N.LIGHT_PER_HIT), (N.STORAGE_FP16, N.LIGHT_CACHE)])
def test_checkpoint_resume_bit_identical(cuda, tmp_path, storage, light):
    import torch

    w = tiny_workload(storage=storage, light=light, prims=6)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    a, b = DDGIVolume(w.volume), DDGIVolume(w.volume)
    a.bind_scene(dev)
    b.bind_scene(dev)
    for f in range(3):
        a.update(frame_rotation(91, f))
    path = tmp_path / "probes.npz"
    a.save_state(path)
    b.load_state(path)
    assert b.frames == a.frames == 3
    for f in range(3, 6):
        if light == N.LIGHT_CACHE and f == 4:
            a.inject_indirect()
            b.inject_indirect()
        a.update(frame_rotation(91, f))
        b.update(frame_rotation(91, f))
    torch.cuda.synchronize()
    for x, y in zip(a.atlases(), b.atlases()):
        assert torch.equal(x, y)
    irr, dist, frames = b.save_atlases()
    assert frames == 6 and np.array_equal(irr, a.atlases()[0].cpu().numpy())


def test_checkpoint_rejects_other_layouts(cuda, tmp_path):
    w = tiny_workload()
    v = DDGIVolume(w.volume)
    path = tmp_path / "probes.npz"
    v.save_state(path)
    other = DDGIVolume(tiny_workload(probe_counts=(3, 2, 4)).volume)
    with pytest.raises(ValueError):
        other.load_state(path)
    fp16 = DDGIVolume(tiny_workload(storage=N.STORAGE_FP16).volume)
    with pytest.raises(ValueError):
        fp16.load_state(path)
