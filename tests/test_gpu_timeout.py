"""The tensor-core blend's bounded device waits, made to run out.

Every mbarrier wait of tc_blend_kernel is bounded by a clock budget
(blend_tc.cu); on expiry the kernel stops issuing work, drains the loads and
matrix multiplies it issued, frees its tensor memory, returns and raises the
volume's status word.  Here one operand load of a probe update is withheld
(luxgi_ddgi_set_blend_wait_test) under a ~1 ms budget, so the consumer's
wait runs out: nothing faults, traps or hangs.  The status reads
LUXGI_ETIMEOUT once, the device stays usable, and the volume restored from
a checkpoint then runs the same frame bit for bit like an untouched volume,
and like the oracle's FP64 blend of its rays within the tensor-core bound
(2e-3)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from luxgi_gb300 import _native as N
from luxgi_gb300.ddgi import DDGIVolume, frame_rotation
from luxgi_gb300.scene import DeviceScene, HostScene
from tests._helpers import rel_err, tiny_workload

pytestmark = pytest.mark.gpu

BUDGET = 2_000_000          # SM clock cycles, ~1 ms at 2 GHz


def _volume(w, dev):
    vol = DDGIVolume(w.volume)
    vol.bind_scene(dev)
    return vol


def test_withheld_load_times_out_and_the_volume_recovers(cuda):
    import torch

    lib = N.ddgi()
    w = tiny_workload(probe_counts=(8, 4, 8), rays=128, blend=N.BLEND_TENSOR)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    vol, clean = _volume(w, dev), _volume(w, dev)
    rots = [frame_rotation(61, f) for f in range(3)]
    for v in (vol, clean):
        v.update(rots[0])
        v.check_status()
    irr0, dist0, frames0 = vol.save_atlases()

    # frame 1 with a withheld operand load: the blend gives up and says so
    assert lib.luxgi_ddgi_set_blend_wait_test(vol.handle, BUDGET, 1) == N.LUXGI_OK
    vol.update(rots[1])
    st = lib.luxgi_ddgi_check_status(vol.handle, torch.cuda.current_stream().cuda_stream)
    assert st == N.LUXGI_ETIMEOUT
    assert lib.luxgi_ddgi_check_status(vol.handle, torch.cuda.current_stream().cuda_stream) == N.LUXGI_OK

    # restored from the checkpoint, frame 1 again (no withheld load, the short
    # budget still in force): equal to the untouched volume's frame 1
    vol.load_atlases(irr0, dist0, frames0)
    vol.update(rots[1])
    vol.check_status()
    clean.update(rots[1])
    clean.check_status()
    a = [t.cpu().numpy() for t in vol.atlases()]
    b = [t.cpu().numpy() for t in clean.atlases()]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])

    # and the frame after that, with the default budget restored, against the
    # FP64 blend of the GPU's own rays
    assert lib.luxgi_ddgi_set_blend_wait_test(vol.handle, 0, 0) == N.LUXGI_OK
    prev = [t.float().cpu().numpy() for t in vol.atlases()]
    vol.trace(rots[2])
    _, rad, _ = vol.rays()
    vol.probe_update()
    vol.end_frame()
    vol.check_status()
    gi, gd = (t.float().cpu().numpy() for t in vol.atlases())
    u = vol.uniform
    ref = oracle.blend(vol.desc, oracle.ray_dirs(rots[2], u.rays_per_probe, 1), rad.float().cpu().numpy(), prev[0],
                       prev[1], first=False, precision=1)
    assert rel_err(gi, ref[0]) < 2e-3
    assert rel_err(gd, ref[1]) < 2e-3


def test_wait_test_rejects_volumes_without_the_tensor_blend(cuda):
    w = tiny_workload(blend=N.BLEND_FP32)
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode)
    vol = _volume(w, dev)
    lib = N.ddgi()
    assert lib.luxgi_ddgi_set_blend_wait_test(vol.handle, BUDGET, 1) == N.LUXGI_EUNSUPPORTED
    assert lib.luxgi_ddgi_set_blend_wait_test(vol.handle, -1, 0) == N.LUXGI_EINVAL
