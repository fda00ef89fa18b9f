"""luxgi_sdf_build_mip_noalloc: the SDF mip build for callers that cannot
allocate device memory (an engine that serves all device memory from its
own fixed-budget pool, or a frame loop that must not call cudaMalloc because
it can synchronise the device).  Its scratch plane is a static device array
inside the library, so it needs no caller-provided scratch and allocates
nothing.

Checked through the C ABI against luxgi_sdf_build_mip (which takes a
caller-allocated scratch plane), bit for bit -- the tolerance the other mip
tests use -- on two calls in a row with different inputs, so a stale
scratch from the first call cannot leak into the second.  Collected last
(file name) so a failure here stops a -x run only after every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from luxgi_gb300 import _native as N
from luxgi_gb300.scene import HostScene
from tests._helpers import tiny_workload

pytestmark = pytest.mark.gpu


def _device_sdf(fmt, seed, res, cascades=1):
    import torch

    host = HostScene(tiny_workload(sdf=res, sdf_format=fmt, seed=seed, prims=8, cascades=cascades).scene)
    sdf = torch.from_numpy(host.sdf.view(np.int16) if fmt == N.STORAGE_FP16 else host.sdf).cuda()
    desc = N.SdfDesc()
    desc.data = host.sdf_data
    desc.format = fmt
    desc.resolution = host.res
    desc.mip_resolution = host.mres
    desc.sdf = sdf.data_ptr()
    return host, sdf, desc


@pytest.mark.parametrize("fmt", [N.STORAGE_FP32, N.STORAGE_FP16])
def test_no_alloc_mip_matches_allocating_entry_point(fmt):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = N.ddgi()
    stream = torch.cuda.current_stream().cuda_stream
    elem = torch.int16 if fmt == N.STORAGE_FP16 else torch.float32
    # two calls in a row, different scenes and sizes (the second call reuses
    # the scratch the first one left behind)
    for seed, res in ((3, 256 if fmt == N.STORAGE_FP32 else 128), (4, 64)):
        host, sdf, desc = _device_sdf(fmt, seed, res)
        m = host.mres
        ref = torch.full((m * m * m,), -1, dtype=elem, device="cuda")
        tmp = torch.zeros(m * m * m, dtype=elem, device="cuda")
        desc.mip = ref.data_ptr()
        assert lib.luxgi_sdf_build_mip(ctypes.byref(desc), ref.data_ptr(), tmp.data_ptr(), stream) == N.LUXGI_OK
        out = torch.full((m * m * m,), -2, dtype=elem, device="cuda")
        assert lib.luxgi_sdf_build_mip_noalloc(ctypes.byref(desc), out.data_ptr(), stream) == N.LUXGI_OK
        torch.cuda.synchronize()
        assert torch.equal(out, ref)


@pytest.mark.parametrize("fmt", [N.STORAGE_FP32, N.STORAGE_FP16])
def test_no_alloc_mip_multi_cascade(fmt):
    """Packed SDFs of 2 and 4 cascades (the mip of each cascade built in
    turn through the one scratch plane), two calls in a row, equal bit for
    bit to luxgi_sdf_build_mip."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = N.ddgi()
    stream = torch.cuda.current_stream().cuda_stream
    elem = torch.int16 if fmt == N.STORAGE_FP16 else torch.float32
    for seed, res, cascades in ((6, 128, 2), (7, 64, 4)):
        host, sdf, desc = _device_sdf(fmt, seed, res, cascades)
        assert host.cascades == cascades
        m = host.mres
        n = m * cascades * m * m
        ref = torch.full((n,), -1, dtype=elem, device="cuda")
        tmp = torch.zeros(m * m * m, dtype=elem, device="cuda")
        desc.mip = ref.data_ptr()
        assert lib.luxgi_sdf_build_mip(ctypes.byref(desc), ref.data_ptr(), tmp.data_ptr(), stream) == N.LUXGI_OK
        out = torch.full((n,), -2, dtype=elem, device="cuda")
        assert lib.luxgi_sdf_build_mip_noalloc(ctypes.byref(desc), out.data_ptr(), stream) == N.LUXGI_OK
        torch.cuda.synchronize()
        assert torch.equal(out, ref)


def test_no_alloc_mip_rejects_inputs_beyond_its_scratch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = N.ddgi()
    # a 512^3 FP32 SDF needs a 128^3 x 4 B = 8 MiB plane: refused before any
    # work is issued (the pointers below are never dereferenced)
    host, sdf, desc = _device_sdf(N.STORAGE_FP32, 5, 32)
    desc.resolution = 512
    desc.mip_resolution = 128
    desc.data.resolution = 512.0
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = lib.luxgi_sdf_build_mip_noalloc(ctypes.byref(desc), dummy.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == N.LUXGI_ESCRATCH
    assert b"static scratch" in lib.luxgi_strerror(st)
