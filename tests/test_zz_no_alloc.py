"""The no-allocation kick (orbit_sc2p5d_track_static) through the C ABI
against the allocating entry points (orbit_sc2p5d_create + orbit_sc2p5d_track)
on the same inputs, on two calls in a row.

Callers that cannot allocate device memory (inside another framework's
memory pool or a fixed budget, loops that must not allocate after start-up)
use the static entry point; its scratch is one static device array shared
by all calls, so the second call must not see anything left by the first.
"""
import ctypes

import numpy as np
import pytest

from helpers import TOL_FIELD, coord_err, rel_err

pytestmark = pytest.mark.gpu


def _inputs(n=20000, seed=17):
    rng = np.random.Generator(np.random.PCG64(seed))
    soa = np.empty((6, n))
    for c, s in enumerate((4e-3, 1e-3, 3e-3, 1e-3, 8.0, 1e-3)):
        soa[c] = rng.normal(0.0, s, n)
    return soa


def _sync(macrosize):
    from bunch import Bunch
    from orbit_gb300 import Sync
    b = Bunch()
    s = b.getSyncParticle()
    s.kinEnergy(1.0)
    return Sync(s.beta(), s.gamma(), s.momentum(), b.mass(), b.charge(), b.classicalRadius(), macrosize, 0.0)


def _static_call(dev, n, grid, length, sync):
    from orbit_gb300 import _native
    ptrs = dev.device_pointers()
    stride = (ptrs[1] - ptrs[0]) // 8
    L = _native.load()
    return L.orbit_sc2p5d_track_static(ctypes.c_void_p(ptrs[0]), n, stride, grid[0], grid[1], grid[2], -1.0,
                                       float(length), ctypes.byref(sync), ctypes.c_void_p(dev.stream_ptr()))


def test_static_kick_matches_allocating_entry_points_twice():
    from orbit_gb300 import DeviceBunch, DeviceSC2p5D
    soa = _inputs()
    n = soa.shape[1]
    grid = (64, 64, 16)
    sync = _sync(2e9)
    dev = DeviceBunch()
    dev.upload(soa)
    dev.set_sync(sync)
    calc = DeviceSC2p5D(*grid)
    calc.track(dev, 0.75)
    ref = dev.download()
    assert rel_err(ref[1], soa[1]) > 1e-6  # the kick acted
    for _ in range(2):
        dev.upload(soa)
        assert _static_call(dev, n, grid, 0.75, sync) == 0
        got = dev.download()
        assert rel_err(got[1] - soa[1], ref[1] - soa[1]) <= TOL_FIELD
        assert rel_err(got[3] - soa[3], ref[3] - soa[3]) <= TOL_FIELD
        assert coord_err(got, ref) <= TOL_FIELD


def test_static_kick_allocates_no_device_memory():
    """The entry point's promise: after a first call (which looks up the
    array's address), a call leaves the device's free memory unchanged
    (cudaMemGetInfo before and after, nothing else running in between)."""
    import torch
    from orbit_gb300 import DeviceBunch
    soa = _inputs(50_000, seed=3)
    grid = (128, 128, 64)
    sync = _sync(1e9)
    dev = DeviceBunch()
    dev.upload(soa)
    dev.set_sync(sync)
    assert _static_call(dev, soa.shape[1], grid, 0.5, sync) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _static_call(dev, soa.shape[1], grid, 0.5, sync) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_static_kick_rejects_grids_above_its_scratch():
    from orbit_gb300 import DeviceBunch, _native
    soa = _inputs(1000)
    dev = DeviceBunch()
    dev.upload(soa)
    rc = _static_call(dev, soa.shape[1], (256, 256, 16), 0.5, _sync(1e9))
    assert rc == _native.ORBIT_ERR_UNSUPPORTED
    assert "static scratch limit" in _native.last_error()
