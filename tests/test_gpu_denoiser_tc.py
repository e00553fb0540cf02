"""The denoiser's tensor-core inference layers (tcgen05 MMA, TF32 operands,
FP32 accumulation in TMEM) against the float64 oracle with the same
rounding of every convolution's input to TF32, and against the CUDA-core
layers.

Tolerances (max-norm relative): 3e-3 against the TF32-rounded oracle and
against the CUDA-core forward, 5e-3 on the correction the network adds to
its input.  Measured on GB300 the tensor-core output sits 3e-4 to 1e-3 from
both, about as far from the oracle that rounds its inputs to TF32 as from
the one that does not: the MMA's own accumulation over up to 1152 products
per output, not the TF32 inputs, sets the difference.  The network's gain
on held-out beams must stay within 2% of the CUDA-core forward's."""
import numpy as np
import pytest

import dn_oracle as D

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _forward(net, x, tc):
    import torch
    net.tensor_cores = tc
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()
    out = torch.empty_like(xd)
    net.forward(xd.data_ptr(), out.data_ptr(), 1)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("h,w,seed", [(32, 32, 3), (128, 128, 9), (64, 32, 5)])
def test_tensor_core_forward_against_oracle(h, w, seed):
    from orbit_gb300 import DeviceDenoiser
    net = DeviceDenoiser(h, w, max_batch=1, seed=seed)
    rng = np.random.default_rng(seed)
    p = net.get_params()
    convs, ow, ob, n = D.layout()
    for (wo, bo, ci, co) in convs:
        p[bo:bo + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.2, 16)
    net.set_params(p)
    x = rng.uniform(0.0, 2.0, (1, 1, h, w)).astype(np.float32)
    y_tc = _forward(net, x, True)
    assert net.tensor_errors() == 0
    y_o, _ = D.forward(p.astype(np.float64), x, tf32_inputs=True)
    assert rel(y_tc, y_o) <= 3e-3
    y_cc = _forward(net, x, False)
    assert rel(y_tc, y_cc) <= 3e-3
    # the correction the network adds, not only the identity part
    assert rel(y_tc - x, y_cc - x) <= 5e-3


def test_tensor_core_forward_follows_parameter_updates():
    """Weights are repacked for the tensor cores after every update."""
    import torch
    from orbit_gb300 import DeviceDenoiser
    net = DeviceDenoiser(32, 32, max_batch=1, seed=4)
    rng = np.random.default_rng(4)
    x = rng.uniform(0.0, 2.0, (1, 1, 32, 32)).astype(np.float32)
    t = (x + rng.normal(0, 0.1, x.shape)).astype(np.float32)
    y0 = _forward(net, x, True)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    net.train_step(xd.data_ptr(), td.data_ptr(), 1, 1e-2, stream=torch.cuda.current_stream().cuda_stream)
    y1 = _forward(net, x, True)
    y1_o, _ = D.forward(net.get_params().astype(np.float64), x, tf32_inputs=True)
    assert rel(y1, y1_o) <= 3e-3
    assert rel(y1, y0) > 1e-2


def test_tensor_core_gain_on_held_out_beams():
    import torch
    from orbit_gb300 import denoiser as DN
    X, T, _ = DN.make_pairs(24, seed=4321)
    net = DN.default_network(max_batch=1)
    gains = {}
    for tc in (False, True):
        net.tensor_cores = tc
        out = torch.empty_like(X)
        s = torch.cuda.current_stream().cuda_stream
        for i in range(X.shape[0]):
            net.forward(X[i:i + 1].data_ptr(), out[i:i + 1].data_ptr(), 1, stream=s)
        torch.cuda.synchronize()
        gains[tc] = float(((X - T) ** 2).mean() / ((out - T) ** 2).mean())
    assert net.tensor_errors() == 0
    assert gains[True] > 20
    assert abs(gains[True] / gains[False] - 1) < 0.02


def test_bounded_wait_runs_out_and_the_closure_falls_back():
    """The failure path of the tensor-core layers, without a GPU fault: the
    network issues no MMA (test hook), so every bounded wait runs out after
    its limit (2e6 cycles, about a millisecond) with nothing in flight.  The
    layers set the error flag, release their tensor memory and return; the
    closure reads the flag and falls back to the plain deposit (the kick
    then equals the calculator's without a closure, bit for bit); the
    network reports the error and runs its single-image forwards on the
    CUDA-core layers from then on."""
    import contextlib
    import io
    from orbit_gb300 import denoiser as DN
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    net = DN.default_network()
    assert net.tensor_cores
    net.set_wait_limit(2_000_000, withhold_mma=True)
    soa = W.c2_coords(100_000, seed=9)
    b1 = W.make_bunch(soa, 1e9)
    b2 = W.make_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(128, 128, 64)
    calc.setDenoiser(net, 10, 1e-3)
    calc.trackBunch(b1, 0.5)
    st = calc.getDenoiserState()
    assert st["fallback"] == 1 and st["trips"] == 1, st
    plain = SpaceChargeCalc2p5D(128, 128, 64)
    plain.trackBunch(b2, 0.5)
    assert np.array_equal(calc.getRhoGrid().getArray(), plain.getRhoGrid().getArray())
    assert np.array_equal(b1.getCoordinates(), b2.getCoordinates())
    assert net.tensor_errors() == 1
    assert not net.tensor_cores
    # a fresh network is unaffected (nothing was left in flight)
    net2 = DN.default_network()
    assert net2.tensor_cores
    # and the calculator keeps tracking with the plain deposit
    with contextlib.redirect_stdout(io.StringIO()):
        lat = W.fodo_lattice(calc, cells=2)
    lat.trackBunch(b1)
    assert calc.getDenoiserState()["fallback"] == 1
