"""Learned denoising closure of the 2.5D kick: training data, training and
evaluation of the denoiser network (orbit_denoiser_*, a 4-level
convolutional encoder-decoder with BF16 weights).

The network maps the normalised charge density that a bunch of few
macroparticles deposits (the plain calculator's own deposit: extrema, grid
set-up and the exact fixed-point 9-point deposit) to the density that a
bunch of many more particles of the same beam deposits on the same grid.
The plain FFT Poisson solve then turns the denoised density into the
potential, so the solver stays exact and only the particle noise is
learned away.

Images are normalised to unit mean over the grid: image = rho * nx * ny /
sum(rho).  Training pairs come from seeded Gaussian, KV and waterbag beams
(transverse rms 2-8 mm, aspect ratio 0.5-2), the input from 1e5 and the
target from 1e7 particles by default."""
from __future__ import annotations

import math
import os

import numpy as np

from . import DeviceDenoiser, _native, call

KINDS = ("gaussian", "kv", "waterbag")


def _beam_params(rng, sizes, ratios):
    kind = int(rng.integers(0, 3))
    sx = math.exp(rng.uniform(math.log(sizes[0]), math.log(sizes[1])))
    ratio = math.exp(rng.uniform(math.log(ratios[0]), math.log(ratios[1])))
    return kind, sx, sx / ratio


def make_pairs(n_pairs, nx=128, ny=128, nz=64, n_lo=100_000, n_hi=10_000_000, seed=1, sizes=(2e-3, 8e-3),
               ratios=(0.5, 2.0)):
    """(inputs, targets, beams) with inputs and targets float32 CUDA tensors
    (n_pairs, 1, nx, ny); beams = [(kind, sx, sy)]."""
    import ctypes

    import torch
    from spacecharge import SpaceChargeCalc2p5D
    from .workloads import make_bunch
    rng = np.random.default_rng(seed)
    soa = np.zeros((6, n_lo))
    soa[4] = rng.uniform(-100.0, 100.0, n_lo)
    bunch = make_bunch(soa, 1.0)
    dev = bunch._device_bunch()
    ptrs = dev.device_pointers()
    calc = SpaceChargeCalc2p5D(nx, ny, nz)
    X = torch.empty((n_pairs, 1, nx, ny), dtype=torch.float32, device="cuda")
    T = torch.empty_like(X)
    g = torch.empty(nx * ny, dtype=torch.float32, device="cuda")
    lim = np.zeros(4)
    beams = []
    for k in range(n_pairs):
        kind, sx, sy = _beam_params(rng, sizes, ratios)
        beams.append((kind, sx, sy))
        s_lo, s_hi = int(rng.integers(1, 2**62)), int(rng.integers(1, 2**62))
        call("orbit_beam_sample", ctypes.c_void_p(ptrs[0]), ctypes.c_void_p(ptrs[2]), n_lo, kind, sx, sy, s_lo)
        calc.trackBunch(bunch, 0.0)  # the calculator's grid set-up and deposit, no kick
        rho = calc._calc.grid(_native.GRID_RHO)
        lim[:] = calc._calc.limits()[:4]
        call("orbit_beam_deposit", ctypes.c_void_p(g.data_ptr()), nx, ny,
             lim.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(n_hi), kind, sx, sy, s_hi)
        X[k, 0] = torch.from_numpy(rho * (nx * ny / rho.sum())).float()
        T[k, 0] = (g * (nx * ny / g.sum())).view(nx, ny)
    return X, T, beams


class _DevArray:
    """A device array of float64 by address, for torch.as_tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3}


def _view(ptr, n):
    import torch
    return torch.as_tensor(_DevArray(ptr, n), device="cuda")


# tracked-beam set-ups: (distribution, rms scale, intensity [protons], FODO k1)
TRACK_SETUPS = (("waterbag", 1.0, 1e14, 0.5), ("gauss", 1.0, 1e14, 0.5), ("waterbag", 0.7, 2e14, 0.4),
                ("gauss", 1.4, 3e14, 0.6), ("waterbag", 1.2, 5e13, 0.6), ("gauss", 0.8, 1.5e14, 0.45))


def make_tracked_pairs(setups=TRACK_SETUPS, turns=10, per_turn=40, nx=128, ny=128, nz=64, n_lo=100_000,
                       n_hi=10_000_000, seed=3, cells=40):
    """Pairs from beams as tracking shapes them: a bunch of n_hi particles
    is tracked with the plain form through a FODO lattice; at the start and
    after each turn, slices of n_lo consecutive particles (independent
    draws of the same distribution) go through the calculator for the
    input, and the whole bunch is deposited on each slice's grid for the
    target."""
    import contextlib
    import ctypes
    import io

    import torch
    from spacecharge import SpaceChargeCalc2p5D
    from . import workloads as W
    lo = W.make_bunch(np.zeros((6, n_lo)), 1.0)
    lo_ptrs = lo._device_bunch().device_pointers()
    lo_x, lo_y, lo_z = (_view(lo_ptrs[c], n_lo) for c in (0, 2, 4))
    calc = SpaceChargeCalc2p5D(nx, ny, nz)
    g = torch.empty(nx * ny, dtype=torch.float32, device="cuda")
    lim = np.zeros(4)
    X, T = [], []
    for k, (dist, scale, intensity, k1) in enumerate(setups):
        soa = W.c2_coords(n_hi, seed=seed * 100 + k) if dist == "waterbag" else W.c3_coords(n_hi, seed * 100 + k)
        soa[:4] *= scale
        hi = W.make_bunch(soa, intensity / n_hi)
        del soa
        with contextlib.redirect_stdout(io.StringIO()):
            lat = W.fodo_lattice(SpaceChargeCalc2p5D(nx, ny, nz), cells=cells, kq=k1)
        for t in range(turns + 1):
            if t > 0:
                lat.trackBunchTurns(hi, 1)
            ptrs = hi._device_bunch().device_pointers()
            hx, hy, hz = (_view(ptrs[c], n_hi) for c in (0, 2, 4))
            for j in range(per_turn):
                off = (j * n_lo) % (n_hi - n_lo + 1)
                lo_x.copy_(hx[off:off + n_lo])
                lo_y.copy_(hy[off:off + n_lo])
                lo_z.copy_(hz[off:off + n_lo])
                torch.cuda.synchronize()
                calc.trackBunch(lo, 0.0)
                rho = calc._calc.grid(_native.GRID_RHO)
                lim[:] = calc._calc.limits()[:4]
                call("orbit_grid_deposit", ctypes.c_void_p(g.data_ptr()), nx, ny,
                     lim.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_void_p(ptrs[0]),
                     ctypes.c_void_p(ptrs[2]), int(n_hi))
                X.append(torch.from_numpy(rho * (nx * ny / rho.sum())).float().cuda())
                T.append((g * (nx * ny / g.sum())).view(nx, ny).clone())
        del hi, lat
        torch.cuda.empty_cache()
    return torch.stack(X)[:, None], torch.stack(T)[:, None]


def _augment(x, t, code):
    """One of the 8 symmetries of the square (flips of x, of y, transpose)."""
    dims = []
    if code & 1:
        dims.append(2)
    if code & 2:
        dims.append(3)
    if dims:
        x, t = x.flip(dims), t.flip(dims)
    if code & 4 and x.shape[2] == x.shape[3]:
        x, t = x.transpose(2, 3), t.transpose(2, 3)
    return x.contiguous(), t.contiguous()


# Multi-scale loss weights 4^s over the output and five 2x2 poolings: a
# stand-in for the force error (the field of the density error weights
# wavenumber k by 1/k^2; pooling s times keeps the modes below k_max / 2^s).
FORCE_LOSS_WEIGHTS = [4.0 ** s for s in range(6)]


def train(net: DeviceDenoiser, X, T, epochs=4, batch=16, lr=1e-3, seed=0, log=None, loss_weights=None,
          tensor_cores=True):
    """Adam on minibatches with random symmetries; cosine learning-rate
    decay.  loss_weights: None, the mean squared error; a list, the
    multi-scale loss (DeviceDenoiser.set_loss).  tensor_cores: the steps'
    3x3 layers (forward, data and weight gradients) on the tensor cores
    (TF32 operands, FP32 accumulation: 1.57x the CUDA-core step on a batch
    of 16 128x128 images, the same held-out gain); the network's batches
    return to the CUDA cores afterwards.  Returns the per-epoch mean
    losses."""
    import torch
    net.set_loss(loss_weights)
    net.set_batch_tensor_cores(tensor_cores)
    try:
        return _train_steps(net, X, T, epochs, batch, lr, seed, log, torch)
    finally:
        net.set_batch_tensor_cores(False)


def _train_steps(net, X, T, epochs, batch, lr, seed, log, torch):
    """The epochs of train()."""
    n = X.shape[0]
    steps = epochs * (n // batch)
    rng = np.random.default_rng(seed)
    stream = torch.cuda.current_stream().cuda_stream  # the stream that builds the minibatches
    out, step = [], 0
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        tot = 0.0
        for b in range(n // batch):
            idx = perm[b * batch:(b + 1) * batch]
            xb, tb = _augment(X.index_select(0, idx), T.index_select(0, idx), int(rng.integers(0, 8)))
            a = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(steps, 1)))
            want = (b % 50) == 0
            loss = net.train_step(xb.data_ptr(), tb.data_ptr(), batch, a, want_loss=want, stream=stream)
            if want:
                tot += loss
            step += 1
        out.append(tot / max(1, (n // batch + 49) // 50))
        if log:
            log("epoch %d: loss %.4g" % (ep, out[-1]))
    return out


def evaluate(net: DeviceDenoiser, X, T, batch=16, force=False):
    """Mean squared error of the raw inputs and of the network outputs
    against the targets and its ratio (`gain`).  With `force`, also the
    ratio of the force errors (`gain_force`, see `force_error`) and the
    ratio of the error spectra per band of |k| (`gain_by_k`, K_BANDS): the
    density error weights all wavelengths alike, the force error weights
    them by 1/k^2, so beam-scale noise, which a single snapshot cannot tell
    from beam structure, dominates it."""
    import torch
    n = X.shape[0]
    out = torch.empty_like(X)
    stream = torch.cuda.current_stream().cuda_stream
    for b in range(0, n, batch):
        m = min(batch, n - b)
        net.forward(X[b:b + m].data_ptr(), out[b:b + m].data_ptr(), m, stream=stream)
    torch.cuda.synchronize()
    mse_raw = float(((X - T) ** 2).mean())
    mse_net = float(((out - T) ** 2).mean())
    ev = {"mse_raw": mse_raw, "mse_net": mse_net, "gain": mse_raw / mse_net}
    if force:
        f_raw, s_raw = force_error(X, T)
        f_net, s_net = force_error(out, T)
        ev.update({"force_raw": f_raw, "force_net": f_net, "gain_force": f_raw / f_net,
                   "gain_by_k": [a / b for a, b in zip(s_raw, s_net)], "k_bands": list(K_BANDS)})
    return ev


K_BANDS = (0.0, 0.02, 0.04, 0.08, 0.16, 0.32, 0.8)  # |k| in cycles per cell


def force_error(Y, T, bands=K_BANDS):
    """How far images Y are from targets T in the force they produce, the
    quantity that moves particles (evaluation only; the kick path uses the
    library's own solver).  Both are (n, 1, nx, ny) densities on a grid of
    unit steps; the potential is the open-boundary convolution with
    -ln(r) / 2 on the doubled grid (the Hockney scheme of the calculator,
    PoissonSolverFFT2D.cc:174-256, at dx = dy), the force its central
    difference.  Returns (force error energy / target force energy, the
    error's power spectrum averaged over the bands of |k|)."""
    import torch
    dev = Y.device
    n, _, nx, ny = Y.shape
    i = torch.arange(2 * nx, device=dev, dtype=torch.float64)
    j = torch.arange(2 * ny, device=dev, dtype=torch.float64)
    i = torch.minimum(i, 2 * nx - i)
    j = torch.minimum(j, 2 * ny - j)
    r2 = i[:, None] ** 2 + j[None, :] ** 2
    G = -0.5 * torch.log(r2.clamp(min=1.0))
    G[0, 0] = 0.0
    Gk = torch.fft.rfft2(G)

    def force(rho):
        p = torch.zeros(rho.shape[0], 2 * nx, 2 * ny, device=dev, dtype=torch.float64)
        p[:, :nx, :ny] = rho
        phi = torch.fft.irfft2(torch.fft.rfft2(p) * Gk, s=(2 * nx, 2 * ny))[:, :nx, :ny]
        return phi[:, 2:, 1:-1] - phi[:, :-2, 1:-1], phi[:, 1:-1, 2:] - phi[:, 1:-1, :-2]

    y, t = Y[:, 0].double(), T[:, 0].double()
    tx, ty = force(t)
    ex, ey = force(y)
    rel = float(((ex - tx) ** 2 + (ey - ty) ** 2).sum() / (tx ** 2 + ty ** 2).sum())
    P = (torch.fft.fft2(y - t).abs() ** 2).mean(0)
    kx = torch.fft.fftfreq(nx, device=dev, dtype=torch.float64).abs()
    ky = torch.fft.fftfreq(ny, device=dev, dtype=torch.float64).abs()
    kr = torch.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    spec = [float(P[(kr >= bands[b]) & (kr < bands[b + 1])].mean()) for b in range(len(bands) - 1)]
    return rel, spec


DATA = os.path.join(os.path.dirname(__file__), "data")
DEFAULT = "denoiser_128x128.npy"


def default_network(max_batch=1, size=128):
    """The shipped network, trained by `train_default` on 128 x 128 images
    (6,000 synthetic-beam pairs and 2,376 tracked-beam pairs, 10 epochs,
    batch 16, Adam 1e-3 with cosine decay) on this library's own kernels.
    The network is convolutional, so the same weights run on a size x size
    grid (size a multiple of 8); they were trained at about 6 input
    particles per cell (1e5 particles on 128 x 128), so a larger grid wants
    proportionally more particles (4e5 on 256 x 256)."""
    net = DeviceDenoiser(size, size, max_batch=max_batch, seed=5)
    net.set_params(np.load(os.path.join(DATA, DEFAULT)))
    return net


def train_default(out_path, n_synth=6000, epochs=10, log=print, loss_weights=None, init=None, lr=1e-3):
    """Generates the training pairs (synthetic beams of seed 11 and the
    tracked set-ups of seed 3), trains the 128 x 128 network (from the
    parameters `init` if given, else from a seeded initialisation) and
    saves its parameters; returns held-out evaluations, density and force
    errors, on both kinds of pairs (200 synthetic pairs, and every tenth
    tracked pair, kept out of training)."""
    import torch
    Xs, Ts, _ = make_pairs(n_synth + 200, seed=11)
    Xk, Tk = make_tracked_pairs()
    test_k = torch.arange(0, Xk.shape[0], 10, device="cuda")
    keep = torch.ones(Xk.shape[0], dtype=torch.bool, device="cuda")
    keep[test_k] = False
    X = torch.cat([Xs[:n_synth], Xk[keep]])
    T = torch.cat([Ts[:n_synth], Tk[keep]])
    net = DeviceDenoiser(128, 128, max_batch=16, seed=5)
    if init is not None:
        net.set_params(np.asarray(init, dtype=np.float32))
    train(net, X, T, epochs=epochs, batch=16, lr=lr, log=log, loss_weights=loss_weights)
    ev = {"synthetic": evaluate(net, Xs[n_synth:], Ts[n_synth:], force=True),
          "tracked": evaluate(net, Xk[test_k].contiguous(), Tk[test_k].contiguous(), force=True),
          "pairs": int(X.shape[0])}
    np.save(out_path, net.get_params())
    return ev


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="train the 128 x 128 denoiser and save its parameters")
    ap.add_argument("--out", default=os.path.join(DATA, DEFAULT))
    ap.add_argument("--loss", choices=["mse", "force"], default="mse",
                    help="mse: squared density error; force: the multi-scale stand-in for the force error")
    ap.add_argument("--init", default=None, help="start from these parameters (.npy) instead of a fresh network")
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--lr", type=float, default=1e-3)
    a = ap.parse_args()
    init = np.load(a.init) if a.init else None
    print(train_default(a.out, epochs=a.epochs, loss_weights=FORCE_LOSS_WEIGHTS if a.loss == "force" else None,
                        init=init, lr=a.lr))
