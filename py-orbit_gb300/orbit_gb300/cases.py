"""One representative run of each part of the library outside the FODO
benchmark, for profiling its kernels (ncu summaries) and for timing them:

  diag      BunchTwissAnalysis.analyzeBunch, computeBunchMoments (order 4)
            and BunchTuneAnalysis.analyzeBunch on a 4e6-particle bunch
  boundary  trackBunch with a 128-point circular conducting boundary,
            128x128x32 grid, 2e6 particles
  rb        SpaceChargeCalc2p5Drb.trackBunch, 128x128x64, 2e6 particles
  fp32      the FP32 field form: eager trackBunch (k_deposit_plain, the
            fixed-point deposit both forms use, and k_kick_fp32) and a
            4-cell FODO program (fused pass with the FP32
            kick), 128x128x64, 4e6 particles
  train     denoiser training steps (CUDA-core convolution forward, data and
            weight gradients, Adam) on batches of 16 128x128 images
  train_tc  the same steps with the 3x3 layers on the tensor cores
            (k_conv3_tcb forward and data gradient, k_conv3_wgrad_tc)
  batch     a 6-bunch batched scan (grids 64x64x32, 128x128x64, 256x256x64)

Usage: python py-orbit_gb300/orbit_gb300/cases.py CASE [--n N] [--repeat R]
Each case repeats its work R times (default 3) after one untimed run and
prints the mean wall time of one repetition.
"""
from __future__ import annotations

import argparse
import contextlib
import io
import os
import sys
import time

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def case_diag(n):
    from bunch import BunchTuneAnalysis, BunchTwissAnalysis
    from orbit_gb300 import workloads as W
    b = W.make_bunch(W.c2_coords(n, seed=5), 1e8)
    b._device_bunch()
    tw, tu = BunchTwissAnalysis(), BunchTuneAnalysis()
    tu.assignTwiss(10.0, -1.2, 0.5, 0.1, 8.0, 0.7)

    def step():
        tw.analyzeBunch(b)
        tw.computeBunchMoments(b, 4)
        tu.analyzeBunch(b)
        b._device_bunch().sync()
    return step


def case_boundary(n):
    from orbit_gb300 import workloads as W
    from spacecharge import Boundary2D, SpaceChargeCalc2p5D
    b = W.make_bunch(W.c2_coords(n, seed=6), 1e8)
    bnd = Boundary2D(128, 10, "Circle", 0.04)
    calc = SpaceChargeCalc2p5D(128, 128, 32)

    def step():
        calc.trackBunch(b, 0.5, bnd)
        b._device_bunch().sync()
    return step


def case_rb(n):
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5Drb
    b = W.make_bunch(W.c2_coords(n, seed=7), 1e8)
    calc = SpaceChargeCalc2p5Drb(128, 128, 64)

    def step():
        calc.trackBunch(b, 0.5, 0.05)
        b._device_bunch().sync()
    return step


def case_fp32(n):
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    b = W.make_bunch(W.c2_coords(n, seed=8), 1e8)
    eager = SpaceChargeCalc2p5D(128, 128, 64, form="fp32")
    with _quiet():
        lat = W.fodo_lattice(SpaceChargeCalc2p5D(128, 128, 64, form="fp32"), cells=4)

    def step():
        eager.trackBunch(b, 0.5)
        lat.trackBunch(b)
        b._device_bunch().sync()
    return step


def case_train(n, tensor_cores=False):
    import torch
    from orbit_gb300 import DeviceDenoiser
    net = DeviceDenoiser(128, 128, max_batch=16, seed=1)
    net.set_batch_tensor_cores(tensor_cores)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((16, 1, 128, 128), device="cuda", generator=g)
    t = torch.rand((16, 1, 128, 128), device="cuda", generator=g)
    s = torch.cuda.current_stream().cuda_stream

    def step():
        net.train_step(x.data_ptr(), t.data_ptr(), 16, 1e-3, want_loss=False, stream=s)
        torch.cuda.synchronize()
    return step


def case_batch(n):
    from orbit_gb300 import workloads as W
    from orbit_gb300.batch import BunchBatch
    from spacecharge import SpaceChargeCalc2p5D
    members = []
    for k, (npart, grid) in enumerate(((n // 4, (64, 64, 32)), (n // 2, (128, 128, 64)), (n, (256, 256, 64)),
                                       (n // 3, (64, 64, 32)), (n // 5, (128, 128, 64)), (n // 2, (256, 256, 64)))):
        b = W.make_bunch(W.c3_coords(npart, seed=300 + k), 1e13 / npart)
        with _quiet():
            lat = W.fodo_lattice(SpaceChargeCalc2p5D(*grid), cells=2, kq=0.3 + 0.05 * k)
        members.append((b, lat))
    bb = BunchBatch(members)

    def step():
        bb.trackTurns(1)
    return step


CASES = {"diag": (case_diag, 4_000_000), "boundary": (case_boundary, 2_000_000), "rb": (case_rb, 2_000_000),
         "fp32": (case_fp32, 4_000_000), "train": (case_train, 0),
         "train_tc": (lambda n: case_train(n, tensor_cores=True), 0), "batch": (case_batch, 400_000)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args(argv)
    fn, n0 = CASES[a.case]
    step = fn(a.n if a.n else n0)
    step()
    t0 = time.perf_counter()
    for _ in range(a.repeat):
        step()
    print("%s: %.3f ms per repetition" % (a.case, (time.perf_counter() - t0) * 1e3 / max(a.repeat, 1)))


if __name__ == "__main__":
    main()
