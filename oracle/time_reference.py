"""ORACLE / TEST INFRASTRUCTURE ONLY.

Times the compiled reference (oracle/_ref/libpyorbit_ref.so: the reference's
own SpaceChargeCalc2p5D and teapot_base C++, one MPI rank, AoS bunch, FFT =
project shim) against the C restatement (oracle/_build/liborbit_oracle.so)
on the same sample of the benchmark workload: the 40-cell FODO lattice with
4 SC nodes per cell (160 kicks per turn), 128x128x64 grid, 1 GeV protons,
4D waterbag bunch.  Both run the same recorded op sequence; the reference is
driven call by call (trackBunch per SC node, one teapot_base function per
map), as its Python layer would.  It also checks that both end on the same
coordinates bit for bit.

Runs only where the compiled reference exists (the x86 host that has the
reference tree).  Usage:

    python oracle/time_reference.py [--n 100000] [--turns 1] [--threads 1,8]

Prints one JSON line: kicks/s of the reference (1 rank) and of the
restatement at each thread count.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "py-orbit_gb300"))

import oracle as O  # noqa: E402

MAP_NAMES = {"DRIFT": "drift", "QUAD1": "quad1", "QUAD2": "quad2", "QFRIN": "quadfringeIN",
             "QFROUT": "quadfringeOUT"}


def recorded_fodo(n, seed):
    """Coordinates, bunch and the recorded op list of one turn."""
    from orbit.lattice import AccActionsContainer
    from orbit.teapot.recording import BunchRecorder
    from orbit_gb300 import workloads as W

    class _Calc:  # records SC nodes without a GPU calculator
        def trackBunch(self, bunch, length, boundary=None):
            bunch._record_sc(self, length)

    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        lat = W.fodo_lattice(_Calc(), cells=40)
    soa = W.c2_coords(n, seed=seed)
    bunch = W.make_bunch(soa, 1e14 / n)
    rec = BunchRecorder(bunch)
    cont = AccActionsContainer()
    cont.addAction(lambda p: p["node"].track(p), AccActionsContainer.BODY)
    lat.trackActions(cont, {"bunch": rec, "useCharge": 1})
    return soa, bunch, rec.ops


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--turns", type=int, default=1)
    ap.add_argument("--threads", default="1,%d" % (os.cpu_count() or 1))
    args = ap.parse_args()
    if not O.ref_available():
        print(json.dumps({"unavailable": "compiled reference not present on this host"}))
        return
    from orbit_gb300 import OP
    inv = {v: k for k, v in OP.items()}
    soa, bunch, ops = recorded_fodo(args.n, 99)
    kpt = sum(1 for o in ops if o[0] == 32)
    kicks = args.n * kpt * args.turns

    rb = O.RefBunch(soa, 1.0, bunch.macroSize())
    rs = O.RefSC(128, 128, 64)
    t0 = time.perf_counter()
    for _ in range(args.turns):
        for code, iv, dv in ops:
            if code == 32:
                rs.track(rb, dv[0])
            else:
                rb.tpb(MAP_NAMES[inv[code]], *dv)
    t_ref = time.perf_counter() - t0
    ref_coords = rb.coords()

    s = bunch.getSyncParticle()
    out = {"workload": "FODO 40 cells x 4 SC nodes (%d kicks per turn), grid 128x128x64, %d particles, %d turn(s)"
                       % (kpt, args.n, args.turns),
           "host": os.uname().machine, "cpu_count": os.cpu_count(),
           "reference_1rank": {"s": t_ref, "kicks_per_s": kicks / t_ref}, "port": {}}
    for th in (int(t) for t in args.threads.split(",")):
        a = np.ascontiguousarray(soa.copy())
        sync = O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), macrosize=bunch.macroSize())
        t0 = time.perf_counter()
        rc = O.run_program(ops, args.turns, a, sync, [O.OracleSC(128, 128, 64)], nthreads=th)
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError("oracle status %d" % rc)
        same = bool(np.array_equal(a, ref_coords)) if th == 1 else None
        out["port"][str(th)] = {"s": dt, "kicks_per_s": kicks / dt, "bit_identical_to_reference": same}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
