"""GPU parity at the benchmark's own configuration: the bench's 1e6-particle
bunch (4D waterbag, rms 4 mm / 0.8 mrad, z ~ N(0, 10 m), dE ~ N(0, 1 MeV),
1e14 protons at 1 GeV), the 128x128x64 grid and the 40-cell FODO lattice
with 4 SC nodes per cell (160 kicks per turn), tracked by the fused device
program against the oracle on all host threads.

At 1e6 particles the fixed-point deposit rounds each contribution to
2^-40 of a unit weight (K = 39), the coarsest of any tested case, so this
is the configuration whose rounding is least covered by the smaller tests.

Tolerances (max-norm relative, tests/helpers.py): density, potential,
line density and fields 1e-12; kicks 1e-12 plus the rounding of the
stored coordinate (kick_delta_tol); coordinates after 100 and after 160
kicks 1e-10."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import TOL_COORD, TOL_FIELD, coord_err, kick_delta_tol, rel_err

pytestmark = pytest.mark.gpu

N_BENCH = 1_000_000
INTENSITY = 1e14
BENCH_SEED = 1000  # bench.py's rank-0 bunch
THREADS = os.cpu_count() or 1


def oracle_sync_of(b):
    s = b.getSyncParticle()
    return O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), mass=b.mass(),
                       charge=b.charge(), classical_radius=b.classicalRadius(), macrosize=b.macroSize())


def test_benchmark_bunch_first_kick():
    """One SC kick (eager trackBunch) of the bench's bunch: grids, fields at
    every particle and the kick itself against the oracle."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(N_BENCH, seed=BENCH_SEED)
    b = W.make_bunch(soa, INTENSITY / N_BENCH)
    calc = SpaceChargeCalc2p5D(128, 128, 64)
    calc.trackBunch(b, 0.5)
    got = b.getCoordinates()
    sc = O.OracleSC(128, 128, 64)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 0.5, nthreads=THREADS) == 0
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(calc.getLongGrid().getArray(), zg) <= TOL_FIELD
    # fields at the particles (the gradient and the line density the kick uses)
    sub = slice(0, N_BENCH, 7)
    ex, ey, lam = calc.fields(soa[0][sub], soa[2][sub], soa[4][sub])
    oex, oey, olam = sc.fields(soa[0][sub], soa[2][sub], soa[4][sub])
    assert rel_err(ex, oex) <= TOL_FIELD
    assert rel_err(ey, oey) <= TOL_FIELD
    assert rel_err(lam, olam) <= TOL_FIELD
    for c in (1, 3):
        dk = a[c] - soa[c]
        assert rel_err(got[c] - soa[c], dk) <= kick_delta_tol(a[c], dk), c
    assert coord_err(got, a) <= TOL_COORD


def test_benchmark_turn_against_oracle():
    """The bench's step: one full turn (160 SC kicks) of the 40-cell FODO
    lattice on the bench's 1e6-particle bunch, fused device program (CUDA
    graphs) against the oracle's program executor."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(N_BENCH, seed=BENCH_SEED)
    b = W.make_bunch(soa, INTENSITY / N_BENCH)
    calc = SpaceChargeCalc2p5D(128, 128, 64)
    lat = W.fodo_lattice(calc, cells=40)
    prog = lat.fusedProgram(b)
    assert prog is not None
    assert sum(1 for o in prog.ops if o[0] == 32) == 160
    lat.trackBunch(b)
    got = b.getCoordinates()
    ref = np.ascontiguousarray(soa.copy())
    oc = O.OracleSC(128, 128, 64)
    assert O.run_program(prog.ops, 1, ref, oracle_sync_of(b), [oc], nthreads=THREADS) == 0
    assert coord_err(got, ref) <= TOL_COORD
    # the grids of the last kick
    rho, phi, zg, lim = oc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(calc.getLongGrid().getArray(), zg) <= TOL_FIELD
    # space charge acted: the kicks are far above the tolerance
    assert rel_err(got[1], soa[1]) > 1e-3


def test_hundred_kicks_benchmark_grid():
    """100 SC kicks (25 FODO cells, one turn) of a 1e5-particle bunch at the
    benchmark's grid and intensity: coordinates within 1e-10."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    n = 100_000
    soa = W.c2_coords(n, seed=BENCH_SEED + 1)
    b = W.make_bunch(soa, INTENSITY / n)
    calc = SpaceChargeCalc2p5D(128, 128, 64)
    lat = W.fodo_lattice(calc, cells=25)
    prog = lat.fusedProgram(b)
    assert sum(1 for o in prog.ops if o[0] == 32) == 100
    lat.trackBunch(b)
    got = b.getCoordinates()
    ref = np.ascontiguousarray(soa.copy())
    oc = O.OracleSC(128, 128, 64)
    assert O.run_program(prog.ops, 1, ref, oracle_sync_of(b), [oc], nthreads=THREADS) == 0
    assert coord_err(got, ref) <= TOL_COORD
    rho, phi, zg, lim = oc.grids()
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(got[1], soa[1]) > 1e-3
