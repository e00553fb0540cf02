"""Grids too large for one block's shared memory (256x256, 300x180,
400x300, 512x512): the deposit splits the grid into row bands with halo rows, each
block depositing the particles whose centre row it owns.  Against the
oracle after one kick and after several, with uniform and per-particle
macrosizes.

Tolerances (max-norm relative): rho, phi and line density 1e-12; kicks
1e-12 up to 256 x 256 and 5e-12 on the finer grids (KICK_TOL); coordinates
after the kicks 1e-10."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_COORD, TOL_FIELD, coord_err, kick_delta_tol, rel_err

pytestmark = pytest.mark.gpu


def gpu_bunch(soa, macrosize, ek=1.0):
    from bunch import Bunch
    b = Bunch()
    b.getSyncParticle().kinEnergy(ek)
    b.macroSize(macrosize)
    b.setCoordinates(soa)
    return b


def oracle_sync_of(b):
    s = b.getSyncParticle()
    return O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), mass=b.mass(),
                       charge=b.charge(), classical_radius=b.classicalRadius(), macrosize=b.macroSize())


# Kick tolerance per grid.  The kick is the potential's 9-point gradient:
# differences of neighbouring potential values over the cell size, which
# amplify the potential's relative rounding by about
# max|phi| / (dx max|dphi/dx|), a factor that grows with the number of
# cells across the beam.  Up to 256 x 256 (the largest grid of the
# benchmark configurations) the kick stays within 1e-12; on the finer
# 300 x 180 and 400 x 300 grids, with the potential still within 1e-12, it
# measured 2.3e-12, and 5e-12 is required.
# The 512 x 512 grid (a 1024-point doubled grid) also runs the fused
# convolution with fewer resident blocks than work items (each block loops
# over several rows and columns).
KICK_TOL = {(256, 256, 32): TOL_FIELD, (300, 180, 16): 5e-12, (400, 300, 16): 5e-12, (512, 512, 16): 5e-12}


@pytest.mark.parametrize("grid,n", [((256, 256, 32), 200_000), ((300, 180, 16), 120_000), ((400, 300, 16), 150_000),
                                    ((512, 512, 16), 200_000)])
def test_large_grid_deposit_single_kick_against_oracle(grid, n):
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(n, seed=41)
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(*grid)
    calc.trackBunch(b, 0.5)
    got = b.getCoordinates()
    sc = O.OracleSC(*grid)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 0.5, nthreads=8) == 0
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(calc.getLongGrid().getArray(), zg) <= TOL_FIELD
    for c in (1, 3):
        dk = a[c] - soa[c]
        assert rel_err(got[c] - soa[c], dk) <= kick_delta_tol(a[c], dk) - TOL_FIELD + KICK_TOL[grid], c


def test_large_grid_deposit_per_particle_macrosizes_and_many_kicks():
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    n = 100_000
    soa = W.c2_coords(n, seed=43)
    w = np.linspace(0.5e9, 1.5e9, n)
    b = gpu_bunch(soa, 1e9)
    b.addPartAttr("macrosize")
    b._part_attr["macrosize"][:n, 0] = w
    b._host_modified()
    calc = SpaceChargeCalc2p5D(256, 256, 16)
    sc = O.OracleSC(256, 256, 16)
    a = np.ascontiguousarray(soa.copy())
    s = oracle_sync_of(b)
    from orbit.teapot_base import TPB
    for _ in range(5):
        calc.trackBunch(b, 0.5)
        TPB.drift(b, 0.5)
        assert sc.track(a, s, 0.5, msize=w, nthreads=8) == 0
        O.tpb("drift", a, s, 0.5)
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert coord_err(b.getCoordinates(), a) <= TOL_COORD
