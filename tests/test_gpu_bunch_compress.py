"""Deleting particles and tracking (Bunch.compress, Bunch.cc:704-770): the
reference compacts the bunch in place at every deposit (Grid2D.cc:121);
here a bunch with particles flagged dead is compacted before its next
upload, so the kick, the grids and the maps see only the live particles,
in their order.  Against the oracle on the surviving particles.

Tolerances (max-norm relative): grids 1e-12, coordinates 1e-10."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_COORD, TOL_FIELD, coord_err, rel_err

pytestmark = pytest.mark.gpu


def oracle_sync_of(b):
    s = b.getSyncParticle()
    return O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), mass=b.mass(),
                       charge=b.charge(), classical_radius=b.classicalRadius(), macrosize=b.macroSize())


def test_delete_then_track_against_oracle_on_the_survivors():
    from orbit.teapot_base import TPB
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    n = 20_000
    soa = W.c2_coords(n, seed=61)
    b = W.make_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(64, 64, 16)
    sc = O.OracleSC(64, 64, 16)
    sync = oracle_sync_of(b)
    # a first kick with every particle, then deletions made on the host
    # while the coordinates live on the device
    calc.trackBunch(b, 0.5)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, sync, 0.5, nthreads=8) == 0
    rng = np.random.default_rng(5)
    dead = np.sort(rng.choice(n, size=n // 10, replace=False))
    for i in dead:
        b.deleteParticleFast(int(i))
    assert b.getSize() == n  # flagged, not yet compacted
    keep = np.setdiff1d(np.arange(n), dead)
    a = np.ascontiguousarray(a[:, keep])
    for _ in range(3):
        calc.trackBunch(b, 0.5)
        TPB.drift(b, 0.5)
        assert sc.track(a, sync, 0.5, nthreads=8) == 0
        O.tpb("drift", a, sync, 0.5)
    assert b.getSize() == keep.size
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert coord_err(b.getCoordinates(), a) <= TOL_COORD
    # one more deletion through deleteParticle (compacts at once)
    b.deleteParticle(0)
    assert b.getSize() == keep.size - 1
    calc.trackBunch(b, 0.5)
    a = np.ascontiguousarray(a[:, 1:])
    assert sc.track(a, sync, 0.5, nthreads=8) == 0
    assert coord_err(b.getCoordinates(), a) <= TOL_COORD


def test_compress_keeps_particle_attributes_aligned():
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    n = 5000
    soa = W.c2_coords(n, seed=62)
    b = W.make_bunch(soa, 1e9)
    b.addPartAttr("ParticleIdNumber")
    for i in range(n):
        b.partAttrValue("ParticleIdNumber", i, 0, i)
    for i in range(0, n, 3):
        b.deleteParticleFast(i)
    SpaceChargeCalc2p5D(32, 32, 8).trackBunch(b, 0.5)
    ids = np.array([b.partAttrValue("ParticleIdNumber", i, 0) for i in range(b.getSize())])
    assert np.array_equal(ids, np.array([i for i in range(n) if i % 3 != 0], dtype=float))
    # positions of the survivors are untouched by the kick (it changes xp, yp)
    got = b.getCoordinates()
    assert np.array_equal(got[0], soa[0][ids.astype(int)])
