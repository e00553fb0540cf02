"""The fused convolution (k_conv_fused in py-orbit_gb300/csrc/sc2p5d.cu: the
Green rebuild, the forward rows with the line-density finalization, the
columns with the Green multiply and the backward rows in one cooperative
launch) against the separate kernels it replaces.  It runs the same
operations in the same order, so grids and coordinates are bit-identical,
in both forms (the deposit is exact in both): eagerly with Green rebuilds
on reshaped beams, in the recorded FODO program (CUDA graphs) and on a
non-square grid of mixed radices.
Its barrier waits are bounded: with a block withheld from the first
barrier, the other blocks' waits run out, the bunch's status reports it,
and the next kick runs normally."""
import numpy as np
import pytest

from helpers import TOL_FIELD, rel_err

pytestmark = pytest.mark.gpu


def _calcs(nx, ny, nz, form="plain"):
    from spacecharge import SpaceChargeCalc2p5D
    fused = SpaceChargeCalc2p5D(nx, ny, nz, form=form)
    sep = SpaceChargeCalc2p5D(nx, ny, nz, form=form)
    assert fused._calc.set_fused_conv(True)
    assert not sep._calc.set_fused_conv(False)
    return fused, sep


def _grids(calc):
    return (calc.getRhoGrid().getArray().copy(), calc.getPhiGrid().getArray().copy(),
            calc.getLongGrid().getArray().copy())


@pytest.mark.parametrize("form,grid", [("plain", (128, 128, 64)), ("fp32", (128, 128, 64)),
                                       ("plain", (96, 60, 16))])
def test_eager_kicks_bit_identical_with_rebuilds(form, grid):
    from orbit_gb300 import workloads as W
    nx, ny, nz = grid
    fused, sep = _calcs(nx, ny, nz, form)
    soa = W.c2_coords(200_000, seed=31)
    ba = W.make_bunch(soa.copy(), 1e8)
    bb = W.make_bunch(soa.copy(), 1e8)
    for k in range(6):
        if k in (2, 4):
            # reshape the beam beyond the 25% aspect-ratio rule: the solver
            # grid is reset and the Green spectrum rebuilt
            for b in (ba, bb):
                c = b.getCoordinates()
                c[0] *= 1.6 if k == 2 else 0.5
                b.setCoordinates(c)
        fused.trackBunch(ba, 0.5)
        sep.trackBunch(bb, 0.5)
        for g1, g2 in zip(_grids(fused), _grids(sep)):
            assert np.array_equal(g1, g2), k
    assert np.array_equal(ba.getCoordinates(), bb.getCoordinates())
    kf, gf = fused._calc.counters()
    ks, gs = sep._calc.counters()
    assert (kf, gf) == (ks, gs) and kf == 6 and gf >= 3


def test_fodo_program_bit_identical():
    """Two turns of a 10-cell FODO lattice (40 kicks per turn, graph replay)."""
    from orbit_gb300 import workloads as W
    fused, sep = _calcs(128, 128, 64)
    soa = W.c2_coords(100_000, seed=32)
    out = []
    for calc in (fused, sep):
        b = W.make_bunch(soa.copy(), 1e13 / 100_000)
        lat = W.fodo_lattice(calc, cells=10)
        lat.trackBunch(b)
        lat.trackBunch(b)
        out.append((b.getCoordinates(), _grids(calc), calc._calc.counters()))
    assert np.array_equal(out[0][0], out[1][0])
    for g1, g2 in zip(out[0][1], out[1][1]):
        assert np.array_equal(g1, g2)
    assert out[0][2] == out[1][2]


def test_fused_against_oracle():
    """One eager kick through the fused launch against the oracle."""
    import oracle as O
    from orbit_gb300 import workloads as W
    fused, _ = _calcs(64, 64, 16)
    soa = W.c2_coords(50_000, seed=33)
    b = W.make_bunch(soa.copy(), 1e9)
    fused.trackBunch(b, 0.5)
    oc = O.OracleSC(64, 64, 16)
    s = b.getSyncParticle()
    sync = O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), mass=b.mass(), charge=b.charge(),
                       classical_radius=b.classicalRadius(), macrosize=b.macroSize())
    ref = np.ascontiguousarray(soa.copy())
    oc.track(ref, sync, 0.5)
    rho, phi, zg, lim = oc.grids()
    assert rel_err(fused.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(fused.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(fused.getLongGrid().getArray(), zg) <= TOL_FIELD


def test_barrier_wait_runs_out_and_is_reported():
    from orbit_gb300 import OrbitError
    from orbit_gb300 import workloads as W
    fused, sep = _calcs(64, 64, 16)
    soa = W.c2_coords(20_000, seed=34)
    b = W.make_bunch(soa.copy(), 1e9)
    b2 = W.make_bunch(soa.copy(), 1e9)
    fused._calc.set_conv_wait(2000, withhold=0)
    with pytest.raises(OrbitError):
        fused.trackBunch(b, 0.5)
        b._device_bunch().sync()
    sep.trackBunch(b2, 0.5)
    # the next kick runs normally (the set-up zeroes the barrier counters);
    # both calculators have now seen the same beam twice
    fused._calc.set_conv_wait(1 << 20, withhold=-1)
    b.setCoordinates(soa.copy())
    b2.setCoordinates(soa.copy())
    fused.trackBunch(b, 0.5)
    sep.trackBunch(b2, 0.5)
    b._device_bunch().sync()
    assert np.array_equal(fused.getPhiGrid().getArray(), sep.getPhiGrid().getArray())
    assert np.array_equal(b.getCoordinates(), b2.getCoordinates())


def test_host_edits_after_an_overlapped_upload():
    """trackBunch enqueues the bunch's upload before the lattice walk and
    does not wait for it; host reads and edits of the coordinates afterwards
    wait for that upload first.  The same sequence with every upload waited
    for beforehand gives the same coordinates."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(50_000, seed=36)
    edited = soa.copy()
    edited[0, :10] += 1e-4
    out = []
    for wait in (False, True):
        calc = SpaceChargeCalc2p5D(64, 64, 16)
        lat = W.fodo_lattice(calc, cells=4)
        b = W.make_bunch(soa.copy(), 1e9)
        steps = [lambda: None,
                 lambda: b.setCoordinates(edited.copy()),
                 lambda: [b.x(i, b.x(i) + 1e-5) for i in range(10)]]
        for edit in steps:
            edit()
            if wait:
                b._device_bunch()        # upload now and wait for it
            lat.trackBunch(b)
        out.append(b.getCoordinates())
    assert np.array_equal(out[0], out[1])
