"""GPU parity of the 2.5D kick with a conducting boundary
(SpaceChargeCalc2p5D.trackBunch(bunch, length, boundary)) against the
reference's golden vectors and the oracle: grid on the boundary extents,
boundary potential subtracted, particles outside the boundary not kicked.

Tolerances (max-norm relative): rho, phi, line density and kicks 1e-12;
coordinates after up to 100 kicks 1e-10."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_COORD, TOL_FIELD, coord_err, kick_delta_tol, load_golden, parse_sequence, rel_err

pytestmark = pytest.mark.gpu

CASES = ["bnd_circle_64x64x16", "bnd_ellipse_48x40x8", "bnd_rect_32x32x4", "bnd_points_40x40x8"]


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


@pytest.mark.parametrize("case", CASES)
def test_boundary_against_golden(case):
    from orbit.teapot_base import TPB
    from spacecharge import SpaceChargeCalc2p5D
    from test_boundary_host import boundary_of
    g = load_golden(case)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    bnd = boundary_of(g)
    b = gpu_bunch(g["init"], float(g["macrosize"]))
    calc = SpaceChargeCalc2p5D(nx, ny, nz)
    k = 0
    for step in parse_sequence(g["sequence"]):
        if step[0] == "sc":
            before = b.getCoordinates().copy()
            calc.trackBunch(b, step[1], bnd)
            got = b.getCoordinates()
            lim = g["lim_%d" % k]
            rho = calc.getRhoGrid()
            assert [rho.getMinX(), rho.getMaxX(), rho.getMinY(), rho.getMaxY()] == list(lim[:4])
            assert rel_err(rho.getArray(), g["rho_%d" % k]) <= TOL_FIELD
            assert rel_err(calc.getPhiGrid().getArray(), g["phi_%d" % k]) <= TOL_FIELD
            assert rel_err(calc.getLongGrid().getArray(), g["zg_%d" % k]) <= TOL_FIELD
            ref = g["coords_%d" % k]
            if k == 0:
                for c in (1, 3):
                    dk = ref[c] - before[c]
                    assert rel_err(got[c] - before[c], dk) <= kick_delta_tol(ref[c], dk), (case, c)
                outside = np.array([bnd.isInside(x, y) != 1 for x, y in zip(before[0], before[2])])
                assert np.array_equal(got[1][outside], before[1][outside])  # not kicked
            assert coord_err(got, ref) <= TOL_COORD
            k += 1
        else:
            getattr(TPB, step[0])(b, *step[1])
    assert k == int(g["nkicks"])


def test_boundary_fused_program_equals_eager_and_oracle():
    """FODO with boundary SC nodes: the captured program equals node-by-node
    tracking and the oracle."""
    from orbit.lattice import AccActionsContainer
    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import DriftTEAPOT, QuadTEAPOT, TEAPOT_Lattice
    from orbit.teapot.recording import BunchRecorder
    from orbit_gb300 import workloads as W
    from spacecharge import Boundary2D, SpaceChargeCalc2p5D

    bnd = Boundary2D(128, 10, "Circle", 0.03)

    def lattice(calc):
        lat = TEAPOT_Lattice("fodo_bnd")
        for c in range(4):
            for name, kq in (("qf", 0.5), ("qd", -0.5)):
                q = QuadTEAPOT("%s%d" % (name, c))
                q.setLength(0.5)
                q.addParam("kq", kq)
                d = DriftTEAPOT("d%s%d" % (name, c))
                d.setLength(2.0)
                lat.addNode(q)
                lat.addNode(d)
        lat.initialize()
        setSC2p5DAccNodes(lat, 0.3, calc, bnd)
        return lat

    soa = W.c2_coords(20_000, seed=23)
    b1 = gpu_bunch(soa, 1e10)
    b2 = gpu_bunch(soa, 1e10)
    l1 = lattice(SpaceChargeCalc2p5D(64, 64, 32))
    l2 = lattice(SpaceChargeCalc2p5D(64, 64, 32))
    l2.setFusedTracking(False)
    for _ in range(4):
        l1.trackBunch(b1)
        l2.trackBunch(b2)
    got, eager = b1.getCoordinates(), b2.getCoordinates()
    # the same arithmetic up to multiply-add contraction in the fused and the
    # per-map kernels; a particle at the boundary that a rounding difference
    # moves across it is kicked on one side only
    assert coord_err(got, eager) <= 1e-11
    rec = BunchRecorder(b1)
    cont = AccActionsContainer()
    cont.addAction(lambda p: p["node"].track(p), AccActionsContainer.BODY)
    l1.trackActions(cont, {"bunch": rec, "useCharge": 1})
    assert rec.boundaries == [bnd] and all(o[1][1] == 1 for o in rec.ops if o[0] == 32)
    a = np.ascontiguousarray(soa.copy())
    sc = O.OracleSC(64, 64, 32)
    ob = O.OracleBoundary(128, 10, "Circle", 0.03)
    s = oracle_sync_of(gpu_bunch(soa, 1e10))
    for _ in range(4):
        for code, iv, dv in rec.ops:
            if code == 32:
                assert O.sc_track_bnd(sc, a, s, dv[0], ob, nthreads=8) == 0
            else:
                assert O.run_program([(code, iv, dv)], 1, a, s, [sc], nthreads=1) == 0
    assert coord_err(got, a) <= TOL_COORD
