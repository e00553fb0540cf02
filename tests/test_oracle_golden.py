"""The C restatement (oracle) against golden vectors produced by the
reference's own C++ (tests/golden/make_golden.py).  This pins the oracle
before the GPU tests compare against it."""
import numpy as np
import pytest

import oracle as O
from helpers import golden_maps, kin_sync, load_golden, parse_sequence, rel_err

# On the x86 build host the oracle reproduces the reference bit for bit; on
# another host libm (log, cos, cosh) may differ in the last bit.
TOL = 1e-13


def test_maps_sequence():
    g = load_golden("maps")
    soa = np.ascontiguousarray(g["init"].copy())
    s = kin_sync(g["kin"], 1e9)
    s.time = 0.0
    for k, (name, args) in enumerate(golden_maps(g)):
        O.tpb(name, soa, s, *args)
        ref = g["after_%02d" % k]
        for c in range(6):
            assert rel_err(soa[c], ref[c]) <= TOL, (k, name, c, rel_err(soa[c], ref[c]))
    assert abs(s.time - g["kin"][6]) <= 1e-15 * abs(g["kin"][6])


@pytest.mark.parametrize("case", ["sc_round_32x32x8", "c1_64x64x1", "flat_40x24x16", "ratio2_16x16x2"])
def test_sc_cases(case):
    g = load_golden(case)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    sc = O.OracleSC(nx, ny, nz, float(g["xy_ratio"]))
    s = kin_sync(g["kin"], float(g["macrosize"]))
    soa = np.ascontiguousarray(g["init"].copy())
    k = 0
    for step in parse_sequence(g["sequence"]):
        if step[0] == "sc":
            assert sc.track(soa, s, step[1]) == 0
            rho, phi, zg, lim = sc.grids()
            assert rel_err(rho, g["rho_%d" % k]) <= TOL
            assert rel_err(phi, g["phi_%d" % k]) <= TOL
            assert rel_err(zg, g["zg_%d" % k]) <= TOL
            assert np.allclose(lim[:9], g["lim_%d" % k], rtol=1e-15, atol=0)
            if k == 0:
                ex, ey, lam = sc.fields(soa[0], soa[2], soa[4])
                assert rel_err(ex, g["ex_0"]) <= TOL
                assert rel_err(ey, g["ey_0"]) <= TOL
                assert rel_err(lam, g["lam_0"]) <= TOL
                for c in range(6):
                    assert rel_err(soa[c], g["coords_0"][c]) <= TOL
            k += 1
        else:
            O.tpb(step[0], soa, s, *step[1])
    assert k == int(g["nkicks"])
    for c in range(6):
        assert rel_err(soa[c], g["final"][c]) <= TOL, (case, c)


@pytest.mark.parametrize("case", ["rb_32x32x16", "rb_40x24x8_avg5", "rb_16x16x2", "rb_16x16x1"])
def test_scrb_cases(case):
    """SpaceChargeCalc2p5Drb: grids, smoothed line-density derivative and all
    six coordinates (the longitudinal kick changes dE) after every kick."""
    g = load_golden(case)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    sc = O.OracleSCrb(nx, ny, nz, float(g["xy_ratio"]))
    sc.setLongAveragingPointsN(int(g["navg"]))
    s = kin_sync(g["kin"], float(g["macrosize"]))
    soa = np.ascontiguousarray(g["init"].copy())
    k = 0
    for step in parse_sequence(g["sequence"]):
        if step[0] == "sc":
            assert sc.track(soa, s, step[1], float(g["pipe_radius"])) == 0
            rho, phi, zg, lim = sc.grids()
            zd = sc.extra()[0]
            assert rel_err(rho, g["rho_%d" % k]) <= TOL
            assert rel_err(phi, g["phi_%d" % k]) <= TOL
            assert rel_err(zg, g["zg_%d" % k]) <= TOL
            assert rel_err(zd, g["zd_%d" % k]) <= TOL
            assert np.allclose(lim[:9], g["lim_%d" % k], rtol=1e-15, atol=0)
            for c in range(6):
                assert rel_err(soa[c], g["coords_%d" % k][c]) <= TOL, (case, k, c)
            k += 1
        else:
            O.tpb(step[0], soa, s, *step[1])
    assert k == int(g["nkicks"])
    assert np.max(np.abs(soa[5] - g["init"][5])) > 0 or nz == 1  # the longitudinal kick acted


def oracle_boundary_of(g):
    shape = str(g["bnd_shape"])
    if shape:
        return O.OracleBoundary(int(g["bnd_np"]), int(g["bnd_nm"]), shape, float(g["bnd_xdim"]),
                                float(g["bnd_ydim"]))
    b = O.OracleBoundary(int(g["bnd_np"]), int(g["bnd_nm"]))
    for i, (x, y) in enumerate(zip(g["bnd_x"], g["bnd_y"])):
        b.setBoundaryPoint(i, x, y)
    assert b.initialize() == 0
    return b


@pytest.mark.parametrize("case", ["bnd_circle_64x64x16", "bnd_ellipse_48x40x8", "bnd_rect_32x32x4",
                                  "bnd_points_40x40x8"])
def test_boundary_cases(case):
    """Conducting boundaries: points, extents and the inside test of the
    shapes, and the kicks with the boundary potential subtracted."""
    g = load_golden(case)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    bnd = oracle_boundary_of(g)
    head, bx, by, lsq = bnd.data()
    assert np.array_equal(bx, g["bnd_x"]) and np.array_equal(by, g["bnd_y"])
    assert np.array_equal(head[:6], g["bnd_head"][:6])
    probe = np.linspace(-0.03, 0.03, 41)
    assert np.array_equal(np.array([[bnd.isInside(x, y) for y in probe] for x in probe]), g["inside"])
    sc = O.OracleSC(nx, ny, nz)
    s = kin_sync(g["kin"], float(g["macrosize"]))
    soa = np.ascontiguousarray(g["init"].copy())
    k = 0
    for step in parse_sequence(g["sequence"]):
        if step[0] == "sc":
            assert O.sc_track_bnd(sc, soa, s, step[1], bnd) == 0
            rho, phi, zg, lim = sc.grids()
            assert rel_err(rho, g["rho_%d" % k]) <= TOL
            assert rel_err(phi, g["phi_%d" % k]) <= TOL
            assert rel_err(zg, g["zg_%d" % k]) <= TOL
            for c in range(6):
                assert rel_err(soa[c], g["coords_%d" % k][c]) <= TOL, (case, k, c)
            k += 1
        else:
            O.tpb(step[0], soa, s, *step[1])
    assert k == int(g["nkicks"])


def test_multithreaded_slices_match_within_summation_order():
    """The rank-sliced oracle differs from one slice only by the order of the
    grid sums (the reference's MPI decomposition)."""
    g = load_golden("sc_round_32x32x8")
    s = kin_sync(g["kin"], float(g["macrosize"]))
    a = np.ascontiguousarray(g["init"].copy())
    b = a.copy()
    s1 = O.OracleSC(32, 32, 8)
    s2 = O.OracleSC(32, 32, 8)
    s1.track(a, s, 0.5, nthreads=1)
    s2.track(b, s, 0.5, nthreads=7)
    assert rel_err(s2.grids()[1], s1.grids()[1]) <= 1e-14
    assert rel_err(b[1] - g["init"][1], a[1] - g["init"][1]) <= 1e-12


def centered(mom):
    """The 29 moments with <c_i c_j> replaced by the centered correlation
    <c_i c_j> - <c_i><c_j> (BunchTwissAnalysis::getCorrelation)."""
    out = np.array(mom, dtype=np.float64)
    k = 8
    for i in range(6):
        for j in range(i + 1):
            out[k] = mom[k] - mom[2 + i] * mom[2 + j]
            k += 1
    return out


def twiss_getters(t):
    """The 27 getters in the order the golden fixture stores them."""
    g = []
    for ic in range(3):
        g += [t.getEmittance(ic), t.getEmittanceNormalized(ic), t.getAlpha(ic), t.getBeta(ic), t.getGamma(ic)]
    for ic in range(2):
        g += [t.getDispersion(ic), t.getDispersionDerivative(ic), t.getEffectiveEmittance(ic),
              t.getEffectiveAlpha(ic), t.getEffectiveBeta(ic), t.getEffectiveGamma(ic)]
    return np.array(g)


def test_diag_oracle_and_host_getters():
    """BunchTwissAnalysis moments (oracle) and the product's host getters
    over them, and the BunchTuneAnalysis phases, tunes and actions after each
    map, bit for bit against the reference."""
    from bunch import Bunch, BunchTwissAnalysis
    g = load_golden("diag_twiss_tune")
    mom = O.twiss_moments(g["init"])
    assert np.array_equal(centered(mom), g["moments"])
    b = Bunch()
    b.getSyncParticle().kinEnergy(float(g["ek"]))
    t = BunchTwissAnalysis()
    t._load(mom, b.getSyncParticle())
    assert np.array_equal(twiss_getters(t), g["getters"])
    assert t.getGlobalCount() == g["init"].shape[1]
    # tune analysis over the reference's coordinates after each map
    s = b.getSyncParticle()
    n = g["init"].shape[1]
    ph = np.zeros((6, n))
    O.tune_analysis(g["init"], s.beta(), s.kinEnergy() + s.mass(), g["twiss"], ph)
    assert np.array_equal(ph, g["phase_0"])
    k = 1
    while "coords_%d" % k in g:
        O.tune_analysis(g["coords_%d" % k], s.beta(), s.kinEnergy() + s.mass(), g["twiss"], ph)
        assert np.array_equal(ph, g["phase_%d" % k]), k
        k += 1
    assert k == 4


def test_diag_oracle_macrosize_weights():
    """With a macrosize attribute the moments are weighted sums."""
    g = load_golden("diag_twiss_tune")
    soa = g["init"]
    w = np.linspace(0.5, 1.5, soa.shape[1])
    mom = O.twiss_moments(soa, w)
    assert mom[1] == pytest.approx(w.sum(), rel=1e-14)
    # the centroids are small against the coordinates: scale by <|c_i|>
    scale = (np.abs(soa) * w).sum(axis=1) / w.sum()
    assert np.all(np.abs(mom[2:8] - (soa * w).sum(axis=1) / w.sum()) <= 1e-13 * scale)


def _moments_uniform_restated(soa, order, D, ekm, b2, xa, ya, xb, yb):
    """The uniform-macrosize branch of BunchTwissAnalysis::computeBunchMoments
    (BunchTwissAnalysis.cc:264-336) restated in numpy: the normalised term
    for j < order, i <= order - j; the raw product momX[i] momY[j] that the
    reference adds once per particle after its loops (i = 2, j = order: its
    braces close the loops before that statement), left unnormalised."""
    disp = D * soa[5] / ekm / b2 if D != 0.0 else 0.0
    dx, dy = (soa[0] - disp) - xa, soa[2] - ya
    w = order + 1
    out = np.zeros((w, w))
    mx, my = [np.ones_like(dx)], [np.ones_like(dy)]
    for _ in range(order):
        mx.append(mx[-1] * dx)
        my.append(my[-1] * dy)
    for j in range(order):
        for i in range(order + 1 - j):
            out[i, j] = np.sum(mx[i] / xb ** i * my[j] / yb ** j)
    out[2, order] += np.sum(mx[2] * my[order])
    n = soa.shape[1]
    for i in range(w):
        for j in range(w - i):
            out[i, j] /= n
    out[0, 0], out[1, 0], out[0, 1] = 1.0, xa, ya
    return out


def test_bunch_moments_restatement_against_golden():
    """The restated computeBunchMoments (its stray cell included) against
    the compiled reference's tables, cell by cell to 1e-9 (zeros exactly):
    the semantics the device kernel reproduces."""
    from bunch import Bunch, BunchTwissAnalysis
    g = load_golden("diag_moments")
    soa = g["init"]
    b = Bunch()
    b.getSyncParticle().kinEnergy(float(g["ek"]))
    t = BunchTwissAnalysis()
    t._load(O.twiss_moments(soa), b.getSyncParticle())
    s = b.getSyncParticle()
    for order in (2, 3, 4):
        for disp in (0, 1):
            for norm in (0, 1):
                D = t.getDispersion(0) if disp else 0.0
                xb = np.sqrt(t.getBeta(0) * t.getEmittance(0)) if norm else np.sqrt(t.getBeta(0))
                yb = np.sqrt(t.getBeta(1) * t.getEmittance(1)) if norm else np.sqrt(t.getBeta(1))
                got = _moments_uniform_restated(soa, order, D, s.kinEnergy() + s.mass(), s.beta() ** 2,
                                                t.getAverage(0), t.getAverage(2), xb, yb)
                ref = g["m_%d_%d_%d" % (order, disp, norm)]
                zero = ref == 0.0
                assert np.array_equal(got[zero], ref[zero])
                rel = np.abs(got[~zero] - ref[~zero]) / np.abs(ref[~zero])
                assert rel.max() <= 1e-9, (order, disp, norm, rel.max())
