"""GPU bunch diagnostics: BunchTwissAnalysis moments reduced on the device
and BunchTuneAnalysis with its per-particle attributes kept on the device,
against the reference's golden vectors and the oracle.

Tolerances.  The device sums the moments in a different order than the
reference (per-thread strided partials, warp shuffles, per-block partials,
then the blocks in a fixed order), so a moment differs from the reference's
by a few ulp of the sum of the absolute terms: the bound is 1e-13 of
<|c_i c_j|> (and of <|c_i|> for the centroids).  The getters divide
correlations that cancel; they are held to 1e-10 relative.  Phases use the
device atan2, within a few ulp of the host's: phases and actions 1e-13
relative, the tunes (differences of phases over 2 pi, modulo 1) 1e-12
absolute."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_COORD, coord_err, load_golden, parse_sequence
from test_oracle_golden import twiss_getters

pytestmark = pytest.mark.gpu

TOL_MOM = 1e-13
TOL_GETTER = 1e-10
TOL_PHASE = 1e-13
TOL_TUNE = 1e-12


def gpu_bunch(soa, macrosize, ek=1.0):
    from bunch import Bunch
    b = Bunch()
    b.getSyncParticle().kinEnergy(ek)
    b.macroSize(macrosize)
    b.setCoordinates(soa)
    return b


def moment_scales(soa, w=None):
    """<|c_i|> and <|c_i c_j|> (i >= j) in the order of the moments."""
    w = np.ones(soa.shape[1]) if w is None else w
    a = np.abs(soa)
    tot = w.sum()
    out = [(a[i] * w).sum() / tot for i in range(6)]
    for i in range(6):
        for j in range(i + 1):
            out.append((a[i] * a[j] * w).sum() / tot)
    return np.array(out)


def check_moments(got, ref, soa, w=None):
    assert got[0] == ref[0]
    assert abs(got[1] - ref[1]) <= 1e-14 * abs(ref[1])
    scale = moment_scales(soa, w)
    assert np.all(np.abs(got[2:] - ref[2:]) <= TOL_MOM * scale), np.abs(got[2:] - ref[2:]) / scale


def tune_dist(a, b):
    d = np.abs(a - b) % 1.0
    return np.minimum(d, 1.0 - d)


def check_phase(got, ref):
    for r in (0, 1, 4, 5):
        assert np.max(np.abs(got[r] - ref[r])) <= TOL_PHASE * np.max(np.abs(ref[r])), r
    for r in (2, 3):
        assert np.max(tune_dist(got[r], ref[r])) <= TOL_TUNE, r


def test_twiss_analysis_against_golden():
    from bunch import BunchTwissAnalysis
    g = load_golden("diag_twiss_tune")
    b = gpu_bunch(g["init"], float(g["macrosize"]), float(g["ek"]))
    b._device_bunch()
    t = BunchTwissAnalysis()
    t.analyzeBunch(b)
    assert b._host_ok  # nothing was downloaded to analyse
    mom = np.zeros(29)
    mom[0], mom[1] = t.getGlobalCount(), t.getGlobalMacrosize()
    mom[2:8] = [t.getAverage(i) for i in range(6)]
    k = 8
    for i in range(6):
        for j in range(i + 1):
            mom[k] = t.getCorrelation(i, j)
            k += 1
    ref = g["moments"]
    # compare centered correlations against the scale of the raw terms
    assert mom[0] == ref[0] and mom[1] == ref[1]
    scale = moment_scales(g["init"])
    assert np.all(np.abs(mom[2:] - ref[2:]) <= TOL_MOM * 4 * scale)
    got = twiss_getters(t)
    exp = g["getters"]
    assert np.all(np.abs(got - exp) <= TOL_GETTER * np.abs(exp))


def test_moments_on_device_after_tracking_match_oracle():
    """After device maps the moments come from the device copy without a
    download; they equal the oracle's sums over the downloaded coordinates."""
    from bunch import BunchTwissAnalysis
    from orbit.teapot_base import TPB
    from orbit_gb300 import workloads as W
    soa = W.c2_coords(1_000_003, seed=5)
    b = gpu_bunch(soa, 1e9)
    TPB.drift(b, 1.0)
    TPB.quad1(b, 0.5, 0.3)
    assert not b._host_ok
    t = BunchTwissAnalysis()
    t.analyzeBunch(b)
    assert not b._host_ok  # still only on the device
    got = b._dev.moments()
    c = b.getCoordinates()
    ref = O.twiss_moments(c)
    check_moments(got, ref, c)
    t_ref = BunchTwissAnalysis()
    t_ref._load(ref, b.getSyncParticle())
    exp = twiss_getters(t_ref)
    assert np.all(np.abs(twiss_getters(t) - exp) <= TOL_GETTER * np.abs(exp))


def test_moments_with_macrosize_attribute():
    from orbit_gb300 import workloads as W
    soa = W.c2_coords(200_000, seed=9)
    b = gpu_bunch(soa, 1e9)
    b.addPartAttr("macrosize")
    w = np.linspace(0.25, 2.0, soa.shape[1])
    b._part_attr["macrosize"][: soa.shape[1], 0] = w
    b._host_modified()
    got = b._device_bunch().moments()
    check_moments(got, O.twiss_moments(soa, w), soa, w)


def test_moments_empty_and_tiny_bunches():
    from bunch import Bunch
    b = Bunch()
    b.getSyncParticle().kinEnergy(1.0)
    assert np.array_equal(b._device_bunch().moments(), np.zeros(29))
    b.addParticle(1e-3, 2e-4, -3e-3, 0.0, 0.5, 1e-4)
    got = b._device_bunch().moments()
    ref = O.twiss_moments(b.getCoordinates())
    assert np.array_equal(got, ref)  # one particle: no summation order


def test_tune_analysis_against_golden():
    """Device tune analysis after each map, the attribute rows staying on the
    device between analyses and read back through the host attribute."""
    from bunch import BunchTuneAnalysis
    from orbit.teapot_base import TPB
    g = load_golden("diag_twiss_tune")
    b = gpu_bunch(g["init"], float(g["macrosize"]), float(g["ek"]))
    tune = BunchTuneAnalysis()
    tune.assignTwiss(*g["twiss"])
    tune.analyzeBunch(b)
    assert b.hasPartAttr("ParticlePhaseAttributes") and b.getPartAttrSize("ParticlePhaseAttributes") == 6
    check_phase(b._dev.phase_get(), g["phase_0"])
    for k, step in enumerate(parse_sequence(g["sequence"]), start=1):
        getattr(TPB, step[0])(b, *step[1])
        tune.analyzeBunch(b)
        assert b._phase_dev
        check_phase(b._dev.phase_get(), g["phase_%d" % k])
    assert coord_err(b.getCoordinates(), g["coords_3"]) <= TOL_COORD
    # the host attribute holds the device rows once read
    n = b.getSize()
    host = np.array([[b.partAttrValue("ParticlePhaseAttributes", i, r) for i in range(n)] for r in range(6)])
    check_phase(host, g["phase_3"])
    assert not b._phase_dev


def test_tune_attribute_host_edits_reach_the_device():
    """A host edit of the phase attribute between analyses is uploaded before
    the next device analysis (the reference reads the attribute each call)."""
    from bunch import BunchTuneAnalysis
    g = load_golden("diag_twiss_tune")
    soa = g["init"]
    s_ek = float(g["ek"])
    b = gpu_bunch(soa, 1e9, s_ek)
    tune = BunchTuneAnalysis()
    tune.assignTwiss(*g["twiss"])
    tune.analyzeBunch(b)
    b.partAttrValue("ParticlePhaseAttributes", 0, 0, 1.0)  # xLastPhase of particle 0
    tune.analyzeBunch(b)
    got = b._dev.phase_get()
    s = b.getSyncParticle()
    ph = np.ascontiguousarray(g["phase_0"].copy())
    ph[0, 0] = 1.0
    O.tune_analysis(soa, s.beta(), s.kinEnergy() + s.mass(), g["twiss"], ph)
    check_phase(got, ph)


def test_tune_analysis_large_bunch_matches_oracle():
    from bunch import BunchTuneAnalysis
    from orbit.teapot_base import TPB
    from orbit_gb300 import workloads as W
    soa = W.c2_coords(500_000, seed=13)
    b = gpu_bunch(soa, 1e9)
    tw = [12.0, 0.8, 1.2, -0.05, 9.0, -0.6]
    tune = BunchTuneAnalysis()
    tune.assignTwiss(*tw)
    tune.analyzeBunch(b)
    TPB.drift(b, 0.7)
    tune.analyzeBunch(b)
    s = b.getSyncParticle()
    ph = np.zeros((6, soa.shape[1]))
    O.tune_analysis(soa, s.beta(), s.kinEnergy() + s.mass(), tw, ph)
    O.tune_analysis(b.getCoordinates(), s.beta(), s.kinEnergy() + s.mass(), tw, ph)
    check_phase(b._dev.phase_get(), ph)


def _moment_table_close(got, ref, tol=1e-9):
    """Cell by cell: zeros exactly, the others within tol relative (the
    table spans many orders of magnitude; sums differ in order only)."""
    got, ref = np.asarray(got), np.asarray(ref)
    zero = ref == 0.0
    assert np.array_equal(got[zero], ref[zero])
    nz = ~zero
    rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    return float(rel.max()) if rel.size else 0.0


def test_bunch_moments_against_golden():
    """BunchTwissAnalysis.computeBunchMoments / getBunchMoment against the
    compiled reference: orders 2-4, with and without the dispersion and the
    emittance-normalisation flags (the reference's stray cell [2][order]
    included)."""
    from bunch import BunchTwissAnalysis
    g = load_golden("diag_moments")
    b = gpu_bunch(g["init"], float(g["macrosize"]), float(g["ek"]))
    tw = BunchTwissAnalysis()
    for order in (2, 3, 4):
        for disp in (0, 1):
            for norm in (0, 1):
                tw.computeBunchMoments(b, order, disp, norm)
                got = np.array([[tw.getBunchMoment(i, j) for j in range(order + 1)] for i in range(order + 1)])
                err = _moment_table_close(got, g["m_%d_%d_%d" % (order, disp, norm)])
                assert err <= 1e-9, (order, disp, norm, err)
    assert tw.getBunchMoment(5, 0) == 0.0 and tw.getBunchMoment(-1, 0) == 0.0


def _moments_msize_restated(soa, m, order, D, ekm, b2, xa, ya, xb, yb):
    """The per-particle-macrosize branch of computeBunchMoments
    (BunchTwissAnalysis.cc:229-262, 325-336) restated in numpy."""
    disp = D * soa[5] / ekm / b2 if D != 0.0 else 0.0
    dx, dy = (soa[0] - disp) - xa, soa[2] - ya
    w = order + 1
    out = np.zeros((w, w))
    mx = [np.ones_like(dx)]
    my = [np.ones_like(dy)]
    for k in range(order):
        mx.append(mx[-1] * m * dx)
        my.append(my[-1] * m * dy)
    for j in range(order):
        for i in range(order + 1 - j):
            out[i, j] = np.sum(mx[i] / xb ** i * my[j] / yb ** j + mx[i] * my[j])
    tot = m.sum()
    for i in range(w):
        for j in range(w - i):
            out[i, j] /= tot
    out[0, 0], out[1, 0], out[0, 1] = 1.0, xa, ya
    return out


def test_bunch_moments_with_macrosize_attribute():
    from bunch import BunchTwissAnalysis
    g = load_golden("diag_moments")
    soa = g["init"]
    m = np.random.default_rng(5).uniform(0.5, 1.5, soa.shape[1])
    b = gpu_bunch(soa, 1e9)
    b.addPartAttr("macrosize")
    b._part_attr["macrosize"][: soa.shape[1], 0] = m
    b._host_modified()
    tw = BunchTwissAnalysis()
    for order, disp, norm in ((2, 0, 0), (3, 1, 1), (4, 0, 1)):
        tw.computeBunchMoments(b, order, disp, norm)
        got = np.array([[tw.getBunchMoment(i, j) for j in range(order + 1)] for i in range(order + 1)])
        D = tw.getDispersion(0) if disp else 0.0
        xb = np.sqrt(tw.getBeta(0) * tw.getEmittance(0)) if norm else np.sqrt(tw.getBeta(0))
        yb = np.sqrt(tw.getBeta(1) * tw.getEmittance(1)) if norm else np.sqrt(tw.getBeta(1))
        s = b.getSyncParticle()
        ref = _moments_msize_restated(soa, m, order, D, s.kinEnergy() + b.mass(), s.beta() ** 2,
                                      tw.getAverage(0), tw.getAverage(2), xb, yb)
        err = _moment_table_close(got, ref)
        assert err <= 1e-9, (order, disp, norm, err)
