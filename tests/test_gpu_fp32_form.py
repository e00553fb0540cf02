"""The FP32 field form (the plain form's exact fixed-point deposit; FFT and
gradient in FP32; coordinates, maps and kick accumulation in FP64) against
the FP64 oracle and the plain form.

Tolerances: density within 1e-12 (the deposit is the plain form's),
potential within 1e-5 and kicks within 2e-4 (max-norm relative) of the
FP64 oracle after one kick; rms emittances within 1% of the plain form
after 200 kicks.  The kick bound is the FP32 noise floor: the grid
coordinate formed in float (the coordinate, 1/dx and the offset each
rounded to float, a few ulps at 64-128 cells, about 1e-5 of a cell, move
the 9-point weights) and the potential's FP32 error (about 1e-6 of its
maximum, amplified some 50 times by the gradient's differences over one
cell) each reach a few 1e-5 of the largest kick; measured 0.99-1.00e-4 on
this test's bunch."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_FIELD, rel_err

pytestmark = pytest.mark.gpu

TOL_PHI_FP32 = 1e-5
TOL_KICK_FP32 = 2e-4
TOL_EMITTANCE_FP32 = 1e-2


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


def test_fp32_single_kick_accuracy():
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(100_000, seed=5)
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(128, 128, 64, form="fp32")
    calc.trackBunch(b, 1.0)
    got = b.getCoordinates()
    sc = O.OracleSC(128, 128, 64)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 1.0, nthreads=8) == 0
    assert rel_err(got[1] - soa[1], a[1] - soa[1]) < TOL_KICK_FP32
    assert rel_err(got[3] - soa[3], a[3] - soa[3]) < TOL_KICK_FP32
    assert np.array_equal(got[0], soa[0]) and np.array_equal(got[2], soa[2]) and np.array_equal(got[4], soa[4])
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getPhiGrid().getArray(), phi) < TOL_PHI_FP32
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD


def test_fp32_fused_program_matches_eager():
    """The fused lattice program and node-by-node tracking of the FP32 form
    agree to FP32 accumulation-order noise."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(50_000, seed=3)
    out = []
    for fused in (True, False):
        b = gpu_bunch(soa, 1e9)
        calc = SpaceChargeCalc2p5D(64, 64, 16, form="fp32")
        lat = W.fodo_lattice(calc, cells=2)
        lat.setFusedTracking(fused)
        lat.trackBunch(b)
        out.append(b.getCoordinates())
    d = out[0] - soa
    e = out[1] - soa
    assert rel_err(d[1], e[1]) < TOL_KICK_FP32 and rel_err(d[3], e[3]) < TOL_KICK_FP32


def test_fp32_emittance_over_many_kicks():
    """FODO, 10 turns x 20 kicks: rms emittances of the FP32 form within 1%
    of the plain form (which is parity-tested against the oracle)."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(200_000, seed=9)
    out = {}
    for form in ("plain", "fp32"):
        b = gpu_bunch(soa, 2e9)
        calc = SpaceChargeCalc2p5D(64, 64, 32, form=form)
        lat = W.fodo_lattice(calc, cells=5)
        lat.trackBunchTurns(b, 10)
        out[form] = b.getCoordinates()
    e64 = O.rms_emittance(np.ascontiguousarray(out["plain"]))
    e32 = O.rms_emittance(np.ascontiguousarray(out["fp32"]))
    e0 = O.rms_emittance(np.ascontiguousarray(soa))
    growth = max(abs(e64[0] / e0[0] - 1), abs(e64[1] / e0[1] - 1))
    assert growth > 1e-4  # space charge acted
    for k in range(2):
        assert abs(e32[k] / e64[k] - 1) < TOL_EMITTANCE_FP32, (k, e32, e64)


def test_fp32_tune_shift_and_emittance_error_report():
    """The error report of the FP32 form at the FODO benchmark's intensity
    (1e14 protons): the beam's mean space-charge tune shift and its tune
    spread (device tune analysis over the turns) within 1% of the FP64
    form's mean shift, rms emittances within 1%."""
    from orbit_gb300 import workloads as W
    from orbit_gb300.form_report import form_error
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(100_000, seed=21)

    def make_lattice(form):
        return W.fodo_lattice(None if form is None else SpaceChargeCalc2p5D(64, 64, 32, form=form), cells=10)

    r = form_error(soa, 1e9, make_lattice, "fp32", turns=30)
    for k in range(2):
        assert 0.0 <= r["bare_tune"][k] < 1.0
        shift = abs(r["tune_shift_fp64_mean"][k])
        assert r["tune_shift_fp64_mean"][k] < -1e-4  # space charge depresses the tunes
        assert r["tune_shift_mean_err"][k] < 0.01 * shift, r
        assert r["tune_spread_err"][k] < 0.01 * shift, r
        assert r["emittance_rel_err"][k] < TOL_EMITTANCE_FP32, r


@pytest.mark.parametrize("offset", [0.03, 2.0])
def test_fp32_offset_beam(offset):
    """A beam displaced from the coordinate origin: by 0.03 m the grid origin
    stays within four grid extents and the kick's grid coordinates are formed
    in float from the converted coordinates; by 2 m (a hundred extents) the
    kick forms them with one FP64 FMA each.  Both within the single-kick
    tolerance of the oracle."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(100_000, seed=6)
    soa[0] += offset
    soa[2] -= 0.5 * offset
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(128, 128, 64, form="fp32")
    calc.trackBunch(b, 1.0)
    got = b.getCoordinates()
    sc = O.OracleSC(128, 128, 64)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 1.0, nthreads=8) == 0
    assert rel_err(got[1] - soa[1], a[1] - soa[1]) < TOL_KICK_FP32
    assert rel_err(got[3] - soa[3], a[3] - soa[3]) < TOL_KICK_FP32
