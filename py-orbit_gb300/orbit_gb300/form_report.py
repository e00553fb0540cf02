"""Accuracy of a reduced-precision space-charge form against the FP64 plain
form on the same bunch and lattice: the relative rms-emittance error and the
per-particle tune-shift error, both measured on the device with the
BunchTwissAnalysis and BunchTuneAnalysis diagnostics (no coordinate
download).

The tunes are the turn-by-turn phase advances of BunchTuneAnalysis
(src/orbit/BunchDiagnostics/BunchTuneAnalysis.cc:36-108) in the normalised
coordinates of the bare lattice's periodic Twiss functions, averaged over
the turns.  The bare lattice's Twiss functions come from its one-turn
matrix, taken by finite differences of the device maps."""
from __future__ import annotations

import math

import numpy as np


def wrap_tune(d):
    """Signed difference of fractional tunes folded into [-1/2, 1/2)."""
    return (np.asarray(d) + 0.5) % 1.0 - 0.5


def one_turn_matrix(lattice, kin_energy=1.0, eps=1e-7):
    """4x4 transverse one-turn matrix of a lattice without space charge:
    five particles (the reference orbit and one offset per coordinate)
    tracked through the device maps."""
    from .workloads import make_bunch
    soa = np.zeros((6, 5))
    for j in range(4):
        soa[j, j + 1] = eps
    b = make_bunch(soa, 1.0, kin_energy)
    lattice.trackBunch(b)
    c = b.getCoordinates()
    m = np.zeros((4, 4))
    for j in range(4):
        m[:, j] = (c[:4, j + 1] - c[:4, 0]) / eps
    return m


def plane_twiss(m2):
    """(beta, alpha, fractional tune) of a stable 2x2 one-turn block."""
    cos_mu = 0.5 * (m2[0, 0] + m2[1, 1])
    if abs(cos_mu) >= 1.0:
        raise ValueError("the lattice is not stable in this plane")
    sin_mu = math.copysign(math.sqrt(1.0 - cos_mu * cos_mu), m2[0, 1])
    beta = m2[0, 1] / sin_mu
    alpha = (m2[0, 0] - m2[1, 1]) / (2.0 * sin_mu)
    mu = math.atan2(sin_mu, cos_mu) % (2.0 * math.pi)
    return beta, alpha, mu / (2.0 * math.pi)


def _track_with_diagnostics(soa, macrosize, lattice, twiss, q0, turns, skip):
    """Per-particle tune shifts from q0 averaged over the turns after
    ``skip`` (each turn's phase advance folded around q0 first, so a tune
    near an integer averages correctly), and the final rms emittances."""
    from bunch import BunchTuneAnalysis, BunchTwissAnalysis
    from .workloads import make_bunch
    b = make_bunch(soa, macrosize)
    tune = BunchTuneAnalysis()
    tune.assignTwiss(*twiss)
    tune.analyzeBunch(b)
    acc = np.zeros((2, soa.shape[1]))
    q0 = np.asarray(q0, dtype=np.float64).reshape(2, 1)
    for t in range(turns):
        lattice.trackBunch(b)
        tune.analyzeBunch(b)
        if t >= skip:
            acc += wrap_tune(b._dev.phase_get()[2:4] - q0)
    tw = BunchTwissAnalysis()
    tw.analyzeBunch(b)
    return acc / (turns - skip), np.array([tw.getEmittance(0), tw.getEmittance(1)])


def form_error(soa, macrosize, make_lattice, form, turns=100, skip=None):
    """Tracks the same bunch with the plain and the given form for ``turns``
    turns of ``make_lattice(calc_form)`` and returns the error report.
    ``make_lattice(None)`` must give the lattice without space charge."""
    skip = turns // 5 if skip is None else skip
    m = one_turn_matrix(make_lattice(None))
    bx, ax, qx0 = plane_twiss(m[:2, :2])
    by, ay, qy0 = plane_twiss(m[2:, 2:])
    twiss = (bx, ax, 0.0, 0.0, by, ay)  # no bends: no dispersion
    q0 = (qx0, qy0)
    shift64, e64 = _track_with_diagnostics(soa, macrosize, make_lattice("plain"), twiss, q0, turns, skip)
    shift, e = _track_with_diagnostics(soa, macrosize, make_lattice(form), twiss, q0, turns, skip)
    err = np.abs(shift - shift64)
    return {
        "turns": turns, "tunes_averaged_over": turns - skip,
        "bare_tune": [qx0, qy0],
        "emittance_fp64": e64.tolist(), "emittance": e.tolist(),
        "emittance_rel_err": (np.abs(e / e64 - 1.0)).tolist(),
        "tune_shift_fp64_mean": shift64.mean(axis=1).tolist(),
        "tune_shift_fp64_min": shift64.min(axis=1).tolist(),
        "tune_shift_mean": shift.mean(axis=1).tolist(),
        # error of the beam's tune shift and tune spread (distribution level)
        "tune_shift_mean_err": np.abs(shift.mean(axis=1) - shift64.mean(axis=1)).tolist(),
        "tune_spread_err": np.abs(shift.std(axis=1) - shift64.std(axis=1)).tolist(),
        # particle by particle; in a strongly space-charge-dominated beam the
        # trajectories of the two forms separate, so this measures that
        # separation as well as the field error
        "tune_err_rms": np.sqrt((err ** 2).mean(axis=1)).tolist(),
        "tune_err_median": np.median(err, axis=1).tolist(),
    }
