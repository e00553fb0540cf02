"""Host arithmetic of the precision-form error report: Twiss functions and
tunes from a one-turn matrix, tune differences folded modulo 1."""
import math

import numpy as np

from orbit_gb300.form_report import plane_twiss, wrap_tune


def test_plane_twiss_of_a_rotation():
    beta, alpha, mu = 7.0, -0.8, 2 * math.pi * 0.23
    gamma = (1 + alpha * alpha) / beta
    m = np.array([[math.cos(mu) + alpha * math.sin(mu), beta * math.sin(mu)],
                  [-gamma * math.sin(mu), math.cos(mu) - alpha * math.sin(mu)]])
    b, a, q = plane_twiss(m)
    assert abs(b - beta) < 1e-12 and abs(a - alpha) < 1e-12 and abs(q - 0.23) < 1e-12


def test_wrap_tune():
    assert np.allclose(wrap_tune([0.98 - 0.01, 0.01 - 0.98, 0.2]), [-0.03, 0.03, 0.2])
