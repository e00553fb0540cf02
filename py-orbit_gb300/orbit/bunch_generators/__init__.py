"""Seeded, vectorised restatement of the reference's transverse distribution
generators (py/orbit/bunch_generators/distribution_generators.py:12-330).

Each generator keeps the reference's constructor (Twiss containers holding
rms emittances) and per-particle ``getCoordinates()``, and adds
``generate(n, rng)`` which draws n particles at once from a
``numpy.random.Generator`` (the synthetic inputs of the tests and benchmarks).
"""
from __future__ import annotations

import math

import numpy as np

_default_rng = np.random.Generator(np.random.PCG64(12345))


class TwissContainer:
    """alpha, beta, emittance; u = sqrt(beta eps) u_n,
    u' = sqrt(eps/beta) (u'_n - alpha u_n) (distribution_generators.py:12-71)."""

    def __init__(self, alpha, beta, emittance):
        self.alpha, self.beta, self.emittance = float(alpha), float(beta), float(emittance)
        self._init()

    def _init(self):
        self.gamma = (1.0 + self.alpha ** 2) / self.beta
        self.u_max = math.sqrt(self.beta * self.emittance)
        self.up_coeff = math.sqrt(self.emittance / self.beta)
        self.up_max = math.sqrt(self.gamma * self.emittance)

    def setEmittance(self, e):
        self.emittance = float(e)
        self._init()

    def getNormalizedH(self, u, up):
        return (u ** 2 + (self.alpha * u + self.beta * up) ** 2) / (self.beta * self.emittance)

    def getU_Max(self):
        return self.u_max

    def getUP_Max(self):
        return self.up_max

    def getU_UP(self, u_norm, up_norm):
        return self.u_max * u_norm, self.up_coeff * (up_norm - self.alpha * u_norm)

    def getAlphaBetaGammaEmitt(self):
        return self.alpha, self.beta, self.gamma, self.emittance

    def getAlphaBetaEmitt(self):
        return self.alpha, self.beta, self.emittance


class _Dist:
    def getCoordinates(self):
        c = self.generate(1, _default_rng)
        return tuple(float(v[0]) for v in c)


class KVDist1D(_Dist):
    """1D KV; 100% emittance = 2 x rms (distribution_generators.py:74-96)."""

    def __init__(self, twiss=None):
        twiss = twiss or TwissContainer(0.0, 1.0, 1.0)
        a, b, e = twiss.getAlphaBetaEmitt()
        self.twiss = TwissContainer(a, b, 2 * e)

    def generate(self, n, rng):
        xn = np.sin(2 * math.pi * (rng.random(n) - 0.5))
        sgn = np.where(rng.random(n) < 0.5, -1.0, 1.0)
        xpn = sgn * np.sqrt(1.0 - xn ** 2)
        return self.twiss.getU_UP(xn, xpn)

    def getTwissContainers(self):
        return (self.twiss,)


class WaterBagDist1D(_Dist):
    """1D waterbag; 100% emittance = 4 x rms (distribution_generators.py:99-120)."""

    def __init__(self, twiss=None):
        twiss = twiss or TwissContainer(0.0, 1.0, 1.0)
        a, b, e = twiss.getAlphaBetaEmitt()
        self.kv = KVDist1D(TwissContainer(a, b, 2 * e))

    def generate(self, n, rng):
        u, up = self.kv.generate(n, rng)
        g = np.sqrt(rng.random(n))
        return g * u, g * up

    def getTwissContainers(self):
        return self.kv.getTwissContainers()


class KVDist2D(_Dist):
    """4D KV; 100% emittance = 4 x rms (distribution_generators.py:123-149)."""

    def __init__(self, twissX=None, twissY=None):
        twissX = twissX or TwissContainer(0.0, 1.0, 1.0)
        twissY = twissY or TwissContainer(0.0, 1.0, 1.0)
        ax, bx, ex = twissX.getAlphaBetaEmitt()
        ay, by, ey = twissY.getAlphaBetaEmitt()
        self.twissX = TwissContainer(ax, bx, 4 * ex)
        self.twissY = TwissContainer(ay, by, 4 * ey)

    def generate(self, n, rng):
        phi = 2 * math.pi * (rng.random(n) - 0.5)
        rho = np.sqrt(rng.random(n))
        xn, yn = rho * np.cos(phi), rho * np.sin(phi)
        p0 = np.sqrt(np.fabs(1.0 - rho ** 2))
        phi = 2 * math.pi * (rng.random(n) - 0.5)
        xpn, ypn = p0 * np.cos(phi), p0 * np.sin(phi)
        x, xp = self.twissX.getU_UP(xn, xpn)
        y, yp = self.twissY.getU_UP(yn, ypn)
        return x, xp, y, yp

    def getTwissContainers(self):
        return self.twissX, self.twissY


class WaterBagDist2D(_Dist):
    """4D waterbag; 100% emittance = 6 x rms (distribution_generators.py:152-175)."""

    def __init__(self, twissX=None, twissY=None):
        twissX = twissX or TwissContainer(0.0, 1.0, 1.0)
        twissY = twissY or TwissContainer(0.0, 1.0, 1.0)
        ax, bx, ex = twissX.getAlphaBetaEmitt()
        ay, by, ey = twissY.getAlphaBetaEmitt()
        self.kv = KVDist2D(TwissContainer(ax, bx, 6.0 * ex / 4.0), TwissContainer(ay, by, 6.0 * ey / 4.0))

    def generate(self, n, rng):
        x, xp, y, yp = self.kv.generate(n, rng)
        g = np.sqrt(np.sqrt(rng.random(n)))
        return g * x, g * xp, g * y, g * yp

    def getTwissContainers(self):
        return self.kv.getTwissContainers()


class GaussDist1D(_Dist):
    """Gaussian with optional cut-off in units of sigma (distribution_generators.py:254-275)."""

    def __init__(self, twiss=None, cut_off=-1.0):
        self.twiss = twiss or TwissContainer(0.0, 1.0, 1.0)
        self.cut_off = float(cut_off)

    def generate(self, n, rng):
        xn = rng.standard_normal(n)
        xpn = rng.standard_normal(n)
        if self.cut_off > 0.0:
            bad = xn ** 2 + xpn ** 2 > self.cut_off ** 2
            while bad.any():
                k = int(bad.sum())
                xn[bad] = rng.standard_normal(k)
                xpn[bad] = rng.standard_normal(k)
                bad = xn ** 2 + xpn ** 2 > self.cut_off ** 2
        return self.twiss.getU_UP(xn, xpn)

    def getTwissContainers(self):
        return self.twiss


class GaussDist2D(_Dist):
    def __init__(self, twissX=None, twissY=None, cut_off=-1.0):
        self.gx = GaussDist1D(twissX, cut_off)
        self.gy = GaussDist1D(twissY, cut_off)

    def generate(self, n, rng):
        x, xp = self.gx.generate(n, rng)
        y, yp = self.gy.generate(n, rng)
        return x, xp, y, yp

    def getTwissContainers(self):
        return self.gx.twiss, self.gy.twiss


class GaussDist3D(_Dist):
    def __init__(self, twissX=None, twissY=None, twissZ=None, cut_off=-1.0):
        self.gx = GaussDist1D(twissX, cut_off)
        self.gy = GaussDist1D(twissY, cut_off)
        self.gz = GaussDist1D(twissZ, cut_off)

    def generate(self, n, rng):
        return self.gx.generate(n, rng) + self.gy.generate(n, rng) + self.gz.generate(n, rng)

    def getTwissContainers(self):
        return self.gx.twiss, self.gy.twiss, self.gz.twiss


def twiss_for_rms(sigma_u, sigma_up):
    """Upright Twiss (alpha = 0) whose rms sizes are sigma_u, sigma_up:
    beta = sigma_u / sigma_up, eps = sigma_u * sigma_up."""
    return TwissContainer(0.0, sigma_u / sigma_up, sigma_u * sigma_up)


__all__ = ["TwissContainer", "KVDist1D", "WaterBagDist1D", "KVDist2D", "WaterBagDist2D", "GaussDist1D",
           "GaussDist2D", "GaussDist3D", "twiss_for_rms"]
