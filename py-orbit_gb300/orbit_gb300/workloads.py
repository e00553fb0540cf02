"""Synthetic workloads of the benchmark configurations, built through the
reference-compatible API.  All inputs are seeded (numpy PCG64); the
reference publishes no datasets for this path.

C1  plain FP64, CPU-runnable: 1e5 protons at 1 GeV, macrosize 1e9,
    x, y ~ N(0, 5 mm), x', y' ~ N(0, 1 mrad), z ~ U(-100, 100) m, dE = 0;
    grid 64x64x1; lattice (0.5 m drift + SC kick) x 10.
C2  FODO tracking: 1e6 protons at 1 GeV, 4D waterbag with rms 4 mm /
    0.8 mrad, z ~ N(0, 10 m), dE ~ N(0, 1 MeV); grid 128x128x64; 40 FODO
    cells (quads k1 = +-0.5 m^-2, 0.5 m long; 2 m drifts; 4 SC nodes per
    cell).  The configuration names no intensity; 1e14 protons
    (macrosize 1e8 at 1e6 particles) is used.
C3  batched scan: 64 bunches, particle counts log-uniform in [5e4, 2e6],
    Gaussian 6D (rms 4 mm / 0.8 mrad transverse, z ~ N(0, 10 m),
    dE ~ N(0, 1 MeV)), intensities log-uniform in [1e12, 2e14] protons,
    FODO k1 uniform in [0.3, 0.7] m^-2 (the C2 lattice otherwise), grids
    drawn from 64x64x32, 128x128x64 and 256x256x64.
C5  large ring: 1.6e7 protons at 1 GeV, 4D KV with rms 6 mm / 1 mrad,
    parabolic line density over 250 m, dE ~ N(0, 1 MeV) (not named by the
    configuration); grid 256x256x128; 32 cells of 7.8 m (249.6 m) with FODO
    quads, sector bends of 2 pi/32 and sextupoles of k2 = +-2 m^-3, 300
    TEAPOT elements, 128 SC nodes.  The configuration names no intensity:
    1e14 protons is used.
"""
from __future__ import annotations

import numpy as np

from orbit.bunch_generators import WaterBagDist2D, twiss_for_rms

KIN_ENERGY = 1.0  # GeV


def c1_coords(n=100_000, seed=20240601):
    rng = np.random.Generator(np.random.PCG64(seed))
    soa = np.empty((6, n))
    soa[0] = rng.normal(0.0, 5e-3, n)
    soa[1] = rng.normal(0.0, 1e-3, n)
    soa[2] = rng.normal(0.0, 5e-3, n)
    soa[3] = rng.normal(0.0, 1e-3, n)
    soa[4] = rng.uniform(-100.0, 100.0, n)
    soa[5] = 0.0
    return soa


def c2_coords(n=1_000_000, seed=20240602):
    rng = np.random.Generator(np.random.PCG64(seed))
    tw = twiss_for_rms(4e-3, 0.8e-3)
    dist = WaterBagDist2D(tw, tw)
    x, xp, y, yp = dist.generate(n, rng)
    soa = np.empty((6, n))
    soa[0], soa[1], soa[2], soa[3] = x, xp, y, yp
    soa[4] = rng.normal(0.0, 10.0, n)
    soa[5] = rng.normal(0.0, 1e-3, n)
    return soa


C1_MACROSIZE = 1e9
C2_MACROSIZE = 1e8

C3_GRIDS = ((64, 64, 32), (128, 128, 64), (256, 256, 64))


def c3_scan(members=64, seed=20240603):
    """[(particles, grid, k1, intensity)] of the batched scan."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(members):
        n = int(round(np.exp(rng.uniform(np.log(5e4), np.log(2e6)))))
        grid = C3_GRIDS[int(rng.integers(0, len(C3_GRIDS)))]
        k1 = float(rng.uniform(0.3, 0.7))
        intensity = float(np.exp(rng.uniform(np.log(1e12), np.log(2e14))))
        out.append((n, grid, k1, intensity))
    return out


def c3_coords(n, seed):
    """Gaussian 6D bunch of the scan."""
    rng = np.random.Generator(np.random.PCG64(seed))
    soa = np.empty((6, n))
    soa[0] = rng.normal(0.0, 4e-3, n)
    soa[1] = rng.normal(0.0, 0.8e-3, n)
    soa[2] = rng.normal(0.0, 4e-3, n)
    soa[3] = rng.normal(0.0, 0.8e-3, n)
    soa[4] = rng.normal(0.0, 10.0, n)
    soa[5] = rng.normal(0.0, 1e-3, n)
    return soa


def make_bunch(soa, macrosize, kin_energy=KIN_ENERGY):
    from bunch import Bunch
    b = Bunch()
    b.getSyncParticle().kinEnergy(kin_energy)
    b.macroSize(macrosize)
    b.setCoordinates(soa)
    return b


def c1_lattice(calc, cells=10, drift=0.5):
    """(drift + SC kick) x cells as a TEAPOT lattice with 2.5D SC nodes."""
    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import DriftTEAPOT, TEAPOT_Lattice
    lat = TEAPOT_Lattice("c1")
    for i in range(cells):
        d = DriftTEAPOT("d%d" % i)
        d.setLength(drift)
        lat.addNode(d)
    lat.initialize()
    setSC2p5DAccNodes(lat, 0.4 * drift, calc)
    return lat


def fodo_lattice(calc, cells=40, kq=0.5, lq=0.5, ld=2.0, sc_min=0.3):
    """FODO cells QF-D-QD-D with quads of 2 parts (fringes on, the
    reference default) and 2.5D SC nodes every ~0.5 / 2 m (4 per cell)."""
    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import DriftTEAPOT, QuadTEAPOT, TEAPOT_Lattice
    lat = TEAPOT_Lattice("fodo")
    for c in range(cells):
        qf = QuadTEAPOT("qf%d" % c)
        qf.setLength(lq)
        qf.addParam("kq", kq)
        d1 = DriftTEAPOT("d1_%d" % c)
        d1.setLength(ld)
        qd = QuadTEAPOT("qd%d" % c)
        qd.setLength(lq)
        qd.addParam("kq", -kq)
        d2 = DriftTEAPOT("d2_%d" % c)
        d2.setLength(ld)
        for node in (qf, d1, qd, d2):
            lat.addNode(node)
    lat.initialize()
    if calc is not None:
        setSC2p5DAccNodes(lat, sc_min, calc)
    return lat


C5_INTENSITY = 1e14


def c5_coords(n=16_000_000, seed=20240605):
    """4D KV beam (points on the surface of the 4D unit sphere, scaled to
    rms 6 mm / 1 mrad: semi-axes twice the rms), parabolic line density on
    [-125, 125] m (the median of three uniforms has the density
    3/4 (1 - u^2)), dE ~ N(0, 1 MeV)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    soa = np.empty((6, n))
    g = rng.normal(size=(4, n))
    g /= np.sqrt((g * g).sum(axis=0))
    soa[0], soa[1], soa[2], soa[3] = 12e-3 * g[0], 2e-3 * g[1], 12e-3 * g[2], 2e-3 * g[3]
    del g
    u = rng.uniform(-1.0, 1.0, (3, n))
    soa[4] = 125.0 * np.median(u, axis=0)
    del u
    soa[5] = rng.normal(0.0, 1e-3, n)
    return soa


def ring_lattice(calc, cells=32, kq=0.5, k2=2.0, sc_min=1.4):
    """cells x [QF, D, SF, D, B, D, QD, D, SD] (7.8 m), the first drift of
    the first 12 cells in two halves: 300 TEAPOT elements for 32 cells;
    sector bends of 2 pi/32, sextupoles of k2 = +-k2 (MultipoleTEAPOT, pole
    2, kl = k2 * 0.2 m), 2.5D SC nodes placed by the reference rule with
    sc_min = 1.4 m (129 nodes for 32 cells)."""
    import math

    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import BendTEAPOT, DriftTEAPOT, MultipoleTEAPOT, QuadTEAPOT, TEAPOT_Lattice
    lat = TEAPOT_Lattice("ring")

    def drift(name, length):
        d = DriftTEAPOT(name)
        d.setLength(length)
        return d

    def quad(name, k):
        q = QuadTEAPOT(name)
        q.setLength(0.5)
        q.addParam("kq", k)
        return q

    def sext(name, k):
        m = MultipoleTEAPOT(name)
        m.setLength(0.2)
        m.addParam("poles", [2])
        m.addParam("kls", [k * 0.2])
        m.addParam("skews", [0])
        return m

    for c in range(cells):
        b = BendTEAPOT("b%d" % c)
        b.setLength(2.0)
        b.addParam("theta", 2.0 * math.pi / 32)
        first = [drift("d1a_%d" % c, 0.85), drift("d1b_%d" % c, 0.85)] if c < 12 else [drift("d1_%d" % c, 1.7)]
        for node in [quad("qf%d" % c, kq)] + first + [sext("sf%d" % c, k2), drift("d2_%d" % c, 0.5), b,
                                                      drift("d3_%d" % c, 0.5), quad("qd%d" % c, -kq),
                                                      drift("d4_%d" % c, 1.7), sext("sd%d" % c, -k2)]:
            lat.addNode(node)
    lat.initialize()
    if calc is not None:
        setSC2p5DAccNodes(lat, sc_min, calc)
    return lat
