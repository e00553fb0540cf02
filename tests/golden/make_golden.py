"""Generates the golden vectors in tests/golden/*.npz by running the
REFERENCE's own C++ (compiled from the reference tree by oracle/build_ref.sh,
FFT = project shim because FFTW is unavailable) on seeded inputs.

Run here, where the reference tree exists:
    python tests/golden/make_golden.py
The fixtures are committed; nothing reads the reference tree at test time.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402


def gaussian(n, seed, sx=5e-3, sxp=1e-3, sy=4e-3, syp=1e-3, sz=10.0, sde=1e-3):
    rng = np.random.Generator(np.random.PCG64(seed))
    soa = np.empty((6, n))
    soa[0] = rng.normal(0, sx, n)
    soa[1] = rng.normal(0, sxp, n)
    soa[2] = rng.normal(0, sy, n)
    soa[3] = rng.normal(0, syp, n)
    soa[4] = rng.normal(0, sz, n)
    soa[5] = rng.normal(0, sde, n)
    return soa


MAPS = [
    ("drift", (0.7,)), ("drift", (-0.3,)), ("quad1", (0.25, 0.5)), ("quad1", (0.25, -0.5)), ("quad1", (0.3, 0.0)),
    ("quad2", (0.25,)), ("quadfringeIN", (0.5,)), ("quadfringeOUT", (-0.5,)), ("bend1", (0.5, 0.1)),
    ("bend2", (0.5,)), ("bend3", (0.05,)), ("bend4", (0.05,)), ("bendfringeIN", (5.0,)),
    ("bendfringeOUT", (5.0,)), ("multp", (2, 0.3, 0)), ("multp", (1, -0.2, 1)), ("multp", (3, 5.0, 0)),
    ("multpfringeIN", (2, 0.4, 0)), ("multpfringeOUT", (2, 0.4, 1)), ("multpfringeIN", (1, 0.3, 0)),
    ("rotatexy", (0.1,)), ("wrapbunch", (20.0,)), ("kick", (1e-4, -2e-4, 1e-5)),
    ("wedgerotate", (0.05, 0)), ("wedgerotate", (0.05, 1)), ("wedgedrift", (0.3, 0)), ("wedgedrift", (0.3, 1)),
    ("wedgebend", (0.3, 0, 10.0, 4)), ("wedgebend", (0.3, 1, 10.0, 5)),
]


def sc_case(name, soa, nx, ny, nz, xy_ratio, seq, ek=1.0, msize=1e9):
    """seq: list of ("sc", L) or (map, args) applied in order; records the
    grids after each SC kick and the coordinates at the end."""
    b = O.RefBunch(soa, ek, msize)
    sc = O.RefSC(nx, ny, nz, xy_ratio)
    out = {"init": soa, "nx": nx, "ny": ny, "nz": nz, "xy_ratio": xy_ratio, "ek": ek, "macrosize": msize}
    k = 0
    seq_txt = []
    for step in seq:
        if step[0] == "sc":
            sc.track(b, step[1])
            rho, phi, zg, lim = sc.grids()
            c = b.coords()
            ex, ey, lam = sc.fields(c[0], c[2], c[4])
            out["rho_%d" % k] = rho
            out["phi_%d" % k] = phi
            out["zg_%d" % k] = zg
            out["lim_%d" % k] = lim
            if k == 0:
                out["ex_0"] = ex
                out["ey_0"] = ey
                out["lam_0"] = lam
                out["coords_0"] = c
            k += 1
            seq_txt.append("sc:%r" % (step[1],))
        else:
            b.tpb(step[0], *step[1])
            seq_txt.append("%s:%r" % (step[0], tuple(step[1])))
    out["final"] = b.coords()
    out["nkicks"] = k
    out["sequence"] = np.array(seq_txt)
    out["kin"] = np.array([b.kinematics()[q] for q in ("beta", "gamma", "momentum", "kin_energy", "mass",
                                                      "classical_radius", "time")])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "kicks", k)


def scrb_case(name, soa, nx, ny, nz, xy_ratio, navg, pipe_radius, seq, ek=1.0, msize=1e9):
    """SpaceChargeCalc2p5Drb: seq of ("sc", L) or maps; records the grids, the
    derivative grid and the coordinates after each kick."""
    b = O.RefBunch(soa, ek, msize)
    sc = O.RefSCrb(nx, ny, nz, xy_ratio)
    sc.setLongAveragingPointsN(navg)
    out = {"init": soa, "nx": nx, "ny": ny, "nz": nz, "xy_ratio": xy_ratio, "ek": ek, "macrosize": msize,
           "navg": navg, "pipe_radius": pipe_radius}
    k = 0
    seq_txt = []
    for step in seq:
        if step[0] == "sc":
            sc.track(b, step[1], pipe_radius)
            rho, phi, zg, zd, lim = sc.grids()
            out["rho_%d" % k] = rho
            out["phi_%d" % k] = phi
            out["zg_%d" % k] = zg
            out["zd_%d" % k] = zd
            out["lim_%d" % k] = lim
            out["coords_%d" % k] = b.coords()
            k += 1
            seq_txt.append("sc:%r" % (step[1],))
        else:
            b.tpb(step[0], *step[1])
            seq_txt.append("%s:%r" % (step[0], tuple(step[1])))
    out["final"] = b.coords()
    out["nkicks"] = k
    out["sequence"] = np.array(seq_txt)
    out["kin"] = np.array([b.kinematics()[q] for q in ("beta", "gamma", "momentum", "kin_energy", "mass",
                                                      "classical_radius", "time")])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "kicks", k)


def bnd_case(name, soa, nx, ny, nz, bnd_args, seq, points=None, ek=1.0, msize=1e9):
    """SpaceChargeCalc2p5D with a conducting boundary: bnd_args = (nPoints,
    nModes[, shape, xDim, yDim]); points: explicit boundary points for the
    base class.  Records the boundary points, the grids and the coordinates
    after each kick."""
    b = O.RefBunch(soa, ek, msize)
    sc = O.RefSC(nx, ny, nz, -1.0)
    bnd = O.RefBoundary(*bnd_args)
    if points is not None:
        for i, (x, y) in enumerate(points):
            bnd.setBoundaryPoint(i, x, y)
        bnd.initialize()
    head, bx, by = bnd.data()
    out = {"init": soa, "nx": nx, "ny": ny, "nz": nz, "ek": ek, "macrosize": msize,
           "bnd_np": int(bnd_args[0]), "bnd_nm": int(bnd_args[1]),
           "bnd_shape": "" if len(bnd_args) < 3 else bnd_args[2],
           "bnd_xdim": 0.0 if len(bnd_args) < 4 else float(bnd_args[3]),
           "bnd_ydim": (0.0 if len(bnd_args) < 4 else float(bnd_args[3])) if len(bnd_args) < 5 else float(bnd_args[4]),
           "bnd_head": head, "bnd_x": bx, "bnd_y": by}
    probe = np.linspace(-0.03, 0.03, 41)
    out["inside"] = np.array([[bnd.isInside(x, y) for y in probe] for x in probe])
    k = 0
    seq_txt = []
    for step in seq:
        if step[0] == "sc":
            O.ref_sc_track_bnd(sc, b, step[1], bnd)
            rho, phi, zg, lim = sc.grids()
            out["rho_%d" % k] = rho
            out["phi_%d" % k] = phi
            out["zg_%d" % k] = zg
            out["lim_%d" % k] = lim
            out["coords_%d" % k] = b.coords()
            k += 1
            seq_txt.append("sc:%r" % (step[1],))
        else:
            b.tpb(step[0], *step[1])
            seq_txt.append("%s:%r" % (step[0], tuple(step[1])))
    out["final"] = b.coords()
    out["nkicks"] = k
    out["sequence"] = np.array(seq_txt)
    out["kin"] = np.array([b.kinematics()[q] for q in ("beta", "gamma", "momentum", "kin_energy", "mass",
                                                      "classical_radius", "time")])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "kicks", k)


def diag_case(name, soa, twiss, steps, ek=1.0, msize=1e9):
    """BunchTwissAnalysis moments and getters, and BunchTuneAnalysis
    attributes after each analysis; steps: maps applied between analyses."""
    b = O.RefBunch(soa, ek, msize)
    out = {"init": soa, "ek": ek, "macrosize": msize, "twiss": np.array(twiss)}
    mom, g = O.ref_twiss(b)
    out["moments"] = mom
    out["getters"] = g
    tune = O.RefTune(twiss)
    out["phase_0"] = tune.analyze(b)
    seq_txt = []
    for k, step in enumerate(steps):
        b.tpb(step[0], *step[1])
        seq_txt.append("%s:%r" % (step[0], tuple(step[1])))
        out["coords_%d" % (k + 1)] = b.coords()
        out["phase_%d" % (k + 1)] = tune.analyze(b)
    out["sequence"] = np.array(seq_txt)
    out["kin"] = np.array([b.kinematics()[q] for q in ("beta", "gamma", "momentum", "kin_energy", "mass",
                                                      "classical_radius", "time")])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name)


def bunch_io_case():
    """Bunch::print of a bunch with particle attributes (macrosize, the
    particle id and a 3-wide "Amplitudes" set, whose size goes into its
    PARTICLE_ATTRIBUTES_CONTROLLER_DICT line), bunch attributes and a sync
    particle time: the reference's own text file, plus its coordinates and
    attributes as the reference holds them."""
    soa = gaussian(40, 151)
    b = O.RefBunch(soa, 1.3, 2.5e9)
    b.add_attr("macrosize")
    b.add_attr("ParticleIdNumber")
    b.add_attr("Amplitudes", 3)
    for i in range(soa.shape[1]):
        b.attr("macrosize", i, 0, 1e9 * (1.0 + 0.01 * i))
        b.attr("ParticleIdNumber", i, 0, 1000 + i)
        for j in range(3):
            b.attr("Amplitudes", i, j, 0.1 * j - 0.003 * i)
    b.bunch_attr_int("TurnNumber", 7)
    b.bunch_attr_double("beam_current", 0.0123456789)
    b.set_time(1.234567890123e-6)
    path = os.path.join(HERE, "bunch_dump_ref.txt")
    b.dump(path)
    # the reference reading its own file into a new bunch and writing it
    # again (the mass comes back at the 6 digits the file holds, which moves
    # the kinematics lines)
    r = O.RefBunch(np.zeros((6, 0)), 1.0, 1.0)
    r.read(path)
    r.dump(os.path.join(HERE, "bunch_dump_ref_reread.txt"))
    print("wrote bunch_dump_ref.txt, bunch_dump_ref_reread.txt")


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "bunch_io":
        bunch_io_case()
        return
    if not O.ref_available():
        if not O.build_reference():
            raise SystemExit("the compiled reference is not available")
    # 1) every TEAPOT map in sequence, 256 particles
    soa = gaussian(256, 11)
    b = O.RefBunch(soa, 1.0, 1e9)
    out = {"init": soa}
    for k, (name, args) in enumerate(MAPS):
        b.tpb(name, *args)
        out["after_%02d" % k] = b.coords()
    out["kin"] = np.array([b.kinematics()[q] for q in ("beta", "gamma", "momentum", "kin_energy", "mass",
                                                      "classical_radius", "time")])
    out["names"] = np.array([m[0] for m in MAPS])
    out["args"] = np.array([repr(tuple(m[1])) for m in MAPS])
    np.savez_compressed(os.path.join(HERE, "maps.npz"), **out)
    print("wrote maps")
    # 2) one kick, round beam, 32x32x8
    sc_case("sc_round_32x32x8", gaussian(4096, 21, sy=5e-3), 32, 32, 8, -1.0, [("sc", 0.5)])
    # 3) C1-like: nz = 1, 64x64x1, drift + kick x 5
    rng = np.random.Generator(np.random.PCG64(31))
    c1 = gaussian(3000, 31, sy=5e-3, sde=0.0)
    c1[4] = rng.uniform(-100, 100, 3000)
    c1[5] = 0.0
    sc_case("c1_64x64x1", c1, 64, 64, 1, -1.0, [("drift", (0.5,)), ("sc", 0.5)] * 5)
    # 4) flat beam (aspect ratio far from 1: the Green function is rebuilt),
    #    odd sizes (40 x 24 -> doubled 80 x 48), per-kick maps between
    flat = gaussian(3000, 41, sx=8e-3, sy=2e-3)
    sc_case("flat_40x24x16", flat, 40, 24, 16, -1.0,
            [("sc", 0.4), ("quad1", (0.25, 0.5)), ("sc", 0.4), ("drift", (1.0,)), ("sc", 0.4)])
    # 5) explicit xy_ratio and nz = 2
    sc_case("ratio2_16x16x2", gaussian(2048, 51, sx=6e-3, sy=3e-3), 16, 16, 2, 2.0,
            [("sc", 1.0), ("drift", (0.5,)), ("sc", 1.0)])
    # 6) SpaceChargeCalc2p5Drb: longitudinal kick, default 3-point smoothing,
    #    a 5-point case with an explicit ratio, nz = 2 and nz = 1
    scrb_case("rb_32x32x16", gaussian(3000, 61), 32, 32, 16, -1.0, 3, 0.05,
              [("sc", 0.5), ("drift", (0.5,)), ("sc", 0.5)])
    scrb_case("rb_40x24x8_avg5", gaussian(3000, 71, sx=6e-3, sy=3e-3), 40, 24, 8, 1.5, 5, 0.03,
              [("sc", 0.4), ("quad1", (0.25, 0.5)), ("sc", 0.4)])
    scrb_case("rb_16x16x2", gaussian(2048, 81), 16, 16, 2, -1.0, 3, 0.1, [("sc", 1.0), ("sc", 1.0)])
    scrb_case("rb_16x16x1", gaussian(2048, 91), 16, 16, 1, -1.0, 3, 0.1, [("sc", 1.0)])
    # 7) conducting boundaries: circle, ellipse, rectangle and explicit points
    #    (some particles outside the boundary are not kicked)
    bnd_case("bnd_circle_64x64x16", gaussian(3000, 101, sx=6e-3, sy=6e-3), 64, 64, 16, (128, 10, "Circle", 0.04),
             [("sc", 0.5), ("drift", (0.5,)), ("sc", 0.5)])
    bnd_case("bnd_ellipse_48x40x8", gaussian(3000, 111, sx=8e-3, sy=4e-3), 48, 40, 8,
             (120, 8, "Ellipse", 0.05, 0.03), [("sc", 0.5), ("sc", 0.5)])
    bnd_case("bnd_rect_32x32x4", gaussian(2048, 121, sx=6e-3, sy=5e-3), 32, 32, 4,
             (128, 12, "Rectangle", 0.05, 0.04), [("sc", 1.0)])
    t = 2 * np.pi * np.arange(64) / 64
    bnd_case("bnd_points_40x40x8", gaussian(2048, 131), 40, 40, 8, (64, 6), [("sc", 0.5)],
             points=list(zip(0.03 * np.cos(t) + 0.002, 0.02 * np.sin(t))))
    # 8) bunch diagnostics: a correlated bunch with offsets and dispersion
    d = gaussian(3000, 141)
    d[0] += 1e-3
    d[1] += 0.1 * d[0]
    d[0] += 2.0 * d[5]
    diag_case("diag_twiss_tune", d, [10.0, -1.2, 0.5, 0.1, 8.0, 0.7],
              [("quad1", (0.5, 0.5)), ("drift", (1.0,)), ("quad1", (0.5, -0.5))])
    # 9) BunchTwissAnalysis::computeBunchMoments / getBunchMoment on the same
    # bunch (orders 2-4, with and without the dispersion and emittance flags)
    moments_case("diag_moments", d)
    # 10) the bunch text file (Bunch::print) with attributes
    bunch_io_case()


def moments_case(name, soa, ek=1.0, msize=1e9):
    b = O.RefBunch(soa, ek, msize)
    out = {"init": soa, "ek": ek, "macrosize": msize}
    for order in (2, 3, 4):
        for disp in (0, 1):
            for norm in (0, 1):
                out["m_%d_%d_%d" % (order, disp, norm)] = O.ref_bunch_moments(b, order, disp, norm)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name)


if __name__ == "__main__":
    main()
