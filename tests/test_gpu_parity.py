"""GPU parity: the CUDA path (through the C ABI, via the reference-compatible
Python API) against the reference's golden vectors and the CPU oracle.

Tolerances (max-norm relative): potential, density and kicks 1e-12;
coordinates after up to 100 kicks 1e-10; grid limits bit-exact."""
import numpy as np
import pytest

import oracle as O
from helpers import (TOL_COORD, TOL_FIELD, coord_err, golden_maps, kick_delta_tol, kin_sync, load_golden,
                     parse_sequence, rel_err)

pytestmark = pytest.mark.gpu


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


def test_library_loads_native():
    import orbit_gb300
    assert "sm_103a" in orbit_gb300.version()


def test_maps_against_golden():
    from orbit.teapot_base import TPB
    g = load_golden("maps")
    b = gpu_bunch(g["init"], 1e9)
    for k, (name, args) in enumerate(golden_maps(g)):
        getattr(TPB, name)(b, *args)
        got = b.getCoordinates()
        err = coord_err(got, g["after_%02d" % k])
        assert err <= TOL_FIELD, (k, name, err)
    assert abs(b.getSyncParticle().time() - g["kin"][6]) <= 1e-15 * abs(g["kin"][6])


@pytest.mark.parametrize("case", ["sc_round_32x32x8", "c1_64x64x1", "flat_40x24x16", "ratio2_16x16x2"])
def test_sc_against_golden(case):
    from orbit.teapot_base import TPB
    from spacecharge import SpaceChargeCalc2p5D
    g = load_golden(case)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    b = gpu_bunch(g["init"], float(g["macrosize"]))
    calc = SpaceChargeCalc2p5D(nx, ny, nz, float(g["xy_ratio"]))
    k = 0
    for step in parse_sequence(g["sequence"]):
        if step[0] == "sc":
            calc.trackBunch(b, step[1])
            rho, phi = calc.getRhoGrid(), calc.getPhiGrid()
            zg = calc.getLongGrid()
            lim = g["lim_%d" % k]
            got_lim = [rho.getMinX(), rho.getMaxX(), rho.getMinY(), rho.getMaxY(), zg.getMinZ(), zg.getMaxZ(),
                       rho.getStepX(), rho.getStepY(), zg.getStepZ()]
            if k == 0:
                # on identical coordinates the grid limits are exact
                # (integer-key extrema, unfused scalar set-up)
                assert got_lim == list(lim)
            else:
                # later kicks see coordinates that differ at the rounding level
                assert np.allclose(got_lim, lim, rtol=1e-13, atol=0)
            assert rel_err(rho.getArray(), g["rho_%d" % k]) <= TOL_FIELD, ("rho", k)
            assert rel_err(phi.getArray(), g["phi_%d" % k]) <= TOL_FIELD, ("phi", k)
            assert rel_err(zg.getArray(), g["zg_%d" % k]) <= TOL_FIELD, ("lambda", k)
            if k == 0:
                c = b.getCoordinates()
                ex, ey, lam = calc.fields(c[0], c[2], c[4])
                assert rel_err(ex, g["ex_0"]) <= TOL_FIELD
                assert rel_err(ey, g["ey_0"]) <= TOL_FIELD
                assert rel_err(lam, g["lam_0"]) <= TOL_FIELD
                # the kick itself: xp, yp changes
                dk = g["coords_0"][1] - g["init"][1]
                assert rel_err(c[1] - g["init"][1], dk) <= kick_delta_tol(g["coords_0"][1], dk)
            k += 1
        else:
            getattr(TPB, step[0])(b, *step[1])
    assert coord_err(b.getCoordinates(), g["final"]) <= TOL_COORD


def run_oracle_program(prog, soa, sync, calcs_shape, turns=1, nthreads=8):
    calcs = [O.OracleSC(*s) for s in calcs_shape]
    a = np.ascontiguousarray(soa.copy())
    rc = O.run_program(prog, turns, a, sync, calcs, nthreads=nthreads)
    assert rc == 0
    return a, calcs


def test_c1_config_full_size():
    """C1: 1e5 particles, 64x64x1, (0.5 m drift + SC kick) x 10, fused on
    the GPU against the oracle."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c1_coords(100_000)
    b = gpu_bunch(soa, W.C1_MACROSIZE)
    calc = SpaceChargeCalc2p5D(64, 64, 1)
    lat = W.c1_lattice(calc)
    prog = lat.fusedProgram(b)
    assert prog is not None
    lat.trackBunch(b)
    got = b.getCoordinates()
    ref, ocalcs = run_oracle_program(prog.ops, soa, oracle_sync_of(b), [(64, 64, 1)])
    assert coord_err(got, ref) <= TOL_COORD
    rho, phi, zg, lim = ocalcs[0].grids()
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD


def test_hundred_kicks_fodo():
    """100 SC kicks through FODO cells (fringes on): coordinates within 1e-10."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(20_000, seed=7)
    b = gpu_bunch(soa, 5e9)
    calc = SpaceChargeCalc2p5D(32, 32, 16)
    lat = W.fodo_lattice(calc, cells=5)   # 20 kicks per turn
    prog = lat.fusedProgram(b)
    lat.trackBunchTurns(b, 5)             # 100 kicks
    got = b.getCoordinates()
    ref, _ = run_oracle_program(prog.ops, soa, oracle_sync_of(b), [(32, 32, 16)], turns=5)
    assert coord_err(got, ref) <= TOL_COORD
    # the kicks moved the beam: a sanity check that SC acted
    assert rel_err(got[1], soa[1]) > 1e-3


def test_ring_cells_fused_program():
    """Four cells of the large-ring lattice (sector bends with their four
    maps and fringes, sextupoles with multp and the multipole fringes,
    quads, drifts) fused on the GPU, two turns (32 kicks), against the
    oracle within 1e-10."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c5_coords(20_000, seed=11)
    b = gpu_bunch(soa, 5e9)
    calc = SpaceChargeCalc2p5D(32, 32, 16)
    lat = W.ring_lattice(calc, cells=4)
    prog = lat.fusedProgram(b)
    from orbit_gb300 import OP
    inv = {v: k for k, v in OP.items()}
    assert {"MPFRIN", "MPFROUT", "MULTP", "BEND3", "BEND4", "BFRIN", "BFROUT"} <= {inv[c] for c, _, _ in prog.ops}
    lat.trackBunchTurns(b, 2)
    got = b.getCoordinates()
    ref, _ = run_oracle_program(prog.ops, soa, oracle_sync_of(b), [(32, 32, 16)], turns=2)
    assert coord_err(got, ref) <= TOL_COORD
    assert rel_err(got[1], soa[1]) > 1e-3


def test_benchmark_grid_fused_program():
    """The benchmark's grid (128x128x64): shared-memory grids of 128 KiB, one
    block per SM, register-limited block sizes; fused program vs oracle."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(100_000, seed=21)
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(128, 128, 64)
    lat = W.fodo_lattice(calc, cells=2)
    prog = lat.fusedProgram(b)
    lat.trackBunchTurns(b, 2)
    got = b.getCoordinates()
    ref, ocalcs = run_oracle_program(prog.ops, soa, oracle_sync_of(b), [(128, 128, 64)], turns=2)
    assert coord_err(got, ref) <= TOL_COORD
    rho, phi, zg, lim = ocalcs[0].grids()
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    # the eager path on the same grid (stand-alone kernels with 1024-thread blocks)
    b2 = gpu_bunch(soa, 1e9)
    c2 = SpaceChargeCalc2p5D(128, 128, 64)
    c2.trackBunch(b2, 0.5)
    s2 = O.OracleSC(128, 128, 64)
    a = np.ascontiguousarray(soa.copy())
    assert s2.track(a, oracle_sync_of(b2), 0.5, nthreads=8) == 0
    assert rel_err(b2.getCoordinates()[1] - soa[1], a[1] - soa[1]) <= kick_delta_tol(a[1], a[1] - soa[1])


def test_fused_equals_eager():
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(10_000, seed=3)
    b1 = gpu_bunch(soa, 1e10)
    b2 = gpu_bunch(soa, 1e10)
    c1 = SpaceChargeCalc2p5D(32, 32, 8)
    c2 = SpaceChargeCalc2p5D(32, 32, 8)
    l1 = W.fodo_lattice(c1, cells=2)
    l2 = W.fodo_lattice(c2, cells=2)
    l2.setFusedTracking(False)
    for _ in range(3):
        l1.trackBunch(b1)
        l2.trackBunch(b2)
    assert coord_err(b1.getCoordinates(), b2.getCoordinates()) <= 1e-13
    assert abs(b1.getSyncParticle().time() - b2.getSyncParticle().time()) <= 1e-15 * b2.getSyncParticle().time()
    # the captured program rebuilds the Green spectrum (a conditional graph
    # branch) exactly when node-by-node tracking does
    k1, g1 = c1._calc.counters()
    k2, g2 = c2._calc.counters()
    assert k1 == k2 == 3 * 8 and g1 == g2 and 1 <= g1 <= k1


def test_fused_with_energy_kicks_equals_eager():
    """Kickers that change dE inside the fused program: the passes after
    them must use the new 1/(1+dp_p), not the one kept from the start of
    the run, and the next run starts from the bunch's current dE."""
    from orbit.teapot import KickTEAPOT, QuadTEAPOT
    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import DriftTEAPOT, TEAPOT_Lattice
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D

    def lattice(calc):
        lat = TEAPOT_Lattice("kicked")
        for c in range(3):
            q = QuadTEAPOT("q%d" % c)
            q.setLength(0.5)
            q.addParam("kq", 0.5 if c % 2 == 0 else -0.5)
            k = KickTEAPOT("k%d" % c)
            k.setLength(0.4)
            k.addParam("kx", 1e-5)
            k.addParam("dE", 2e-4 * (c + 1))
            d = DriftTEAPOT("d%d" % c)
            d.setLength(1.0)
            for node in (q, k, d):
                lat.addNode(node)
        lat.initialize()
        setSC2p5DAccNodes(lat, 0.3, calc)
        return lat

    soa = W.c2_coords(10_000, seed=21)
    b1 = gpu_bunch(soa, 1e10)
    b2 = gpu_bunch(soa, 1e10)
    l1 = lattice(SpaceChargeCalc2p5D(32, 32, 8))
    l2 = lattice(SpaceChargeCalc2p5D(32, 32, 8))
    l2.setFusedTracking(False)
    for _ in range(3):
        l1.trackBunch(b1)
        l2.trackBunch(b2)
    got, ref = b1.getCoordinates(), b2.getCoordinates()
    assert np.max(np.abs(got[5] - soa[5])) > 1e-4  # the kickers acted
    assert coord_err(got, ref) <= 1e-13


def test_large_grid_global_path():
    """256x256x64 (the C3/C5 grid): deposit and kick use the global-memory
    path and the FFT runs at N = 512."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(50_000, seed=11)
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(256, 256, 64)
    calc.trackBunch(b, 1.0)
    got = b.getCoordinates()
    sc = O.OracleSC(256, 256, 64)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 1.0, nthreads=8) == 0
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getRhoGrid().getArray(), rho) <= TOL_FIELD
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert rel_err(got[1] - soa[1], a[1] - soa[1]) <= kick_delta_tol(a[1], a[1] - soa[1])
    assert coord_err(got, a) <= TOL_COORD


@pytest.mark.parametrize("shape", [(3, 3, 1), (50, 30, 7), (48, 64, 3), (7, 11, 2)])
def test_odd_grids(shape):
    """Minimum grid and sizes whose doubled FFT lengths are not powers of two."""
    from spacecharge import SpaceChargeCalc2p5D
    rng = np.random.Generator(np.random.PCG64(sum(shape)))
    n = 5000
    soa = np.empty((6, n))
    soa[0] = rng.normal(0, 3e-3, n); soa[1] = rng.normal(0, 1e-3, n)
    soa[2] = rng.normal(0, 2e-3, n); soa[3] = rng.normal(0, 1e-3, n)
    soa[4] = rng.normal(0, 5.0, n); soa[5] = rng.normal(0, 1e-3, n)
    b = gpu_bunch(soa, 1e10)
    calc = SpaceChargeCalc2p5D(*shape)
    sc = O.OracleSC(*shape)
    a = np.ascontiguousarray(soa.copy())
    for _ in range(3):
        calc.trackBunch(b, 0.7)
        assert sc.track(a, oracle_sync_of(b), 0.7) == 0
    rho, phi, zg, lim = sc.grids()
    assert rel_err(calc.getPhiGrid().getArray(), phi) <= TOL_FIELD
    assert coord_err(b.getCoordinates(), a) <= TOL_COORD


def test_per_particle_macrosize():
    from spacecharge import SpaceChargeCalc2p5D
    rng = np.random.Generator(np.random.PCG64(99))
    n = 8000
    soa = np.empty((6, n))
    for c, s in enumerate((4e-3, 1e-3, 4e-3, 1e-3, 8.0, 1e-3)):
        soa[c] = rng.normal(0, s, n)
    m = rng.uniform(0.5e9, 1.5e9, n)
    b = gpu_bunch(soa, 0.0)
    b.addPartAttr("macrosize")
    for i in range(n):
        b.partAttrValue("macrosize", i, 0, m[i])
    calc = SpaceChargeCalc2p5D(32, 32, 16)
    calc.trackBunch(b, 0.5)
    sc = O.OracleSC(32, 32, 16)
    a = np.ascontiguousarray(soa.copy())
    assert sc.track(a, oracle_sync_of(b), 0.5, msize=m) == 0
    assert rel_err(calc.getRhoGrid().getArray(), sc.grids()[0]) <= TOL_FIELD
    assert coord_err(b.getCoordinates(), a) <= TOL_COORD


def test_tiny_bunches_are_noops():
    from spacecharge import SpaceChargeCalc2p5D
    calc = SpaceChargeCalc2p5D(16, 16, 4)
    for n in (0, 1):
        soa = np.full((6, n), 1e-3)
        b = gpu_bunch(soa, 1e9)
        calc.trackBunch(b, 1.0)  # SpaceChargeCalc2p5D.cc:79-80
        assert np.array_equal(b.getCoordinates(), soa)


def test_zero_extent_raises():
    from orbit_gb300 import SpaceChargeError
    from spacecharge import SpaceChargeCalc2p5D
    soa = np.zeros((6, 100))
    soa[0] = np.linspace(-1e-3, 1e-3, 100)
    soa[4] = np.linspace(-1, 1, 100)  # y has zero extent
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(16, 16, 4)
    with pytest.raises(SpaceChargeError):
        calc.trackBunch(b, 1.0)
    # the kick was skipped and the calculator still works afterwards
    assert np.array_equal(b.getCoordinates(), soa)
    soa[2] = np.linspace(-1e-3, 1e-3, 100)
    b2 = gpu_bunch(soa, 1e9)
    calc.trackBunch(b2, 1.0)


def test_nan_coordinate_raises():
    from orbit_gb300 import OrbitError
    from spacecharge import SpaceChargeCalc2p5D
    rng = np.random.Generator(np.random.PCG64(5))
    soa = rng.normal(0, 1e-3, (6, 1000))
    soa[0, 17] = np.nan
    b = gpu_bunch(soa, 1e9)
    calc = SpaceChargeCalc2p5D(16, 16, 4)
    with pytest.raises(OrbitError) as ei:
        calc.trackBunch(b, 1.0)
    assert ei.value.code == -5
