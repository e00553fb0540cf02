"""Host set-up of the conducting boundaries (no GPU): boundary points,
extents, the inside test and the least-squares matrix of the product
library against the reference's golden vectors and the oracle."""
import numpy as np
import pytest

import oracle as O
from helpers import load_golden, rel_err

CASES = ["bnd_circle_64x64x16", "bnd_ellipse_48x40x8", "bnd_rect_32x32x4", "bnd_points_40x40x8"]


def boundary_of(g):
    from spacecharge import Boundary2D
    shape = str(g["bnd_shape"])
    if shape:
        return Boundary2D(int(g["bnd_np"]), int(g["bnd_nm"]), shape, float(g["bnd_xdim"]), float(g["bnd_ydim"]))
    b = Boundary2D(int(g["bnd_np"]), int(g["bnd_nm"]))
    for i, (x, y) in enumerate(zip(g["bnd_x"], g["bnd_y"])):
        b.setBoundaryPoint(i, x, y)
    assert b.isInitialized() == 0
    b.initialize()
    return b


@pytest.mark.parametrize("case", CASES)
def test_boundary_setup_matches_reference(case):
    g = load_golden(case)
    b = boundary_of(g)
    assert b.isInitialized() == 1
    n = b.getNumberOfPoints()
    assert n == len(g["bnd_x"]) and b.getNumberOfModes() == int(g["bnd_nm"])
    pts = np.array([b.getBoundaryPoint(i) for i in range(n)])
    assert np.array_equal(pts[:, 0], g["bnd_x"]) and np.array_equal(pts[:, 1], g["bnd_y"])
    head = g["bnd_head"]
    assert (b.getMinX(), b.getMaxX(), b.getMinY(), b.getMaxY()) == tuple(head[2:6])
    probe = np.linspace(-0.03, 0.03, 41)
    assert np.array_equal(np.array([[b.isInside(x, y) for y in probe] for x in probe]), g["inside"])
    # the least-squares matrix: same algorithm as the oracle's restatement
    from test_oracle_golden import oracle_boundary_of
    _, _, _, lsq_o = oracle_boundary_of(g).data()
    lsq, rnorm = b._dev.lsq()
    assert rel_err(lsq, lsq_o) <= 1e-12


def test_boundary_errors():
    from orbit_gb300 import OrbitError
    from spacecharge import Boundary2D
    with pytest.raises(OrbitError):
        Boundary2D(10, 5)  # 2*nModes+1 >= nPoints
    with pytest.raises(OrbitError):
        Boundary2D(64, 4, "Circle", 0.04, 0.03)  # a circle needs equal sizes
    with pytest.raises(OrbitError):
        Boundary2D(64, 4, "Hexagon", 0.04)
    b = Boundary2D(64, 4, "Rectangle", 0.04, 0.02)
    with pytest.raises(OrbitError):
        b.setBoundaryPoint(0, 0.0, 0.0)  # the shape fixed the points
    assert b.getShapeName() == "Rectangle" and b.getNumberOfPoints() == 64


def test_add_boundary_potential_on_host_grids():
    """Boundary2D.addBoundaryPotential on host Grid2D objects equals the
    oracle's correction of the same potential."""
    from spacecharge import Boundary2D, Grid2D
    b = Boundary2D(128, 10, "Circle", 0.04)
    ob = O.OracleBoundary(128, 10, "Circle", 0.04)
    rng = np.random.default_rng(2)
    n = 33
    phi0 = rng.normal(0, 1.0, (n, n))
    rho = Grid2D(n, n, b.getMinX(), b.getMaxX(), b.getMinY(), b.getMaxY())
    phi = Grid2D(n, n, b.getMinX(), b.getMaxX(), b.getMinY(), b.getMaxY())
    for i in range(n):
        for j in range(n):
            phi.setValue(phi0[i, j], i, j)
    b.addBoundaryPotential(rho, phi)
    # the same correction written out with the oracle's matrix
    head, bx, by, lsq = ob.data()
    ref = Grid2D(n, n, b.getMinX(), b.getMaxX(), b.getMinY(), b.getMaxY())
    for i in range(n):
        for j in range(n):
            ref.setValue(phi0[i, j], i, j)
    bphi = np.array([ref.getValue(x, y) for x, y in zip(bx, by)])
    coef = lsq @ bphi
    rnorm = head[6]
    expect = phi0.copy()
    for i in range(n):
        for j in range(n):
            x, y = ref.getGridX(i), ref.getGridY(j)
            r = np.hypot(x, y)
            f = [1.0]
            for m in range(1, 11):
                f += [(r / rnorm) ** m * np.cos(m * np.arctan2(y, x)), (r / rnorm) ** m * np.sin(m * np.arctan2(y, x))]
            expect[i, j] -= float(np.dot(coef, f))
    assert rel_err(phi.getArray(), expect) <= 1e-12
