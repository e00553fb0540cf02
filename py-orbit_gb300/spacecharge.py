"""Module ``spacecharge``: ``SpaceChargeCalc2p5D``, ``Grid2D`` and ``Grid1D``
with the reference's Python interface (src/spacecharge/wrap_spacechargecalc2p5d.cc,
wrap_grid2D.cc, wrap_grid1D.cc).

``SpaceChargeCalc2p5D.trackBunch`` runs entirely on the GPU
(liborbit_gb300: extrema, deposit, FFT Poisson solve, kick).  The grids it
returns are host views of the device grids, fetched when first read after a
kick.  Stand-alone ``Grid2D``/``Grid1D`` objects are host-side numpy grids
with the reference's indexing and weights (diagnostics, not the hot path).
"""
from __future__ import annotations

import math

import numpy as np


def _finalize(msg):
    raise ValueError(msg)


class Grid2D:
    """Node-centred 2D grid, 9-point quadratic weights (src/spacecharge/Grid2D.cc)."""

    def __init__(self, xSize, ySize, xMin=-1.0, xMax=1.0, yMin=-1.0, yMax=1.0):
        if xSize < 3 or ySize < 3:  # Grid2D.cc:40-51
            _finalize("Grid2D: the grid size too small (should be more than 3)")
        self._nx, self._ny = int(xSize), int(ySize)
        self._arr = np.zeros((self._nx, self._ny))
        self._src = None
        self.setGridX(xMin, xMax)
        self.setGridY(yMin, yMax)

    # lazily refreshed from a device calculator
    def _bind(self, src):
        self._src = src

    def _pull(self):
        if self._src is not None:
            self._src(self)

    def setGridX(self, xMin, xMax):
        self._pull()
        self._xmin, self._xmax = float(xMin), float(xMax)
        self._dx = (self._xmax - self._xmin) / (self._nx - 1)

    def setGridY(self, yMin, yMax):
        self._pull()
        self._ymin, self._ymax = float(yMin), float(yMax)
        self._dy = (self._ymax - self._ymin) / (self._ny - 1)

    def getSizeX(self): return self._nx
    def getSizeY(self): return self._ny
    def getMinX(self): self._pull(); return self._xmin
    def getMaxX(self): self._pull(); return self._xmax
    def getMinY(self): self._pull(); return self._ymin
    def getMaxY(self): self._pull(); return self._ymax
    def getStepX(self): self._pull(); return self._dx
    def getStepY(self): self._pull(); return self._dy
    def getGridX(self, i): self._pull(); return self._xmin + i * self._dx
    def getGridY(self, i): self._pull(); return self._ymin + i * self._dy

    def setZero(self):
        self._pull()
        self._arr[:] = 0.0

    def setValue(self, value, ix, iy):
        self._pull()
        self._arr[ix, iy] = value

    def getValueOnGrid(self, ix, iy):
        self._pull()
        return float(self._arr[ix, iy])

    def getArray(self) -> np.ndarray:
        """The (nx, ny) values as a numpy array (copy)."""
        self._pull()
        return self._arr.copy()

    def getSum(self):
        self._pull()
        s = 0.0
        for v in self._arr.ravel():
            s += v
        return s

    def multiply(self, coeff):
        self._pull()
        self._arr *= coeff

    def isInside(self, x, y):
        self._pull()
        return 0 if (x < self._xmin or x > self._xmax or y < self._ymin or y > self._ymax) else 1

    # Grid2D::getIndAndFracX/Y (Grid2D.cc:337-349)
    def _ind(self, v, vmin, dv, n):
        i = int((v - vmin) / dv + 0.5)
        i = min(max(i, 1), n - 2)
        return i, (v - (vmin + i * dv)) / dv

    @staticmethod
    def _w(f):
        f2 = f * f
        return 0.5 * (0.25 - f + f2), 0.75 - f2, 0.5 * (0.25 + f + f2)

    def getValue(self, x, y):
        self._pull()
        ix, fx = self._ind(x, self._xmin, self._dx, self._nx)
        iy, fy = self._ind(y, self._ymin, self._dy, self._ny)
        wx, wy = self._w(fx), self._w(fy)
        a = self._arr
        return sum(wx[i] * wy[j] * a[ix - 1 + i, iy - 1 + j] for i in range(3) for j in range(3))

    def binValue(self, value, x, y):
        self._pull()
        if x < self._xmin or x > self._xmax or y < self._ymin or y > self._ymax:
            return
        ix, fx = self._ind(x, self._xmin, self._dx, self._nx)
        iy, fy = self._ind(y, self._ymin, self._dy, self._ny)
        wx, wy = self._w(fx), self._w(fy)
        for i in range(3):
            for j in range(3):
                self._arr[ix - 1 + i, iy - 1 + j] += wx[i] * wy[j] * value

    def binBunch(self, bunch, ind0=0, ind1=2):
        """Grid2D::binBunch (Grid2D.cc:113-138), vectorised on the host."""
        self._pull()
        bunch.compress()
        c = bunch.getCoordinates()
        n = c.shape[1]
        if bunch.hasPartAttr("macrosize"):
            m = np.array([bunch.partAttrValue("macrosize", i, 0) for i in range(n)])
        else:
            m = np.full(n, bunch.macroSize())
        x, y = c[ind0], c[ind1]
        ok = ~((x < self._xmin) | (x > self._xmax) | (y < self._ymin) | (y > self._ymax))
        x, y, m = x[ok], y[ok], m[ok]
        ix = np.clip(((x - self._xmin) / self._dx + 0.5).astype(np.int64), 1, self._nx - 2)
        iy = np.clip(((y - self._ymin) / self._dy + 0.5).astype(np.int64), 1, self._ny - 2)
        fx = (x - (self._xmin + ix * self._dx)) / self._dx
        fy = (y - (self._ymin + iy * self._dy)) / self._dy
        wx, wy = self._w(fx), self._w(fy)
        for i in range(3):
            for j in range(3):
                np.add.at(self._arr, (ix - 1 + i, iy - 1 + j), wx[i] * wy[j] * m)

    def calcGradient(self, x, y):
        """Returns (ex, ey) by the 9-point scheme (Grid2D.cc:212-256)."""
        self._pull()
        ix, fx = self._ind(x, self._xmin, self._dx, self._nx)
        iy, fy = self._ind(y, self._ymin, self._dy, self._ny)
        wx, wy = self._w(fx), self._w(fy)
        dwx = ((-1.0) * (0.5 - fx), (-1.0) * (+2.0) * fx, (-1.0) * (-(0.5 + fx)))
        dwy = ((-1.0) * (0.5 - fy), (-1.0) * (+2.0) * fy, (-1.0) * (-(0.5 + fy)))
        a = self._arr
        ex = 0.0
        ey = 0.0
        for i in range(3):
            for j in range(3):
                v = a[ix - 1 + i, iy - 1 + j]
                ex += dwx[i] * wy[j] * v
                ey += wx[i] * dwy[j] * v
        return ex / self._dx, ey / self._dy

    # bilinear variants (Grid2D.cc:168-208, 284-312, 351-366)
    def _bind_lin(self, v, vmin, dv, n):
        i = int((v - vmin) / dv)
        i = min(max(i, 0), n - 2)
        return i, (v - (vmin + i * dv)) / dv

    def getValueBilinear(self, x, y):
        self._pull()
        ix, fx = self._bind_lin(x, self._xmin, self._dx, self._nx)
        iy, fy = self._bind_lin(y, self._ymin, self._dy, self._ny)
        a = self._arr
        return ((1. - fx) * (1. - fy) * a[ix, iy] + fx * (1. - fy) * a[ix + 1, iy]
                + (1. - fx) * fy * a[ix, iy + 1] + fx * fy * a[ix + 1, iy + 1])

    def binValueBilinear(self, value, x, y):
        self._pull()
        ix, fx = self._bind_lin(x, self._xmin, self._dx, self._nx)
        iy, fy = self._bind_lin(y, self._ymin, self._dy, self._ny)
        self._arr[ix, iy] += ((1. - fx) * (1. - fy)) * value
        self._arr[ix, iy + 1] += ((1. - fx) * fy) * value
        self._arr[ix + 1, iy] += (fx * (1. - fy)) * value
        self._arr[ix + 1, iy + 1] += (fx * fy) * value

    def binBunchBilinear(self, bunch, ind0=0, ind1=2):
        bunch.compress()
        c = bunch.getCoordinates()
        m = bunch.macroSize()
        for i in range(c.shape[1]):
            self.binValueBilinear(m, c[ind0, i], c[ind1, i])

    def calcGradientBilinear(self, x, y):
        self._pull()
        ix, fx = self._bind_lin(x, self._xmin, self._dx, self._nx)
        iy, fy = self._bind_lin(y, self._ymin, self._dy, self._ny)
        a = self._arr
        ex = (a[ix + 1, iy] - a[ix, iy]) * (1.0 - fy) + fy * (a[ix + 1, iy + 1] - a[ix, iy + 1])
        ey = (a[ix, iy + 1] - a[ix, iy]) * (1.0 - fx) + fx * (a[ix + 1, iy + 1] - a[ix + 1, iy])
        return ex / self._dx, ey / self._dy

    def synchronizeMPI(self, comm=None):
        """Single process per GPU: nothing to reduce."""
        return None


class Grid1D:
    """Periodic cell-centred 1D grid, linear weights (src/spacecharge/Grid1D.cc)."""

    def __init__(self, zSize, zMin=-0.5, zMax=0.5):
        if zSize < 1:  # Grid1D.cc:70-82
            _finalize("Grid1D: the grid size is too small (should be more than 0)")
        self._nz = int(zSize)
        self._arr = np.zeros(self._nz)
        self._src = None
        self.setGridZ(zMin, zMax)

    def _bind(self, src):
        self._src = src

    def _pull(self):
        if self._src is not None:
            self._src(self)

    def setGridZ(self, zMin, zMax):
        self._pull()
        self._zmin, self._zmax = float(zMin), float(zMax)
        self._dz = (self._zmax - self._zmin) / self._nz

    def getMinZ(self): self._pull(); return self._zmin
    def getMaxZ(self): self._pull(); return self._zmax
    def getSizeZ(self): return self._nz
    def getStepZ(self): self._pull(); return self._dz
    def getGridZ(self, i): self._pull(); return self._zmin + (i + 0.5) * self._dz

    def getSum(self):
        self._pull()
        s = 0.0
        for v in self._arr:
            s += v
        return s

    def setZero(self):
        self._pull()
        self._arr[:] = 0.0

    def setValue(self, value, iz):
        self._pull()
        self._arr[iz] = value

    def multiply(self, coeff):
        self._pull()
        self._arr *= coeff

    def getValueOnGrid(self, iz):
        self._pull()
        return float(self._arr[iz])

    def getArray(self) -> np.ndarray:
        self._pull()
        return self._arr.copy()

    def isInside(self, z):
        self._pull()
        return 0 if (z < self._zmin or z > self._zmax) else 1

    # Grid1D::getIndAndWZ (Grid1D.cc:568-627)
    def _ind(self, z):
        nz = self._nz
        if nz > 1:
            ind_dbl = ((z - self._zmin) / self._dz) - 0.5
            i0 = int(ind_dbl)
            zf = (z - (self._zmin + (i0 + 0.5) * self._dz)) / self._dz
            if i0 < 0 or i0 > nz - 1:
                raise ValueError("Grid1D::getIndAndWZ Wrong z value.")
            if i0 == 0 and zf < 0.0:
                return nz - 1, 0, -zf, 1.0 + zf
            if i0 == nz - 1:
                if zf > 0.0:
                    return i0, 0, 1.0 - zf, zf
                return nz - 2, i0, -zf, 1.0 + zf
            return i0, i0 + 1, 1.0 - zf, zf
        return 0, 0, 1.0, 0.0

    def getValue(self, z):
        self._pull()
        if z < self._zmin or z > self._zmax:
            return 0.0
        i0, ip, w0, wp = self._ind(z)
        if self._nz > 1:
            return w0 * self._arr[i0] + wp * self._arr[ip]
        return float(self._arr[0])

    def binValue(self, value, z):
        self._pull()
        if z < self._zmin or z > self._zmax:
            return
        i0, ip, w0, wp = self._ind(z)
        if self._nz > 1:
            self._arr[i0] += w0 * value
            self._arr[ip] += wp * value
        else:
            self._arr[i0] += value

    def binBunch(self, bunch, axis_ind=4):
        if axis_ind < 0 or axis_ind > 5:
            _finalize("Grid1D::binBunch: axis_ind should be between 0 and 5")
        bunch.compress()
        c = bunch.getCoordinates()
        m = bunch.macroSize()
        has_m = bunch.hasPartAttr("macrosize")
        for i in range(c.shape[1]):
            self.binValue(bunch.partAttrValue("macrosize", i, 0) if has_m else m, c[axis_ind, i])

    def calcGradient(self, z):
        self._pull()
        if z < self._zmin or z > self._zmax:
            return 0.0
        i0, ip, _, _ = self._ind(z)
        if self._nz > 1:
            return (self._arr[ip] - self._arr[i0]) / self._dz
        return 0.0

    def synchronizeMPI(self, comm=None):
        return None


class Boundary2D:
    """``Boundary2D(nPoints, nModes)`` (points set with setBoundaryPoint, then
    initialize()) or ``Boundary2D(nPoints, nModes, shape, xDim[, yDim])`` with
    shape "Circle", "Ellipse" or "Rectangle" (src/spacecharge/wrap_boundary2d.cc,
    BaseBoundary2D.cc, ShapedBoundary2D.cc): a conducting boundary for the
    2.5D space-charge kick."""

    IS_INSIDE = 1
    IS_OUTSIDE = -1

    def __init__(self, nPoints, nModes, shape=None, xDim=None, yDim=None):
        from orbit_gb300 import DeviceBoundary
        if shape is None:
            self._dev = DeviceBoundary(nPoints, nModes)
            self._shape = "noshape"
        else:
            self._dev = DeviceBoundary(nPoints, nModes, shape, xDim, yDim)
            self._shape = shape

    def _info(self):
        return self._dev.info()

    def getMaxX(self): return float(self._info()[3][1])
    def getMinX(self): return float(self._info()[3][0])
    def getMaxY(self): return float(self._info()[3][3])
    def getMinY(self): return float(self._info()[3][2])
    def getNumberOfModes(self): return self._info()[1]
    def getNumberOfPoints(self): return self._info()[0]
    def getShapeName(self): return self._shape
    def isInitialized(self): return 1 if self._info()[4] else 0

    def isInside(self, x, y):
        return self._dev.is_inside(x, y)

    def initialize(self):
        self._dev.initialize()

    def getBoundaryPoint(self, index):
        return self._dev.get_point(index)

    def setBoundaryPoint(self, index, x, y):
        self._dev.set_point(index, x, y)

    def addBoundaryPotential(self, rhoGrid, phiGrid):
        """Subtracts the fitted free-space field of the boundary charges from
        phiGrid (BaseBoundary2D::addBoundaryPotential, BaseBoundary2D.cc:352-460)."""
        npnt, nm, _, lim, init = self._info()
        if not init:
            _finalize("Boundary2D: the boundary was not initialized! Call initialize() method!")
        if (rhoGrid.getMinX() > lim[0] or rhoGrid.getMaxX() < lim[1] or rhoGrid.getMinY() > lim[2]
                or rhoGrid.getMaxY() < lim[3]):
            _finalize("Boundary2D: some boundary points are outside the grids")
        lsq, rnorm = self._dev.lsq()
        bphi = np.array([phiGrid.getValue(*self.getBoundaryPoint(j)) for j in range(npnt)])
        coef = np.array([sum(lsq[i, j] * bphi[j] for j in range(npnt)) for i in range(2 * nm + 1)])
        arr = phiGrid.getArray()
        for i in range(phiGrid.getSizeX()):
            for j in range(phiGrid.getSizeY()):
                x, y = phiGrid.getGridX(i), phiGrid.getGridY(j)
                r2 = x * x + y * y
                if r2 == 0.0:
                    f = [1.0] + [0.0] * (2 * nm)
                else:
                    r = math.sqrt(r2)
                    s = y / r
                    c = x / r
                    s0, c0, rfac, rj = s, c, r / rnorm, 1.0
                    f = [1.0]
                    for _ in range(nm):
                        rj *= rfac
                        f += [rj * c0, rj * s0]
                        s0, c0 = s * c0 + c * s0, c * c0 - s * s0
                p = 0.0
                for k in range(2 * nm + 1):
                    p += coef[k] * f[k]
                phiGrid.setValue(arr[i, j] - p, i, j)


class SpaceChargeCalc2p5D:
    """``SpaceChargeCalc2p5D(xSize, ySize, zSize[, xy_ratio])``
    (src/spacecharge/SpaceChargeCalc2p5D.cc, wrap_spacechargecalc2p5d.cc:38-52).

    ``form`` selects the arithmetic: ``"plain"`` (FP64 throughout, the
    drop-in) or ``"fp32"`` (the plain form's exact fixed-point deposit, FFT
    and gradient in FP32; coordinates and kick accumulation FP64).
    """

    _FORMS = {"plain": 0, "fp32": 1}

    def __init__(self, xSize, ySize, zSize, xy_ratio=-1.0, form="plain"):
        from orbit_gb300 import DeviceSC2p5D
        if form not in self._FORMS:
            raise ValueError("form must be 'plain' or 'fp32'")
        if xSize < 3 or ySize < 3:
            _finalize("Grid2D: the grid size too small (should be more than 3)")
        if zSize < 1:
            _finalize("Grid1D: the grid size is too small (should be more than 0)")
        self.form = form
        self._calc = DeviceSC2p5D(xSize, ySize, zSize, xy_ratio, self._FORMS[form])
        self._nx, self._ny, self._nz = int(xSize), int(ySize), int(zSize)
        self._version = 0
        self._seen = {}
        self._rho = Grid2D(xSize, ySize)
        self._phi = Grid2D(xSize, ySize)
        self._long = Grid1D(zSize)
        self._rho._bind(lambda g: self._refresh(g, 0))
        self._phi._bind(lambda g: self._refresh(g, 1))
        self._long._bind(lambda g: self._refresh(g, 2))

    # ---- learned closure (a form of this library; no reference counterpart)
    def setDenoiser(self, denoiser, checkEvery=10, bound=1e-3):
        """Denoise every kick's deposit with a trained network
        (orbit_gb300.DeviceDenoiser of the grid's size) before the FFT solve;
        every checkEvery-th kick the raw deposit is solved as well and the
        calculator falls back to it for good when the relative rms difference
        of the two potentials exceeds `bound` (default 1e-3: the shipped
        network scores 0.6-1.3e-4 on in-distribution beams and 1-7e-4 while
        tracking).  A network that reports a failed tensor-core wait also
        makes the calculator fall back.  None removes the closure."""
        self._calc.set_denoiser(denoiser, checkEvery, bound)

    def getDenoiserState(self):
        return self._calc.denoiser_state()

    def resetDenoiser(self):
        self._calc.denoiser_reset()

    def _refresh(self, g, which):
        if self._version == 0 or self._seen.get(which) == self._version:
            return
        self._seen[which] = self._version
        src = g._src
        g._src = None  # avoid recursion through the setters
        try:
            lim = self._calc.limits()
            arr = self._calc.grid(which)
            if which == 2:
                g.setGridZ(lim[4], lim[5])
                g._dz = lim[8]
                g._arr = np.array(arr)
            else:
                g.setGridX(lim[0], lim[1])
                g.setGridY(lim[2], lim[3])
                g._dx, g._dy = lim[6], lim[7]
                g._arr = np.array(arr)
        finally:
            g._src = src

    def trackBunch(self, bunch, length, boundary=None):
        """Applies the 2.5D space-charge kick of a lattice part of the given
        length, with an optional conducting boundary
        (SpaceChargeCalc2p5D.cc:77-120)."""
        rec = getattr(bunch, "_record_sc", None)
        if rec is not None:
            rec(self, float(length), 0.0, boundary)
            return
        if bunch.getSizeGlobal() < 2:
            return
        dev = bunch._device_bunch()
        if boundary is not None:
            self._calc.track_boundary(dev, float(length), boundary._dev)
        else:
            self._calc.track(dev, float(length))
        bunch._device_modified()
        self._version += 1
        dev.sync()

    def getRhoGrid(self) -> Grid2D:
        return self._rho

    def getPhiGrid(self) -> Grid2D:
        return self._phi

    def getLongGrid(self) -> Grid1D:
        return self._long

    def fields(self, x, y, z):
        """(ex, ey, lambda) at host points from the current device grids."""
        return self._calc.fields(x, y, z)


class SpaceChargeCalc2p5Drb(SpaceChargeCalc2p5D):
    """``SpaceChargeCalc2p5Drb(xSize, ySize, zSize[, xy_ratio])``
    (src/spacecharge/SpaceChargeCalc2p5Drb.cc, wrap_spacechargecalc2p5d_rb.cc:37-50):
    the 2.5D transverse kick plus a longitudinal kick of dE from the
    smoothed derivative of the line density and a pipe radius.  The grid
    keeps the calculator's aspect ratio and the Poisson solver grid is never
    reshaped.  Plain FP64 form."""

    def __init__(self, xSize, ySize, zSize, xy_ratio=-1.0):
        from orbit_gb300 import DeviceSC2p5Drb
        if xSize < 3 or ySize < 3:
            _finalize("Grid2D: the grid size too small (should be more than 3)")
        if zSize < 1:
            _finalize("Grid1D: the grid size is too small (should be more than 0)")
        self.form = "plain"
        self._calc = DeviceSC2p5Drb(xSize, ySize, zSize, xy_ratio)
        self._nx, self._ny, self._nz = int(xSize), int(ySize), int(zSize)
        self._version = 0
        self._seen = {}
        self._rho = Grid2D(xSize, ySize)
        self._phi = Grid2D(xSize, ySize)
        self._long = Grid1D(zSize)
        self._deriv = Grid1D(zSize)
        self._rho._bind(lambda g: self._refresh(g, 0))
        self._phi._bind(lambda g: self._refresh(g, 1))
        self._long._bind(lambda g: self._refresh(g, 2))
        self._deriv._bind(lambda g: self._refresh(g, 3))

    def _refresh(self, g, which):
        if which != 3:
            return SpaceChargeCalc2p5D._refresh(self, g, which)
        if self._version == 0 or self._seen.get(which) == self._version:
            return
        self._seen[which] = self._version
        src = g._src
        g._src = None
        try:
            lim = self._calc.limits()
            g.setGridZ(lim[4], lim[5])
            g._dz = lim[8]
            g._arr = np.array(self._calc.grid(3))
        finally:
            g._src = src

    def trackBunch(self, bunch, length, pipe_radius):
        """Transverse and longitudinal space-charge kicks of a lattice part of
        the given length (SpaceChargeCalc2p5Drb.cc:107-155)."""
        rec = getattr(bunch, "_record_sc", None)
        if rec is not None:
            rec(self, float(length), float(pipe_radius))
            return
        if bunch.getSizeGlobal() < 2:
            return
        dev = bunch._device_bunch()
        self._calc.track_rb(dev, float(length), float(pipe_radius))
        bunch._device_modified()
        self._version += 1
        dev.sync()

    def getLongDerivativeGrid(self) -> Grid1D:
        return self._deriv

    def setLongAveragingPointsN(self, n_points):
        self._calc.set_long_avg(int(n_points))

    def getLongAveragingPointsN(self) -> int:
        return self._calc.get_long_avg()


__all__ = ["SpaceChargeCalc2p5D", "SpaceChargeCalc2p5Drb", "Boundary2D", "Grid2D", "Grid1D"]
