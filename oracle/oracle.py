"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes access to
  * ``liborbit_oracle.so`` -- the plain-C restatement of the PyORBIT 2.5D
    space-charge + TEAPOT hot path (oracle/orbit_oracle.c), built on any host
    by :func:`build_oracle`;
  * ``_ref/libpyorbit_ref.so`` -- the reference's own C++ compiled from the
    reference tree by oracle/build_ref.sh (only where that tree exists).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import
this module.  The product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "liborbit_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpyorbit_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


def _P(a):
    return a.ctypes.data_as(_dp)


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement with -ffp-contract=off (no fused multiply-add,
    matching the reference's x86-64 build) for whatever host this runs on."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("orbit_oracle.c", "fft.c")]
    hdrs = [os.path.join(HERE, f) for f in ("orbit_oracle.h", "fft.h")]
    if not force and os.path.exists(ORACLE_SO):
        t = os.path.getmtime(ORACLE_SO)
        if all(os.path.getmtime(s) < t for s in srcs + hdrs):
            return ORACLE_SO
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp] + srcs + ["-lpthread", "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference() -> bool:
    """Compile the reference C++ (only where the reference tree exists)."""
    script = os.path.join(HERE, "build_ref.sh")
    try:
        subprocess.check_call(["bash", script])
    except (subprocess.CalledProcessError, OSError):
        return False
    return os.path.exists(REF_SO)


class OracleSync(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("beta", "gamma", "momentum", "mass", "charge", "classical_radius",
                 "macrosize", "time")]


class OracleOp(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("i0", ctypes.c_int32), ("i1", ctypes.c_int32),
                ("i2", ctypes.c_int32), ("d", ctypes.c_double * 6)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.oracle_sc_new.restype = _vp
        L.oracle_sc_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.oracle_sc_free.argtypes = [_vp]
        L.oracle_sc_track.restype = ctypes.c_int
        L.oracle_sc_track.argtypes = [_vp, _dp, ctypes.c_int, _dp, ctypes.POINTER(OracleSync),
                                      ctypes.c_double, ctypes.c_int]
        L.oracle_sc_grids.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.oracle_sc_fields.argtypes = [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_run_program.restype = ctypes.c_int
        L.oracle_run_program.argtypes = [ctypes.POINTER(OracleOp), ctypes.c_int, ctypes.c_int, _dp,
                                         ctypes.c_int, _dp, ctypes.POINTER(OracleSync),
                                         ctypes.POINTER(_vp), ctypes.c_int]
        L.oracle_rms_emittance.argtypes = [_dp, ctypes.c_int, _dp, _dp]
        L.oracle_scrb_new.restype = _vp
        L.oracle_scrb_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.oracle_scrb_set_long_avg.argtypes = [_vp, ctypes.c_int]
        L.oracle_scrb_track.restype = ctypes.c_int
        L.oracle_scrb_track.argtypes = [_vp, _dp, ctypes.c_int, _dp, ctypes.POINTER(OracleSync), ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int]
        L.oracle_scrb_extra.argtypes = [_vp, _dp, _dp]
        L.oracle_bnd_new.restype = _vp
        L.oracle_bnd_new.argtypes = [ctypes.c_int, ctypes.c_int]
        L.oracle_bnd_new_shape.restype = _vp
        L.oracle_bnd_new_shape.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double]
        L.oracle_bnd_free.argtypes = [_vp]
        L.oracle_bnd_set_point.argtypes = [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_bnd_initialize.restype = ctypes.c_int
        L.oracle_bnd_initialize.argtypes = [_vp]
        L.oracle_bnd_is_inside.restype = ctypes.c_int
        L.oracle_bnd_is_inside.argtypes = [_vp, ctypes.c_double, ctypes.c_double]
        L.oracle_bnd_get.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.oracle_twiss_moments.argtypes = [_dp, ctypes.c_int, _dp, _dp]
        L.oracle_tune_analysis.argtypes = [_dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp]
        L.oracle_sc_track_bnd.restype = ctypes.c_int
        L.oracle_sc_track_bnd.argtypes = [_vp, _dp, ctypes.c_int, _dp, ctypes.POINTER(OracleSync), ctypes.c_double,
                                          _vp, ctypes.c_int]
        _lib = L
    return _lib


def make_sync(beta, gamma, momentum, mass=0.938272013, charge=1.0,
              classical_radius=1.534698e-18, macrosize=0.0, time=0.0) -> OracleSync:
    return OracleSync(beta, gamma, momentum, mass, charge, classical_radius, macrosize, time)


class OracleSC:
    """SpaceChargeCalc2p5D restated in C."""

    def __init__(self, nx, ny, nz, xy_ratio=-1.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = lib().oracle_sc_new(nx, ny, nz, float(xy_ratio))
        if not self.h:
            raise ValueError("bad grid size")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_sc_free(self.h)
            self.h = None

    def track(self, soa: np.ndarray, sync: OracleSync, length: float, msize=None, nthreads=1) -> int:
        assert soa.dtype == np.float64 and soa.flags.c_contiguous and soa.shape[0] == 6
        m = None if msize is None else _P(np.ascontiguousarray(msize, dtype=np.float64))
        return lib().oracle_sc_track(self.h, _P(soa), soa.shape[1], m, ctypes.byref(sync),
                                     float(length), int(nthreads))

    def grids(self):
        rho = np.zeros(self.nx * self.ny)
        phi = np.zeros(self.nx * self.ny)
        zg = np.zeros(self.nz)
        lim = np.zeros(11)
        lib().oracle_sc_grids(self.h, _P(rho), _P(phi), _P(zg), _P(lim))
        return rho.reshape(self.nx, self.ny), phi.reshape(self.nx, self.ny), zg, lim

    def fields(self, x, y, z):
        n = len(x)
        ex, ey, lam = np.zeros(n), np.zeros(n), np.zeros(n)
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        lib().oracle_sc_fields(self.h, n, _P(x), _P(y), _P(z), _P(ex), _P(ey), _P(lam))
        return ex, ey, lam


class OracleSCrb(OracleSC):
    """SpaceChargeCalc2p5Drb restated in C."""

    def __init__(self, nx, ny, nz, xy_ratio=-1.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = lib().oracle_scrb_new(nx, ny, nz, float(xy_ratio))
        if not self.h:
            raise ValueError("bad grid size")

    def setLongAveragingPointsN(self, n):
        lib().oracle_scrb_set_long_avg(self.h, int(n))

    def track(self, soa: np.ndarray, sync: OracleSync, length: float, pipe_radius: float, msize=None,
              nthreads=1) -> int:
        assert soa.dtype == np.float64 and soa.flags.c_contiguous and soa.shape[0] == 6
        m = None if msize is None else _P(np.ascontiguousarray(msize, dtype=np.float64))
        return lib().oracle_scrb_track(self.h, _P(soa), soa.shape[1], m, ctypes.byref(sync), float(length),
                                       float(pipe_radius), int(nthreads))

    def extra(self):
        """(derivative grid [nz], a_bunch, x_center, y_center)."""
        zd = np.zeros(self.nz)
        abx = np.zeros(3)
        lib().oracle_scrb_extra(self.h, _P(zd), _P(abx))
        return zd, abx[0], abx[1], abx[2]


SHAPES = {"Circle": 1, "Ellipse": 2, "Rectangle": 3}


class OracleBoundary:
    """BaseBoundary2D / ShapedBoundary2D restated in C.  Boundary(np, nm) or
    Boundary(np, nm, shape, xDim[, yDim]) as the reference's Boundary2D."""

    def __init__(self, np_, nm, shape=None, xdim=0.0, ydim=None):
        L = lib()
        if shape is None:
            self.h = L.oracle_bnd_new(int(np_), int(nm))
        else:
            self.h = L.oracle_bnd_new_shape(int(np_), int(nm), SHAPES[shape], float(xdim),
                                            float(xdim if ydim is None else ydim))
        if not self.h:
            raise ValueError("bad boundary parameters")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_bnd_free(self.h)
            self.h = None

    def setBoundaryPoint(self, i, x, y):
        lib().oracle_bnd_set_point(self.h, int(i), float(x), float(y))

    def initialize(self):
        return lib().oracle_bnd_initialize(self.h)

    def isInside(self, x, y):
        return lib().oracle_bnd_is_inside(self.h, float(x), float(y))

    def data(self):
        head = np.zeros(7)
        lib().oracle_bnd_get(self.h, _P(head), None, None, None)
        np_, nm = int(head[0]), int(head[1])
        bx, by = np.zeros(np_), np.zeros(np_)
        lsq = np.zeros((2 * nm + 1) * np_)
        lib().oracle_bnd_get(self.h, _P(head), _P(bx), _P(by), _P(lsq))
        return head, bx, by, lsq.reshape(2 * nm + 1, np_)


def twiss_moments(soa, msize=None):
    """{count, total macrosize, <c_i>[6], <c_i c_j> i >= j [21]} as
    BunchTwissAnalysis::analyzeBunch accumulates them."""
    soa = np.ascontiguousarray(soa, dtype=np.float64)
    out = np.zeros(29)
    m = None if msize is None else _P(np.ascontiguousarray(msize, dtype=np.float64))
    lib().oracle_twiss_moments(_P(soa), soa.shape[1], m, _P(out))
    return out


def tune_analysis(soa, beta, etot, twiss, ph):
    """BunchTuneAnalysis::analyzeBunch; ph (6, n) is updated in place."""
    soa = np.ascontiguousarray(soa, dtype=np.float64)
    tw = np.ascontiguousarray(twiss, dtype=np.float64)
    assert ph.dtype == np.float64 and ph.flags.c_contiguous and ph.shape == (6, soa.shape[1])
    lib().oracle_tune_analysis(_P(soa), soa.shape[1], float(beta), float(etot), _P(tw), _P(ph))


def sc_track_bnd(sc, soa, sync, length, bnd, msize=None, nthreads=1):
    m = None if msize is None else _P(np.ascontiguousarray(msize, dtype=np.float64))
    return lib().oracle_sc_track_bnd(sc.h, _P(soa), soa.shape[1], m, ctypes.byref(sync), float(length), bnd.h,
                                     int(nthreads))


def tpb(name: str, soa: np.ndarray, sync: OracleSync, *args):
    """Apply one TEAPOT map by its reference name (drift, quad1, ...)."""
    L = lib()
    f = getattr(L, "oracle_" + name)
    n = soa.shape[1]
    ints = {"multp", "multpfringeIN", "multpfringeOUT"}
    if name in ("rotatexy", "wrapbunch"):
        f.argtypes = [_dp, ctypes.c_int, ctypes.c_double]
        return f(_P(soa), n, float(args[0]))
    if name == "kick":
        f.argtypes = [_dp, ctypes.c_int] + [ctypes.c_double] * 3
        return f(_P(soa), n, *map(float, args[:3]))
    if name in ints:
        f.argtypes = [_dp, ctypes.c_int, ctypes.POINTER(OracleSync), ctypes.c_int, ctypes.c_double,
                      ctypes.c_int]
        return f(_P(soa), n, ctypes.byref(sync), int(args[0]), float(args[1]), int(args[2]))
    if name in ("wedgerotate", "wedgedrift"):
        f.argtypes = [_dp, ctypes.c_int, ctypes.POINTER(OracleSync), ctypes.c_double, ctypes.c_int]
        return f(_P(soa), n, ctypes.byref(sync), float(args[0]), int(args[1]))
    if name == "wedgebend":
        f.argtypes = [_dp, ctypes.c_int, ctypes.POINTER(OracleSync), ctypes.c_double, ctypes.c_int,
                      ctypes.c_double, ctypes.c_int]
        return f(_P(soa), n, ctypes.byref(sync), float(args[0]), int(args[1]), float(args[2]),
                 int(args[3]))
    f.argtypes = [_dp, ctypes.c_int, ctypes.POINTER(OracleSync)] + [ctypes.c_double] * len(args)
    return f(_P(soa), n, ctypes.byref(sync), *map(float, args))


def run_program(ops, turns, soa, sync, calcs, msize=None, nthreads=1) -> int:
    """Run a recorded op list (list of (code, (i0,i1,i2), (d0..d5)))."""
    arr = (OracleOp * len(ops))()
    for k, (code, iv, dv) in enumerate(ops):
        arr[k].code = code
        arr[k].i0, arr[k].i1, arr[k].i2 = (list(iv) + [0, 0, 0])[:3]
        for j, v in enumerate((list(dv) + [0.0] * 6)[:6]):
            arr[k].d[j] = v
    hs = (_vp * max(1, len(calcs)))(*[c.h for c in calcs])
    m = None if msize is None else _P(np.ascontiguousarray(msize, dtype=np.float64))
    return lib().oracle_run_program(arr, len(ops), int(turns), _P(soa), soa.shape[1], m,
                                    ctypes.byref(sync), hs, int(nthreads))


def rms_emittance(soa):
    ex, ey = ctypes.c_double(), ctypes.c_double()
    lib().oracle_rms_emittance(_P(soa), soa.shape[1], ctypes.byref(ex), ctypes.byref(ey))
    return ex.value, ey.value


# ----------------------------------------------------------------------
# The compiled reference (x86 container only)
# ----------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    """True where the compiled reference exists and loads on this host."""
    if not os.path.exists(REF_SO):
        return False
    try:
        ref()
    except OSError:
        return False
    return True


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        L.ref_bunch_new.restype = _vp
        L.ref_bunch_free.argtypes = [_vp]
        L.ref_bunch_set_kin_energy.restype = ctypes.c_double
        L.ref_bunch_set_kin_energy.argtypes = [_vp, ctypes.c_double]
        L.ref_bunch_set_macrosize.argtypes = [_vp, ctypes.c_double]
        L.ref_bunch_size.restype = ctypes.c_int
        L.ref_bunch_size.argtypes = [_vp]
        L.ref_bunch_kinematics.argtypes = [_vp, _dp]
        L.ref_bunch_add.argtypes = [_vp, ctypes.c_int, _dp]
        L.ref_bunch_get.argtypes = [_vp, _dp]
        L.ref_bunch_set.argtypes = [_vp, _dp]
        L.ref_sc_new.restype = _vp
        L.ref_sc_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ref_sc_free.argtypes = [_vp]
        L.ref_sc_track.argtypes = [_vp, _vp, ctypes.c_double]
        L.ref_sc_grids.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.ref_sc_fields.argtypes = [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_scrb_new.restype = _vp
        L.ref_scrb_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ref_scrb_free.argtypes = [_vp]
        L.ref_scrb_set_long_avg.argtypes = [_vp, ctypes.c_int]
        L.ref_scrb_track.argtypes = [_vp, _vp, ctypes.c_double, ctypes.c_double]
        L.ref_scrb_grids.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp]
        L.ref_bnd_new.restype = _vp
        L.ref_bnd_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.ref_bnd_free.argtypes = [_vp]
        L.ref_bnd_set_point.argtypes = [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.ref_bnd_initialize.argtypes = [_vp]
        L.ref_bnd_is_inside.restype = ctypes.c_int
        L.ref_bnd_is_inside.argtypes = [_vp, ctypes.c_double, ctypes.c_double]
        L.ref_bnd_get.argtypes = [_vp, _dp, _dp, _dp]
        L.ref_sc_track_bnd.argtypes = [_vp, _vp, ctypes.c_double, _vp]
        L.ref_twiss.argtypes = [_vp, _dp, _dp]
        L.ref_bunch_moments.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
        L.ref_tune_new.restype = _vp
        L.ref_tune_free.argtypes = [_vp]
        L.ref_tune_assign.argtypes = [_vp, _dp]
        L.ref_tune_analyze.argtypes = [_vp, _vp, _dp]
        _cp = ctypes.c_char_p
        L.ref_bunch_dump.argtypes = [_vp, _cp]
        L.ref_bunch_read.argtypes = [_vp, _cp]
        L.ref_bunch_add_attr.argtypes = [_vp, _cp, ctypes.c_int]
        L.ref_bunch_attr_size.restype = ctypes.c_int
        L.ref_bunch_attr_size.argtypes = [_vp, _cp]
        L.ref_bunch_attr_set.argtypes = [_vp, _cp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ref_bunch_attr_get.restype = ctypes.c_double
        L.ref_bunch_attr_get.argtypes = [_vp, _cp, ctypes.c_int, ctypes.c_int]
        L.ref_bunch_set_int_attr.argtypes = [_vp, _cp, ctypes.c_int]
        L.ref_bunch_set_double_attr.argtypes = [_vp, _cp, ctypes.c_double]
        L.ref_bunch_get_int_attr.restype = ctypes.c_int
        L.ref_bunch_get_int_attr.argtypes = [_vp, _cp]
        L.ref_bunch_get_double_attr.restype = ctypes.c_double
        L.ref_bunch_get_double_attr.argtypes = [_vp, _cp]
        L.ref_bunch_set_time.argtypes = [_vp, ctypes.c_double]
        _ref = L
    return _ref


class RefBunch:
    """A reference ``Bunch`` (AoS, src/orbit/Bunch.cc) driven through the harness."""

    def __init__(self, soa: np.ndarray, kin_energy: float, macrosize: float):
        L = ref()
        self.h = L.ref_bunch_new()
        L.ref_bunch_set_kin_energy(self.h, float(kin_energy))
        L.ref_bunch_set_macrosize(self.h, float(macrosize))
        soa = np.ascontiguousarray(soa, dtype=np.float64)
        L.ref_bunch_add(self.h, soa.shape[1], _P(soa))
        self.n = soa.shape[1]

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_bunch_free(self.h)
            self.h = None

    def coords(self) -> np.ndarray:
        self.n = ref().ref_bunch_size(self.h)
        out = np.zeros((6, self.n))
        ref().ref_bunch_get(self.h, _P(out))
        return out

    # text I/O (Bunch::print / readBunch) and attributes
    def dump(self, path: str):
        ref().ref_bunch_dump(self.h, path.encode())

    def read(self, path: str):
        ref().ref_bunch_read(self.h, path.encode())
        self.n = ref().ref_bunch_size(self.h)

    def add_attr(self, name: str, size: int = 0):
        ref().ref_bunch_add_attr(self.h, name.encode(), int(size))

    def attr_size(self, name: str) -> int:
        return ref().ref_bunch_attr_size(self.h, name.encode())

    def attr(self, name: str, i: int, j: int, value=None) -> float:
        if value is not None:
            ref().ref_bunch_attr_set(self.h, name.encode(), int(i), int(j), float(value))
        return ref().ref_bunch_attr_get(self.h, name.encode(), int(i), int(j))

    def bunch_attr_int(self, name: str, value=None) -> int:
        if value is not None:
            ref().ref_bunch_set_int_attr(self.h, name.encode(), int(value))
        return ref().ref_bunch_get_int_attr(self.h, name.encode())

    def bunch_attr_double(self, name: str, value=None) -> float:
        if value is not None:
            ref().ref_bunch_set_double_attr(self.h, name.encode(), float(value))
        return ref().ref_bunch_get_double_attr(self.h, name.encode())

    def set_time(self, t: float):
        ref().ref_bunch_set_time(self.h, float(t))

    def kinematics(self):
        k = np.zeros(7)
        ref().ref_bunch_kinematics(self.h, _P(k))
        return dict(beta=k[0], gamma=k[1], momentum=k[2], kin_energy=k[3], mass=k[4],
                    classical_radius=k[5], time=k[6])

    def tpb(self, name: str, *args):
        L = ref()
        f = getattr(L, "ref_tpb_" + name)
        types = {
            "rotatexy": "d", "drift": "d", "wrapbunch": "d", "kick": "ddd", "multp": "idi",
            "multpfringeIN": "idi", "multpfringeOUT": "idi", "quad1": "dd", "quad2": "d",
            "quadfringeIN": "d", "quadfringeOUT": "d", "wedgerotate": "di", "wedgedrift": "di",
            "wedgebend": "didi", "bend1": "dd", "bend2": "d", "bend3": "d", "bend4": "d",
            "bendfringeIN": "d", "bendfringeOUT": "d",
        }[name]
        f.argtypes = [_vp] + [ctypes.c_int if c == "i" else ctypes.c_double for c in types]
        conv = [int if c == "i" else float for c in types]
        f(self.h, *[cv(a) for cv, a in zip(conv, args)])


class RefSC:
    """A reference ``SpaceChargeCalc2p5D`` driven through the harness."""

    def __init__(self, nx, ny, nz, xy_ratio=-1.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = ref().ref_sc_new(nx, ny, nz, float(xy_ratio))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_sc_free(self.h)
            self.h = None

    def track(self, bunch: RefBunch, length: float):
        ref().ref_sc_track(self.h, bunch.h, float(length))

    def grids(self):
        rho = np.zeros(self.nx * self.ny)
        phi = np.zeros(self.nx * self.ny)
        zg = np.zeros(self.nz)
        lim = np.zeros(9)
        ref().ref_sc_grids(self.h, _P(rho), _P(phi), _P(zg), _P(lim))
        return rho.reshape(self.nx, self.ny), phi.reshape(self.nx, self.ny), zg, lim

    def fields(self, x, y, z):
        n = len(x)
        ex, ey, lam = np.zeros(n), np.zeros(n), np.zeros(n)
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        ref().ref_sc_fields(self.h, n, _P(x), _P(y), _P(z), _P(ex), _P(ey), _P(lam))
        return ex, ey, lam


class RefSCrb:
    """A reference ``SpaceChargeCalc2p5Drb`` driven through the harness."""

    def __init__(self, nx, ny, nz, xy_ratio=-1.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = ref().ref_scrb_new(nx, ny, nz, float(xy_ratio))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_scrb_free(self.h)
            self.h = None

    def setLongAveragingPointsN(self, n):
        ref().ref_scrb_set_long_avg(self.h, int(n))

    def track(self, bunch: RefBunch, length: float, pipe_radius: float):
        ref().ref_scrb_track(self.h, bunch.h, float(length), float(pipe_radius))

    def grids(self):
        rho = np.zeros(self.nx * self.ny)
        phi = np.zeros(self.nx * self.ny)
        zg = np.zeros(self.nz)
        zd = np.zeros(self.nz)
        lim = np.zeros(9)
        ref().ref_scrb_grids(self.h, _P(rho), _P(phi), _P(zg), _P(zd), _P(lim))
        return rho.reshape(self.nx, self.ny), phi.reshape(self.nx, self.ny), zg, zd, lim


class RefBoundary:
    """A reference BaseBoundary2D / ShapedBoundary2D driven through the harness."""

    def __init__(self, np_, nm, shape=None, xdim=0.0, ydim=None):
        self.h = ref().ref_bnd_new(int(np_), int(nm), 0 if shape is None else SHAPES[shape], float(xdim),
                                   float(xdim if ydim is None else ydim))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_bnd_free(self.h)
            self.h = None

    def setBoundaryPoint(self, i, x, y):
        ref().ref_bnd_set_point(self.h, int(i), float(x), float(y))

    def initialize(self):
        ref().ref_bnd_initialize(self.h)

    def isInside(self, x, y):
        return ref().ref_bnd_is_inside(self.h, float(x), float(y))

    def data(self):
        head = np.zeros(6)
        bx = np.zeros(4096)
        by = np.zeros(4096)
        ref().ref_bnd_get(self.h, _P(head), _P(bx), _P(by))
        n = int(head[0])
        return head, bx[:n].copy(), by[:n].copy()


def ref_sc_track_bnd(sc: "RefSC", bunch: RefBunch, length: float, bnd: RefBoundary):
    ref().ref_sc_track_bnd(sc.h, bunch.h, float(length), bnd.h)


def ref_bunch_moments(bunch: RefBunch, order, dispersion=0, emitnorm=0):
    """getBunchMoment(i, j), i, j = 0..order, after the reference's
    BunchTwissAnalysis::computeBunchMoments(bunch, order, dispersion,
    emitnorm) (order >= 2)."""
    if order < 2:
        raise ValueError("order >= 2: for order 1 the reference writes outside its moment table")
    out = np.zeros((order + 1) * (order + 1))
    ref().ref_bunch_moments(bunch.h, int(order), int(dispersion), int(emitnorm), _P(out))
    return out.reshape(order + 1, order + 1)


def ref_twiss(bunch: RefBunch):
    """(moments[29], getters[27]) of the reference's BunchTwissAnalysis."""
    out, g = np.zeros(29), np.zeros(27)
    ref().ref_twiss(bunch.h, _P(out), _P(g))
    return out, g


class RefTune:
    """A reference BunchTuneAnalysis driven through the harness."""

    def __init__(self, twiss):
        self.h = ref().ref_tune_new()
        ref().ref_tune_assign(self.h, _P(np.ascontiguousarray(twiss, dtype=np.float64)))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_tune_free(self.h)
            self.h = None

    def analyze(self, bunch: RefBunch):
        ph = np.zeros((6, bunch.n))
        ref().ref_tune_analyze(self.h, bunch.h, _P(ph))
        return ph
