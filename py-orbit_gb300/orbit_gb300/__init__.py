"""orbit_gb300: GB300-native (sm_103a) PyORBIT 2.5D space-charge and TEAPOT
tracking hot path behind the C ABI of include/orbit_gb300.h.

The reference-compatible Python modules live beside this package
(``bunch``, ``spacecharge``, ``orbit.*``); this package holds the thin
native layer they call.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import (FORM_FP32, FORM_PLAIN, OP, OrbitError, SpaceChargeError, Sync, call, load,
                      library_path)

__all__ = ["DeviceBunch", "DeviceSC2p5D", "DeviceSC2p5Drb", "DeviceBoundary", "DeviceProgram", "DeviceBatch", "DeviceDenoiser", "OrbitError", "SpaceChargeError", "load",
           "FORM_PLAIN", "FORM_FP32", "OP", "library_path", "version"]

_dp = ctypes.POINTER(ctypes.c_double)


def version() -> str:
    return load().orbit_version().decode()


def device_peaks():
    """(FP64 FMA TFLOP/s, copy GB/s) measured on the current GPU."""
    f, g = ctypes.c_double(), ctypes.c_double()
    call("orbit_device_peaks", ctypes.byref(f), ctypes.byref(g))
    return f.value, g.value


def device_mul_rates():
    """Binary64 multiply rates (G multiplies/s) on the current GPU: FP64 pipe
    alone, integer pipes alone (the correctly rounded integer multiply of
    the maps), half on each."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    call("orbit_device_mul_rates", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def softf64_check(n, seed=1):
    """Mismatch counts (mul, add, fma, scale2, to_float, from_float) of the
    integer-pipe binary64 routines against the hardware instructions on n
    generated device cases."""
    out = (ctypes.c_longlong * 6)()
    call("orbit_softf64_check", ctypes.c_longlong(n), ctypes.c_ulonglong(seed), out)
    return tuple(out)


def _ptr_array(arrs):
    return (_dp * 6)(*[a.ctypes.data_as(_dp) for a in arrs])


class DeviceBunch:
    """A device-resident SoA bunch (six FP64 arrays in HBM)."""

    def __init__(self, capacity: int = 0):
        h = ctypes.c_void_p()
        call("orbit_bunch_create", ctypes.byref(h), int(capacity))
        self.h = h
        self._n = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_bunch_destroy(h)
            self.h = None

    @property
    def n(self) -> int:
        return self._n

    def upload(self, soa: np.ndarray):
        soa = np.ascontiguousarray(soa, dtype=np.float64)
        if soa.ndim != 2 or soa.shape[0] != 6:
            raise ValueError("expected a (6, n) array")
        n = soa.shape[1]
        rows = [np.ascontiguousarray(soa[c]) for c in range(6)]
        call("orbit_bunch_upload", self.h, _ptr_array(rows), n)
        self._n = n
        # the upload is asynchronous from pinned or pageable memory; make the
        # host arrays' lifetime irrelevant by waiting here
        call("orbit_bunch_sync", self.h)

    def upload_rows(self, rows, n: int):
        """Upload from six host arrays without copying them into one block."""
        call("orbit_bunch_upload", self.h, _ptr_array(rows), int(n))
        self._n = int(n)

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((6, self._n), dtype=np.float64)
        rows = [out[c] for c in range(6)]
        if not all(r.flags.c_contiguous for r in rows):
            raise ValueError("output rows must be contiguous")
        call("orbit_bunch_download", self.h, _ptr_array(rows))
        return out

    def download_rows(self, rows):
        call("orbit_bunch_download", self.h, _ptr_array(rows))

    def set_sync(self, s: Sync):
        call("orbit_bunch_set_sync", self.h, ctypes.byref(s))

    def get_sync(self) -> Sync:
        s = Sync()
        call("orbit_bunch_get_sync", self.h, ctypes.byref(s))
        return s

    def set_macrosizes(self, m):
        if m is None:
            call("orbit_bunch_set_macrosizes", self.h, None, 0)
        else:
            m = np.ascontiguousarray(m, dtype=np.float64)
            call("orbit_bunch_set_macrosizes", self.h, m.ctypes.data_as(_dp), m.shape[0])

    def sync(self):
        call("orbit_bunch_sync", self.h)

    # ------------------------------------------------- diagnostics
    def moments(self) -> np.ndarray:
        """{count, total macrosize, <c_i>[6], <c_i c_j> (i >= j)[21]}: the
        sums of BunchTwissAnalysis::analyzeBunch reduced on the device."""
        out = np.zeros(29)
        call("orbit_bunch_moments", self.h, out.ctypes.data_as(_dp))
        return out

    def xy_moments(self, order: int, params) -> np.ndarray:
        """The (order+1) x (order+1) table of BunchTwissAnalysis::
        computeBunchMoments summed on the device; params = {D, E_kin + mass,
        beta^2, xAvg, yAvg, xbetaterm, ybetaterm} (D = 0 without the
        dispersion term)."""
        out = np.zeros((order + 1) * (order + 1))
        p = np.ascontiguousarray(params, dtype=np.float64)
        call("orbit_bunch_xy_moments", self.h, int(order), p.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
        return out.reshape(order + 1, order + 1)

    def tune_analysis(self, twiss, etot: float):
        """BunchTuneAnalysis::analyzeBunch on the device; twiss = {betax,
        alphax, etax, etapx, betay, alphay}, etot = kinetic energy + mass."""
        tw = np.ascontiguousarray(twiss, dtype=np.float64)
        if tw.shape != (6,):
            raise ValueError("expected six lattice functions")
        call("orbit_bunch_tune_analysis", self.h, tw.ctypes.data_as(_dp), float(etot))

    def phase_get(self) -> np.ndarray:
        """(6, n) rows {xLastPhase, yLastPhase, xLastTune, yLastTune,
        xAction, yAction}."""
        out = np.zeros((6, self._n))
        call("orbit_bunch_phase_get", self.h, out.ctypes.data_as(_dp))
        return out

    def phase_set(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        if rows.shape != (6, self._n):
            raise ValueError("expected a (6, n) array")
        call("orbit_bunch_phase_set", self.h, rows.ctypes.data_as(_dp))

    def stream_ptr(self) -> int:
        """The bunch's cudaStream_t as an integer."""
        v = ctypes.c_void_p()
        call("orbit_bunch_stream", self.h, ctypes.byref(v))
        return v.value or 0

    def device_pointers(self):
        ptrs = (_dp * 6)()
        call("orbit_bunch_device_coords", self.h, ptrs)
        return [ctypes.cast(p, ctypes.c_void_p).value for p in ptrs]

    def tpb(self, name: str, *args):
        conv = [int if t is ctypes.c_int else float for t in _native.TPB_SIGS[name]]
        call("orbit_tpb_" + name, self.h, *[c(a) for c, a in zip(conv, args)])


class DeviceSC2p5D:
    """The device SpaceChargeCalc2p5D (FP64 plain or FP32 form)."""

    def __init__(self, nx: int, ny: int, nz: int, xy_ratio: float = -1.0, form: int = FORM_PLAIN):
        h = ctypes.c_void_p()
        call("orbit_sc2p5d_create", ctypes.byref(h), int(nx), int(ny), int(nz), float(xy_ratio), int(form))
        self.h = h
        self.nx, self.ny, self.nz, self.form = int(nx), int(ny), int(nz), int(form)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_sc2p5d_destroy(h)
            self.h = None

    def track(self, bunch: DeviceBunch, length: float):
        call("orbit_sc2p5d_track", self.h, bunch.h, float(length))

    def track_boundary(self, bunch: DeviceBunch, length: float, boundary: "DeviceBoundary"):
        call("orbit_sc2p5d_track_boundary", self.h, bunch.h, float(length), boundary.h)

    def grid(self, which: int) -> np.ndarray:
        n = self.nz if which in (_native.GRID_LONG, _native.GRID_LONG_DERIV) else self.nx * self.ny
        out = np.empty(n, dtype=np.float64)
        call("orbit_sc2p5d_get_grid", self.h, int(which), out.ctypes.data_as(_dp))
        return out if which in (_native.GRID_LONG, _native.GRID_LONG_DERIV) else out.reshape(self.nx, self.ny)

    def limits(self) -> np.ndarray:
        lim = np.empty(11, dtype=np.float64)
        call("orbit_sc2p5d_get_limits", self.h, lim.ctypes.data_as(_dp))
        return lim

    def set_fused_conv(self, on: bool) -> bool:
        """The convolution of each kick as one cooperative launch (True, the
        default) or as separate kernels; returns whether the fused launch
        will run (orbit_sc2p5d_set_fused_conv)."""
        act = ctypes.c_int()
        call("orbit_sc2p5d_set_fused_conv", self.h, int(bool(on)), ctypes.byref(act))
        return bool(act.value)

    def set_conv_wait(self, polls: int, withhold: int = -1):
        """Barrier wait limit of the fused convolution and its test hook
        (orbit_sc2p5d_set_conv_wait)."""
        call("orbit_sc2p5d_set_conv_wait", self.h, int(polls), int(withhold))

    def set_denoiser(self, dn, check_every: int = 10, bound: float = 0.05):
        """Learned closure (orbit_sc2p5d_set_denoiser); dn None removes it."""
        call("orbit_sc2p5d_set_denoiser", self.h, dn.h if dn is not None else None, int(check_every), float(bound))
        self._dn = dn  # kept alive while the calculator uses it

    def denoiser_state(self):
        """{fallback, checks, trips, last_err} of the learned closure."""
        f, c, t, e = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_double()
        call("orbit_sc2p5d_denoiser_state", self.h, ctypes.byref(f), ctypes.byref(c), ctypes.byref(t), ctypes.byref(e))
        return {"fallback": f.value, "checks": c.value, "trips": t.value, "last_err": e.value}

    def denoiser_reset(self):
        call("orbit_sc2p5d_denoiser_reset", self.h)

    def counters(self):
        """(kicks solved, Green spectra rebuilt) since creation."""
        k, g = ctypes.c_longlong(), ctypes.c_longlong()
        call("orbit_sc2p5d_counters", self.h, ctypes.byref(k), ctypes.byref(g))
        return k.value, g.value

    def fields(self, x, y, z):
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        n = x.shape[0]
        ex, ey, lam = np.empty(n), np.empty(n), np.empty(n)
        call("orbit_sc2p5d_fields", self.h, n, *[a.ctypes.data_as(_dp) for a in (x, y, z, ex, ey, lam)])
        return ex, ey, lam


class DeviceSC2p5Drb(DeviceSC2p5D):
    """The device SpaceChargeCalc2p5Drb (plain FP64 form)."""

    def __init__(self, nx: int, ny: int, nz: int, xy_ratio: float = -1.0):
        h = ctypes.c_void_p()
        call("orbit_sc2p5drb_create", ctypes.byref(h), int(nx), int(ny), int(nz), float(xy_ratio))
        self.h = h
        self.nx, self.ny, self.nz, self.form = int(nx), int(ny), int(nz), FORM_PLAIN

    def track_rb(self, bunch: DeviceBunch, length: float, pipe_radius: float):
        call("orbit_sc2p5drb_track", self.h, bunch.h, float(length), float(pipe_radius))

    def set_long_avg(self, n: int):
        call("orbit_sc2p5drb_set_long_avg", self.h, int(n))

    def get_long_avg(self) -> int:
        v = ctypes.c_int()
        call("orbit_sc2p5drb_get_long_avg", self.h, ctypes.byref(v))
        return v.value

    def beam(self):
        """(a_bunch, x_center, y_center) of the last kick."""
        out = np.zeros(3)
        call("orbit_sc2p5drb_beam", self.h, out.ctypes.data_as(_dp))
        return float(out[0]), float(out[1]), float(out[2])


class DeviceBoundary:
    """A conducting boundary (Boundary2D): points given one by one, or a
    Circle / Ellipse / Rectangle shape."""

    SHAPES = {"Circle": 1, "Ellipse": 2, "Rectangle": 3}

    def __init__(self, n_points: int, n_modes: int, shape=None, xdim: float = 0.0, ydim=None):
        h = ctypes.c_void_p()
        if shape is None:
            call("orbit_boundary_create", ctypes.byref(h), int(n_points), int(n_modes))
        else:
            if shape not in self.SHAPES:
                raise OrbitError(_native.ORBIT_ERR_ARG, "Boundary2D: the shape should be Circle, Ellipse or Rectangle")
            call("orbit_boundary_create_shape", ctypes.byref(h), int(n_points), int(n_modes), self.SHAPES[shape],
                 float(xdim), float(xdim if ydim is None else ydim))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_boundary_destroy(h)
            self.h = None

    def info(self):
        npnt, nm, shape, init = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lim = np.zeros(4)
        call("orbit_boundary_info", self.h, ctypes.byref(npnt), ctypes.byref(nm), ctypes.byref(shape),
             lim.ctypes.data_as(_dp), ctypes.byref(init))
        return npnt.value, nm.value, shape.value, lim, bool(init.value)

    def set_point(self, i, x, y):
        call("orbit_boundary_set_point", self.h, int(i), float(x), float(y))

    def initialize(self):
        call("orbit_boundary_initialize", self.h)

    def get_point(self, i):
        x, y = ctypes.c_double(), ctypes.c_double()
        call("orbit_boundary_get_point", self.h, int(i), ctypes.byref(x), ctypes.byref(y))
        return x.value, y.value

    def is_inside(self, x, y) -> int:
        return _native.load().orbit_boundary_is_inside(self.h, float(x), float(y))

    def lsq(self):
        npnt, nm, _, _, _ = self.info()
        out = np.empty((2 * nm + 1, npnt))
        call("orbit_boundary_lsq", self.h, out.ctypes.data_as(_dp))
        r = ctypes.c_double()
        call("orbit_boundary_rnorm", self.h, ctypes.byref(r))
        return out, r.value


class DeviceDenoiser:
    """The learned denoiser network (orbit_denoiser_*): images are device
    arrays given by address (e.g. ``tensor.data_ptr()``), NCHW float32."""

    def __init__(self, h: int, w: int, max_batch: int = 1, seed: int = 1):
        hd = ctypes.c_void_p()
        call("orbit_denoiser_create", ctypes.byref(hd), int(max_batch), int(h), int(w), int(seed))
        self.h = hd
        n, hh, ww, mb = (ctypes.c_int() for _ in range(4))
        call("orbit_denoiser_info", self.h, ctypes.byref(n), ctypes.byref(hh), ctypes.byref(ww), ctypes.byref(mb))
        self.nparam, self.height, self.width, self.max_batch = n.value, hh.value, ww.value, mb.value

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_denoiser_destroy(h)
            self.h = None

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        call("orbit_denoiser_get_params", self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.nparam,):
            raise ValueError("expected %d parameters" % self.nparam)
        call("orbit_denoiser_set_params", self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    # The stream argument (a cudaStream_t as an integer) orders the network's
    # work after whatever wrote its inputs; 0 is the denoiser's own stream.
    def forward(self, dev_in: int, dev_out: int, nb: int = 1, stream: int = 0):
        call("orbit_denoiser_forward", self.h, ctypes.c_void_p(dev_in), ctypes.c_void_p(dev_out), int(nb),
             ctypes.c_void_p(stream) if stream else None)

    @property
    def tensor_cores(self) -> bool:
        """Single-image forwards run their 3x3 layers on the tensor cores
        (tcgen05, TF32 operands, FP32 accumulation); batches and training
        use the CUDA-core layers."""
        on = ctypes.c_int()
        call("orbit_denoiser_tensor_status", self.h, ctypes.byref(on), None)
        return bool(on.value)

    @tensor_cores.setter
    def tensor_cores(self, on: bool):
        call("orbit_denoiser_set_tensor_cores", self.h, int(bool(on)))

    def set_batch_tensor_cores(self, on: bool = True):
        """Batches (training steps, gradients, batched forwards): the 3x3
        layers' forward, data gradient and weight gradient on the tensor
        cores (TF32 operands, FP32 accumulation).  Off by default."""
        call("orbit_denoiser_set_batch_tensor_cores", self.h, int(bool(on)))

    def tensor_errors(self) -> int:
        """Error bits of the tensor-core layers since the last call (then
        cleared): 1 = a bounded wait gave up, 2 = an MMA had not completed
        after a second wait either.  After any error this network's
        single-image forwards run on the CUDA-core layers."""
        err = ctypes.c_int()
        call("orbit_denoiser_tensor_status", self.h, None, ctypes.byref(err))
        return err.value

    def set_loss(self, weights=None):
        """Training loss: None, the mean squared error; a list of L + 1
        weights, the multi-scale loss sum_s w_s mean((P^s y - P^s t)^2)
        over s = 0..L 2x2 poolings (weights 4^s: a stand-in for the force
        error)."""
        if not weights:
            call("orbit_denoiser_set_loss", self.h, 0, None)
            return
        w = (ctypes.c_float * len(weights))(*[float(v) for v in weights])
        call("orbit_denoiser_set_loss", self.h, len(weights) - 1, w)

    def set_wait_limit(self, cycles: int, withhold_mma: bool = False):
        """Clock-cycle limit of each bounded wait of the tensor-core layers
        (default 2e9); withhold_mma issues no MMA, so the waits run out with
        nothing in flight (for testing the failure path)."""
        call("orbit_denoiser_set_wait_limit", self.h, ctypes.c_longlong(int(cycles)), int(bool(withhold_mma)))

    def train_step(self, dev_in: int, dev_target: int, nb: int, lr: float, want_loss: bool = True, stream: int = 0):
        loss = ctypes.c_float()
        call("orbit_denoiser_train_step", self.h, ctypes.c_void_p(dev_in), ctypes.c_void_p(dev_target), int(nb),
             float(lr), ctypes.byref(loss) if want_loss else None, ctypes.c_void_p(stream) if stream else None)
        return loss.value if want_loss else None

    def gradients(self, dev_in: int, dev_target: int, nb: int, dev_out: int = 0, stream: int = 0):
        """(loss, gradient of every parameter) without an update."""
        g = np.empty(self.nparam, dtype=np.float32)
        loss = ctypes.c_float()
        call("orbit_denoiser_gradients", self.h, ctypes.c_void_p(dev_in), ctypes.c_void_p(dev_target), int(nb),
             g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss),
             ctypes.c_void_p(dev_out) if dev_out else None, ctypes.c_void_p(stream) if stream else None)
        return loss.value, g


class DeviceBatch:
    """Members (program i tracking device bunch i) advanced together; one
    kernel launch per stage per grid class (orbit_batch_*)."""

    def __init__(self, programs, bunches):
        if len(programs) != len(bunches) or not programs:
            raise ValueError("one program per bunch")
        n = len(programs)
        ph = (ctypes.c_void_p * n)(*[p.h.value for p in programs])
        bh = (ctypes.c_void_p * n)(*[b.h.value for b in bunches])
        h = ctypes.c_void_p()
        call("orbit_batch_create", ctypes.byref(h), ph, bh, n)
        self.h = h
        self.programs = list(programs)  # kept alive with the batch
        self.bunches = list(bunches)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_batch_destroy(h)
            self.h = None

    def run(self, turns: int = 1):
        call("orbit_batch_run", self.h, int(turns))

    def enqueue(self, turns: int = 1):
        call("orbit_batch_enqueue", self.h, int(turns))

    def sync(self):
        call("orbit_batch_sync", self.h)

    def info(self):
        """(number of grid classes, kernel launches per captured turn)."""
        nc, nl = ctypes.c_int(), ctypes.c_int()
        call("orbit_batch_info", self.h, ctypes.byref(nc), ctypes.byref(nl))
        return nc.value, nl.value

    def classes(self):
        """Per grid class: {grid, members, dep_threads, dep_chunk,
        pass_threads, pass_chunk, fft_radix2, tuned}."""
        nc, _ = self.info()
        out = []
        for k in range(nc):
            g = (ctypes.c_int * 3)()
            m = ctypes.c_int()
            t = (ctypes.c_int * 6)()
            call("orbit_batch_class", self.h, k, g, ctypes.byref(m), t)
            out.append({"grid": tuple(g), "members": m.value, "dep_threads": t[0], "dep_chunk": t[1],
                        "pass_threads": t[2], "pass_chunk": t[3], "fft_radix2": t[4], "tuned": t[5]})
        return out

    def set_tuning(self, cls, dep_threads, dep_chunk, pass_threads, pass_chunk, fft_radix2):
        t = (ctypes.c_int * 5)(dep_threads, dep_chunk, pass_threads, pass_chunk, fft_radix2)
        call("orbit_batch_set_tuning", self.h, int(cls), t)

    def stream_ptr(self) -> int:
        v = ctypes.c_void_p()
        call("orbit_batch_stream", self.h, ctypes.byref(v))
        return v.value or 0

    def profile(self, max_kinds: int = 32):
        """One eager turn with every launch timed: {kernel kind: (total ms, launches)}."""
        names = ctypes.create_string_buffer(32 * max_kinds)
        ms = (ctypes.c_double * max_kinds)()
        cnt = (ctypes.c_int * max_kinds)()
        nk = ctypes.c_int()
        call("orbit_batch_profile", self.h, max_kinds, names, ms, cnt, ctypes.byref(nk))
        out = {}
        for k in range(nk.value):
            nm = names.raw[32 * k: 32 * k + 32].split(b"\0", 1)[0].decode()
            out[nm] = (ms[k], cnt[k])
        return out


class DeviceProgram:
    """A compiled lattice program: ops (code, (i0,i1,i2), (d0..d5)) plus calculators."""

    def __init__(self, ops, calcs, boundaries=()):
        arr = (_native.Op * max(1, len(ops)))()
        for k, (code, iv, dv) in enumerate(ops):
            arr[k].code = int(code)
            iv = list(iv) + [0, 0, 0]
            arr[k].i0, arr[k].i1, arr[k].i2 = int(iv[0]), int(iv[1]), int(iv[2])
            dv = list(dv) + [0.0] * 6
            for j in range(6):
                arr[k].d[j] = float(dv[j])
        hs = (ctypes.c_void_p * max(1, len(calcs)))(*[c.h.value for c in calcs])
        h = ctypes.c_void_p()
        call("orbit_program_create", ctypes.byref(h), arr, len(ops), hs, len(calcs))
        self.h = h
        self.calcs = list(calcs)  # keep the calculators alive
        self.nops = len(ops)
        self.boundaries = list(boundaries)  # kept alive with the program
        if self.boundaries:
            bh = (ctypes.c_void_p * len(self.boundaries))(*[b.h.value for b in self.boundaries])
            call("orbit_program_set_boundaries", self.h, bh, len(self.boundaries))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.orbit_program_destroy(h)
            self.h = None

    def run(self, bunch: DeviceBunch, turns: int = 1):
        call("orbit_program_run", self.h, bunch.h, int(turns))

    def enqueue(self, bunch: DeviceBunch, turns: int = 1):
        """Enqueue without waiting; bunch.sync() waits and reports errors."""
        call("orbit_program_enqueue", self.h, bunch.h, int(turns))

    def launches_per_turn(self) -> int:
        v = ctypes.c_int()
        call("orbit_program_launches", self.h, ctypes.byref(v))
        return v.value

    def profile(self, bunch: DeviceBunch, max_kinds: int = 32):
        """One eager turn with every launch timed by CUDA events:
        {kernel kind: (total ms, launches)}."""
        names = ctypes.create_string_buffer(32 * max_kinds)
        ms = (ctypes.c_double * max_kinds)()
        cnt = (ctypes.c_int * max_kinds)()
        nk = ctypes.c_int()
        call("orbit_program_profile", self.h, bunch.h, max_kinds, names, ms, cnt, ctypes.byref(nk))
        out = {}
        for k in range(nk.value):
            nm = names.raw[32 * k: 32 * k + 32].split(b"\0", 1)[0].decode()
            out[nm] = (ms[k], cnt[k])
        return out
