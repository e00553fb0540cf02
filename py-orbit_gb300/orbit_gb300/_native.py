"""ctypes binding of liborbit_gb300.so (the C ABI declared in
include/orbit_gb300.h).  There is no CPU fallback: if the library is missing
or cannot run, every call raises."""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

ORBIT_OK = 0
ORBIT_ERR_ARG = -1
ORBIT_ERR_EXTENT = -2
ORBIT_ERR_GRID = -3
ORBIT_ERR_CUDA = -4
ORBIT_ERR_NAN = -5
ORBIT_ERR_DEVICE = -6
ORBIT_ERR_NOMEM = -8
ORBIT_ERR_UNSUPPORTED = -9

FORM_PLAIN = 0
FORM_FP32 = 1

GRID_RHO, GRID_PHI, GRID_LONG, GRID_LONG_DERIV = 0, 1, 2, 3

# op codes (ORBIT_OP_* in include/orbit_gb300.h)
OP = dict(DRIFT=1, QUAD1=2, QUAD2=3, QFRIN=4, QFROUT=5, BEND1=6, BEND2=7, BEND3=8, BEND4=9, BFRIN=10,
          BFROUT=11, MULTP=12, MPFRIN=13, MPFROUT=14, ROTXY=15, WRAP=16, KICK=17, WEDGEROT=18,
          WEDGEDRIFT=19, WEDGEBEND=20, SC=32)


class OrbitError(RuntimeError):
    """A non-zero status from liborbit_gb300."""

    def __init__(self, code: int, msg: str):
        super().__init__("orbit_gb300 error %d: %s" % (code, msg))
        self.code = code


class SpaceChargeError(OrbitError):
    """Zero beam extent at a space-charge kick (the reference aborts there)."""


class Sync(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("beta", "gamma", "momentum", "mass", "charge", "classical_radius", "macrosize", "time")]


class Op(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("i0", ctypes.c_int32), ("i1", ctypes.c_int32),
                ("i2", ctypes.c_int32), ("d", ctypes.c_double * 6)]


_lib = None
_lock = threading.Lock()

_SIGS = {
    "orbit_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "orbit_version": (ctypes.c_char_p, []),
    "orbit_device_peaks": (ctypes.c_int, [_dp, _dp]),
    "orbit_device_mul_rates": (ctypes.c_int, [_dp, _dp, _dp]),
    "orbit_softf64_check": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_longlong)]),
    "orbit_bunch_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int]),
    "orbit_bunch_destroy": (ctypes.c_int, [_vp]),
    "orbit_bunch_upload": (ctypes.c_int, [_vp, ctypes.POINTER(_dp), ctypes.c_int]),
    "orbit_bunch_download": (ctypes.c_int, [_vp, ctypes.POINTER(_dp)]),
    "orbit_bunch_upload_device": (ctypes.c_int, [_vp, ctypes.POINTER(_dp), ctypes.c_int]),
    "orbit_bunch_size": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "orbit_bunch_set_sync": (ctypes.c_int, [_vp, ctypes.POINTER(Sync)]),
    "orbit_bunch_get_sync": (ctypes.c_int, [_vp, ctypes.POINTER(Sync)]),
    "orbit_bunch_set_macrosizes": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "orbit_bunch_device_coords": (ctypes.c_int, [_vp, ctypes.POINTER(_dp)]),
    "orbit_bunch_sync": (ctypes.c_int, [_vp]),
    "orbit_bunch_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "orbit_sc2p5d_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_int]),
    "orbit_sc2p5d_destroy": (ctypes.c_int, [_vp]),
    "orbit_sc2p5d_track": (ctypes.c_int, [_vp, _vp, ctypes.c_double]),
    "orbit_sc2p5d_get_grid": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "orbit_sc2p5d_get_limits": (ctypes.c_int, [_vp, _dp]),
    "orbit_sc2p5d_get_sizes": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_int)] * 4),
    "orbit_sc2p5d_set_fused_conv": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "orbit_sc2p5d_set_conv_wait": (ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.c_int]),
    "orbit_sc2p5d_counters": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "orbit_sc2p5drb_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double]),
    "orbit_sc2p5drb_track": (ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_double]),
    "orbit_sc2p5drb_set_long_avg": (ctypes.c_int, [_vp, ctypes.c_int]),
    "orbit_sc2p5drb_get_long_avg": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "orbit_sc2p5drb_beam": (ctypes.c_int, [_vp, _dp]),
    "orbit_sc2p5d_fields": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]),
    "orbit_sc2p5d_track_static": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                 ctypes.POINTER(Sync), _vp]),
    "orbit_program_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.POINTER(Op), ctypes.c_int,
                                            ctypes.POINTER(_vp), ctypes.c_int]),
    "orbit_program_destroy": (ctypes.c_int, [_vp]),
    "orbit_program_set_boundaries": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.c_int]),
    "orbit_bunch_moments": (ctypes.c_int, [_vp, _dp]),
    "orbit_bunch_xy_moments": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "orbit_bunch_tune_analysis": (ctypes.c_int, [_vp, _dp, ctypes.c_double]),
    "orbit_bunch_phase_get": (ctypes.c_int, [_vp, _dp]),
    "orbit_bunch_phase_set": (ctypes.c_int, [_vp, _dp]),
    "orbit_boundary_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int]),
    "orbit_boundary_create_shape": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_double, ctypes.c_double]),
    "orbit_boundary_destroy": (ctypes.c_int, [_vp]),
    "orbit_boundary_set_point": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    "orbit_boundary_initialize": (ctypes.c_int, [_vp]),
    "orbit_boundary_get_point": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "orbit_boundary_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int), _dp, ctypes.POINTER(ctypes.c_int)]),
    "orbit_boundary_is_inside": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double]),
    "orbit_boundary_lsq": (ctypes.c_int, [_vp, _dp]),
    "orbit_boundary_rnorm": (ctypes.c_int, [_vp, _dp]),
    "orbit_sc2p5d_track_boundary": (ctypes.c_int, [_vp, _vp, ctypes.c_double, _vp]),
    "orbit_program_run": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "orbit_program_enqueue": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "orbit_program_launches": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "orbit_program_profile": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_char_p, _dp,
                                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "orbit_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                          ctypes.c_int]),
    "orbit_batch_destroy": (ctypes.c_int, [_vp]),
    "orbit_batch_enqueue": (ctypes.c_int, [_vp, ctypes.c_int]),
    "orbit_batch_sync": (ctypes.c_int, [_vp]),
    "orbit_batch_run": (ctypes.c_int, [_vp, ctypes.c_int]),
    "orbit_batch_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "orbit_batch_class": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "orbit_batch_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "orbit_batch_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "orbit_denoiser_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_ulonglong]),
    "orbit_denoiser_destroy": (ctypes.c_int, [_vp]),
    "orbit_sc2p5d_set_denoiser": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_double]),
    "orbit_sc2p5d_denoiser_state": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong),
                                                   ctypes.POINTER(ctypes.c_longlong), _dp]),
    "orbit_sc2p5d_denoiser_reset": (ctypes.c_int, [_vp]),
    "orbit_grid_deposit": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _vp, _vp, ctypes.c_longlong]),
    "orbit_beam_sample": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_ulonglong]),
    "orbit_beam_deposit": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_longlong, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong]),
    "orbit_denoiser_info": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_int)] * 4),
    "orbit_denoiser_get_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "orbit_denoiser_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "orbit_denoiser_forward": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp]),
    "orbit_denoiser_set_tensor_cores": (ctypes.c_int, [_vp, ctypes.c_int]),
    "orbit_denoiser_set_batch_tensor_cores": (ctypes.c_int, [_vp, ctypes.c_int]),
    "orbit_denoiser_tensor_status": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "orbit_denoiser_set_wait_limit": (ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.c_int]),
    "orbit_denoiser_set_loss": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "orbit_nvtx_push": (ctypes.c_int, [ctypes.c_char_p]),
    "orbit_nvtx_pop": (ctypes.c_int, []),
    "orbit_denoiser_train_step": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_float,
                                                 ctypes.POINTER(ctypes.c_float), _vp]),
    "orbit_denoiser_gradients": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                                ctypes.POINTER(ctypes.c_float), _vp, _vp]),
    "orbit_batch_profile": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, _dp, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)]),
}

_D, _I = ctypes.c_double, ctypes.c_int
TPB_SIGS = {
    "rotatexy": [_D], "drift": [_D], "wrapbunch": [_D], "kick": [_D, _D, _D],
    "multp": [_I, _D, _I], "multpfringeIN": [_I, _D, _I], "multpfringeOUT": [_I, _D, _I],
    "quad1": [_D, _D], "quad2": [_D], "quadfringeIN": [_D], "quadfringeOUT": [_D],
    "wedgerotate": [_D, _I], "wedgedrift": [_D, _I], "wedgebend": [_D, _I, _D, _I],
    "bend1": [_D, _D], "bend2": [_D], "bend3": [_D], "bend4": [_D],
    "bendfringeIN": [_D], "bendfringeOUT": [_D],
}
for _name, _args in TPB_SIGS.items():
    _SIGS["orbit_tpb_" + _name] = (ctypes.c_int, [_vp] + _args)


def exported_symbols():
    """Every entry point include/orbit_gb300.h declares."""
    return sorted(_SIGS)


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (building first if needed) liborbit_gb300.so and bind signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not os.path.exists(path):
            if not build_if_missing:
                raise ImportError("liborbit_gb300.so is not built (run __graft_entry__.build())")
            _build.build_library()
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def last_error() -> str:
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.orbit_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != ORBIT_OK:
        msg = last_error()
        if rc == ORBIT_ERR_EXTENT:
            raise SpaceChargeError(rc, msg)
        raise OrbitError(rc, msg)
    return rc


def call(name: str, *args):
    return check(getattr(load(), name)(*args))
