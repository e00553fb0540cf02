"""Module ``teapot_base`` (TPB): the TEAPOT maps with the argument tuples of
src/teapot/wrap_teapotbase.cc:25-512, each one GPU kernel over the bunch.

While a lattice is being recorded for fused execution the bunch argument is
a recorder (orbit.teapot.recording) and the call is appended to the
program instead of being executed.
"""
from __future__ import annotations

from orbit_gb300 import OP

_OPS = {
    "rotatexy": (OP["ROTXY"], "d"), "drift": (OP["DRIFT"], "d"), "wrapbunch": (OP["WRAP"], "d"),
    "kick": (OP["KICK"], "ddd"), "multp": (OP["MULTP"], "idi"), "multpfringeIN": (OP["MPFRIN"], "idi"),
    "multpfringeOUT": (OP["MPFROUT"], "idi"), "quad1": (OP["QUAD1"], "dd"), "quad2": (OP["QUAD2"], "d"),
    "quadfringeIN": (OP["QFRIN"], "d"), "quadfringeOUT": (OP["QFROUT"], "d"),
    "wedgerotate": (OP["WEDGEROT"], "di"), "wedgedrift": (OP["WEDGEDRIFT"], "di"),
    "wedgebend": (OP["WEDGEBEND"], "didi"), "bend1": (OP["BEND1"], "dd"), "bend2": (OP["BEND2"], "d"),
    "bend3": (OP["BEND3"], "d"), "bend4": (OP["BEND4"], "d"), "bendfringeIN": (OP["BFRIN"], "d"),
    "bendfringeOUT": (OP["BFROUT"], "d"),
}


# the maps whose parameters are all doubles (most of them): their program
# tuples are built without the per-argument type dispatch (the lattice walk
# records every map call on every trackBunch)
_ALL_D = {name for name, (_, types) in _OPS.items() if "i" not in types}


def op_tuple(name, args):
    """(code, ints, doubles) of one map call in the program format."""
    code, types = _OPS[name]
    if name in _ALL_D:
        return code, (), tuple(map(float, args))
    ints, dbls = [], []
    for t, a in zip(types, args):
        (ints if t == "i" else dbls).append(int(a) if t == "i" else float(a))
    return code, tuple(ints), tuple(dbls)


def _apply(name, bunch, args):
    code, types = _OPS[name]
    if len(args) < len(types):
        raise TypeError("teapot_base.%s: expected %d parameters after the bunch" % (name, len(types)))
    args = args[: len(types)]
    rec = getattr(bunch, "_record_op", None)
    if rec is not None:
        rec(*op_tuple(name, args))
        return None
    dev = bunch._device_bunch()
    dev.tpb(name, *args)
    bunch._device_modified()
    return None


def rotatexy(bunch, angle):
    return _apply("rotatexy", bunch, (angle,))


def drift(bunch, length):
    return _apply("drift", bunch, (length,))


def wrapbunch(bunch, length):
    return _apply("wrapbunch", bunch, (length,))


def kick(bunch, kx, ky, kE, useCharge=1):
    return _apply("kick", bunch, (kx, ky, kE))


def multp(bunch, pole, kl, skew, useCharge=1):
    return _apply("multp", bunch, (pole, kl, skew))


def multpfringeIN(bunch, pole, kl, skew, useCharge=1):
    return _apply("multpfringeIN", bunch, (pole, kl, skew))


def multpfringeOUT(bunch, pole, kl, skew, useCharge=1):
    return _apply("multpfringeOUT", bunch, (pole, kl, skew))


def quad1(bunch, length, kq, useCharge=1):
    return _apply("quad1", bunch, (length, kq))


def quad2(bunch, length):
    return _apply("quad2", bunch, (length,))


def quad3(bunch, length, kq, useCharge=1):
    """Empty in the reference (teapotbase.cc:761-764)."""
    return None


def quadfringeIN(bunch, kq, useCharge=1):
    return _apply("quadfringeIN", bunch, (kq,))


def quadfringeOUT(bunch, kq, useCharge=1):
    return _apply("quadfringeOUT", bunch, (kq,))


def wedgerotate(bunch, e, frinout):
    return _apply("wedgerotate", bunch, (e, frinout))


def wedgedrift(bunch, e, inout):
    return _apply("wedgedrift", bunch, (e, inout))


def wedgebend(bunch, e, inout, rho, nsteps):
    return _apply("wedgebend", bunch, (e, inout, rho, nsteps))


def bend1(bunch, length, th):
    return _apply("bend1", bunch, (length, th))


def bend2(bunch, length):
    return _apply("bend2", bunch, (length,))


def bend3(bunch, th):
    return _apply("bend3", bunch, (th,))


def bend4(bunch, th):
    return _apply("bend4", bunch, (th,))


def bendfringeIN(bunch, rho):
    return _apply("bendfringeIN", bunch, (rho,))


def bendfringeOUT(bunch, rho):
    return _apply("bendfringeOUT", bunch, (rho,))


def _not_built(name):
    def f(*args, **kw):
        raise NotImplementedError("teapot_base.%s is outside the GPU hot path and is not built" % name)
    f.__name__ = name
    return f


soln = _not_built("soln")
wedgebendCF = _not_built("wedgebendCF")
RingRF = _not_built("RingRF")
drifti = _not_built("drifti")
