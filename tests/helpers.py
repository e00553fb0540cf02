"""Shared helpers of the test-suite: tolerances, golden fixtures and the
oracle runners."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# Required parity (max-norm relative): potential and kicks 1e-12,
# coordinates after 100 kicks 1e-10.
TOL_FIELD = 1e-12
TOL_COORD = 1e-10


def rel_err(a, b):
    """max |a - b| / max |b| (max-norm relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if a.size else 0.0
    if den == 0.0:
        return float(num)
    return float(num / den)


def coord_err(a, b):
    """Worst per-coordinate max-norm relative error of (6, n) arrays."""
    return max(rel_err(a[c], b[c]) for c in range(6))


def kick_delta_tol(p_after, dp_ref):
    """Tolerance on a kick read back from coordinates, dp = p_after - p_before.

    The kick itself is held to TOL_FIELD, but the coordinate stores
    fl(p_before + kick): that addition rounds by up to half an ulp of
    p_after, in this code and in the reference alike, and the subtraction
    that recovers the kick keeps that rounding.  Relative to max |kick| the
    two roundings add 2 * 2^-53 max|p_after| / max|kick|; for a 1 mrad
    angle kicked by 1e-5 that is 2.2e-14.  The bound is that term plus
    TOL_FIELD."""
    den = float(np.max(np.abs(dp_ref)))
    if den == 0.0:
        return TOL_FIELD
    return TOL_FIELD + 2.0 * 2.0 ** -53 * float(np.max(np.abs(p_after))) / den


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def kin_sync(kin, macrosize):
    """Oracle sync struct from the golden kinematics vector
    (beta, gamma, momentum, kin_energy, mass, classical_radius, time)."""
    import oracle as O
    return O.make_sync(beta=kin[0], gamma=kin[1], momentum=kin[2], mass=kin[4], classical_radius=kin[5],
                       macrosize=macrosize)


def parse_sequence(seq):
    """Golden sequence strings ("sc:0.5", "drift:(0.5,)") to python steps."""
    import ast
    out = []
    for s in seq:
        name, _, arg = str(s).partition(":")
        if name == "sc":
            out.append(("sc", float(ast.literal_eval(arg))))
        else:
            out.append((name, tuple(ast.literal_eval(arg))))
    return out


def golden_maps(g):
    """[(map name, args)] of the maps fixture."""
    import ast
    return [(str(n), tuple(ast.literal_eval(str(a)))) for n, a in zip(g["names"], g["args"])]
