"""Host-side checks of the denoiser's evaluation measures (no GPU): the force
error is linear in the density error and weights long wavelengths by 1/k^2,
so a beam-scale density error moves particles far more than a grid-scale one
of the same size."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _disk(n=64, r=12.0):
    i = torch.arange(n, dtype=torch.float64) - (n - 1) / 2
    return ((i[:, None] ** 2 + i[None, :] ** 2) <= r * r).double()[None, None]


def test_force_error_zero_and_linear():
    from orbit_gb300.denoiser import force_error
    t = _disk()
    rel, spec = force_error(t.clone(), t)
    assert rel == 0.0 and max(spec) == 0.0
    rel2, _ = force_error(2.0 * t, t)  # error = t itself: its force equals the target's
    assert abs(rel2 - 1.0) < 1e-12
    rel3, _ = force_error(3.0 * t, t)
    assert abs(rel3 - 4.0) < 1e-12


def test_uniform_disk_force_is_linear_inside():
    """Gauss's law for the -ln(r)/2 kernel: inside a uniform disk the field
    is radial and proportional to r, which the doubled-grid convolution
    reproduces away from the disk's edge."""
    from orbit_gb300 import denoiser as D
    n = 64
    t = _disk(n, 20.0)
    z = torch.zeros_like(t)
    # the error of a zero image is minus the target: recover the target's force
    rel, _ = D.force_error(z, t)
    assert abs(rel - 1.0) < 1e-12
    import torch.fft as F
    i = torch.arange(2 * n, dtype=torch.float64)
    i = torch.minimum(i, 2 * n - i)
    G = -0.5 * torch.log((i[:, None] ** 2 + i[None, :] ** 2).clamp(min=1.0))
    G[0, 0] = 0.0
    p = torch.zeros(2 * n, 2 * n, dtype=torch.float64)
    p[:n, :n] = t[0, 0]
    phi = F.irfft2(F.rfft2(p) * F.rfft2(G), s=(2 * n, 2 * n))[:n, :n]
    ex = (phi[2:, 1:-1] - phi[:-2, 1:-1]).numpy()
    c = (n - 1) / 2
    xs = np.arange(1, n - 1) - c
    row = ex[:, n // 2 - 1]
    inner = np.abs(xs) < 10
    slope = np.polyfit(xs[inner], row[inner], 1)[0]
    assert np.max(np.abs(row[inner] - slope * xs[inner])) < 0.03 * np.max(np.abs(row[inner]))
    assert slope < 0  # -grad(phi) points outward: phi falls off, its difference is negative


def test_long_wavelengths_dominate_the_force_error():
    from orbit_gb300.denoiser import force_error
    n = 64
    t = _disk(n, 20.0) + 0.5
    i = torch.arange(n, dtype=torch.float64)
    checker = ((i[:, None] + i[None, :]) % 2 * 2 - 1)[None, None]
    bump = torch.exp(-((i[:, None] - 40) ** 2 + (i[None, :] - 28) ** 2) / (2 * 8.0 ** 2))[None, None]
    bump = bump - bump.mean()
    bump = bump * (checker.norm() / bump.norm())  # same density error energy
    f_checker, s_checker = force_error(t + 0.01 * checker, t)
    f_bump, s_bump = force_error(t + 0.01 * bump, t)
    assert f_bump > 100 * f_checker
    assert int(np.argmax(s_checker)) == len(s_checker) - 1  # |k| = 0.707: the top band
    assert int(np.argmax(s_bump)) <= 1
