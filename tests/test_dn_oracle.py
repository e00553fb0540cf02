"""The numpy restatement of the denoiser network (the oracle of the
device kernels): its analytic gradients against central finite
differences on a small image, and the BF16 rounding it shares with the
device."""
import numpy as np

import dn_oracle as D


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = D.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(5)
    convs, ow, ob, n = D.layout()
    assert n == 302561
    # parameters exactly representable in BF16, so that the finite
    # differences (steps of whole BF16 units are too coarse) see a smooth
    # function: perturb only FP32 parameters (biases and the output layer)
    # and check the 3x3 weight gradients through their bilinear structure
    p = np.zeros(n, dtype=np.float32)
    for (w, b, ci, co) in convs:
        p[w:w + ci * co * 9] = D.bf16(rng.normal(0, np.sqrt(2.0 / (9 * ci)), ci * co * 9))
        p[b:b + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.1, 16)
    p[ob] = 0.01
    x = rng.uniform(0, 2, (1, 1, 8, 8))
    t = rng.uniform(0, 2, (1, 1, 8, 8))
    loss, g, _ = D.loss_and_grads(p.astype(np.float64), x, t)
    pd = p.astype(np.float64)
    idx = [ow + 3, ob] + [convs[k][1] + 1 for k in (0, 4, 8, 13)]
    for i in idx:
        h = 1e-6
        a, b = pd.copy(), pd.copy()
        a[i] += h
        b[i] -= h
        fd = (D.loss_and_grads(a, x, t)[0] - D.loss_and_grads(b, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    # 3x3 weights: the loss is a polynomial in each weight; a difference
    # step of a BF16 unit of that weight (exact in both directions)
    for k in (1, 6, 10):
        w = convs[k][0] + 5
        u = float(np.spacing(np.float32(abs(pd[w])))) * 65536.0  # one BF16 unit
        a, b = pd.copy(), pd.copy()
        a[w] += u
        b[w] -= u
        assert D.bf16(a[w:w + 1])[0] == a[w] and D.bf16(b[w:w + 1])[0] == b[w]
        fd = (D.loss_and_grads(a, x, t)[0] - D.loss_and_grads(b, x, t)[0]) / (2 * u)
        assert abs(fd - g[w]) <= 1e-3 * max(1e-3, abs(g[w])) + 1e-9, (k, fd, g[w])


def test_oracle_multiscale_loss_gradient_by_finite_differences():
    """The multi-scale loss (squared errors of the output and of its 2x2
    poolings, weighted 4^s): its gradient with respect to the output bias
    and output weights against central differences, on a 16x16 image (three
    pooling levels)."""
    rng = np.random.default_rng(6)
    convs, ow, ob, n = D.layout()
    p = np.zeros(n)
    for (w, b, ci, co) in convs:
        p[w:w + ci * co * 9] = D.bf16(rng.normal(0, np.sqrt(2.0 / (9 * ci)), ci * co * 9))
        p[b:b + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.1, 16)
    x = rng.uniform(0, 2, (2, 1, 16, 16))
    t = rng.uniform(0, 2, (2, 1, 16, 16))
    wts = [1.0, 4.0, 16.0, 64.0]
    loss, g, y = D.loss_and_grads(p, x, t, weights=wts)
    # the loss itself, from its definition
    ref, ys, ts = 0.0, y, t
    for s, w in enumerate(wts):
        if s:
            ys, ts = D.pool(ys), D.pool(ts)
        ref += w * np.mean((ys - ts) ** 2)
    assert abs(loss - ref) <= 1e-12 * ref
    for i in [ob, ow, ow + 7, convs[13][1] + 2, convs[2][1]]:
        h = 1e-6
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        fd = (D.loss_and_grads(a, x, t, wts)[0] - D.loss_and_grads(b, x, t, wts)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_tf32_rounding_and_the_rounded_operand_model():
    """TF32 rounding (10 mantissa bits, to nearest, ties away from zero) and
    the oracle's model of the batched tensor-core layers: its output is the
    forward pass with TF32 conv inputs, and its gradients differ from the
    unrounded ones by about the TF32 rounding, not more."""
    x = np.array([1.0, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, -2.5, 0.0], dtype=np.float32)
    r = D.tf32(x)
    assert r[0] == 1.0 and r[4] == 0.0 and r[3] == -2.5
    assert r[1] == 1.0 + 2.0 ** -10          # a tie rounds away from zero
    assert r[2] == 1.0 + 2.0 ** -9
    rng = np.random.default_rng(8)
    convs, ow, ob, n = D.layout()
    p = np.zeros(n, dtype=np.float32)
    for (w, b, ci, co) in convs:
        p[w:w + ci * co * 9] = D.bf16(rng.normal(0, np.sqrt(2.0 / (9 * ci)), ci * co * 9))
        p[b:b + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.1, 16)
    x0 = rng.uniform(0.0, 2.0, (1, 1, 16, 16)).astype(np.float32)
    t = (x0 + rng.normal(0, 0.1, x0.shape)).astype(np.float32)
    pd = p.astype(np.float64)
    loss_r, g_r, y_r = D.loss_and_grads(pd, x0, t, tf32_operands=True)
    y_f, _ = D.forward(pd, x0, tf32_inputs=True)
    assert np.array_equal(y_r, y_f)
    loss, g, y = D.loss_and_grads(pd, x0, t)
    assert 0 < np.abs(y_r - y).max() <= 1e-2 * np.abs(y).max()
    assert np.abs(g_r - g).max() <= 5e-2 * np.abs(g).max()
    assert not np.array_equal(g_r, g)
