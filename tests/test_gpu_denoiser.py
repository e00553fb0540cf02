"""The denoiser network's device kernels (hand-written BF16-weight
convolutions, pooling, upsampling, loss and Adam) against the float64
numpy restatement in oracle/dn_oracle.py, on two 32x32 images.

Tolerances: the device accumulates in FP32, the oracle in float64, both
with the same BF16 convolution weights: output 1e-5 relative (max-norm),
loss 1e-5, every layer's weight and bias gradients 1e-4 (max-norm relative
per layer)."""
import numpy as np
import pytest

import dn_oracle as D

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _net(h=32, w=32, nb=2, seed=3):
    import torch
    from orbit_gb300 import DeviceDenoiser
    net = DeviceDenoiser(h, w, max_batch=nb, seed=seed)
    rng = np.random.default_rng(seed)
    p = net.get_params()
    # non-zero biases and output weights so every path carries gradient
    convs, ow, ob, n = D.layout()
    for (wo, bo, ci, co) in convs:
        p[bo:bo + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.2, 16)
    net.set_params(p)
    x = rng.uniform(0.0, 2.0, (nb, 1, h, w)).astype(np.float32)
    t = (x + rng.normal(0, 0.1, x.shape)).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(t).cuda()
    return net, p, x, t, xd, td


def test_gradients_against_oracle():
    import torch
    net, p, x, t, xd, td = _net()
    out = torch.empty_like(xd)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 2, out.data_ptr())
    loss_o, g_o, y_o = D.loss_and_grads(p.astype(np.float64), x, t)
    assert rel(out.cpu().numpy(), y_o) <= 1e-5
    assert abs(loss - loss_o) <= 1e-5 * abs(loss_o)
    convs, ow, ob, n = D.layout()
    for k, (wo, bo, ci, co) in enumerate(convs):
        assert rel(g[wo:wo + ci * co * 9], g_o[wo:wo + ci * co * 9]) <= 1e-4, ("weights", k)
        assert rel(g[bo:bo + co], g_o[bo:bo + co]) <= 1e-4, ("bias", k)
    assert rel(g[ow:ow + 17], g_o[ow:ow + 17]) <= 1e-4
    # a second call gives the same gradients (they are cleared in between;
    # the float atomic sums may round differently)
    loss2, g2 = net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    assert rel(g2, g) <= 1e-6 and abs(loss2 - loss) <= 1e-6 * abs(loss)


def test_forward_matches_gradients_output_and_adam_step():
    import torch
    net, p, x, t, xd, td = _net(h=64, w=32, nb=2, seed=7)
    out = torch.empty_like(xd)
    net.forward(xd.data_ptr(), out.data_ptr(), 2)
    torch.cuda.synchronize()
    _, _, y_o = D.loss_and_grads(p.astype(np.float64), x, t)
    assert rel(out.cpu().numpy(), y_o) <= 1e-5
    # first Adam step: m_hat = g, v_hat = g^2, so p moves by lr g / (|g| + eps)
    loss0, g = net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    lr = 1e-3
    loss1 = net.train_step(xd.data_ptr(), td.data_ptr(), 2, lr)
    assert abs(loss1 - loss0) <= 1e-6 * abs(loss0)
    p1 = net.get_params()
    expect = p.astype(np.float64) - lr * g / (np.abs(g) + 1e-8)
    # (the step's own gradient may differ from g in the last bits: the
    # single-image forward sums input channels with float atomics; where
    # |g| is near the Adam epsilon that changes the step, which stays <= lr)
    big = np.abs(g) > 1e-5
    assert np.abs(p1 - expect)[big].max() <= 1e-6
    assert np.abs(p1.astype(np.float64) - p.astype(np.float64)).max() <= lr * (1 + 1e-4)
    # and the loss goes down over a few steps on this pair
    for _ in range(20):
        last = net.train_step(xd.data_ptr(), td.data_ptr(), 2, lr)
    assert last < loss0


def test_gradients_against_oracle_full_size():
    """The same check at the 128 x 128 size the closure uses (several
    16x16 tiles and weight-gradient splits per layer), one image."""
    import torch
    net, p, x, t, xd, td = _net(h=128, w=128, nb=1, seed=9)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 1)
    loss_o, g_o, y_o = D.loss_and_grads(p.astype(np.float64), x, t)
    assert abs(loss - loss_o) <= 1e-5 * abs(loss_o)
    convs, ow, ob, n = D.layout()
    for k, (wo, bo, ci, co) in enumerate(convs):
        assert rel(g[wo:wo + ci * co * 9], g_o[wo:wo + ci * co * 9]) <= 1e-4, ("weights", k)
        assert rel(g[bo:bo + co], g_o[bo:bo + co]) <= 1e-4, ("bias", k)
    assert rel(g[ow:ow + 17], g_o[ow:ow + 17]) <= 1e-4


def test_multiscale_loss_gradients_against_oracle():
    """The multi-scale training loss (weights 4^s over the output and three
    2x2 poolings) on the device against the oracle: loss 1e-5, gradients
    1e-4, as the mean-squared-error test."""
    import torch
    net, p, x, t, xd, td = _net()
    wts = [1.0, 4.0, 16.0, 64.0]
    net.set_loss(wts)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    loss_o, g_o, _ = D.loss_and_grads(p.astype(np.float64), x, t, weights=wts)
    assert abs(loss - loss_o) <= 1e-5 * abs(loss_o)
    convs, ow, ob, n = D.layout()
    for k, (wo, bo, ci, co) in enumerate(convs):
        assert rel(g[wo:wo + ci * co * 9], g_o[wo:wo + ci * co * 9]) <= 1e-4, ("weights", k)
        assert rel(g[bo:bo + co], g_o[bo:bo + co]) <= 1e-4, ("bias", k)
    assert rel(g[ow:ow + 17], g_o[ow:ow + 17]) <= 1e-4
    # back to the mean squared error
    net.set_loss(None)
    loss_m, _ = net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    loss_mo, _, _ = D.loss_and_grads(p.astype(np.float64), x, t)
    assert abs(loss_m - loss_mo) <= 1e-5 * abs(loss_mo)
