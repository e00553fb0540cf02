"""Batches on the tensor cores (orbit_denoiser_set_batch_tensor_cores): the
denoiser's 3x3 layers, forward, data gradient and weight gradient, as
tcgen05 MMAs (TF32 operands, FP32 accumulation in tensor memory: every K
stage of a 128-pixel tile for the forward and data gradient, a slice of
the batch's pixels for the weight gradient).

Against the float64 oracle that rounds the same operands to TF32 (every
3x3 convolution's input in the forward pass; the layer input and the
output gradient entering the weight and data gradients) and against the
CUDA-core layers; a short training
run on the tensor cores gains as much as one on the CUDA cores; a bounded
wait that runs out (no MMA issued, a test hook) makes the step report the
error and the network fall back to the CUDA cores.

Tolerances (max-norm relative): output 3e-3 against the oracle and the
CUDA-core forward, as for the single-image tensor-core layers (the MMA's
FP32 accumulation order, not the TF32 operands, sets most of it); loss
1e-3; each layer's weight and bias gradients 2e-2 (they sum products of the
network's activations with output gradients that both carry the forward's
differences)."""
import numpy as np
import pytest

import dn_oracle as D

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _net(h, w, nb, seed):
    import torch
    from orbit_gb300 import DeviceDenoiser
    net = DeviceDenoiser(h, w, max_batch=nb, seed=seed)
    rng = np.random.default_rng(seed)
    p = net.get_params()
    convs, ow, ob, n = D.layout()
    for (wo, bo, ci, co) in convs:
        p[bo:bo + co] = rng.normal(0, 0.05, co)
    p[ow:ow + 16] = rng.normal(0, 0.2, 16)
    net.set_params(p)
    x = rng.uniform(0.0, 2.0, (nb, 1, h, w)).astype(np.float32)
    t = (x + rng.normal(0, 0.1, x.shape)).astype(np.float32)
    return net, p, x, t, torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()


def _forward(net, xd, nb, tcb):
    import torch
    net.set_batch_tensor_cores(tcb)
    out = torch.empty_like(xd)
    net.forward(xd.data_ptr(), out.data_ptr(), nb)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("h,w,nb,seed", [(32, 32, 3, 11), (128, 128, 2, 12)])
def test_batched_forward_against_oracle(h, w, nb, seed):
    """32x32 images in a batch of 3: the 8x8 and 4x4 levels put pixels of
    two images in one 128-pixel tile."""
    net, p, x, t, xd, td = _net(h, w, nb, seed)
    y_tc = _forward(net, xd, nb, True)
    y_o, _ = D.forward(p.astype(np.float64), x, tf32_inputs=True)
    e_o = rel(y_tc, y_o)
    y_cc = _forward(net, xd, nb, False)
    e_cc = rel(y_tc, y_cc)
    print("batched forward: vs oracle %.2e, vs CUDA cores %.2e" % (e_o, e_cc))
    assert e_o <= 3e-3 and e_cc <= 3e-3
    assert rel(y_tc - x, y_cc - x) <= 5e-3
    assert net.tensor_errors() == 0


def test_batched_gradients_against_oracle():
    import torch
    net, p, x, t, xd, td = _net(32, 32, 2, 3)
    net.set_batch_tensor_cores(True)
    out = torch.empty_like(xd)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 2, out.data_ptr())
    loss_o, g_o, y_o = D.loss_and_grads(p.astype(np.float64), x, t, tf32_operands=True)
    e_y = rel(out.cpu().numpy(), y_o)
    e_l = abs(loss - loss_o) / abs(loss_o)
    convs, ow, ob, n = D.layout()
    e_w = max(rel(g[wo:wo + ci * co * 9], g_o[wo:wo + ci * co * 9]) for (wo, bo, ci, co) in convs)
    e_b = max(rel(g[bo:bo + co], g_o[bo:bo + co]) for (wo, bo, ci, co) in convs)
    e_out = rel(g[ow:ow + 17], g_o[ow:ow + 17])
    print("batched gradients: output %.2e loss %.2e weights %.2e biases %.2e output layer %.2e"
          % (e_y, e_l, e_w, e_b, e_out))
    assert e_y <= 3e-3 and e_l <= 1e-3
    assert e_w <= 2e-2 and e_b <= 2e-2 and e_out <= 2e-2
    assert net.tensor_errors() == 0


def test_training_on_tensor_cores_gains_like_cuda_cores():
    """The same short run (512 pairs from the plain calculator, 4 epochs,
    Adam) on each path; held-out gains within 10% of each other and at
    least 2."""
    from orbit_gb300 import DeviceDenoiser
    from orbit_gb300 import denoiser as DN
    X, T, _ = DN.make_pairs(544, seed=7)
    gains = {}
    for tcb in (True, False):
        net = DeviceDenoiser(128, 128, max_batch=16, seed=3)
        DN.train(net, X[:512], T[:512], epochs=4, batch=16, lr=1e-3, tensor_cores=tcb)
        gains[tcb] = DN.evaluate(net, X[512:], T[512:])["gain"]
    print("held-out gain: tensor cores %.2f, CUDA cores %.2f" % (gains[True], gains[False]))
    assert gains[True] >= 2.0
    assert abs(gains[True] / gains[False] - 1) <= 0.1


def test_bounded_wait_runs_out_and_training_falls_back():
    """No MMA issued (test hook): every wait runs out after 2e6 cycles with
    nothing in flight, the step reports the error, and the network runs on
    the CUDA cores from then on (its gradients are then the CUDA-core
    ones)."""
    from orbit_gb300 import OrbitError
    net, p, x, t, xd, td = _net(32, 32, 2, 3)
    ref = _net(32, 32, 2, 3)[0]
    net.set_batch_tensor_cores(True)
    net.set_wait_limit(2_000_000, withhold_mma=True)
    with pytest.raises(OrbitError):
        net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    assert not net.tensor_cores
    net.set_wait_limit(2_000_000_000, withhold_mma=False)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 2)
    loss_r, g_r = ref.gradients(xd.data_ptr(), td.data_ptr(), 2)
    assert rel(g, g_r) <= 1e-6 and abs(loss - loss_r) <= 1e-6 * abs(loss_r)
