"""Test infrastructure only: a float64 numpy restatement of the learned
denoiser network of the library (py-orbit_gb300/csrc/dn.cu), its loss and
its gradients, against which the tests hold the device forward and
backward kernels.  The network has no counterpart in the reference.

Parameters are one flat array in the library's order: for each of the 14
3x3 convolutions W[cout][cin][3][3] then b[cout]; then the 16 weights and
the bias of the 1x1 output convolution.  The device computes with the 3x3
weights rounded to BF16; `bf16` does that rounding (round to nearest even)
so that both sides use the same weights."""
import numpy as np

CIN = [1, 16, 16, 32, 32, 64, 64, 64, 128, 64, 96, 32, 48, 16]
COUT = [16, 16, 32, 32, 64, 64, 64, 64, 64, 64, 32, 32, 16, 16]


def layout():
    """[(w_off, b_off, cin, cout)] for the 14 convolutions, out_w, out_b, n."""
    off, out = 0, []
    for ci, co in zip(CIN, COUT):
        w = off
        off += ci * co * 9
        out.append((w, off, ci, co))
        off += co
    ow = off
    off += 16
    ob = off
    off += 1
    return out, ow, ob, off


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    v = ((u + r) >> 16) << 16
    return v.astype(np.uint32).view(np.float32).astype(np.float64)


def tf32(a):
    """Round to TF32 (10 mantissa bits; to nearest, ties away from zero, as
    cvt.rna.tf32.f32 does) through float32, as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x1000) & 0xFFFFE000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def unpack(p):
    convs, ow, ob, _ = layout()
    ws = []
    for (w, b, ci, co) in convs:
        W = bf16(p[w:w + ci * co * 9]).reshape(co, ci, 3, 3)
        ws.append((W, np.asarray(p[b:b + co], dtype=np.float64)))
    return ws, np.asarray(p[ow:ow + 16], dtype=np.float64), float(p[ob])


def conv3(x, W, b):
    n, ci, h, w = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    out = np.zeros((n, W.shape[0], h, w))
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("oi,niyx->noyx", W[:, :, ky, kx], xp[:, :, ky:ky + h, kx:kx + w])
    return out + b[None, :, None, None]


def conv3_bwd(x, W, dy):
    n, ci, h, w = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dW = np.zeros_like(W)
    dxp = np.zeros_like(xp)
    for ky in range(3):
        for kx in range(3):
            dW[:, :, ky, kx] = np.einsum("noyx,niyx->oi", dy, xp[:, :, ky:ky + h, kx:kx + w])
            dxp[:, :, ky:ky + h, kx:kx + w] += np.einsum("oi,noyx->niyx", W[:, :, ky, kx], dy)
    return dW, dy.sum(axis=(0, 2, 3)), dxp[:, :, 1:-1, 1:-1]


def pool(x):
    return 0.25 * (x[:, :, 0::2, 0::2] + x[:, :, 1::2, 0::2] + x[:, :, 0::2, 1::2] + x[:, :, 1::2, 1::2])


def pool_bwd(dy):
    return 0.25 * np.repeat(np.repeat(dy, 2, axis=2), 2, axis=3)


def up(x):
    return np.repeat(np.repeat(x, 2, axis=2), 2, axis=3)


def up_bwd(dy):
    return dy[:, :, 0::2, 0::2] + dy[:, :, 1::2, 0::2] + dy[:, :, 0::2, 1::2] + dy[:, :, 1::2, 1::2]


def forward(p, x0, tf32_inputs=False):
    """Network output and the activations the backward pass needs.  With
    tf32_inputs, the input of every 3x3 convolution is rounded to TF32 (the
    device's tensor-core layers do so; their weights are BF16, exact in
    TF32)."""
    ws, ow, ob = unpack(p)
    A = {"x0": np.asarray(x0, dtype=np.float64)}

    def c(name, src, k):
        a = tf32(A[src]) if tf32_inputs else A[src]
        A[name] = np.maximum(conv3(a, *ws[k]), 0.0)

    c("a1", "x0", 0); c("s1", "a1", 1); A["p1"] = pool(A["s1"])
    c("a2", "p1", 2); c("s2", "a2", 3); A["p2"] = pool(A["s2"])
    c("a3", "p2", 4); c("s3", "a3", 5); A["p3"] = pool(A["s3"])
    c("a4", "p3", 6); c("b4", "a4", 7)
    A["c3"] = np.concatenate([up(A["b4"]), A["s3"]], axis=1)
    c("d3a", "c3", 8); c("d3", "d3a", 9)
    A["c2"] = np.concatenate([up(A["d3"]), A["s2"]], axis=1)
    c("d2a", "c2", 10); c("d2", "d2a", 11)
    A["c1"] = np.concatenate([up(A["d2"]), A["s1"]], axis=1)
    c("d1a", "c1", 12); c("d1", "d1a", 13)
    A["y"] = A["x0"] + ob + np.einsum("c,ncyx->nyx", ow, A["d1"])[:, None]
    return A["y"], A


def loss_and_grads(p, x0, t, weights=None, tf32_operands=False):
    """The loss, the flat parameter gradient and the output.  Loss: the mean
    squared error, or with `weights` (w_0..w_L) the multi-scale loss
    sum_s w_s mean((P^s y - P^s t)^2), P the 2x2 average pooling, whose
    gradient is sum_s w_s (P^T)^s 2 (P^s y - P^s t) / n_s.  With
    tf32_operands, the operands the device's batched tensor-core layers
    round to TF32 are rounded here too: the input of every 3x3 convolution
    in the forward pass, and in the backward pass the layer input and the
    output gradient entering the weight and data gradients (the bias
    gradient sums the unrounded output gradient)."""
    ws, ow, ob = unpack(p)
    y, A = forward(p, x0, tf32_inputs=tf32_operands)
    t = np.asarray(t, dtype=np.float64)
    n = y.size
    if not weights:
        loss = float(((y - t) ** 2).sum() / n)
        dy = 2.0 * (y - t) / n
    else:
        loss = 0.0
        dy = np.zeros_like(y)
        ys, ts = y, t
        for s, w in enumerate(weights):
            if s > 0:
                ys, ts = pool(ys), pool(ts)
            e = ys - ts
            loss += float(w * (e ** 2).sum() / e.size)
            g = 2.0 * w * e / e.size
            for _ in range(s):
                g = pool_bwd(g)
            dy = dy + g
    convs, owo, obo, total = layout()
    g = np.zeros(total)
    g[owo:owo + 16] = np.einsum("nyx,ncyx->c", dy[:, 0], A["d1"])
    g[obo] = dy.sum()
    D = {"d1": ow[None, :, None, None] * dy}
    srcs = ["x0", "a1", "p1", "a2", "p2", "a3", "p3", "a4", "c3", "d3a", "c2", "d2a", "c1", "d1a"]
    outs = ["a1", "s1", "a2", "s2", "a3", "s3", "a4", "b4", "d3a", "d3", "d2a", "d2", "d1a", "d1"]

    def cb(k):
        dpre = D[outs[k]] * (A[outs[k]] > 0)
        dW, db, dx = conv3_bwd(A[srcs[k]], ws[k][0], dpre)
        if tf32_operands:
            dW, _, dx = conv3_bwd(tf32(A[srcs[k]]), ws[k][0], tf32(dpre))
        w, b, ci, co = convs[k]
        g[w:w + ci * co * 9] = dW.ravel()
        g[b:b + co] = db
        D[srcs[k]] = D.get(srcs[k], 0) + dx

    cb(13); cb(12)
    D["d2"] = up_bwd(D["c1"][:, :32]); D["s1"] = D["c1"][:, 32:].copy()
    cb(11); cb(10)
    D["d3"] = up_bwd(D["c2"][:, :64]); D["s2"] = D["c2"][:, 64:].copy()
    cb(9); cb(8)
    D["b4"] = up_bwd(D["c3"][:, :64]); D["s3"] = D["c3"][:, 64:].copy()
    cb(7); cb(6)
    D["s3"] = D["s3"] + pool_bwd(D["p3"])
    cb(5); cb(4)
    D["s2"] = D["s2"] + pool_bwd(D["p2"])
    cb(3); cb(2)
    D["s1"] = D["s1"] + pool_bwd(D["p1"])
    cb(1); cb(0)
    return loss, g, y
