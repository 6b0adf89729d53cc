"""CPU oracle of the learned-preconditioner MLP (test infrastructure only).

No reference counterpart exists (the reference's NJPCG solver is declared only).
The network of include/mps_learned.h restated in numpy, in FP64 arithmetic with the
BF16 roundings the GPU path applies at the same points: weights, network inputs,
hidden activations and back-propagated gradients are rounded to BF16 (round to
nearest even) before each product, accumulation is exact(ish) FP64 here and FP32 on
the tensor cores.  Used by tests/test_gpu_learned.py to check the GPU forward pass,
the gradients of the backward pass and the training loop.

Parameter vector layout: W1[12][128] b1[128] W2[128][128] b2[128] W3[128][128] b3[128]
W4[128][2] b4[2] (34,946 floats).
"""
import numpy as np

FIN, H, FOUT = 12, 128, 2
NPARAMS = FIN * H + H + H * H + H + H * H + H + H * FOUT + FOUT


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = []
    for fi, fo in ((FIN, H), (H, H), (H, H), (H, FOUT)):
        W = p[o:o + fi * fo].reshape(fi, fo)
        o += fi * fo
        b = p[o:o + fo]
        o += fo
        out.append((W, b))
    assert o == NPARAMS
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, keep=False):
    layers = unpack(p)
    h = bf16(X)
    zs, hs = [], [h]
    for li, (W, b) in enumerate(layers):
        z = h @ bf16(W) + b
        if li < 3:
            zs.append(z)
            h = bf16(silu(z))
            hs.append(h)
        else:
            y = z
    return (y, zs, hs) if keep else y


def loss_grad(p, X, T, w1=0.25):
    """Mean loss (y0-t0)^2 + w1 (y1-t1)^2 and its gradient (FP64, BF16 points)."""
    layers = unpack(p)
    y, zs, hs = forward(p, X, keep=True)
    M = X.shape[0]
    e = y - T
    loss = float(np.mean(e[:, 0] ** 2 + w1 * e[:, 1] ** 2))
    dy = np.stack([2.0 / M * e[:, 0], 2.0 / M * w1 * e[:, 1]], 1)
    grads = [None] * 4
    d = bf16(dy)
    for li in range(3, -1, -1):
        W, _ = layers[li]
        dW = hs[li].T @ d
        db = (dy if li == 3 else dz).sum(0)
        grads[li] = (dW, db)
        if li > 0:
            dh = d @ bf16(W).T
            dz = dh * silu_grad(zs[li - 1])
            d = bf16(dz)
    g = []
    for dW, db in grads:
        g.append(dW.ravel())
        g.append(db)
    return loss, np.concatenate(g)
