"""CPU restatement of the learned residual network (forward and backward).

TEST INFRASTRUCTURE ONLY: the checker for the GPU's tcgen05 MLP kernels.
The network has no counterpart in grav_sim; this module restates its
mathematics in numpy FP64, rounding to BF16 exactly where the GPU feeds a
tensor-core operand (inputs, weights, hidden activations, back-propagated
deltas), so the GPU result differs only by FP32 accumulation order and the
hardware exp.

Parameter layout (FP32, contiguous): W1[64][32] b1[64] W2[64][64] b2[64]
W3[64][64] b3[64] W4[16][64] b4[16]; the loss is mean over samples of the
squared error summed over the 3 outputs.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT, OUT_PAD = 32, 64, 3, 16
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
         ("b3", (H,)), ("W4", (OUT_PAD, H)), ("b4", (OUT_PAD,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + k], dtype=np.float64).reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).ravel() for name, _ in SIZES])


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(v):
    return v / (1.0 + np.exp(-v))


def silu_grad(v):
    s = 1.0 / (1.0 + np.exp(-v))
    return s * (1.0 + v * (1.0 - s))


def forward(p, x, keep=False):
    P = unpack(p)
    X = bf16(x)
    W = [bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3"]), bf16(P["W4"])]
    b = [P["b1"], P["b2"], P["b3"], P["b4"]]
    acts, pre = [X], []
    h = X
    for l in range(3):
        v = h @ W[l].T + b[l]
        pre.append(v)
        h = bf16(silu(v))
        acts.append(h)
    out = h @ W[3].T + b[3]
    pred = out[:, :OUT]
    if keep:
        return pred, (W, b, acts, pre)
    return pred


def gradients(p, x, t):
    """(gradient vector, loss sum) of mean_n sum_k (pred - t)^2."""
    n = x.shape[0]
    pred, (W, b, acts, pre) = forward(p, x, keep=True)
    err = pred - t
    loss_sum = float((err * err).sum())
    d = np.zeros((n, OUT_PAD))
    d[:, :OUT] = 2.0 / n * err
    g = {"b4": d.sum(0)}
    g["b4"][OUT:] = 0.0
    db = bf16(d)
    g["W4"] = db.T @ acts[3]
    g["W4"][OUT:] = 0.0
    for l in (2, 1, 0):
        dx = db @ W[l + 1]
        d = dx * silu_grad(pre[l])
        g[f"b{l + 1}"] = d.sum(0)
        db = bf16(d)
        g[f"W{l + 1}"] = db.T @ acts[l]
    return pack(g).astype(np.float64), loss_sum
