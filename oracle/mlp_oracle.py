"""TEST INFRASTRUCTURE. CPU oracle of the learned QED weight's network
(hlbl_gb300/csrc/surrogate.cu): forward and backward of the MLP
3 -> 128 -> 128 -> 128 -> 6 (SiLU) and its mean-squared-error loss, in FP64,
with the GPU's numerics as options: the operands of the three tensor-core
layers rounded to BF16 (round to nearest even), as the training GEMMs stage
them. Only tests use it, to check the GPU's gradients.

Parameter layout (FP32 master copy on the GPU): W1[128][3], b1[128],
W2[128][128], b2, W3[128][128], b3, W4[6][128], b4[6].
"""
from __future__ import annotations

import numpy as np

H, NIN, NOUT = 128, 3, 6
SHAPES = [("W1", (H, NIN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
          ("b3", (H,)), ("W4", (NOUT, H)), ("b4", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_and_grad(p, feat, target, round_bf16=True):
    """Mean over rows of sum_j (out - target)^2 and its gradient (layout of p)."""
    P = unpack(p)
    r = bf16 if round_bf16 else (lambda x: np.asarray(x, dtype=np.float64))
    X = np.asarray(feat, dtype=np.float64)
    T = np.asarray(target, dtype=np.float64)
    B = X.shape[0]
    z1 = X @ P["W1"].T + P["b1"]
    h1 = silu(z1)
    z2 = r(h1) @ r(P["W2"]).T + P["b2"]
    h2 = silu(z2)
    z3 = r(h2) @ r(P["W3"]).T + P["b3"]
    h3 = silu(z3)
    o = r(h3) @ r(P["W4"]).T + P["b4"]
    d = o - T
    loss = float(np.sum(d * d) / B)
    do = 2.0 * d / B
    g = {}
    g["W4"] = r(do).T @ r(h3)
    g["b4"] = do.sum(0)
    dh3 = r(do) @ r(P["W4"])
    dz3 = dh3 * dsilu(z3)
    g["W3"] = r(dz3).T @ r(h2)
    g["b3"] = dz3.sum(0)
    dh2 = r(dz3) @ r(P["W3"])
    dz2 = dh2 * dsilu(z2)
    g["W2"] = r(dz2).T @ r(h1)
    g["b2"] = dz2.sum(0)
    dh1 = r(dz2) @ r(P["W2"])
    dz1 = dh1 * dsilu(z1)
    g["W1"] = r(dz1).T @ r(X)
    g["b1"] = dz1.sum(0)
    return loss, pack(g)


def forward(p, feat, round_bf16=True):
    """Network outputs for rows feat[n][3]."""
    P = unpack(p)
    r = bf16 if round_bf16 else (lambda x: np.asarray(x, dtype=np.float64))
    X = np.asarray(feat, dtype=np.float64)
    h1 = silu(X @ P["W1"].T + P["b1"])
    h2 = silu(r(h1) @ r(P["W2"]).T + P["b2"])
    h3 = silu(r(h2) @ r(P["W3"]).T + P["b3"])
    return r(h3) @ r(P["W4"]).T + P["b4"]
