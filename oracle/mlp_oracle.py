"""TEST INFRASTRUCTURE ONLY — FP64 numpy restatement of the tau / block-shape
MLP of sptc-smat_gb300/csrc/mlp.cu (64-128-128-12, ReLU, two softmax heads:
logits 0..8 tau, 9..11 block shape; loss = sum of the heads' cross-entropies,
mean over the batch), used to check the GPU gradients."""
from __future__ import annotations

import numpy as np

IN, H, OUT, TAU = 64, 128, 12, 9
SIZES = [("W1", (IN, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, OUT)), ("b3", (OUT,))]


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SIZES])


def loss_and_grad(p, X, yt, yb):
    P = unpack(p)
    X = np.asarray(X, np.float64)
    B = X.shape[0]
    z1 = X @ P["W1"] + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"] + P["b2"]
    h2 = np.maximum(z2, 0)
    L = h2 @ P["W3"] + P["b3"]
    dL = np.zeros_like(L)
    loss = 0.0
    for lo, hi, y in ((0, TAU, np.asarray(yt)), (TAU, OUT, TAU + np.asarray(yb))):
        seg = L[:, lo:hi]
        m = seg.max(1, keepdims=True)
        lse = m[:, 0] + np.log(np.exp(seg - m).sum(1))
        p_ = np.exp(seg - lse[:, None])
        oh = np.zeros_like(seg)
        oh[np.arange(B), y - lo] = 1.0
        dL[:, lo:hi] = (p_ - oh) / B
        loss += float(np.mean(lse - L[np.arange(B), y]))
    g = {"W3": h2.T @ dL, "b3": dL.sum(0)}
    dh2 = (dL @ P["W3"].T) * (h2 > 0)
    g["W2"], g["b2"] = h1.T @ dh2, dh2.sum(0)
    dh1 = (dh2 @ P["W2"].T) * (h1 > 0)
    g["W1"], g["b1"] = X.T @ dh1, dh1.sum(0)
    return loss, pack(g), L
