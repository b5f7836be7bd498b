"""CHECKER INFRASTRUCTURE (oracle): FP64 restatement of the cons2prim MLP
(disco_gb300/csrc/cuda/mlp.cuh, mlp_train.cuh) -- forward pass, loss and
gradients -- for checking the device's tensor-core kernels.

With bf16=True it rounds the same operands to BF16 that the device feeds
the tensor cores (standardised inputs, weights, hidden activations after
tanh, dY and the backpropagated deltas) and does everything else in FP64;
with bf16=False it is the plain FP64 network, whose gradient
tests/test_mlp_ref.py checks by finite differences.  Not product code."""
from __future__ import annotations

import numpy as np

OFF = {"W1": (0, (64, 16)), "b1": (1024, (64,)), "W2": (1088, (64, 64)), "b2": (5184, (64,)),
       "W3": (5248, (8, 64)), "b3": (5760, (8,))}
NPARAMS = 5768


def to_bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    return np.where(np.isnan(f), np.nan, out)


def unpack(p) -> dict:
    p = np.asarray(p, dtype=np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFF.items()}


def pack(d: dict) -> np.ndarray:
    out = np.zeros(NPARAMS)
    for k, (o, s) in OFF.items():
        out[o:o + int(np.prod(s))] = np.asarray(d[k], dtype=np.float64).ravel()
    return out


def forward_backward(p, norm, X, Y, bf16: bool = True):
    """(summed squared error of the standardised outputs, gradient of its
    mean over the samples, the raw outputs) for raw features X [n][F] and
    raw targets Y [n][2]; norm = (x mean[F], x scale[F], y mean[2], y
    scale[2]) as the flat 2 F + 4 floats of the model."""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    F = X.shape[1]
    nm = np.asarray(norm, dtype=np.float64)
    xm, xs, ym, ys = nm[0:F], nm[F:2 * F], nm[2 * F:2 * F + 2], nm[2 * F + 2:2 * F + 4]
    n = len(X)
    xn = (X.astype(np.float32) - xm.astype(np.float32)) / xs.astype(np.float32) if bf16 else (X - xm) / xs
    x = np.zeros((n, 16))
    x[:, :F] = r(xn)
    W1, W2, W3 = r(w["W1"]), r(w["W2"]), r(w["W3"])
    h1 = np.tanh(x @ W1.T + w["b1"])
    h1b = r(h1)
    h2 = np.tanh(h1b @ W2.T + w["b2"])
    h2b = r(h2)
    y = h2b @ W3.T + w["b3"]
    tn = (Y - ym) / ys
    d = y[:, :2] - tn
    loss = float((d * d).sum())
    dy = np.zeros((n, 8))
    dy[:, :2] = 2.0 * d / n
    dyb = r(dy)
    dz2 = (dyb @ W3) * (1.0 - h2 * h2)
    dz2b = r(dz2)
    dz1 = (dz2b @ W2) * (1.0 - h1 * h1)
    dz1b = r(dz1)
    g = {"W3": dyb.T @ h2b, "b3": dyb.sum(0), "W2": dz2b.T @ h1b, "b2": dz2b.sum(0),
         "W1": dz1b.T @ x, "b1": dz1b.sum(0)}
    return loss, pack(g), y[:, :2] * ys + ym
