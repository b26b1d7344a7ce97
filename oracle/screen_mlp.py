"""CPU oracle of the pair-screen network -- TEST INFRASTRUCTURE ONLY.

The screen network (12 -> 64 -> 64 -> 1, ReLU) has no counterpart in the
reference; this restates the forward and backward passes the GPU kernels
run, in float64 with the same bf16 rounding points, so the kernels'
gradients can be checked:

* weights and input features are rounded to bf16 (round to nearest even);
* z1 = W1 x + b1, h1 = bf16(relu(z1)); z2 = W2 h1 + b2, h2 = bf16(relu(z2));
  out = W3 . h2 + b3;
* loss = mean((out - y)^2); gradients of that loss with respect to the
  (bf16-rounded) parameters, ReLU derivative 1 where z > 0.

Parameter layout: W1 [64][12], b1 [64], W2 [64][64], b2 [64], W3 [64], b3.
"""
from __future__ import annotations

import numpy as np

NFEAT, NHID = 12, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NHID * NFEAT
OFF_W2 = OFF_B1 + NHID
OFF_B2 = OFF_W2 + NHID * NHID
OFF_W3 = OFF_B2 + NHID
OFF_B3 = OFF_W3 + NHID
NPARAMS = OFF_B3 + 1


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    nan = np.isnan(a)
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[OFF_W1:OFF_B1].reshape(NHID, NFEAT), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(NHID, NHID),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3], w[OFF_B3])


def forward_backward(weights, feats, targets, round_bf16=True):
    """(pred [n], grad [NPARAMS], loss) of the mean squared error."""
    wr = bf16(weights) if round_bf16 else np.asarray(weights, np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(wr)
    x = bf16(feats) if round_bf16 else np.asarray(feats, np.float64)
    y = np.asarray(targets, np.float64)
    n = len(y)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    if round_bf16:
        h1 = bf16(h1)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    if round_bf16:
        h2 = bf16(h2)
    out = h2 @ W3 + b3
    e = out - y
    loss = float(np.mean(e * e))
    dout = 2.0 * e / n
    g = np.zeros(NPARAMS)
    g[OFF_W3:OFF_B3] = dout @ h2
    g[OFF_B3] = dout.sum()
    dh2 = np.outer(dout, W3) * (z2 > 0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ W2) * (z1 > 0)
    g[OFF_W1:OFF_B1] = (dh1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return out, g, loss
