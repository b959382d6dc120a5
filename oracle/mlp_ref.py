"""CPU oracle of the learned seeding's network (test infrastructure: only the
tests import it, to verify the CUDA kernels in c2a_gb300/csrc/mlp.cu).

A numpy restatement of the forward and backward passes with BF16 rounding at
the points where the CUDA path rounds (inputs, weight copies, hidden
activations, the gradients that feed a GEMM) and FP32 elsewhere; with
``rounding=False`` the same code runs in FP64 without rounding, for the
finite-difference check of the backward formulas themselves.

Layers: x -> GELU(x W0^T + b0) -> GELU(. W1^T + b1) -> GELU(. W2^T + b2) ->
. W3^T + b3 = logits; loss = mean softmax cross-entropy.  x = [features
(18), E[ia] (16), E[ib] (16), 0 ...].
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

NFEAT = 18
EMBED = 16


def bf16(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def assemble(feat, ia, ib, E, width):
    n = len(feat)
    x = np.zeros((n, width), dtype=E.dtype)
    x[:, :NFEAT] = feat
    x[:, NFEAT:NFEAT + EMBED] = E[ia]
    x[:, NFEAT + EMBED:NFEAT + 2 * EMBED] = E[ib]
    return x


def forward_backward(W, b, E, feat, ia, ib, labels, rounding: bool = True):
    """Returns (mean loss, logits, gradients dict: W[i], b[i], E)."""
    dt = np.float32 if rounding else np.float64
    r = bf16 if rounding else (lambda v: v)
    W = [np.asarray(w, dtype=dt) for w in W]
    b = [np.asarray(v, dtype=dt) for v in b]
    E = np.asarray(E, dtype=dt)
    n = len(feat)
    x = r(assemble(np.asarray(feat, dtype=dt), ia, ib, E, W[0].shape[1]))
    Wr = [r(w) for w in W]
    acts, pres = [x], []
    h = x
    for i in range(3):
        pre = (h @ Wr[i].T + b[i]).astype(dt)
        pres.append(pre)
        h = r(gelu(pre).astype(dt))
        acts.append(h)
    logits = (h @ Wr[3].T + b[3]).astype(dt)
    z = logits - logits.max(axis=1, keepdims=True)
    ez = np.exp(z)
    p = ez / ez.sum(axis=1, keepdims=True)
    loss = float(np.mean(np.log(ez.sum(axis=1)) - z[np.arange(n), labels]))
    onehot = np.zeros_like(p)
    onehot[np.arange(n), labels] = 1.0
    d = r(((p - onehot) / n).astype(dt))
    gW, gb = [None] * 4, [None] * 4
    for i in (3, 2, 1, 0):
        gW[i] = (d.T @ acts[i]).astype(dt)
        gb[i] = d.sum(axis=0).astype(dt)
        dh = (d @ Wr[i]).astype(dt)
        if i > 0:
            d = r((dh * gelu_grad(pres[i - 1])).astype(dt))
        else:
            gE = np.zeros_like(E)
            np.add.at(gE, ia, dh[:, NFEAT:NFEAT + EMBED])
            np.add.at(gE, ib, dh[:, NFEAT + EMBED:NFEAT + 2 * EMBED])
    return loss, logits, {"W": gW, "b": gb, "E": gE}
