"""FP64 numpy restatement of the guiding network (test infrastructure only).

The learned proposal has no counterpart in the reference path tracer; its
output distribution is the reference's VonMisesFisherDistribution<8>
(Include/Xitils/VonMisesFisherDistribution.h: pdf :205-211). This module is the
CPU checker for the GPU kernels of xitils_gb300/csrc/guide.cu: feature
encoding, the 64-64-64-64-40 MLP forward pass, the mixture decoding, the
normalised NLL and its gradient, and the backward pass. ``bf16=True`` rounds
operands where the GPU stores BF16 (inputs, activations, weights, gradients of
activations) so the comparison isolates accumulation order from quantisation.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT, LOBES = 64, 64, 40, 8
SHAPES = [("W0", (64, 64)), ("b0", (64,)), ("W1", (64, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)),
          ("W3", (40, 64)), ("b3", (40,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
KMIN, KMAX = -6.0, 8.0


def split(params):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def join(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def features(pos, nrm, wo, lo, hi):
    pos, nrm, wo = (np.asarray(a, dtype=np.float64).reshape(-1, 3) for a in (pos, nrm, wo))
    p = (pos - np.asarray(lo, np.float64)) / (np.asarray(hi, np.float64) - np.asarray(lo, np.float64))
    n = p.shape[0]
    X = np.zeros((n, 64))
    for i in range(36):
        band, rem = i // 6, i % 6
        axis = rem >> 1
        arg = p[:, axis] * (2.0 ** band) * np.pi
        X[:, i] = np.cos(arg) if rem & 1 else np.sin(arg)
    X[:, 36:39] = p
    X[:, 39:42] = nrm
    X[:, 42:45] = wo
    return X


def forward(params, X, quant=True):
    q = bf16 if quant else (lambda a: np.asarray(a, np.float64))
    P = split(params)
    acts = [q(X)]
    h = acts[0]
    for l in range(3):
        z = h @ q(P[f"W{l}"]).T + P[f"b{l}"]
        h = q(np.maximum(z, 0.0))
        acts.append(h)
    Y = h @ q(P["W3"]).T + P["b3"]
    return Y, acts


def decode(Y):
    Y = np.asarray(Y, np.float64).reshape(-1, LOBES, 5)
    m = Y[:, :, 0:3]
    mu = m / np.linalg.norm(m, axis=2, keepdims=True)
    kappa = np.exp(np.clip(Y[:, :, 3], KMIN, KMAX))
    l = Y[:, :, 4]
    a = np.exp(l - l.max(axis=1, keepdims=True))
    alpha = a / a.sum(axis=1, keepdims=True)
    return mu, kappa, alpha


def vmf_pdf(mu, kappa, w):
    """kappa / (2 pi (1 - exp(-2 kappa))) exp(kappa (mu . w - 1))."""
    c = kappa / (2 * np.pi * -np.expm1(-2 * kappa))
    return c * np.exp(kappa * (np.sum(mu * w, axis=-1) - 1.0))


def mixture_pdf(Y, w):
    mu, kappa, alpha = decode(Y)
    w = np.asarray(w, np.float64).reshape(-1, 1, 3)
    return np.sum(alpha * vmf_pdf(mu, kappa, w), axis=1)


def loss_and_output_grad(Y, wdir, weight):
    """loss = sum_i -(w_i / sum w) log q_i; returns (loss, dL/dY [n, 40])."""
    Y = np.asarray(Y, np.float64)
    n = Y.shape[0]
    wn = np.asarray(weight, np.float64) / np.sum(weight)
    mu, kappa, alpha = decode(Y)
    wv = np.asarray(wdir, np.float64).reshape(-1, 1, 3)
    v = vmf_pdf(mu, kappa, wv)
    q = np.sum(alpha * v, axis=1)
    loss = float(np.sum(-wn * np.log(q)))
    g = (-wn / q)[:, None]
    Yr = Y.reshape(n, LOBES, 5)
    m = Yr[:, :, 0:3]
    mlen = np.linalg.norm(m, axis=2)
    cosw = np.sum(mu * wv, axis=2)
    av = alpha * v
    dY = np.zeros((n, LOBES, 5))
    s = g * av * kappa / mlen
    dY[:, :, 0:3] = s[:, :, None] * (wv - cosw[:, :, None] * mu)
    k = Yr[:, :, 3]
    inside = (k > KMIN) & (k < KMAX)
    dlogc = 1.0 / kappa - 2.0 / np.expm1(2.0 * kappa)
    dY[:, :, 3] = np.where(inside, g * av * (dlogc + cosw - 1.0) * kappa, 0.0)
    dY[:, :, 4] = g * alpha * (v - q[:, None])
    return loss, dY.reshape(n, 40)


def backward(params, acts, dY, quant=True):
    """Parameter gradients for output gradient dY (with BF16 rounding of the
    stored gradients of activations when quant)."""
    q = bf16 if quant else (lambda a: np.asarray(a, np.float64))
    P = split(params)
    grads = {}
    d = q(dY)
    grads["W3"] = d.T @ acts[3]
    grads["b3"] = d.sum(axis=0)
    dz = d
    for l in (2, 1, 0):
        W = q(P[f"W{l + 1}"])
        dx = dz @ W
        dz = q(dx * (acts[l + 1] > 0))
        grads[f"W{l}"] = dz.T @ acts[l]
        grads[f"b{l}"] = dz.sum(axis=0)
    return join(grads)
