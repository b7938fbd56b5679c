"""FP64 reference of the orientation surrogate (test infrastructure).

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Spherical-harmonic
features restate kernel/utilities/spher_harmon.m (Schmidt-normalised Legendre
functions, orthonormal Y_lm, Condon-Shortley phase for odd positive m); the
multilayer perceptron is written out in numpy with the same BF16 rounding of
the weights the GPU kernels use, so GPU gradients can be checked against it.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf, lpmv


def spher_harmon(l: int, m: int, theta, phi):
    """kernel/utilities/spher_harmon.m: complex Y_lm(theta, phi)."""
    x = np.cos(np.asarray(theta, float))
    am = abs(m)
    # Schmidt semi-normalised associated Legendre function (MATLAB legendre(...,'sch')):
    # S_l^m = sqrt(2 (l-m)!/(l+m)!) P_l^m without the Condon-Shortley phase for m > 0
    P = lpmv(am, l, x) * ((-1.0) ** am)          # remove scipy's Condon-Shortley phase
    S = P if am == 0 else math.sqrt(2.0 * math.factorial(l - am) / math.factorial(l + am)) * P
    Y = math.sqrt((2 * l + 1) / (4 * math.pi)) * S * np.exp(1j * m * np.asarray(phi, float))
    if m != 0:
        Y = Y / math.sqrt(2.0)
    if m > 0 and m % 2 == 1:
        Y = -Y
    return Y


def sh_features(beta, gamma, lmax: int) -> np.ndarray:
    """Per l: Re Y_l0, then Re Y_lm, Im Y_lm for m = 1..l."""
    cols = []
    for l in range(lmax + 1):
        cols.append(spher_harmon(l, 0, beta, gamma).real)
        for m in range(1, l + 1):
            Y = spher_harmon(l, m, beta, gamma)
            cols.append(Y.real)
            cols.append(Y.imag)
    return np.stack(cols, axis=1)


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(a, np.float32).copy()
    u = f.view(np.uint32)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.view(np.float32).astype(np.float64)


def layer_shapes(nin: int, hidden: int, layers: int, nout: int):
    dims = [nin] + [hidden] * layers + [nout]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


def unpack(params: np.ndarray, shapes):
    out, off = [], 0
    for o, i in shapes:
        W = params[off:off + o * i].reshape(o, i)
        off += o * i
        b = params[off:off + o]
        off += o
        out.append((W, b))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)


def forward_backward(params, shapes, X, T, round_weights: bool = True):
    """Loss (mean squared error over all outputs) and gradients of every
    parameter, FP64.  Products use BF16-rounded weights (the rounding is passed
    straight through in the gradient) unless ``round_weights`` is false."""
    layers = unpack(np.asarray(params, np.float64), shapes)
    rnd = bf16_round if round_weights else (lambda a: np.asarray(a, np.float64))
    acts, pre = [X], []
    h = X
    for li, (W, b) in enumerate(layers):
        z = h @ rnd(W).T + b
        pre.append(z)
        h = gelu(z) if li + 1 < len(layers) else z
        acts.append(h)
    n = X.shape[0] * T.shape[1]
    d = acts[-1] - T
    loss = float(np.sum(d * d) / n)
    dA = 2.0 * d / n
    grads = [None] * len(layers)
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        if li + 1 < len(layers):
            dA = dA * gelu_grad(pre[li])
        gW = dA.T @ acts[li]
        gb = dA.sum(axis=0)
        grads[li] = (gW, gb)
        dA = dA @ rnd(W)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
