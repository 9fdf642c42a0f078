"""CPU oracle of the learned-guess MLP (test infrastructure only).

Float64 numpy forward and backward passes of the network in
quiqbox.jl_gb300/guess.py, with BF16 rounding (round to nearest even) applied at the
same points as the GPU kernels: inputs, weights, hidden activations, and the output /
hidden gradients fed to the tensor-core GEMMs.  With round=False it is the exact
float64 network, checked against central finite differences.  The network has no
reference counterpart (the reference has no learned guess), so this is its oracle.
"""
import numpy as np
from math import erf, sqrt, pi


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / sqrt(2.0)))


def gelu_grad(z):
    Phi = 0.5 * (1.0 + _erf(z / sqrt(2.0)))
    return Phi + z * np.exp(-0.5 * z * z) / sqrt(2.0 * pi)


def forward(params, X, round=True):
    r = bf16 if round else (lambda v: np.asarray(v, np.float64))
    L = len([k for k in params if k.startswith("W")])
    acts, zs = [r(X)], []
    x = acts[0]
    for l in range(L):
        z = x @ r(params["W%d" % l]).T + params["b%d" % l]
        if l == L - 1:
            return z, (acts, zs)
        zs.append(z)
        x = r(gelu(z))
        acts.append(x)


def backward(params, saved, dY, round=True):
    r = bf16 if round else (lambda v: np.asarray(v, np.float64))
    acts, zs = saved
    L = len(acts)
    dW, db = [None] * L, [None] * L
    d = np.asarray(dY, np.float64)
    for l in range(L - 1, -1, -1):
        db[l] = d.sum(axis=0)
        dW[l] = r(d).T @ acts[l]
        if l == 0:
            break
        dx = r(d) @ r(params["W%d" % l])
        d = dx * gelu_grad(zs[l - 1])
    return dW, db


def mse(Y, T, W):
    wsum = W.sum()
    return float((W * (Y - T) ** 2).sum() / wsum), 2.0 * W * (Y - T) / wsum
