"""CPU oracle of the surrogate network (test infrastructure: the checker for the GPU
kernels of boltzmann_gb300/csrc/bz_mlp.cu, never part of the product).

The network has no counterpart in the reference (jfabell/boltzmann starts every run from
the plain initial state, boltzmann.py:271-312); this file restates the network the
kernels compute, in float64:

* layers l = 0..4: z_l = a_{l-1} W_l^T + b_l, a_l = GELU(z_l) (tanh form) for the hidden
  layers, y = z_4; a_{-1} = x;
* the matrix operands are rounded to bfloat16 (round to nearest even) exactly where the
  GPU rounds them: x and every a_l before a product, the weights, and the loss gradient
  dZ_l before both products of the backward pass (dW_l = dZ_l^T a_{l-1}, dA = dZ_l W_l)
  and the bias sums;
* GELU with the exact tanh (the GPU uses the hardware tanh approximation, relative error
  about 2^-11, below the BF16 rounding of every activation that follows);
* loss = sum_r sum_c wcol_c (y_rc - t_rc)^2 / (2 n);
* Adam (Kingma & Ba 2015) with bias correction and decoupled weight decay on the
  weights (Loshchilov & Hutter 2019).

``exact=True`` skips every bfloat16 rounding: the float64 network whose analytic
gradient the finite-difference test checks.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT, NL = 16, 128, 80, 5


def dims(l):
    return (IN if l == 0 else H), (OUT if l == NL - 1 else H)


def offsets():
    """(weight offset, bias offset) of every layer in the flat parameter array."""
    o, res = 0, []
    for l in range(NL):
        ni, no = dims(l)
        res.append((o, o + ni * no))
        o += ni * no + no
    return res, o


OFFS, NPARAM = offsets()


def layer(params, l):
    ni, no = dims(l)
    wo, bo = OFFS[l]
    return params[wo:wo + ni * no].reshape(no, ni), params[bo:bo + no]


def bf16(a):
    """float -> float32 -> bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


GC, GA = 0.7978845608028654, 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GC * (z + GA * z ** 3)))


def gelu_grad(z):
    th = np.tanh(GC * (z + GA * z ** 3))
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * GC * (1.0 + 3.0 * GA * z * z)


def forward(params, x, exact=False):
    """y (n x OUT) and the hidden pre-activations [z_0 .. z_3]."""
    r = (lambda v: np.asarray(v, dtype=np.float64)) if exact else bf16
    p = np.asarray(params, dtype=np.float64)
    a = r(x)
    zs = []
    y = None
    for l in range(NL):
        W, b = layer(p, l)
        z = a @ r(W).T + b
        if l < NL - 1:
            zs.append(z)
            a = r(gelu(z))
        else:
            y = z
    return y, zs


def backward(params, x, t, wcol, exact=False):
    """(loss, gradient of the loss with respect to the flat parameters)."""
    r = (lambda v: np.asarray(v, dtype=np.float64)) if exact else bf16
    p = np.asarray(params, dtype=np.float64)
    n = len(x)
    y, zs = forward(p, x, exact)
    e = y - t
    loss = 0.5 * np.sum(wcol * e * e) / n
    dz = wcol * e / n
    g = np.zeros(NPARAM)
    for l in range(NL - 1, -1, -1):
        W, _ = layer(p, l)
        ni, no = dims(l)
        wo, bo = OFFS[l]
        dzb = r(dz)
        a = r(x) if l == 0 else r(gelu(zs[l - 1]))
        g[wo:wo + ni * no] = (dzb.T @ a).reshape(-1)
        g[bo:bo + no] = dzb.sum(axis=0)
        if l > 0:
            dz = (dzb @ r(W)) * gelu_grad(zs[l - 1])
    return loss, g


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
    """One Adam step; returns (params, m, v)."""
    p = np.asarray(params, dtype=np.float64).copy()
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1 = 1 - b1 ** step
    c2 = 1 - b2 ** step
    isw = np.zeros(NPARAM, dtype=bool)
    for l in range(NL):
        wo, bo = OFFS[l]
        isw[wo:bo] = True
    p = np.where(isw, p - lr * wd * p, p)
    p = p - (lr / c1) * m / (np.sqrt(v / c2) + eps)
    return p, m, v
