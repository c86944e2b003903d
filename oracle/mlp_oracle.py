"""CPU oracle of the Nu network (TEST INFRASTRUCTURE ONLY: tests and smoke() import it).

The reference has no neural network -- its Fourier-order field comes from NU_TYPE rules or
a wisdom file (NuWisdom.cpp:19-86) -- so this oracle is the network's mathematical
definition in FP64, the same one include/ax3d.h states for ax3d_mlp_*:

    h1 = gelu(W1 x + b1), h2 = gelu(W2 h1 + b2), h3 = gelu(W3 h2 + b3), y = w4 . h3 + b4
    loss = mean((y - t)^2), Adam(beta1 0.9, beta2 0.999, eps 1e-8)

With mirror=True the BF16 roundings of the CUDA path (features, weights, activations and
back-propagated errors, round to nearest even) are applied at the same places, so the
two differ only by FP32-vs-FP64 accumulation and the rare rounding that this flips.
With mirror=False it is the exact FP64 gradient, which the tests pin against central
finite differences.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

NIN, NHID = 16, 128
_SIZES = (("W1", NHID * NIN), ("b1", NHID), ("W2", NHID * NHID), ("b2", NHID), ("W3", NHID * NHID),
          ("b3", NHID), ("w4", NHID), ("b4", 1))
NPARAM = sum(s for _, s in _SIZES)


def bf16(a):
    """Round to BF16 (nearest even) through FP32, returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, o = {}, 0
    for name, n in _SIZES:
        out[name] = p[o:o + n]
        o += n
    out["W1"] = out["W1"].reshape(NHID, NIN)
    out["W2"] = out["W2"].reshape(NHID, NHID)
    out["W3"] = out["W3"].reshape(NHID, NHID)
    return out


def pack(d):
    return np.concatenate([np.ravel(d[name]) for name, _ in _SIZES])


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def dgelu(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(p, x, mirror=True, keep=False):
    r = bf16 if mirror else (lambda a: np.asarray(a, np.float64))
    P = unpack(p)
    W1, W2, W3, w4 = r(P["W1"]), r(P["W2"]), r(P["W3"]), r(P["w4"])
    x = r(x)
    z1 = x @ W1.T + P["b1"]
    h1 = r(gelu(z1))
    z2 = h1 @ W2.T + P["b2"]
    h2 = r(gelu(z2))
    z3 = h2 @ W3.T + P["b3"]
    h3 = r(gelu(z3))
    y = h3 @ w4 + P["b4"][0]
    if keep:
        return y, dict(x=x, W1=W1, W2=W2, W3=W3, w4=w4, z1=z1, z2=z2, z3=z3, h1=h1, h2=h2, h3=h3)
    return y


def gradient(p, x, t, mirror=True):
    """(gradient vector, loss) of mean((y - t)^2)."""
    r = bf16 if mirror else (lambda a: np.asarray(a, np.float64))
    y, c = forward(p, x, mirror, keep=True)
    n = len(y)
    e = y - np.asarray(t, np.float64)
    dy = 2.0 * e / n
    dz3 = r(c["w4"][None, :] * dy[:, None] * dgelu(c["z3"]))
    dz2 = r((dz3 @ c["W3"]) * dgelu(c["z2"]))
    dz1 = r((dz2 @ c["W2"]) * dgelu(c["z1"]))
    g = dict(W1=dz1.T @ c["x"], b1=dz1.sum(0), W2=dz2.T @ c["h1"], b2=dz2.sum(0), W3=dz3.T @ c["h2"],
             b3=dz3.sum(0), w4=dy @ c["h3"], b4=np.array([dy.sum()]))
    return pack(g), float(np.mean(e * e))


class Adam:
    """FP64 Adam on an FP32-rounded master copy (the CUDA path keeps FP32 masters)."""

    def __init__(self, p):
        self.p = np.asarray(p, np.float64)
        self.m = np.zeros_like(self.p)
        self.v = np.zeros_like(self.p)
        self.t = 0

    def step(self, g, lr):
        self.t += 1
        self.m = 0.9 * self.m + 0.1 * g
        self.v = 0.999 * self.v + 0.001 * g * g
        mh = self.m / (1 - 0.9 ** self.t)
        vh = self.v / (1 - 0.999 ** self.t)
        self.p = np.float32(self.p - lr * mh / (np.sqrt(vh) + 1e-8)).astype(np.float64)
        return self.p
