"""Spectral constants for nPol = 4, computed in FP64 from their definitions.

The reference hard-codes 12-digit tables (SOLVER/src/preloop/spectral/SpectralConstants.cpp:17-144).
Here they are derived:

* GLL nodes: -1, 1 and the zeros of P'_N (= zeros of the Jacobi polynomial P_{N-1}^{(1,1)}).
* GLJ(0,1) nodes used on the axis (xi direction of axial elements): -1, 1 and the zeros
  of P_{N-1}^{(1,2)}.
* GLL weights integrate f on [-1, 1]; GLJ weights integrate (1 + xi) f, exactly for
  polynomials of degree <= 2N - 1 (moments solved in FP64).
* G(i, j) = l_i'(xi_j), the derivative of the i-th Lagrange basis polynomial at node j,
  the layout Gradient::setGMat receives (Map<RDMatPP> of the row-major table).
"""
from __future__ import annotations

from functools import lru_cache

import numpy as np
from scipy.special import roots_jacobi

NPOL = 4
NP = NPOL + 1


def _lagrange_derivative(x: np.ndarray) -> np.ndarray:
    """G[i, j] = l_i'(x_j) for the Lagrange basis on nodes x."""
    n = len(x)
    G = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i == j:
                G[i, j] = sum(1.0 / (x[i] - x[m]) for m in range(n) if m != i)
            else:
                num = np.prod([x[j] - x[m] for m in range(n) if m != i and m != j])
                den = np.prod([x[i] - x[m] for m in range(n) if m != i])
                G[i, j] = num / den
    return G


def _weights(x: np.ndarray, weight_poly) -> np.ndarray:
    """Quadrature weights exact for degree <= len(x) - 1 against weight_poly (moments)."""
    n = len(x)
    V = np.vander(x, n, increasing=True).T  # V[k, i] = x_i^k
    mom = np.array([weight_poly(k) for k in range(n)])
    return np.linalg.solve(V, mom)


@lru_cache(maxsize=None)
def gll(npol: int = NPOL):
    if npol == 1:
        x = np.array([-1.0, 1.0])
    else:
        inner, _ = roots_jacobi(npol - 1, 1, 1)
        x = np.concatenate([[-1.0], np.sort(inner), [1.0]])
    w = _weights(x, lambda k: (1 - (-1) ** (k + 1)) / (k + 1))  # int x^k dx
    return x, w, _lagrange_derivative(x)


@lru_cache(maxsize=None)
def glj(npol: int = NPOL):
    if npol == 1:
        x = np.array([-1.0, 1.0])
    else:
        inner, _ = roots_jacobi(npol - 1, 1, 2)
        x = np.concatenate([[-1.0], np.sort(inner), [1.0]])
    # int (1 + x) x^k dx
    w = _weights(x, lambda k: (1 - (-1) ** (k + 1)) / (k + 1) + (1 - (-1) ** (k + 2)) / (k + 2))
    return x, w, _lagrange_derivative(x)


def xi_eta(ipol: int, jpol: int, axial: bool):
    """SpectralConstants::getXiEta (SpectralConstants.cpp:146-156)."""
    return (glj()[0][ipol] if axial else gll()[0][ipol]), gll()[0][jpol]


def weights(ipol: int, jpol: int, axial: bool):
    """SpectralConstants::getWeights (SpectralConstants.cpp:158-168)."""
    return (glj()[1][ipol] if axial else gll()[1][ipol]), gll()[1][jpol]
