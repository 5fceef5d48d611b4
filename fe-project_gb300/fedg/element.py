"""Reference hexahedral element on Legendre-Gauss-Lobatto (LGL) nodes.

Host-side (numpy) construction of the 1D operators FElib builds for its tensor-product
element: LGL nodes and weights (FElib/src/common/scale_polynomial.F90:250-373), the
orthonormal Legendre Vandermonde V (FElib/src/element/scale_element_hexahedral.F90:243-262),
the Lagrange derivative matrix D1D, the inverse of the exact (non-lumped) 1D mass matrix
(M = (V V^T)^-1, scale_element_base.F90:221-239, hence M^-1 = V V^T), the exponential
modal filter (scale_element_modalfilter.F90:204-236) and the VPOrdM1 truncation
(scale_element_operation_tensorprod3D.F90:5560-5563).

The CUDA library builds the same operators in its own C++ host code; this module serves
coordinates and synthetic initial conditions to Python callers.
"""
from __future__ import annotations

import numpy as np


def legendre(n: int, x):
    x = np.asarray(x, dtype=np.float64)
    if n == 0:
        return np.ones_like(x)
    p0, p1 = np.ones_like(x), x.copy()
    for m in range(1, n):
        p0, p1 = p1, ((2 * m + 1) * x * p1 - m * p0) / (m + 1)
    return p1


def lgl_nodes(N: int):
    """LGL nodes and weights of order N (N+1 points) by Newton iteration on P_N'."""
    x = np.zeros(N + 1)
    x[0], x[N] = -1.0, 1.0
    for i in range(1, N):
        xi = -np.cos(np.pi * i / N)
        for _ in range(100):
            pn, pn1 = legendre(N, xi), legendre(N - 1, xi)
            f = N * (pn1 - xi * pn) / (1 - xi * xi)
            fp = (2 * xi * f - N * (N + 1) * pn) / (1 - xi * xi)
            dx = f / fp
            xi -= dx
            if abs(dx) < 1e-17:
                break
        x[i] = xi
    w = 2.0 / (N * (N + 1) * legendre(N, x) ** 2)
    return x, w


def operators_1d(porder: int, etac=2.0 / 3.0, alpha=36.0, order=16):
    N = porder
    n1 = N + 1
    x, w = lgl_nodes(N)
    V = np.stack([legendre(m, x) * np.sqrt(m + 0.5) for m in range(n1)], axis=1)
    invV = np.linalg.inv(V)
    D = np.zeros((n1, n1))
    PN = legendre(N, x)
    for i in range(n1):
        for l in range(n1):
            if i != l:
                D[i, l] = PN[i] / (PN[l] * (x[i] - x[l]))
    D[0, 0] = -N * (N + 1) / 4.0
    D[N, N] = N * (N + 1) / 4.0
    Minv = V @ V.T
    sig = np.ones(n1)
    for m in range(1, n1):
        eta = m / N
        if eta > etac:
            sig[m] = np.exp(-alpha * ((eta - etac) / (1 - etac)) ** order)
    F = V @ np.diag(sig) @ invV
    trunc = np.ones(n1)
    trunc[-1] = 0.0
    T = V @ np.diag(trunc) @ invV
    return dict(x=x, w=w, V=V, invV=invV, D=D, Minv=Minv, F=F, T=T)
