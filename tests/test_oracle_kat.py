"""Known-answer tests that pin the FP64 oracle to the reference's own test suite.

* LGL nodes/weights N=1..4 (FElib/test/FE/polynomial/test_polynomial.f90:11-44)
* derivative / Lift exactness p=1..7 (FElib/test/FE/element_operation_hexahedral/
  test_element_operation_hexahedral.f90:73-147, 236-259)
* RK convergence orders, SSP 3s3o >= 2.98 and IMEX ARK232 >= 1.98
  (FElib/test/common/timeint_rk/test_timeint_rk.f90:33-43, 173-282)
* Butcher/Shu-Osher consistency of SSP 3s3o (test_timeint_rk.f90:284-320)
"""
import numpy as np
import pytest

import oracle as orc
import timeint_ref
from fedg import element


def _orc(p, ne=(1, 1, 1)):
    return orc.Oracle(p, *ne, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))


LGL_KAT = {
    1: ([-1.0, 1.0], [1.0, 1.0]),
    2: ([-1.0, 0.0, 1.0], [1 / 3, 4 / 3, 1 / 3]),
    3: ([-1.0, -np.sqrt(1 / 5), np.sqrt(1 / 5), 1.0], [1 / 6, 5 / 6, 5 / 6, 1 / 6]),
    4: ([-1.0, -np.sqrt(21) / 7, 0.0, np.sqrt(21) / 7, 1.0], [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10]),
}


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_lgl_nodes_weights(n):
    ops = _orc(n).operators_1d()
    x, w = LGL_KAT[n]
    assert np.max(np.abs(ops["x"] - x)) < 5e-15
    assert np.max(np.abs(ops["w"] - w)) < 5e-15
    xe, we = element.lgl_nodes(n)
    assert np.max(np.abs(xe - x)) < 5e-15 and np.max(np.abs(we - w)) < 5e-15


@pytest.mark.parametrize("p", range(1, 8))
def test_derivative_and_lift_exact(p):
    """D1D differentiates x^m exactly (m <= p); M^-1 = (V V^T) inverts the exact mass matrix;
    the tensor-product Lift equals the dense invM*E of the hexahedral element."""
    o = _orc(p)
    ops = o.operators_1d()
    x, D, Minv = ops["x"], ops["D"], ops["Minv"]
    for m in range(0, p + 1):
        f = x ** m
        df = m * x ** (m - 1) if m > 0 else np.zeros_like(x)
        assert np.max(np.abs(D @ f - df)) < 1e-12 * max(1, m * m)
    # exact 1D mass matrix by Gauss-Legendre quadrature of the Lagrange basis (independent path)
    gx, gw = np.polynomial.legendre.leggauss(p + 2)
    n1 = p + 1
    Lag = np.zeros((n1, gx.size))
    for l in range(n1):
        others = [x[m] for m in range(n1) if m != l]
        Lag[l] = np.prod([(gx - xm) / (x[l] - xm) for xm in others], axis=0) if others else 1.0
    M = (Lag * gw) @ Lag.T
    assert np.max(np.abs(Minv @ M - np.eye(n1))) < 1e-12
    # dense 3D Lift (FElib scale_element_hexahedral.F90:330-401) vs the tensor-product form
    M3 = np.kron(np.kron(M, M), M)  # index n = i + n1*j + n1^2*k -> kron(Mk, Mj, Mi)
    Np = n1 ** 3
    idx = lambda i, j, k: i + n1 * j + n1 * n1 * k
    faces = []
    for f in range(6):
        nodes = []
        for b in range(n1):
            for a in range(n1):
                i, j, k = [(a, 0, b), (p, a, b), (a, p, b), (0, a, b), (a, b, 0), (a, b, p)][f]
                nodes.append(idx(i, j, k))
        faces.append(nodes)
    E = np.zeros((Np, 6 * n1 * n1))
    M2 = np.kron(M, M)
    for f, nodes in enumerate(faces):
        E[np.ix_(nodes, range(f * n1 * n1, (f + 1) * n1 * n1))] = M2
    Lift = np.linalg.solve(M3, E)
    rng = np.random.default_rng(p)
    g = rng.standard_normal(6 * n1 * n1)
    dense = Lift @ g
    tp = np.zeros(Np)
    for k in range(n1):
        for j in range(n1):
            for i in range(n1):
                tp[idx(i, j, k)] = (Minv[j, 0] * g[0 * n1 * n1 + i + n1 * k] + Minv[i, p] * g[1 * n1 * n1 + j + n1 * k]
                                    + Minv[j, p] * g[2 * n1 * n1 + i + n1 * k] + Minv[i, 0] * g[3 * n1 * n1 + j + n1 * k]
                                    + Minv[k, 0] * g[4 * n1 * n1 + i + n1 * j] + Minv[k, p] * g[5 * n1 * n1 + i + n1 * j])
    assert np.max(np.abs(dense - tp)) < 1e-10 * np.max(np.abs(dense))


@pytest.mark.parametrize("p", [3, 7])
def test_filter_and_truncation(p):
    ops = _orc(p).operators_1d()
    V, F, T, invV = ops["V"], ops["F"], ops["T"], ops["invV"]
    n1 = p + 1
    modal_T = invV @ T @ V
    assert np.allclose(modal_T, np.diag([1.0] * p + [0.0]), atol=1e-12)
    modal_F = np.diag(invV @ F @ V)
    for m in range(n1):
        eta = m / p
        s = 1.0 if (eta <= 2 / 3 or m == 0) else np.exp(-36.0 * ((eta - 2 / 3) / (1 / 3)) ** 16)
        assert abs(modal_F[m] - s) < 1e-12
    e = element.operators_1d(p)
    for k in ("D", "Minv", "F", "T", "V"):
        assert np.max(np.abs(e[k] - ops[k])) < 1e-12


@pytest.mark.parametrize("name,order", [("ERK_SSP_3s3o", 2.98), ("IMEX_ARK232", 1.98)])
def test_rk_convergence_order(name, order):
    errs = [timeint_ref.damped_oscillator_error(name, dt) for dt in (1e-2, 5e-3, 2.5e-3)]
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(orders) >= order, (errs, orders)


def test_ssp3_shu_osher_to_butcher():
    """Shu-Osher SSP(3,3) expands to the Butcher tableau A=[[0],[1],[1/4,1/4]], b=[1/6,1/6,2/3]."""
    t = timeint_ref.tables("ERK_SSP_3s3o")
    sig, gam = t["sig"], t["gam"]
    ns = 3
    A = np.zeros((ns + 1, ns))
    for i in range(1, ns + 1):
        for j in range(i):
            A[i, j] = gam[i, j] + sum(sig[i, k] * A[k, j] for k in range(j + 1, i))
    assert np.allclose(A[1:ns, :], [[1, 0, 0], [0.25, 0.25, 0]])
    assert np.allclose(A[ns], [1 / 6, 1 / 6, 2 / 3])
