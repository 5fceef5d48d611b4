"""The pivot order and skip rules of the column solve's element LU (fe-project_gb300/csrc/fedg_vicol.cu,
PivOrder / shfl_fwd / shfl_bwd), restated step for step in numpy and checked against a dense solve.

The element block of the DENS/MOMZ/RHOT system has rows 3k+v (node k, variable v = DENS, MOMZ,
RHOT).  A DENS row has nonzeros only in DENS_k, DENS_0, DENS_N, the MOMZ columns and RHOT_0, so the
kernel pivots on DENS_0 .. DENS_N first (updating the other DENS rows only at the DENS_0 step, and
shuffling only DENS_N, the MOMZ columns and RHOT_0 of a DENS pivot row), then on MOMZ/RHOT node by
node; the back substitution skips the same structural zeros.  Matrices with that sparsity and a
dominant diagonal (no pivoting, as in the kernel) must be solved to roundoff.
"""
import numpy as np
import pytest


def col(s, N1):
    return 3 * s if s < N1 else 3 * ((s - N1) // 2) + 1 + ((s - N1) & 1)


def pos(c, N1):
    return c // 3 if c % 3 == 0 else N1 + 2 * (c // 3) + (c % 3 - 1)


def nz(s, c, N1):
    if pos(c, N1) <= s:
        return False
    if s >= N1:
        return True
    return c == 3 * (N1 - 1) or c % 3 == 1 or c == 2


def structured_solve(A, R, N1):
    n = 3 * N1
    a, r = A.copy(), R.copy()
    for s in range(n):  # forward elimination (shfl_fwd)
        pc = col(s, N1)
        inv = 1.0 / a[pc, pc]
        prow, pr = a[pc].copy(), r[pc].copy()
        for k in range(N1):
            for v in range(3):
                row = 3 * k + v
                if v == 0:
                    if s != 0 or k == 0:
                        continue  # DENS rows: only the DENS_0 step eliminates in them
                    f = a[row, pc] * inv
                elif pos(row, N1) > s:
                    f = a[row, pc] * inv
                else:
                    continue
                for c in range(n):
                    if nz(s, c, N1):
                        a[row, c] -= f * prow[c]
                r[row] -= f * pr
    for s in range(n - 1, -1, -1):  # back substitution (shfl_bwd)
        pc = col(s, N1)
        x = r[pc] / a[pc, pc]
        dcol = pc % 3 == 1 or pc == 2 or pc == 3 * (N1 - 1)
        for k in range(N1):
            for v in range(3):
                row = 3 * k + v
                if row == pc:
                    r[row] = x
                elif v == 0 and not dcol:
                    continue
                elif v > 0 and s < N1:
                    continue
                elif pos(row, N1) < s:
                    r[row] -= a[row, pc] * x
    return r


def test_pivot_order_is_a_permutation():
    for N1 in (4, 8):
        cols = [col(s, N1) for s in range(3 * N1)]
        assert sorted(cols) == list(range(3 * N1))
        assert all(pos(c, N1) == s for s, c in enumerate(cols))


@pytest.mark.parametrize("N1", [4, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_structured_lu_solves_the_dens_sparse_block(N1, seed):
    rng = np.random.default_rng(seed)
    n, N = 3 * N1, N1 - 1
    A = 0.1 * rng.standard_normal((n, n)) + 3.0 * np.eye(n)
    for k in range(N1):
        for c in range(n):
            if not (c == 3 * k or c == 0 or c == 3 * N or c % 3 == 1 or c == 2):
                A[3 * k, c] = 0.0
    R = rng.standard_normal((n, 4))
    X = structured_solve(A, R, N1)
    assert np.max(np.abs(X - np.linalg.solve(A, R))) < 1e-13


def test_structured_lu_needs_the_sparsity():
    """a DENS row with a nonzero the skip rules assume away (DENS_1 of row DENS_2) is solved wrongly"""
    rng = np.random.default_rng(3)
    N1 = 4
    n = 3 * N1
    A = 0.1 * rng.standard_normal((n, n)) + 3.0 * np.eye(n)
    for k in range(N1):
        for c in range(n):
            if not (c == 3 * k or c == 0 or c == 3 * (N1 - 1) or c % 3 == 1 or c == 2):
                A[3 * k, c] = 0.0
    A[6, 3] = 0.5
    R = rng.standard_normal((n, 4))
    assert np.max(np.abs(structured_solve(A, R, N1) - np.linalg.solve(A, R))) > 1e-6
