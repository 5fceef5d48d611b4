"""The pivot order and skip rules of the column solves' element LU (PivOrder, fe-project_gb300/csrc/
fedg_common.cuh), restated step for step in numpy and checked against a dense solve, with the two forms
the kernels use: the blocked form of the FP32 column solve (fedg_vicol.cu, lu_blocked) and the FP64 one
with partial pivoting in the MOMZ/RHOT phase (fedg_vi.cu, warp_lu_dfirst).

The element block of the DENS/MOMZ/RHOT system has rows 3k+v (node k, variable v = DENS, MOMZ,
RHOT).  A DENS row has nonzeros only in DENS_k, DENS_0, DENS_N, the MOMZ columns and RHOT_0, so the
order pivots on DENS_0 .. DENS_N first (updating the other DENS rows only at the DENS_0 step, and
carrying only DENS_N, the MOMZ columns and RHOT_0 of a DENS pivot row), then on MOMZ/RHOT node by
node; the back substitution skips the same structural zeros.  Matrices with that sparsity and a
dominant diagonal (no pivoting, as in the FP32 kernel) must be solved to roundoff.
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
    for s in range(n):  # forward elimination, one pivot at a time
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
    for s in range(n - 1, -1, -1):  # back substitution
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


def dfirst_pivoting_solve(A, R, N1, rows_out=None):
    """The FP64 kernel's variant (fe-project_gb300/csrc/fedg_vi.cu, blk_fwd / blk_bwd): the same DENS-first
    column order, every DENS column pivoted on its own DENS row, the MOMZ/RHOT columns with partial
    pivoting over the rows not yet pivoted (largest |a|, lowest row on ties); the back substitution
    in reverse step order."""
    n = 3 * N1
    a, r = A.copy(), R.copy()
    done = np.zeros(n, bool)
    piv_row = np.zeros(n, int)
    for s in range(n):
        pc = col(s, N1)
        if s < N1:
            p = pc
        else:
            cand = [row for row in range(n) if not done[row]]
            p = max(cand, key=lambda row: (abs(a[row, pc]), -row))
        piv_row[s] = p
        inv = 1.0 / a[p, pc]
        for row in range(n):
            if done[row] or row == p:
                continue
            f = a[row, pc] * inv
            for c in range(n):
                if nz(s, c, N1):
                    a[row, c] -= f * a[p, c]
            r[row] -= f * r[p]
        done[p] = True
    if rows_out is not None:
        rows_out[:] = piv_row
    x = np.zeros_like(r)
    for s in range(n - 1, -1, -1):
        pc = col(s, N1)
        p = piv_row[s]
        rhs = r[p] - sum(a[p, col(t, N1)] * x[col(t, N1)] for t in range(s + 1, n))
        x[pc] = rhs / a[p, pc]
    return x


@pytest.mark.parametrize("N1", [2, 3, 4, 8])
@pytest.mark.parametrize("seed", [0, 1])
def test_dfirst_lu_with_pivoting_solves_the_dens_sparse_block(N1, seed):
    """DENS-sparse blocks with a dominant diagonal only in the DENS block, so that the MOMZ/RHOT phase
    exchanges rows: solved to roundoff."""
    rng = np.random.default_rng(seed)
    n, N = 3 * N1, N1 - 1
    A = rng.standard_normal((n, n))
    for k in range(N1):
        A[3 * k, :] *= 0.1
        A[3 * k, 3 * k] = 3.0
        for c in range(n):
            if not (c == 3 * k or c == 0 or c == 3 * N or c % 3 == 1 or c == 2):
                A[3 * k, c] = 0.0
    for k in range(N1):
        A[3 * k + 1, 3 * k + 1] = 1e-9
    R = rng.standard_normal((n, 4))
    rows = np.zeros(n, int)
    X = dfirst_pivoting_solve(A, R, N1, rows_out=rows)
    ref = np.linalg.solve(A, R)
    assert np.max(np.abs(X - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref)))
    assert any(rows[s] != col(s, N1) for s in range(N1, n))  # rows were exchanged


def dens_sparse_block(rng, N1):
    """A random element block with the DENS rows' sparsity and an FP64-kernel-like conditioning: a
    dominant DENS diagonal, a weak MOMZ diagonal (the MOMZ/RHOT phase exchanges rows)."""
    n, N = 3 * N1, N1 - 1
    A = rng.standard_normal((n, n))
    for k in range(N1):
        A[3 * k, :] *= 0.1
        A[3 * k, 3 * k] = 3.0
        for c in range(n):
            if not (c == 3 * k or c == 0 or c == 3 * N or c % 3 == 1 or c == 2):
                A[3 * k, c] = 0.0
        A[3 * k + 1, 3 * k + 1] = 1e-9
    return A


def two_column_kernel_solve(A, R, N1, zeros_out=None):
    """The FP64 kernel's elimination with the skips of its two-columns-per-warp form (fedg_vi.cu:
    blk_fwd, blk_bwd): the DENS rows eliminate only at step 0; their pivots' reciprocals are formed
    once their rows are final; the column-oriented back substitution updates a DENS row only at the
    MOMZ columns, RHOT_0 and DENS_N, and scales the DENS rows of nodes below N together after the
    DENS_N update.  zeros_out collects the entries the skips assume to be exact zeros."""
    n, N = 3 * N1, N1 - 1
    a, r = A.copy(), R.copy().astype(float)
    done = np.zeros(n, bool)
    piv_row = np.zeros(n, int)
    for s in range(n):
        pc = col(s, N1)
        if s < N1:
            p = pc
        else:
            cand = [row for row in range(n) if not done[row] and row % 3 != 0]
            p = max(cand, key=lambda row: (abs(a[row, pc]), -row))
        piv_row[s] = p
        inv = 1.0 / a[p, pc]
        for row in range(n):
            if done[row] or row == p:
                continue
            if row % 3 == 0 and s > 0:  # a DENS row: skipped past step 0
                if zeros_out is not None:
                    zeros_out.append(a[row, pc])
                continue
            f = a[row, pc] * inv
            for c in range(n):
                if nz(s, c, N1):
                    a[row, c] -= f * a[p, c]
            r[row] -= f * r[p]
        done[p] = True
    mypiv = {piv_row[s]: s for s in range(n)}
    for s in range(n - 1, -1, -1):  # column-oriented: scale the pivot row, then update the rows above it
        pc, p = col(s, N1), piv_row[s]
        if s >= N1 or s == N:
            r[p] = r[p] / a[p, pc]
        for row in range(n):
            if mypiv[row] >= s:
                continue
            dens_row = row % 3 == 0
            if dens_row and s >= N1 and not (pc % 3 == 1 or pc == 2):
                if zeros_out is not None:
                    zeros_out.append(a[row, pc])
                continue
            if dens_row and s < N and s > 0:
                if zeros_out is not None:
                    zeros_out.append(a[row, pc])
                continue
            r[row] -= a[row, pc] * r[p]
        if s == N:  # the DENS rows of the nodes below N are final: scale them together
            for k in range(N):
                r[3 * k] = r[3 * k] / a[3 * k, 3 * k]
    x = np.zeros_like(r)
    for s in range(n):
        x[col(s, N1)] = r[piv_row[s]]
    return x


@pytest.mark.parametrize("N1", [2, 3, 4, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_two_column_kernel_skips_only_exact_zeros(N1, seed):
    """The skips of the two-columns-per-warp FP64 kernel touch only entries that are exactly zero, so
    the kernel's arithmetic is the full DENS-first elimination's (its results are bit-identical to the
    one-column kernel's); and the restated skips still solve the block to roundoff."""
    rng = np.random.default_rng(seed)
    A = dens_sparse_block(rng, N1)
    R = rng.standard_normal((3 * N1, 4))
    zeros = []
    X = two_column_kernel_solve(A, R, N1, zeros_out=zeros)
    assert zeros and all(z == 0.0 for z in zeros)
    ref = np.linalg.solve(A, R)
    assert np.max(np.abs(X - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref)))


def blocked_solve(A, R, N1):
    """The FP32 kernel's blocked form of the same elimination (fe-project_gb300/csrc/fedg_vicol.cu,
    lu_blocked): DENS_0 first; the DENS pivots 1 .. N-1 together (their pivot rows and the other
    rows' multipliers are fixed once DENS_0 is eliminated, so the updates are independent); DENS_N;
    then the MOMZ/RHOT Schur complement node by node with 2x2 pivot blocks (MOMZ_k, RHOT_k), no
    exchanges; back substitution block by block, then DENS_N, then DENS_0 .. N-1 together."""
    n, N = 3 * N1, N1 - 1
    a, r = A.copy(), R.copy()
    mz = [3 * k + v for k in range(N1) for v in (1, 2)]
    sparse_cols = [c for c in range(n) if c == 3 * N or c % 3 == 1 or c == 2]  # DENS-row nonzeros
    for row in range(1, n):  # DENS_0: every other row
        f = a[row, 0] / a[0, 0]
        for c in sparse_cols:
            a[row, c] -= f * a[0, c]
        r[row] -= f * r[0]
    if N1 > 2:  # DENS_1 .. DENS_{N-1}: MOMZ/RHOT rows, multipliers left by the DENS_0 step
        F = {(row, s): a[row, 3 * s] / a[3 * s, 3 * s] for row in mz for s in range(1, N)}
        for row in mz:
            for s in range(1, N):
                for c in sparse_cols:
                    a[row, c] -= F[row, s] * a[3 * s, c]
                r[row] -= F[row, s] * r[3 * s]
    for row in mz:  # DENS_N
        f = a[row, 3 * N] / a[3 * N, 3 * N]
        for c in sparse_cols:
            if c != 3 * N:
                a[row, c] -= f * a[3 * N, c]
        r[row] -= f * r[3 * N]
    Pinv = []
    for k in range(N1):  # MOMZ/RHOT 2x2 blocks
        b = [3 * k + 1, 3 * k + 2]
        Pi = np.linalg.inv(a[np.ix_(b, b)])
        Pinv.append(Pi)
        later = [3 * m + v for m in range(k + 1, N1) for v in (1, 2)]
        for row in later:
            f = a[row, b] @ Pi
            for c in later:
                a[row, c] -= f[0] * a[b[0], c] + f[1] * a[b[1], c]
            r[row] -= f[0] * r[b[0]] + f[1] * r[b[1]]
    x = np.zeros_like(r)
    for k in range(N1 - 1, -1, -1):
        b = [3 * k + 1, 3 * k + 2]
        later = [3 * m + v for m in range(k + 1, N1) for v in (1, 2)]
        y = r[b] - a[np.ix_(b, later)] @ x[later] if later else r[b]
        x[b] = Pinv[k] @ y
    x[3 * N] = (r[3 * N] - a[3 * N, mz] @ x[mz]) / a[3 * N, 3 * N]
    for s in range(N):
        cols = mz + [3 * N]
        x[3 * s] = (r[3 * s] - a[3 * s, cols] @ x[cols]) / a[3 * s, 3 * s]
    return x


@pytest.mark.parametrize("N1", [4, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_blocked_lu_solves_the_dens_sparse_block(N1, seed):
    rng = np.random.default_rng(seed)
    n, N = 3 * N1, N1 - 1
    A = 0.1 * rng.standard_normal((n, n)) + 3.0 * np.eye(n)
    for k in range(N1):
        for c in range(n):
            if not (c == 3 * k or c == 0 or c == 3 * N or c % 3 == 1 or c == 2):
                A[3 * k, c] = 0.0
    R = rng.standard_normal((n, 4))
    assert np.max(np.abs(blocked_solve(A, R, N1) - np.linalg.solve(A, R))) < 1e-13
