"""Sparse test systems of the reference's own GPU-solver tests (gpu/src/solver.rs tests,
gpu/src/precond.rs tests), built as CsrMatrix + right-hand side."""
import numpy as np

import researchuv_gb300 as R


def lap1d(n):
    """solver.rs laplacian_1d: tridiagonal (-1, 2, -1), b = e_0 + e_{n-1} (solution all ones)."""
    vals, cols, rp = [], [], [0]
    for i in range(n):
        if i > 0:
            vals.append(-1.0)
            cols.append(i - 1)
        vals.append(2.0)
        cols.append(i)
        if i + 1 < n:
            vals.append(-1.0)
            cols.append(i + 1)
        rp.append(len(vals))
    b = np.zeros(n)
    b[0] = b[-1] = 1.0
    return R.CsrMatrix(np.array(vals), np.array(cols), np.array(rp)), b


def poisson(side):
    """solver.rs preconditioning_reduces_iterations: 5-point Poisson on side x side, diagonal
    4.05 on every 11th row, b_i = (i mod 97) * 0.01 + 1."""
    n = side * side
    rows, cols, vals = [], [], []
    for rr in range(side):
        for cc in range(side):
            i = rr * side + cc
            for r2, c2 in [(rr - 1, cc), (rr, cc - 1)]:
                if r2 >= 0 and c2 >= 0:
                    rows.append(i); cols.append(r2 * side + c2); vals.append(-1.0)
            rows.append(i); cols.append(i); vals.append(4.05 if i % 11 == 0 else 4.0)
            for r2, c2 in [(rr + 1, cc), (rr, cc + 1)]:
                if r2 < side and c2 < side:
                    rows.append(i); cols.append(r2 * side + c2); vals.append(-1.0)
    rp = np.concatenate([[0], np.cumsum(np.bincount(np.array(rows), minlength=n))])
    return R.CsrMatrix(np.array(vals), np.array(cols), rp), (np.arange(n) % 97) * 0.01 + 1.0


def banded(n, band):
    """precond.rs diag_dominant_banded: off-diagonals -0.25/d, diagonal 4 + (i mod 11) * 0.75."""
    vals, cols, rp = [], [], [0]
    for i in range(n):
        for d in range(1, band + 1):
            if i >= d:
                vals.append(-0.25 / d)
                cols.append(i - d)
        vals.append(4.0 + (i % 11) * 0.75)
        cols.append(i)
        for d in range(1, band + 1):
            if i + d < n:
                vals.append(-0.25 / d)
                cols.append(i + d)
        rp.append(len(vals))
    return R.CsrMatrix(np.array(vals), np.array(cols), np.array(rp))
