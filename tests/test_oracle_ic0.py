"""The oracle's IC(0) / colouring restatement pinned against the assertions of the reference's
own tests (gpu/src/precond.rs:708-760, solver.rs:890-910).  CPU only."""
import numpy as np

from oracle import oracle as O
from systems import banded, lap1d


def test_factor_reproduces_matrix_on_its_pattern():
    """precond.rs:708-735: L L^T equals A on every stored entry (zero fill-in), 1e-9 relative."""
    a = banded(200, 3)
    f = O.Ic0(a.row_ptr, a.cols, a.vals)
    assert f.ok
    n = a.rows()
    L = np.zeros((n, n))
    for i in range(n):
        for k in range(f.l_ptr[i], f.l_ptr[i + 1]):
            L[i, f.l_cols[k]] = f.l_vals[k]
        assert f.l_cols[f.l_ptr[i + 1] - 1] == i  # diagonal last
    LL = L @ L.T
    for i in range(n):
        for k in range(a.row_ptr[i], a.row_ptr[i + 1]):
            j = a.cols[k]
            assert abs(LL[i, j] - a.vals[k]) < 1e-9 * (1.0 + abs(a.vals[k]))


def test_levels_respect_dependencies():
    """precond.rs:737-752 (every row levelled once) and the layering rule of tri_levels."""
    a = banded(150, 2)
    f = O.Ic0(a.row_ptr, a.cols, a.vals)
    for ptr, cols, lev in [(f.l_ptr, f.l_cols, f.fwd_level), (f.lt_ptr, f.lt_cols, f.bwd_level)]:
        for i in range(a.rows()):
            deps = cols[ptr[i]:ptr[i + 1] - 1]
            assert lev[i] == (max(lev[deps]) + 1 if len(deps) else 0)


def test_colored_ordering_bounds_levels():
    """solver.rs:890-910."""
    a, _ = lap1d(20_000)
    c = O.Ic0(a.row_ptr, a.cols, a.vals, colored=True)
    n_colors = int(c.color.max()) + 1
    assert n_colors <= 8
    assert c.fwd_level.max() + 1 <= n_colors + 1 and c.bwd_level.max() + 1 <= n_colors + 1
    assert np.array_equal(np.sort(c.to_orig), np.arange(a.rows()))
    nat = O.Ic0(a.row_ptr, a.cols, a.vals)
    assert nat.fwd_level.max() + 1 > 1000


def test_host_apply_inverts_the_factor():
    a = banded(400, 3)
    f = O.Ic0(a.row_ptr, a.cols, a.vals)
    r = np.array([((i * 7919) % 101) / 101.0 - 0.5 for i in range(a.rows())])
    z = f.apply(r)
    n = a.rows()
    L = np.zeros((n, n))
    for i in range(n):
        for k in range(f.l_ptr[i], f.l_ptr[i + 1]):
            L[i, f.l_cols[k]] = f.l_vals[k]
    assert np.abs(L @ (L.T @ z) - r).max() < 1e-12


def test_zero_pivot_is_none():
    f = O.Ic0(np.array([0, 1, 2]), np.array([0, 1]), np.array([1.0, 0.0]))
    assert not f.ok
