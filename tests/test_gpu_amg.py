"""The device AMG hierarchy against dense references, as the reference's own AMG tests check
its host hierarchy (gpu/src/amg.rs:800-942): the pairwise aggregation covers every row, the
tentative prolongator is the aggregate indicator, the smoothed prolongator is
(I - w D^-1 A) P_t (w = 2/3, amg.rs:308-362), every coarse operator is the Galerkin product
P^T A P of the level above, and the hierarchy stays symmetric positive definite and bottoms
out at a directly solved level.  The system is the 2-D 5-point Poisson matrix."""
import numpy as np
import pytest

import researchuv_gb300 as R

pytestmark = pytest.mark.gpu

OMEGA = 2.0 / 3.0
DIRECT_ROWS = 64  # a chart of at most this many rows is solved directly


def poisson(m):
    rp, cols, vals = [0], [], []
    for i in range(m):
        for j in range(m):
            r = i * m + j
            for c, v, keep in ((r - m, -1.0, i > 0), (r - 1, -1.0, j > 0), (r, 4.0, True),
                               (r + 1, -1.0, j < m - 1), (r + m, -1.0, i < m - 1)):
                if keep:
                    cols.append(c)
                    vals.append(v)
            rp.append(len(cols))
    return R.CsrMatrix(np.array(vals), np.array(cols), np.array(rp))


def dense(ptr, cols, vals, n, m):
    d = np.zeros((n, m))
    rows = np.repeat(np.arange(n), np.diff(ptr))
    np.add.at(d, (rows, cols), np.asarray(vals, np.float64))
    return d


@pytest.fixture(scope="module")
def solver():
    s = R.GpuSolver.new()
    assert s is not None
    return s


@pytest.fixture(scope="module")
def A():
    return poisson(32)


def level(solver, A, k, smoothed):
    L = solver.amg_level(A, k, smoothed)
    n, nc = L["rows"], L["next_rows"]
    L["Ad"] = dense(*L["A"], n, n)
    L["Pd"] = dense(*L["P"], n, nc) if nc > 0 else None
    return L


@pytest.mark.parametrize("smoothed", [False, True])
def test_aggregation_covers_every_row(solver, A, smoothed):
    """amg.rs:800-808: every row in exactly one aggregate, no aggregate empty."""
    L = level(solver, A, 0, smoothed)
    assert L["levels"] >= 2 and L["rows"] == A.rows()
    agg, nc = L["agg"], L["next_rows"]
    assert 0 < nc < L["rows"]
    assert agg.min() >= 0 and agg.max() == nc - 1
    assert np.bincount(agg, minlength=nc).min() >= 1


def test_tentative_prolongator_and_galerkin(solver, A):
    """The tentative prolongator is the aggregate indicator, and the next operator is
    P^T A P (amg.rs:844-874) -- FP64 sums of the level's entries."""
    L0 = level(solver, A, 0, False)
    assert not L0["smoothed"]
    n, nc = L0["rows"], L0["next_rows"]
    indicator = np.zeros((n, nc))
    indicator[np.arange(n), L0["agg"]] = 1.0
    assert np.array_equal(L0["Pd"], indicator)
    assert np.array_equal(L0["Ad"], dense(A.row_ptr, A.cols, A.vals, n, n))
    L1 = level(solver, A, 1, False)
    want = indicator.T @ L0["Ad"] @ indicator
    assert L1["rows"] == nc
    assert np.abs(L1["Ad"] - want).max() <= 1e-12 * np.abs(want).max()


def test_smoothed_prolongator_and_galerkin(solver, A, monkeypatch):
    """The smoothed prolongator without truncation is (I - w D^-1 A) P_t (amg.rs:811-841, FP32
    on the device) and the next operator is P^T A P with those P values (FP64 products)."""
    monkeypatch.setenv("RUV_AMG_PMAX", "48")  # keep every entry of a row
    L0 = level(solver, A, 0, True)
    assert L0["smoothed"]
    n, nc = L0["rows"], L0["next_rows"]
    Ad = L0["Ad"]
    Pt = np.zeros((n, nc))
    Pt[np.arange(n), L0["agg"]] = 1.0
    want_p = Pt - OMEGA * (Ad / np.diag(Ad)[:, None]) @ Pt
    assert np.abs(L0["Pd"] - want_p).max() <= 1e-6
    assert np.array_equal(L0["Pd"] != 0.0, want_p != 0.0)
    L1 = level(solver, A, 1, True)
    P = L0["Pd"]  # the FP32 values the device multiplies with, exactly
    want = P.T @ Ad @ P
    assert L1["rows"] == nc
    assert np.abs(L1["Ad"] - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("smoothed", [False, True])
def test_hierarchy_spd_and_bottoms_out(solver, A, smoothed):
    """amg.rs:890-942: every level symmetric positive definite, each coarser than the last, the
    last one small enough to solve directly."""
    K = level(solver, A, 0, smoothed)["levels"]
    rows = []
    for k in range(K):
        L = level(solver, A, k, smoothed)
        Ad = L["Ad"]
        assert np.abs(Ad - Ad.T).max() <= 1e-12 * np.abs(Ad).max()
        assert np.linalg.eigvalsh(Ad).min() > 0.0
        rows.append(L["rows"])
        assert (L["next_rows"] == 0) == (k == K - 1)
    assert all(b < a for a, b in zip(rows, rows[1:]))
    assert rows[-1] <= DIRECT_ROWS


def test_level_out_of_range_is_bad_input(solver, A):
    K = level(solver, A, 0, True)["levels"]
    with pytest.raises(R.RuvError):
        solver.amg_level(A, K, True)
