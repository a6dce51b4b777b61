"""IC(0) and colour-ordered IC(0) on the GPU against the oracle's restatement of the
reference's factor_ic0 / tri_levels / graph_coloring / permute_csr (gpu/src/precond.rs:49-262),
and the reference's own IC(0) tests (precond.rs:708-760, :886-927; solver.rs:830-935).

Bars: the device factor (pattern and FP64 values) and the colour permutation are
bit-identical to the oracle's; the device apply is within 1e-9 of the host sweeps (the
reference's bar); PCG with IC(0) reaches the plain-CG solution with fewer iterations; the
batched LSCM solve with IC(0) meets the 1e-6 UV bar against FP64 LU.
"""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W
from systems import banded, lap1d, poisson

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    return R.GpuSolver.global_()


def _systems(ctx):
    out = [("banded200", banded(200, 3)), ("poisson30", poisson(30)[0]), ("lap1d1000", lap1d(1000)[0])]
    p, f = O.grid(24, 24)
    C = R.prepare_mesh(p, f)
    R.unfold_charts(ctx, C, R.UnfoldOptions(precision=R.Precision.FP64))
    rp, cols, vals, _ = R.export_chart_system(ctx, 0)
    out.append(("lscm_grid24", R.CsrMatrix(vals, cols, rp)))
    return out


def _same_factor(dev, ref):
    assert np.array_equal(dev["ptr"], ref.l_ptr)
    assert np.array_equal(dev["cols"], ref.l_cols)
    assert np.array_equal(dev["vals"].view(np.uint64), ref.l_vals.view(np.uint64)), "factor values differ (bitwise)"


def test_ic0_factor_bitwise(gpu):
    ctx = R.Context(0)
    for name, a in _systems(ctx):
        ref = O.Ic0(a.row_ptr, a.cols, a.vals)
        assert ref.ok
        dev = gpu.ic0_factor(a)
        _same_factor(dev, ref)
        assert np.array_equal(dev["to_orig"], np.arange(a.rows()))
        assert dev["levels"] == max(ref.fwd_level.max(), ref.bwd_level.max()) + 1, name
        assert dev["colours"] == 0


def test_ic0_colored_factor_bitwise(gpu):
    """precond.rs:49-123: greedy colouring in index order, colour-major permutation."""
    ctx = R.Context(0)
    for name, a in _systems(ctx):
        ref = O.Ic0(a.row_ptr, a.cols, a.vals, colored=True)
        assert ref.ok
        dev = gpu.ic0_factor(a, colored=True)
        assert np.array_equal(dev["to_orig"], ref.to_orig), name
        assert dev["colours"] == ref.color.max() + 1
        _same_factor(dev, ref)
        assert dev["levels"] == max(ref.fwd_level.max(), ref.bwd_level.max()) + 1, name


def test_colored_levels_bounded_on_elongated_system(gpu):
    """solver.rs:890-910: the 1-D system chains natural IC(0) (> 1000 levels) while the colour
    ordering bounds the levels by the colour count (+1)."""
    a, _ = lap1d(20_000)
    col = gpu.ic0_factor(a, colored=True)
    assert col["colours"] <= 8
    assert col["levels"] <= col["colours"] + 1
    nat = gpu.ic0_factor(a)
    assert nat["levels"] > 1000


def test_apply_ic0_matches_host_sweeps(gpu):
    """precond.rs:886-927: device apply vs the host forward/backward sweeps, max diff < 1e-9."""
    a = banded(400, 3)
    n = a.rows()
    r = np.array([((i * 7919) % 101) / 101.0 - 0.5 for i in range(n)])
    ref = O.Ic0(a.row_ptr, a.cols, a.vals)
    z_host = ref.apply(r)
    z = gpu.apply_ic0_for_test(a, r)
    assert z is not None, gpu.last_error
    assert np.abs(z - z_host).max() < 1e-9


def test_apply_ic0_rejects_bad_input(gpu):
    a = banded(10, 1)
    assert gpu.apply_ic0_for_test(a, np.zeros(5)) is None
    z = R.CsrMatrix(np.array([1.0, 0.0]), np.array([0, 1]), np.array([0, 1, 2]))  # zero pivot
    assert gpu.apply_ic0_for_test(z, np.ones(2)) is None and "BREAKDOWN" in gpu.last_error


def test_cg_ic0_poisson(gpu):
    """solver.rs:830-889: IC(0)-PCG reaches the plain-CG solution with fewer iterations."""
    a, b = poisson(400)
    x_none, it_none = gpu.cg_solve_precond(a, b, 100_000, 1e-10, R.Precond.NONE)
    r = gpu.cg_solve_precond(a, b, 100_000, 1e-10, R.Precond.IC0)
    assert r is not None, gpu.last_error
    x, it = r
    n = a.rows()
    for i in [0, n // 2, n - 1]:
        assert abs(x[i] - x_none[i]) < 1e-5
    assert it < it_none, (it, it_none)


def test_cg_ic0color_elongated(gpu):
    """solver.rs:912-935: colour-ordered IC(0) converges on the 200k 1-D system, faster than
    plain CG."""
    a, b = lap1d(200_000)
    x_none, it_none = gpu.cg_solve_precond(a, b, 200_000, 1e-10, R.Precond.NONE)
    r = gpu.cg_solve_precond(a, b, 200_000, 1e-10, R.Precond.IC0_COLOR)
    assert r is not None, gpu.last_error
    for i in [0, 100_000, 199_999]:
        assert abs(r[0][i] - x_none[i]) < 1e-5
    assert r[1] < it_none, (r[1], it_none)


@pytest.mark.parametrize("pc", [R.Precond.IC0, R.Precond.IC0_COLOR])
@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
def test_batched_disks_ic0_match_fp64_lu(pc, precision):
    ctx = R.Context(0)
    vo, to, p3, tr = W.disks(24, t_min=50, t_max=8000, seed=23)
    C = R.prepare_patches(vo, to, p3, tr)
    jac = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=precision, precond=R.Precond.JACOBI))
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=precision, precond=pc))
    big = max(range(len(res)), key=lambda c: res[c].n_free)
    for c in range(len(vo) - 1):
        assert res[c].status == R.Status.OK, (c, res[c].status)
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        assert O.uv_error(res[c].uv, P.superlu_uv(0)) <= 1e-6
    assert res[big].cg_iters < jac[big].cg_iters, (res[big].cg_iters, jac[big].cg_iters)


def _ic0_pair(gpu, a, r, monkeypatch, tickets):
    monkeypatch.setenv("RUV_IC0_TICKETS", "1" if tickets else "0")
    f = gpu.ic0_factor(a)
    z = gpu.apply_ic0_for_test(a, r)
    monkeypatch.delenv("RUV_IC0_TICKETS", raising=False)
    assert z is not None, gpu.last_error
    return f, z


@pytest.mark.parametrize("name", ["poisson300", "lap1d_chain"])
def test_ic0_sync_free_sweeps_bitwise(gpu, monkeypatch, name):
    """The sync-free (ticket) factorization and sweeps, used for charts with many dependency
    levels, against the per-chart level walk: the same factor and the same apply bit for bit,
    and the factor equal to the oracle's factor_ic0.  A 5-point Poisson grid (599 levels of up
    to 300 rows) and a pure chain (40000 levels of one row each)."""
    a = poisson(300)[0] if name == "poisson300" else lap1d(40_000)[0]
    n = a.rows()
    r = np.array([((i * 7919) % 101) / 101.0 - 0.5 for i in range(n)])
    f1, z1 = _ic0_pair(gpu, a, r, monkeypatch, True)
    f0, z0 = _ic0_pair(gpu, a, r, monkeypatch, False)
    for k in ("ptr", "cols"):
        assert np.array_equal(f1[k], f0[k])
    assert np.array_equal(f1["vals"].view(np.uint64), f0["vals"].view(np.uint64))
    assert np.array_equal(z1.view(np.uint64), z0.view(np.uint64))
    _same_factor(f1, O.Ic0(a.row_ptr, a.cols, a.vals))


def test_ic0_sync_free_wait_times_out(monkeypatch):
    """Every device-side dependency wait of the sync-free kernels is bounded: with a spin limit
    of 1 the waits run out, the call returns TIMEOUT, and the same context solves again once
    the limit is back to its default."""
    a, b = poisson(300)
    g = R.GpuSolver.new()
    monkeypatch.setenv("RUV_IC0_TICKETS", "1")
    monkeypatch.setenv("RUV_SPIN_LIMIT", "1")
    assert g.cg_solve_precond(a, b, 1000, 1e-10, R.Precond.IC0) is None
    assert "TIMEOUT" in g.last_error, g.last_error
    assert g.apply_ic0_for_test(a, b) is None and "TIMEOUT" in g.last_error
    monkeypatch.delenv("RUV_SPIN_LIMIT")
    r = g.cg_solve_precond(a, b, 100_000, 1e-10, R.Precond.IC0)
    assert r is not None, g.last_error
    x_none, _ = g.cg_solve_precond(a, b, 100_000, 1e-10, R.Precond.NONE)
    assert np.abs(r[0] - x_none).max() < 1e-5
