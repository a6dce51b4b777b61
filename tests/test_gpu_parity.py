"""GPU parity: the sm_103a path against the oracle, through the C ABI (libruv.so).

Bars (from the reference and the workload definitions):
* CSR pattern, values and right-hand side of every chart: bit-identical to the reference's
  Sparse::to_csr(2 nf) (unwrap/src/sparse.rs:69-84) as the oracle restates it.
* UVs: FP64 PCG <= 1e-10 normalised max-abs vs the CPU LU (the small cube workload);
  mixed precision <= 1e-6 vs FP64 LU; normalisation of unwrap/src/lscm.rs:749-758.
* Driver iterations and err_accum as the reference driver computes them.
* GpuSolver::cg_solve known answers (gpu/src/solver.rs:767-1109).
"""
import ctypes

import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W
from systems import lap1d as _lap1d, poisson as _poisson

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # FP64 PCG vs CPU LU (cube workload)
MIXED_TOL = 1e-6   # FP32 inner CG + FP64 refinement vs FP64 LU


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


def _solve_mesh(ctx, p, f, precision, weld_tol=1e-12, angle=30.0, lu_limit=6000):
    P = O.Pipeline(p, f, weld_tol=weld_tol, angle_deg=angle, lu_limit=lu_limit)
    C = R.prepare_mesh(p, f, weld_tol=weld_tol, angle_min_deg=angle)
    assert C.n_charts == P.n_charts
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=precision, precond=R.Precond.JACOBI))
    return P, C, res


def _check_system(ctx, P, c):
    ref = P.chart(c)
    rp, cols, vals, rhs = R.export_chart_system(ctx, c)
    assert np.array_equal(rp, ref["csr_ptr"]), "CSR row pointers differ"
    assert np.array_equal(cols, ref["csr_cols"]), "CSR pattern differs"
    assert np.array_equal(vals.view(np.uint64), ref["csr_vals"].view(np.uint64)), "CSR values differ (bitwise)"
    n2 = len(rp) - 1
    assert np.array_equal(rhs, ref["rhs"][:n2]), "right-hand side differs"


def test_cube_fp64_matches_cpu_lu(ctx):
    p, f = O.cube(6)
    P, C, res = _solve_mesh(ctx, p, f, R.Precision.FP64)
    for c in range(P.n_charts):
        _check_system(ctx, P, c)
        ref = P.chart(c)
        assert res[c].status == R.Status.OK
        assert O.uv_error(res[c].uv, ref["uv"]) <= FP64_TOL
        assert res[c].iters == ref["iters"] == 2
        assert abs(res[c].err_accum - ref["err_accum"]) <= 1e-9 * abs(ref["err_accum"])


@pytest.mark.parametrize("angle_mix", [0.0, 0.5])
def test_angle_mix_matches_cpu_lu(ctx, angle_mix):
    """#AngleDistanceMix below 1 (mix_b = 1 - angle_mix > 0: the pull towards the frame
    positions enters the right-hand side, lscm.rs:630-638): the same CSR systems and
    right-hand sides bit for bit, and the UVs of the FP64 solve within 1e-10 of the reference
    LU with its damped driver (the default angle_mix = 1 skips those zero terms)."""
    for p, f in (O.cube(6), O.uv_sphere(48, 24)):
        P = O.Pipeline(p, f, angle_mix=angle_mix, lu_limit=6000)
        C = R.prepare_mesh(p, f)
        assert C.n_charts == P.n_charts
        res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=R.Precision.FP64, precond=R.Precond.JACOBI,
                                                      angle_mix=angle_mix))
        for c in range(P.n_charts):
            _check_system(ctx, P, c)
            ref = P.chart(c)
            assert res[c].status == R.Status.OK
            if "uv" in ref:
                assert O.uv_error(res[c].uv, ref["uv"]) <= FP64_TOL
                assert res[c].iters == ref["iters"]


@pytest.mark.parametrize("precision", [R.Precision.FP64, R.Precision.MIXED])
def test_fixtures_match_cpu_lu(ctx, precision):
    tol = FP64_TOL if precision == R.Precision.FP64 else MIXED_TOL
    for name, (p, f) in [("grid32", O.grid(32, 32)), ("sphere", O.uv_sphere(48, 24)),
                         ("annulus", O.torus_annulus(2.0, 0.7, 64, 40)), ("cylinder", O.cylinder(1.0, 2.0, 32, 16))]:
        P, C, res = _solve_mesh(ctx, p, f, precision)
        for c in range(P.n_charts):
            _check_system(ctx, P, c)
            ref = P.chart(c)
            err = O.uv_error(res[c].uv, ref["uv"])
            # sphere: closed chart, 4 anchors -> conditioning ~1e7; FP64 CG to 1e-12 rel-res
            bound = tol if name != "sphere" else max(tol, 1e-6)
            assert err <= bound, f"{name} chart {c}: uv error {err:.3e} > {bound:.1e}"
            assert res[c].iters == ref["iters"]


def test_reference_gpu_parity_grid32(ctx, known):
    """unwrap/src/lscm.rs:733-760: GPU unfold of grid(32,32) within 1e-6 of the CPU solve."""
    p, f = O.grid(32, 32)
    P, C, res = _solve_mesh(ctx, p, f, R.Precision.MIXED)
    assert O.uv_error(res[0].uv, P.chart(0)["uv"]) < known["gpu_parity"]["grid32x32"]["rel_max_abs_lt"]


def test_batched_disks_match_fp64_lu(ctx):
    vo, to, p3, tr = W.disks(48, t_min=50, t_max=5000, seed=11)
    C = R.prepare_patches(vo, to, p3, tr)
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=R.Precision.MIXED))
    for c in range(len(vo) - 1):
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        assert P.n_charts == 1
        rp, cols, vals, rhs = R.export_chart_system(ctx, c)
        ref = P.chart(0)
        assert np.array_equal(cols, ref["csr_cols"]) and np.array_equal(vals, ref["csr_vals"])
        uv_lu = P.superlu_uv(0)
        assert res[c].status == R.Status.OK
        assert O.uv_error(res[c].uv, uv_lu) <= MIXED_TOL


def test_empty_and_fully_pinned_charts(ctx):
    """A chart whose vertices are all pinned (a lone triangle) has nf = 0: UVs are the pins."""
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    f = np.array([[0, 1, 2]])
    P = O.Pipeline(p, f)
    C = R.prepare_mesh(p, f)
    res = R.unfold_charts(ctx, C, R.UnfoldOptions())
    assert res[0].status == R.Status.OK and res[0].n_free == 0
    assert O.uv_error(res[0].uv, P.chart(0)["uv"]) == 0.0


def test_repeatable_bitwise(ctx):
    """Same batch twice -> bitwise identical UVs (deterministic reductions)."""
    vo, to, p3, tr = W.disks(16, t_min=200, t_max=3000, seed=5)
    C = R.prepare_patches(vo, to, p3, tr)
    a = R.unfold_charts(ctx, C)
    b = R.unfold_charts(ctx, C)
    for x, y in zip(a, b):
        assert np.array_equal(x.uv, y.uv)


# ------------------------------------------------------------------ GpuSolver known answers
def test_cg_laplacian_1d(known):
    k = known["gpu_cg"]["laplacian_1d_4096"]
    g = R.GpuSolver.global_()
    a, b = _lap1d(k["n"])
    x = g.cg_solve(a, b, k["max_iter"], k["tol"])
    assert x is not None, g.last_error
    assert np.abs(x - 1.0).max() < k["x_tol"]


def test_cg_banded_500k(known):
    k = known["gpu_cg"]["banded_500k"]
    n, band = k["n"], k["band"]
    i = np.arange(n)
    rows, cols, vals = [], [], []
    for d in range(band, 0, -1):
        m = i >= d
        rows.append(i[m]); cols.append(i[m] - d); vals.append(np.full(m.sum(), -0.25 / d))
    rows.append(i); cols.append(i); vals.append(np.full(n, 4.0))
    for d in range(1, band + 1):
        m = i + d < n
        rows.append(i[m]); cols.append(i[m] + d); vals.append(np.full(m.sum(), -0.25 / d))
    r = np.concatenate(rows); c = np.concatenate(cols); v = np.concatenate(vals)
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    rp = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=n))])
    a = R.CsrMatrix(v, c, rp)
    b = (i % 97) * 0.01 + 1.0
    x = R.GpuSolver.global_().cg_solve(a, b, k["max_iter"], k["tol"])
    assert x is not None
    for row in [0, n // 2, n - 1]:
        s = sum(a.vals[q] * x[a.cols[q]] for q in range(a.row_ptr[row], a.row_ptr[row + 1]))
        assert abs(s - b[row]) < k["row_check_tol"]


def test_cg_poisson_preconditioning(known):
    k = known["gpu_cg"]["poisson_400"]
    a, b = _poisson(400)
    g = R.GpuSolver.global_()
    x_none, it_none = g.cg_solve_precond(a, b, 100_000, k["tol"], R.Precond.NONE)
    x_j, it_j = g.cg_solve_precond(a, b, 100_000, k["tol"], R.Precond.JACOBI)
    n = a.rows()
    for i in [0, n // 2, n - 1]:
        assert abs(x_j[i] - x_none[i]) < k["x_agree_tol"]
    assert it_j <= it_none


def test_cg_mismatched_dimensions():
    a, b = _lap1d(8)
    assert R.GpuSolver.global_().cg_solve(a, b[:4], 10, 1e-10) is None


def test_cg_not_converged_and_breakdown():
    a, b = _lap1d(4096)
    g = R.GpuSolver.global_()
    assert g.cg_solve(a, b, 3, 1e-12) is None and "NOT_CONVERGED" in g.last_error
    z = R.CsrMatrix(np.array([0.0, 0.0]), np.array([0, 1]), np.array([0, 1, 2]))
    assert g.cg_solve(z, np.array([1.0, 1.0]), 10, 1e-12) is None and "BREAKDOWN" in g.last_error
    assert g.cg_solve_precond(z, np.array([1.0, 1.0]), 10, 1e-12, R.Precond.JACOBI) is None


# ------------------------------------------------------------------ AMG preconditioners
@pytest.mark.parametrize("kcycle", ["0", "2"])
@pytest.mark.parametrize("pc", [R.Precond.AMG, R.Precond.AMG_SA])
def test_batched_disks_amg_match_fp64_lu(ctx, pc, kcycle, monkeypatch):
    monkeypatch.setenv("RUV_AMG_KCYCLE", kcycle)
    vo, to, p3, tr = W.disks(40, t_min=50, t_max=20000, seed=21)
    C = R.prepare_patches(vo, to, p3, tr)
    jac = R.unfold_charts(ctx, C, R.UnfoldOptions(precond=R.Precond.JACOBI))
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(precond=pc))
    big = max(range(len(res)), key=lambda c: res[c].n_free)
    for c in range(len(vo) - 1):
        assert res[c].status == R.Status.OK, (c, res[c].status)
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        assert O.uv_error(res[c].uv, P.superlu_uv(0)) <= MIXED_TOL
    # the multigrid cycle needs far fewer Krylov iterations than Jacobi on the largest chart
    assert res[big].cg_iters * 3 < jac[big].cg_iters, (res[big].cg_iters, jac[big].cg_iters)


def test_cg_amg_poisson_and_elongated(known):
    """gpu/src/solver.rs:912-935, :1032-1102: AMG/AMG-SA converge to the plain-CG solution
    with fewer iterations on the 2-D Poisson and the elongated 1-D systems."""
    g = R.GpuSolver.global_()
    a, b = _poisson(400)
    x_none, it_none = g.cg_solve_precond(a, b, 100_000, 1e-10, R.Precond.NONE)
    for pc in (R.Precond.AMG, R.Precond.AMG_SA):
        r = g.cg_solve_precond(a, b, 100_000, 1e-10, pc)
        assert r is not None, g.last_error
        x, it = r
        n = a.rows()
        for i in [0, n // 2, n - 1]:
            assert abs(x[i] - x_none[i]) < 1e-4
        assert it < it_none, (pc, it, it_none)
    # kappa ~ 1e10: at equal residual the FP32 V-cycle leaves more low-mode error than plain
    # FP64 CG, so the multigrid solve runs one decade tighter to meet the 1e-5 agreement
    a, b = _lap1d(200_000)
    x_none, it_none = g.cg_solve_precond(a, b, 200_000, 1e-10, R.Precond.NONE)
    r = g.cg_solve_precond(a, b, 200_000, 1e-11, R.Precond.AMG_SA)
    assert r is not None, g.last_error
    for i in [0, 100_000, 199_999]:
        assert abs(r[0][i] - x_none[i]) < 1e-5
    assert r[1] < it_none


def test_batched_disks_16bit_columns(monkeypatch):
    """The 16-bit column streams (the default; RUV_NARROW_COLS=0 turns them off) give bitwise
    the same UVs as 32-bit columns, for the CG operator and for every AMG level."""
    vo, to, p3, tr = W.disks(16, t_min=200, t_max=6000, seed=17)
    C = R.prepare_patches(vo, to, p3, tr)
    ctx = R.Context(0)
    for pc in (R.Precond.JACOBI, R.Precond.AMG, R.Precond.AMG_SA):
        monkeypatch.setenv("RUV_NARROW_COLS", "0")
        wide = R.unfold_charts(ctx, C, R.UnfoldOptions(precond=pc))
        monkeypatch.delenv("RUV_NARROW_COLS", raising=False)
        narrow = R.unfold_charts(ctx, C, R.UnfoldOptions(precond=pc))
        for a, b in zip(wide, narrow):
            assert a.status == b.status == R.Status.OK
            assert np.array_equal(a.uv, b.uv)


def test_mixed_split_formed_in_fill(monkeypatch):
    """The assembly's fill pass forms the mixed solver's low FP32 halves and double-float row
    sums with the solver's own rounding: bitwise the same UVs as when the solver forms them
    (RUV_SPLIT_IN_FILL=0)."""
    vo, to, p3, tr = W.disks(16, t_min=200, t_max=6000, seed=19)
    C = R.prepare_patches(vo, to, p3, tr)
    ctx = R.Context(0)
    for pc in (R.Precond.JACOBI, R.Precond.AMG_SA):
        opts = R.UnfoldOptions(precond=pc, precision=R.Precision.MIXED)
        monkeypatch.setenv("RUV_SPLIT_IN_FILL", "0")
        solver = R.unfold_charts(ctx, C, opts)
        monkeypatch.delenv("RUV_SPLIT_IN_FILL", raising=False)
        fill = R.unfold_charts(ctx, C, opts)
        for a, b in zip(solver, fill):
            assert a.status == b.status == R.Status.OK
            assert np.array_equal(a.uv, b.uv)


def test_group_graph_bitwise(monkeypatch):
    """The group matching over a group graph built once per level (the default;
    RUV_AMG_GROUP_GRAPH=0 accumulates the group strengths again in every round) sees the same
    strengths in the same order: the same hierarchy, so the same iterations and UVs."""
    vo, to, p3, tr = W.disks(24, t_min=200, t_max=20000, seed=47)
    C = R.prepare_patches(vo, to, p3, tr)
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precond=R.Precond.AMG_SA, precision=R.Precision.MIXED)
    monkeypatch.setenv("RUV_AMG_GROUP_GRAPH", "0")
    old = R.unfold_charts(ctx, C, opts)
    monkeypatch.delenv("RUV_AMG_GROUP_GRAPH", raising=False)
    new = R.unfold_charts(ctx, C, opts)
    for a, b in zip(old, new):
        assert a.status == b.status == R.Status.OK
        assert a.cg_iters == b.cg_iters
        assert np.array_equal(a.uv, b.uv)


@pytest.mark.parametrize("case", ["disks_16bit_columns", "field_row_relative_columns", "field_32bit_columns"])
def test_bulk_copy_spmv_bitwise(monkeypatch, case):
    """The SpMV that stages each tile's row pointers, values and columns into shared memory
    by bulk asynchronous copies (RUV_SPMV_TMA=1) runs the same row loop as the CSR-vector
    kernel reading them from global memory (RUV_SPMV_TMA=0): bitwise the same UVs and iterations,
    with the chart-relative 16-bit column stream (charts of <= 65536 rows), the row-relative
    one (a 258k-row chart) and 32-bit columns (the same chart, RUV_NARROW_COLS=chart)."""
    if case == "disks_16bit_columns":
        vo, to, p3, tr = W.disks(24, t_min=200, t_max=20000, seed=53)
        C = R.prepare_patches(vo, to, p3, tr)
    else:
        p, f = W.height_field(512, 8, 0.15, seed=2)
        C = R.prepare_mesh(p, f)
    if case == "field_32bit_columns":
        monkeypatch.setenv("RUV_NARROW_COLS", "chart")
    ctx = R.Context(0)
    for pc in (R.Precond.JACOBI, R.Precond.AMG_SA):
        opts = R.UnfoldOptions(precond=pc, precision=R.Precision.MIXED)
        monkeypatch.setenv("RUV_SPMV_TMA", "0")
        plain = R.unfold_charts(ctx, C, opts)
        monkeypatch.setenv("RUV_SPMV_TMA", "1")
        staged = R.unfold_charts(ctx, C, opts)
        monkeypatch.delenv("RUV_SPMV_TMA", raising=False)
        for a, b in zip(plain, staged):
            assert a.status == b.status == R.Status.OK
            assert a.cg_iters == b.cg_iters
            assert np.array_equal(a.uv, b.uv)


@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
def test_row_relative_columns_bitwise(monkeypatch, precision):
    """A chart of more than 65536 rows (a 512^2 height field, 258k rows) streams its columns
    as 16-bit offsets from each row (every entry lies within 32767 rows of its row in the
    grid's order) on the system operator and the AMG levels: bitwise the same UVs and
    iterations as with 32-bit columns (RUV_NARROW_COLS=chart)."""
    p, f = W.height_field(512, 8, 0.15, seed=2)
    C = R.prepare_mesh(p, f)
    ctx = R.Context(0)
    for pc in (R.Precond.JACOBI, R.Precond.AMG_SA, R.Precond.AMG):
        opts = R.UnfoldOptions(precond=pc, precision=precision)
        monkeypatch.setenv("RUV_NARROW_COLS", "chart")
        wide = R.unfold_charts(ctx, C, opts)
        monkeypatch.delenv("RUV_NARROW_COLS", raising=False)
        rel = R.unfold_charts(ctx, C, opts)
        for a, b in zip(wide, rel):
            assert a.status == b.status == R.Status.OK
            assert a.cg_iters == b.cg_iters
            assert np.array_equal(a.uv, b.uv)


def test_bulk_copy_spmv_wait_is_bounded(monkeypatch):
    """The staging wait is bounded: with a spin limit of 1 a solve either finishes (the copies
    landed within the first try) or returns TIMEOUT, and the context then solves normally."""
    vo, to, p3, tr = W.disks(8, t_min=2000, t_max=20000, seed=59)
    C = R.prepare_patches(vo, to, p3, tr)
    nv = int(C.i64("chart.vert_off")[-1])
    ctx = R.Context(0)
    monkeypatch.setenv("RUV_SPMV_TMA", "1")
    monkeypatch.setenv("RUV_SPIN_LIMIT", "1")
    _, _, st = R.solve_batch(ctx, C.batch(), R.UnfoldOptions(precond=R.Precond.JACOBI), nv, check=False)
    assert st in (R.Status.OK, R.Status.TIMEOUT), R.Status(st).name
    monkeypatch.delenv("RUV_SPIN_LIMIT")
    _, stats, st = R.solve_batch(ctx, C.batch(), R.UnfoldOptions(precond=R.Precond.JACOBI), nv)
    assert st == R.Status.OK


@pytest.mark.parametrize("kernel,parts", [("1", None), ("0", None), ("1", "1"), ("1", "5"), ("0", "16")])
def test_pinned_inputs_bitwise(monkeypatch, kernel, parts):
    """The one-call entry with its inputs in page-locked host memory (copied by the SMs over
    the buffers' device mapping; RUV_H2D_KERNEL=0: by cudaMemcpyAsync) gives bitwise the UVs
    and statistics of the same batch from pageable memory and of the resident upload, for
    any number of upload parts (RUV_UPLOAD_PARTS; 16 is more than the 12 charts)."""
    monkeypatch.setenv("RUV_H2D_KERNEL", kernel)
    if parts is not None:
        monkeypatch.setenv("RUV_UPLOAD_PARTS", parts)
    vo, to, p3, tr = W.disks(12, t_min=200, t_max=20000, seed=67)
    C = R.prepare_patches(vo, to, p3, tr)
    nv = int(C.i64("chart.vert_off")[-1])
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precond=R.Precond.AMG_SA, precision=R.Precision.MIXED)
    uv_a, st_a, s_a = R.solve_batch(ctx, C.batch(), opts, nv)
    pb, keep = R.pinned_batch(ctx, C)
    out = R.pinned_empty(ctx, (nv, 2), np.float64)
    stats = (R.RuvChartStat * max(pb.n_charts, 1))()
    L = R.lib()
    ctx.check(L.ruv_lscm_solve_batch(ctx.h, ctypes.byref(pb), ctypes.byref(opts.to_c()),
                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), stats), "pinned solve")
    assert s_a == R.Status.OK
    assert np.array_equal(uv_a, out)
    assert [s.cg_iters for s in st_a] == [stats[c].cg_iters for c in range(pb.n_charts)]
    # the resident path (one upload on the main stream, no parts)
    ctx.check(L.ruv_lscm_upload(ctx.h, ctypes.byref(pb)), "upload")
    ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(opts.to_c()), stats), "resident solve")
    res = R.pinned_empty(ctx, (nv, 2), np.float64)
    ctx.check(L.ruv_lscm_download_uv(ctx.h, res.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "download")
    assert np.array_equal(uv_a, res)


def test_staged_smoothers_bitwise(monkeypatch):
    """Level 0's AMG smoothers with their tiles staged into shared memory by bulk copies
    (RUV_AMG_STAGE=1) run the same row loop: bitwise the same UVs and iterations.  Level 0's
    tiles at 1024 rows, whose staged rows always fit the 100 KB cap (at the default 2048 the
    largest tiles may not, and the smoothers then stay unstaged)."""
    vo, to, p3, tr = W.disks(24, t_min=200, t_max=20000, seed=61)
    C = R.prepare_patches(vo, to, p3, tr)
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precond=R.Precond.AMG_SA, precision=R.Precision.MIXED)
    monkeypatch.setenv("RUV_AMG_TILE", "1024")
    monkeypatch.setenv("RUV_AMG_STAGE", "0")
    plain = R.unfold_charts(ctx, C, opts)
    monkeypatch.setenv("RUV_AMG_STAGE", "1")
    staged = R.unfold_charts(ctx, C, opts)
    for a, b in zip(plain, staged):
        assert a.status == b.status == R.Status.OK
        assert a.cg_iters == b.cg_iters
        assert np.array_equal(a.uv, b.uv)
