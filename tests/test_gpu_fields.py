"""GPU parity on the height-field workloads and the cube with IC(0), through the C ABI.

The height fields are the single-large-chart workloads (a 1024^2 grid with 8 sines at
amplitude 0.15, a 2048^2 grid with 16 sines at amplitude 0.3) at reduced sizes: the same
generator, the same chart stages, every chart compared with the FP64 sparse-LU oracle
(SuperLU on the scalar Laplacian, both coordinates, then the reference's damped driver).
Bars: mixed precision <= 1e-6 and FP64 <= 1e-10 in the reference's normalised max-abs
(unwrap/src/lscm.rs:749-758), with the smoothed-aggregation AMG and the colour-ordered IC(0)
preconditioners.  The chart partition and every CSR system are bit-identical to the oracle.

The cube (six 6 x 6 faces) is solved by the FP64 PCG with IC(0) and compared with the
restated reference LU at <= 1e-10.
"""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = {R.Precision.MIXED: 1e-6, R.Precision.FP64: 1e-10}


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


_FIELDS = {}


def _field(n, n_sines, amp):
    """Height field, its oracle pipeline (systems only) and the SuperLU UVs of every chart."""
    key = (n, n_sines, amp)
    if key not in _FIELDS:
        p, f = W.height_field(n, n_sines, amp, seed=2)
        P = O.Pipeline(p, f, lu_limit=0)
        uv_lu = [P.superlu_uv(c) for c in range(P.n_charts)]
        _FIELDS[key] = (p, f, P, uv_lu)
    return _FIELDS[key]


def _check(ctx, key, precision, precond):
    p, f, P, uv_lu = _field(*key)
    C = R.prepare_mesh(p, f)
    assert C.n_charts == P.n_charts
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=precision, precond=precond))
    worst = 0.0
    for c in range(P.n_charts):
        ref = P.chart(c)
        rp, cols, vals, rhs = R.export_chart_system(ctx, c)
        assert np.array_equal(rp, ref["csr_ptr"]) and np.array_equal(cols, ref["csr_cols"])
        assert np.array_equal(vals.view(np.uint64), ref["csr_vals"].view(np.uint64))
        assert res[c].status == R.Status.OK, (c, R.Status(res[c].status).name)
        err = O.uv_error(res[c].uv, uv_lu[c])
        worst = max(worst, err)
        assert err <= TOL[precision], f"chart {c}: uv error {err:.3e}"
    return worst, res


@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
@pytest.mark.parametrize("precond", [R.Precond.AMG_SA, R.Precond.IC0_COLOR])
def test_height_field_256_matches_superlu(ctx, precision, precond):
    """The 1024^2 / 8-sine / 0.15 family at 256^2: one chart of 64k free vertices."""
    _check(ctx, (256, 8, 0.15), precision, precond)


@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
def test_height_field_512_matches_superlu(ctx, precision):
    """The 1024^2 family at 512^2 (a 258k-vertex chart) with AMG-SA."""
    _check(ctx, (512, 8, 0.15), precision, R.Precond.AMG_SA)


@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
def test_height_field_384_natural_ic0_matches_superlu(ctx, precision):
    """Natural-order IC(0) on one 146k-vertex chart: about 760 dependency levels, so the
    factorization and sweeps run sync-free over the whole GPU."""
    _check(ctx, (384, 8, 0.15), precision, R.Precond.IC0)


@pytest.mark.parametrize("precond", [R.Precond.AMG_SA, R.Precond.AMG, R.Precond.IC0_COLOR])
def test_anisotropic_field_512_matches_superlu(ctx, precond):
    """The 2048^2 / 16-sine / 0.3 family at 512^2: ridges cut at 30 degrees into several
    charts, strongly anisotropic triangles; mixed precision."""
    worst, res = _check(ctx, (512, 16, 0.3), R.Precision.MIXED, precond)
    assert len(res) > 1


@pytest.mark.parametrize("precond", [R.Precond.AMG_SA, R.Precond.AMG])
def test_kcycle_field_matches_superlu(ctx, monkeypatch, precond):
    """The K-cycle (two coarse corrections with per-chart CG steplengths on the top two
    levels, gpu/src/amg.rs:468-639) on the anisotropic family: every chart converges and meets
    the same UV bar against SuperLU as the V(1,1) cycle.  (It takes more CG iterations than the
    V(1,1) cycle with its over-corrected coarse space on these charts, which is why it is an
    option and not the default.)"""
    monkeypatch.setenv("RUV_AMG_KCYCLE", "2")
    _check(ctx, (512, 16, 0.3), R.Precision.MIXED, precond)


def test_cube_fp64_ic0_matches_cpu_lu(ctx):
    """cube(6) welded and charted into 6 planar charts, FP64 PCG + IC(0) vs the reference LU."""
    p, f = O.cube(6)
    P = O.Pipeline(p, f)
    C = R.prepare_mesh(p, f)
    assert C.n_charts == P.n_charts == 6
    for pc in (R.Precond.IC0, R.Precond.IC0_COLOR):
        res = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=R.Precision.FP64, precond=pc))
        for c in range(6):
            ref = P.chart(c)
            assert res[c].status == R.Status.OK
            assert O.uv_error(res[c].uv, ref["uv"]) <= 1e-10
            assert res[c].iters == ref["iters"] == 2
