"""Launch shapes on the GPU: every CG SpMV shape the library instantiates solves the batch to
the LU bar, the autotuner keeps one of them and its solves stay on the bar, and the AMG
smoothers' lane rules and one-lane shapes are interchangeable (the one-lane shapes bit for
bit: one lane sums its row in entry order whatever the number of rows in flight).

Bars: mixed precision <= 1e-6 normalised max-abs against the FP64 sparse LU of each chart
(unwrap/src/lscm.rs:749-758 normalisation), as in test_gpu_parity.py.
"""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6

# (lanes per row, rows in flight) of every instantiated CG SpMV shape (pcg.cu RUV_SHAPES)
SHAPES = [(1, 2), (2, 2), (2, 4), (4, 1), (4, 2), (4, 4), (8, 1), (8, 2), (8, 4), (16, 1), (32, 1)]


@pytest.fixture(scope="module")
def disks():
    vo, to, p3, tr = W.disks(10, t_min=100, t_max=8000, seed=29)
    C = R.prepare_patches(vo, to, p3, tr)
    ref = []
    for c in range(len(vo) - 1):
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        ref.append(P.superlu_uv(0))
    return C, ref


def _check(res, ref):
    for c, r in enumerate(res):
        assert r.status == R.Status.OK, (c, r.status)
        assert O.uv_error(r.uv, ref[c]) <= MIXED_TOL, c


@pytest.mark.parametrize("lpr,unroll", SHAPES)
def test_every_spmv_shape_meets_the_lu_bar(monkeypatch, disks, lpr, unroll):
    C, ref = disks
    monkeypatch.setenv("RUV_LPR", str(lpr))  # read when the context is created
    monkeypatch.setenv("RUV_UNROLL", str(unroll))
    monkeypatch.setenv("RUV_TILE_ROWS", "256")
    ctx = R.Context(0)
    for pc in (R.Precond.JACOBI, R.Precond.AMG_SA):
        _check(R.unfold_charts(ctx, C, R.UnfoldOptions(precond=pc)), ref)


def test_autotuner_keeps_an_instantiated_shape(disks):
    C, ref = disks
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precond=R.Precond.AMG_SA)
    _check(R.unfold_charts(ctx, C, opts), ref)  # assembles the batch the tuner times
    lpr, unroll, tile, ms = R.autotune(ctx, R.Precision.MIXED, reps=2)
    assert (lpr, unroll) in SHAPES
    assert tile in (128, 256, 512, 1024)
    assert ms > 0.0
    assert R.spmv_form(ctx) in (0, 1)
    _check(R.unfold_charts(ctx, C, opts), ref)


def test_smoother_lane_rules_and_one_lane_shapes(monkeypatch, disks):
    """The smoothers' lane rule (one lane per row at level 0) against the transfer rule
    (RUV_AMG_SMOOTH_LANES=0) and per-level overrides: all on the LU bar with the same CG
    iterations; the two one-lane shapes (RUV_AMG_L1SHAPE 1 and 0) and the two two-lane shapes
    (RUV_AMG_L2SHAPE 0 and 1) bit for bit."""
    C, ref = disks
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precond=R.Precond.AMG_SA)
    base = R.unfold_charts(ctx, C, opts)
    _check(base, ref)
    for knob, v in (("RUV_AMG_L1SHAPE", "0"), ("RUV_AMG_L2SHAPE", "1")):
        monkeypatch.setenv(knob, v)
        other = R.unfold_charts(ctx, C, opts)
        for a, b in zip(base, other):
            assert a.cg_iters == b.cg_iters
            assert np.array_equal(a.uv, b.uv)
        monkeypatch.delenv(knob)
    for env in ({"RUV_AMG_SMOOTH_LANES": "0"}, {"RUV_AMG_LANES": "2/4/16/1"}, {"RUV_AMG_TLANES": "1,8"}):
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        res = R.unfold_charts(ctx, C, opts)
        _check(res, ref)
        for k in env:
            monkeypatch.delenv(k)
