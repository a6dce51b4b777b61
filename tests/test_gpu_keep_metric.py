"""KeepMetric on the GPU (ruv_lscm_solve_batch_keep_metric: the bordered system solved by its
Schur complement over two batched PCG solves) against the oracle's restatement of the
reference (lscm.rs:544-568, :642-727: the bordered system factored by the sparse LU every
driver iteration).  Bars: the same driver iteration counts, and UVs within 1e-6 (the UV
error of lscm.rs:749-758) -- on charts whose loop converges in two iterations (annulus,
cylinder), a flat chart whose bordered system is singular (the reference's LU fails on the
first iteration and the UVs stay at the tangent frame), closed charts (four anchors), the
cube's charts and a disk whose fully pinned border fixes the area (the loop runs to
max_iter)."""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _disk():
    vo, to, p3, tr = W.disks(3, t_min=200, t_max=600, seed=5)
    return p3[vo[0]:vo[1]], tr[to[0]:to[1]]


CASES = {
    "annulus": lambda: O.torus_annulus(2.0, 0.7, 32, 20),
    "cylinder": lambda: O.cylinder(1.0, 2.0, 24, 8),
    "grid_singular": lambda: O.grid(12, 12),
    "torus_closed": lambda: O.torus(2.0, 0.7, 24, 12),
    "sphere_closed": lambda: O.uv_sphere(16, 8),
    "cube": lambda: O.cube(4),
    "disk_max_iter": _disk,
}


@pytest.mark.parametrize("precision", [R.Precision.FP64, R.Precision.MIXED])
@pytest.mark.parametrize("name", sorted(CASES))
def test_keep_metric_matches_reference_lu(name, precision):
    ctx = R.Context(0)
    p, f = CASES[name]()
    P = O.Pipeline(p, f, keep_metric=True, lu_limit=100000)
    C = R.prepare_mesh(p, f)
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(keep_metric=True, precision=precision, precond=R.Precond.JACOBI))
    assert len(res) == P.n_charts
    for c in range(P.n_charts):
        uv_ref = P.bag.f64(f"c{c}.uv").reshape(-1, 2)
        it_ref = int(P.bag.i64(f"c{c}.iters")[0])
        assert res[c].iters == it_ref, (c, res[c].iters, it_ref)
        assert O.uv_error(res[c].uv, uv_ref) <= 1e-6, (c, O.uv_error(res[c].uv, uv_ref))


def test_keep_metric_target_area_and_default_path_unchanged():
    """An explicit target_area reaches the area row; the default path is untouched."""
    ctx = R.Context(0)
    p, f = O.torus_annulus(2.0, 0.7, 32, 20)
    C = R.prepare_mesh(p, f)
    P = O.Pipeline(p, f, keep_metric=True, target_area=30.0, lu_limit=100000)
    res = R.unfold_charts(ctx, C, R.UnfoldOptions(keep_metric=True, target_area=30.0, precision=R.Precision.FP64))
    assert O.uv_error(res[0].uv, P.bag.f64("c0.uv").reshape(-1, 2)) <= 1e-6
    D = O.Pipeline(p, f, lu_limit=100000)
    res0 = R.unfold_charts(ctx, C, R.UnfoldOptions(precision=R.Precision.FP64))
    assert O.uv_error(res0[0].uv, D.bag.f64("c0.uv").reshape(-1, 2)) <= 1e-6
