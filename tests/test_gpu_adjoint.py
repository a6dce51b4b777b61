"""Differentiation and distortion metrics on the GPU (ruv_lscm_forward / ruv_lscm_backward,
ruv_distortion_loss, ruv_chart_distortion) against the oracle:

* chart_distortion (unwrap/src/metrics.rs:73-141): bit-identical to the reference's
  (per-triangle values without FMA contraction, per-chart sums in triangle order);
* the distortion loss and its explicit gradients: within 1e-10 relative of the oracle's;
* the position gradient of loss = sum_t area_t (s1/s2 - 1)^2 + lam |uv - target|^2 through
  the solve: within 1e-5 relative of the CPU LU adjoint and of FP64 central differences
  (h = 1e-6) on 64 random vertices (norm over the picked components).
"""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _sphere(n_lat, n_lon, seed=4):
    p, f = W.sh_sphere(n_lat, n_lon, seed=seed)
    C = R.prepare_patches(np.array([0, len(p)]), np.array([0, len(f)]), p, f)
    ch = C.chart(0)
    rng = np.random.Generator(np.random.PCG64(11))
    target = ch["p2"] + 0.01 * rng.standard_normal(ch["p2"].shape)
    return p, C, ch, target


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_chart_distortion_matches_reference_metric():
    ctx = R.Context(0)
    for p, f in [O.grid(32, 32), O.uv_sphere(48, 24), O.torus_annulus(2.0, 0.7, 64, 40), O.cube(6)]:
        P = O.Pipeline(p, f)
        C = R.prepare_mesh(p, f)
        vo = C.i64("chart.vert_off")
        uv, _, _ = R.solve_batch(ctx, C.batch(), R.UnfoldOptions(precision=R.Precision.FP64), int(vo[-1]))
        m = R.chart_distortion(ctx, uv, C.n_charts)
        for c in range(C.n_charts):
            ref = P.metrics(c, uv[vo[c]:vo[c + 1]])
            assert np.array_equal(m[c], ref), (c, m[c], ref)


def test_distortion_loss_and_gradients_match_oracle():
    ctx = R.Context(0)
    p, C, ch, _ = _sphere(24, 48)
    n = len(p)
    uv, _ = R.lscm_forward(ctx, C.batch(), R.UnfoldOptions(precision=R.Precision.FP64), n)
    loss, duv, dp = R.distortion_loss(ctx, uv, 1)
    F = O.FixedPinChart(p, ch["tris"], ch["pinned"].astype(np.int64), ch["pin_uv"])
    l_ref, duv_ref, dp_ref, _ = F.distortion(uv)
    assert abs(loss[0] - l_ref) <= 1e-10 * abs(l_ref)
    assert _rel(duv, duv_ref) <= 1e-10
    assert _rel(dp, dp_ref) <= 1e-10


@pytest.mark.parametrize("precision", [R.Precision.FP64, R.Precision.MIXED])
def test_adjoint_matches_lu_adjoint_and_finite_differences(precision):
    ctx = R.Context(0)
    p, C, ch, target = _sphere(24, 48)
    n = len(p)
    lam = 1.0 / n
    opts = R.UnfoldOptions(precision=precision, precond=R.Precond.AMG)
    uv, _ = R.lscm_forward(ctx, C.batch(), opts, n)
    _, duv, dp_dist = R.distortion_loss(ctx, uv, 1)
    g = duv + 2.0 * lam * (uv - target)
    dp_solve, st = R.lscm_backward(ctx, g, opts, 1)
    assert st[0].status == R.Status.OK
    grad = dp_dist + dp_solve
    pinned = ch["pinned"].astype(np.int64)
    ref, _ = O.lu_adjoint_gradient(p, ch["tris"], pinned, ch["pin_uv"], lam, target)
    assert _rel(grad, ref) <= 1e-6, _rel(grad, ref)
    rng = np.random.Generator(np.random.PCG64(5))
    picks = [(int(v), k) for v in rng.choice(n, 64, replace=False) for k in range(3)]
    fd = O.fd_gradient(p, ch["tris"], pinned, ch["pin_uv"], lam, target, picks, h=1e-6)
    ad = np.array([grad[v, k] for v, k in picks])
    assert _rel(ad, fd) <= 1e-5, _rel(ad, fd)


def test_batched_adjoint_matches_per_chart_lu():
    """All charts of a batch in one forward / backward pair; each chart's gradient equals the
    single-chart CPU LU adjoint."""
    ctx = R.Context(0)
    vo, to, p3, tr = W.disks(12, t_min=100, t_max=4000, seed=31)
    C = R.prepare_patches(vo, to, p3, tr)
    n = int(vo[-1])
    opts = R.UnfoldOptions(precision=R.Precision.MIXED, precond=R.Precond.AMG)
    uv, _ = R.lscm_forward(ctx, C.batch(), opts, n)
    rng = np.random.Generator(np.random.PCG64(2))
    target = uv + 0.01 * rng.standard_normal(uv.shape)
    lam = 0.5
    loss, duv, dp_dist = R.distortion_loss(ctx, uv, C.n_charts)
    dp_solve, st = R.lscm_backward(ctx, duv + 2.0 * lam * (uv - target), opts, C.n_charts)
    grad = dp_dist + dp_solve
    for c in range(C.n_charts):
        ch = C.chart(c)
        sl = slice(vo[c], vo[c + 1])
        ref, _ = O.lu_adjoint_gradient(p3[sl], ch["tris"], ch["pinned"].astype(np.int64), ch["pin_uv"], lam,
                                       target[sl])
        assert _rel(grad[sl], ref) <= 1e-6, (c, _rel(grad[sl], ref))


def test_rectangularize_matches_reference():
    """rectangularize (metrics.rs:147-227) of every chart on the device: bit-identical to the
    reference restatement (same host libm angle table, no FMA contraction)."""
    ctx = R.Context(0)
    cases = [R.prepare_mesh(*O.grid(32, 32)), R.prepare_mesh(*O.cube(6)),
             R.prepare_mesh(*O.torus_annulus(2.0, 0.7, 64, 40)), R.prepare_mesh(*O.uv_sphere(48, 24)),
             R.prepare_patches(*W.disks(24, t_min=50, t_max=5000, seed=7))]
    for C in cases:
        vo = C.i64("chart.vert_off")
        uv, _, _ = R.solve_batch(ctx, C.batch(), R.UnfoldOptions(), int(vo[-1]))
        border = R.border_flags(C)
        q, ext = R.rectangularize(ctx, uv, border, C.n_charts)
        for c in range(C.n_charts):
            sl = slice(vo[c], vo[c + 1])
            q_ref, e_ref = O.rectangularize(uv[sl], border[sl])
            assert np.array_equal(q[sl], q_ref), c
            assert np.array_equal(ext[c], e_ref), c
