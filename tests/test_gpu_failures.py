"""Failure paths of the batched solve, made on the host (no GPU fault).

* Device allocation failure: ruv_debug_fail_alloc makes the k-th allocation of a context
  fail as cudaMalloc would when the device is full.  For every k up to the number of
  allocations one solve makes, the call returns OOM with the allocation named, and the same
  context then solves the batch again to bit-identical UVs (the reference's counterpart is
  DeviceMem::alloc returning None, gpu/src/solver.rs:671-729, after which the caller falls
  back to its CPU LU, unwrap/src/lscm.rs:677-678).
* Per-chart non-convergence in the batched entry: with one CG iteration allowed, every chart
  that has free vertices reports NOT_CONVERGED and the call returns NOT_CONVERGED; charts
  without free vertices (all pinned) are OK.
"""

import numpy as np
import pytest

import researchuv_gb300 as R
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _disks():
    vo, to, p3, tr = W.disks(6, t_min=200, t_max=4000, seed=23)
    return R.prepare_patches(vo, to, p3, tr)


@pytest.mark.parametrize("precond", [R.Precond.AMG_SA, R.Precond.JACOBI, R.Precond.IC0])
def test_injected_oom_at_every_allocation(precond):
    C = _disks()
    nv = int(C.i64("chart.vert_off")[-1])
    opts = R.UnfoldOptions(precision=R.Precision.MIXED, precond=precond)
    ref_uv, _, st = R.solve_batch(R.Context(0), C.batch(), opts, nv)
    assert st == R.Status.OK
    L = R.lib()
    failed = 0
    for k in range(1, 400):
        ctx = R.Context(0)
        assert L.ruv_debug_fail_alloc(ctx.h, k) == 0
        uv, _, st = R.solve_batch(ctx, C.batch(), opts, nv, check=False)
        if st == R.Status.OK:  # fewer than k allocations in one solve: every point was covered
            L.ruv_debug_fail_alloc(ctx.h, 0)
            break
        failed += 1
        assert st == R.Status.OOM, (k, R.Status(st).name, ctx.last_error())
        assert "injected allocation failure" in ctx.last_error()
        uv, _, st = R.solve_batch(ctx, C.batch(), opts, nv, check=False)  # same context, no injection left
        assert st == R.Status.OK, (k, R.Status(st).name, ctx.last_error())
        assert np.array_equal(uv, ref_uv), f"solve after an injected failure at allocation {k} differs"
        ctx.close()
    else:
        pytest.fail("more than 400 allocations in one solve")
    assert failed >= 5


def test_injected_oom_in_cg_solve():
    from systems import poisson

    a, b = poisson(64)
    g = R.GpuSolver.new()
    ref = g.cg_solve_precond(a, b, 10_000, 1e-10, R.Precond.AMG_SA)
    assert ref is not None
    L = R.lib()
    for k in (1, 2, 5, 10):
        g2 = R.GpuSolver.new()
        L.ruv_debug_fail_alloc(g2.ctx.h, k)
        r = g2.cg_solve_precond(a, b, 10_000, 1e-10, R.Precond.AMG_SA)
        if r is not None:
            break
        assert "OOM" in g2.last_error and "injected" in g2.last_error
        r = g2.cg_solve_precond(a, b, 10_000, 1e-10, R.Precond.AMG_SA)
        assert r is not None and np.array_equal(r[0], ref[0]) and r[1] == ref[1]


@pytest.mark.parametrize("precond", [R.Precond.JACOBI, R.Precond.AMG_SA])
@pytest.mark.parametrize("precision", [R.Precision.MIXED, R.Precision.FP64])
def test_batched_not_converged_per_chart(precond, precision):
    vo, to, p3, tr = W.disks(8, t_min=300, t_max=6000, seed=29)
    # one lone triangle: all three vertices pinned, nothing to solve
    vo = np.concatenate([vo, [vo[-1] + 3]])
    to = np.concatenate([to, [to[-1] + 1]])
    p3 = np.concatenate([p3, [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]])
    tr = np.concatenate([tr, [[0, 1, 2]]]).astype(np.int32)
    C = R.prepare_patches(vo, to, p3, tr)
    nv = int(C.i64("chart.vert_off")[-1])
    ctx = R.Context(0)
    opts = R.UnfoldOptions(precision=precision, precond=precond, max_cg_iter=1)
    _, stats, st = R.solve_batch(ctx, C.batch(), opts, nv)
    assert st == R.Status.NOT_CONVERGED
    for c, s in enumerate(stats):
        if s.n_free == 0:
            assert s.status == R.Status.OK, c
        else:
            assert s.status == R.Status.NOT_CONVERGED, (c, R.Status(s.status).name)
            assert s.cg_iters <= 8  # one block of captured iterations at most
    # the context is still usable: the same batch with the default limit converges
    _, stats, st = R.solve_batch(ctx, C.batch(), R.UnfoldOptions(precision=precision, precond=precond), nv)
    assert st == R.Status.OK and all(s.status == R.Status.OK for s in stats)
