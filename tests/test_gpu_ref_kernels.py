"""The reference's own single-system GPU CG — its CG kernels (gpu/src/kernels.cu:7-102,
compute_80 PTX built from the reference's source as gpu/build.rs:41-49 does, JIT-loaded)
driven by the oracle's C++ restatement of GpuSolver::cg_solve_precond (gpu/src/solver.rs:
284-565).  It is the measuring stick of the batched solve, so it is pinned here: to the
reference's GPU CG known answer (solver.rs:767-779) and to ruv_cg_solve on the same systems
(FP64 Jacobi PCG with the same stopping rule: the same solution, iteration counts within a
couple of iterations of each other since the dot products are summed in different orders)."""
import os

import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W
from systems import lap1d, poisson

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(O.REF_PTX):
        pytest.skip("the reference kernels' PTX was not built (needs the reference source tree at build time)")
    return O.RefGpuCG()


def test_reference_cg_known_answer(ref, known):
    k = known["gpu_cg"]["laplacian_1d_4096"]
    a, b = lap1d(k["n"])
    r = ref.solve(a.row_ptr, a.cols, a.vals, b, k["max_iter"], k["tol"], jacobi=False)
    assert r is not None
    assert np.abs(r[0] - 1.0).max() < k["x_tol"]


@pytest.mark.parametrize("jacobi", [False, True])
def test_reference_cg_matches_ruv_cg_solve(ref, jacobi):
    g = R.GpuSolver.global_()
    pc = R.Precond.JACOBI if jacobi else R.Precond.NONE
    systems = [poisson(60)]
    ctx = R.Context(0)
    vo, to, p3, tr = W.disks(3, t_min=500, t_max=6000, seed=43)
    R.unfold_charts(ctx, R.prepare_patches(vo, to, p3, tr), R.UnfoldOptions(precision=R.Precision.FP64))
    for c in range(3):
        rp, cols, vals, rhs = R.export_chart_system(ctx, c)
        systems.append((R.CsrMatrix(vals, cols, rp), rhs))
    for a, b in systems:
        mine = g.cg_solve_precond(a, b, 16384, 1e-12, pc)
        theirs = ref.solve(a.row_ptr, a.cols, a.vals, b, 16384, 1e-12, jacobi=jacobi)
        assert mine is not None and theirs is not None
        scale = max(1.0, np.abs(mine[0]).max())
        assert np.abs(mine[0] - theirs[0]).max() <= 1e-9 * scale
        assert abs(mine[1] - theirs[1]) <= 3, (mine[1], theirs[1])


def test_reference_cg_returns_none_like_the_reference(ref):
    a, b = lap1d(4096)
    assert ref.solve(a.row_ptr, a.cols, a.vals, b, 3, 1e-12, jacobi=False) is None  # not converged
    z = R.CsrMatrix(np.array([0.0, 0.0]), np.array([0, 1]), np.array([0, 1, 2]))
    assert ref.solve(z.row_ptr, z.cols, z.vals, np.ones(2), 10, 1e-12, jacobi=True) is None  # zero diagonal
