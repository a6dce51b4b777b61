"""The oracle's fixed-pin LU adjoint gradient pinned against central finite differences
(the check the differentiation workload asks for: FP64 central differences, h = 1e-6,
agreement to <= 1e-5 relative).  CPU only: a small instance of the spherical-harmonic sphere."""
import numpy as np

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W


def _instance(n_lat=20, n_lon=40, seed=4):
    p, f = W.sh_sphere(n_lat, n_lon, seed=seed)
    C = R.prepare_patches(np.array([0, len(p)]), np.array([0, len(f)]), p, f)
    ch = C.chart(0)
    rng = np.random.Generator(np.random.PCG64(11))
    target = ch["p2"] + 0.01 * rng.standard_normal(ch["p2"].shape)
    return p, ch["tris"], ch["pinned"].astype(np.int64), ch["pin_uv"], target


def test_lu_adjoint_matches_finite_differences():
    p, tris, pinned, pin_uv, target = _instance()
    lam_l2 = 1.0 / len(p)
    g, _ = O.lu_adjoint_gradient(p, tris, pinned, pin_uv, lam_l2, target)
    rng = np.random.Generator(np.random.PCG64(5))
    verts = rng.choice(len(p), 32, replace=False)
    picks = [(int(v), k) for v in verts for k in range(3)]
    fd = O.fd_gradient(p, tris, pinned, pin_uv, lam_l2, target, picks)
    ad = np.array([g[v, k] for v, k in picks])
    rel = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    assert rel <= 1e-5, rel
    assert np.abs(ad - fd).max() <= 1e-5 * np.abs(fd).max()


def test_fixed_system_matches_unfold_solution():
    """With the pins of the unfold, the fixed-pin solve is the unfold's own solve."""
    p, tris, pinned, pin_uv, _ = _instance(24, 48)
    ch = O.FixedPinChart(p, tris, pinned, pin_uv)
    uv = ch.uv()
    P = O.Pipeline(p, tris, weld_tol=0.0, lu_limit=0)
    assert P.n_charts == 1
    assert O.uv_error(uv, P.superlu_uv(0)) < 1e-12


def test_fd_steps_avoid_the_clamps_and_low_rank_solves_agree():
    """The FD check's step selection (the largest of 1e-6 ... 1e-9 at which +-h moves no clamp
    of the assembly around the vertex) and its low-rank (Woodbury) perturbed solves: on a
    smooth instance every pick keeps h = 1e-6, and the quotients equal those of refactoring
    every perturbed system and agree with the LU adjoint."""
    p, tris, pinned, pin_uv, target = _instance()
    lam_l2 = 1.0 / len(p)
    g, _ = O.lu_adjoint_gradient(p, tris, pinned, pin_uv, lam_l2, target)
    rng = np.random.Generator(np.random.PCG64(9))
    picks = [(int(v), k) for v in rng.choice(len(p), 12, replace=False) for k in range(3)]
    fd, hs = O.fd_gradient(p, tris, pinned, pin_uv, lam_l2, target, picks, reuse_base=True,
                           smooth_steps=(1e-6, 1e-7, 1e-8, 1e-9))
    assert np.all(hs == 1e-6)
    plain = O.fd_gradient(p, tris, pinned, pin_uv, lam_l2, target, picks, h=1e-6)
    assert np.abs(fd - plain).max() <= 1e-9 * np.abs(plain).max()
    ad = np.array([g[v, k] for v, k in picks])
    assert np.linalg.norm(ad - fd) / np.linalg.norm(fd) <= 1e-5
