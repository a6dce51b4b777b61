"""Mesh preparation with its data-parallel stages on the device (ruv_prepare_mesh_gpu: weld,
edge-face lists, dihedral cut flags, chart vertex sets) against the host preparation
(ruv_prepare_mesh, itself pinned to the oracle's restatement of weld.rs:19-57 and
segment.rs:61-331): every exported array equal, bit for bit, on meshes that exercise the
weld (duplicated vertices, collapsed faces), one and many charts, closed charts, two border
loops, no welding, and the extreme dihedral angles."""
import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

pytestmark = pytest.mark.gpu

I64 = ["chart.vert_off", "chart.tri_off", "chart.vertex_ids", "chart.face_ids", "chart.tris", "chart.border_off",
       "chart.border", "chart.loop_off", "chart.loop_seg", "chart.loop_ids", "chart.pinned", "mesh.faces",
       "mesh.n_cut_slots"]
F64 = ["chart.area3d", "mesh.pos", "chart.pin_uv", "chart.p2", "chart.p3"]


def _same(a, b):
    for w in I64:
        assert np.array_equal(a.i64(w), b.i64(w)), w
    for w in F64:
        x, y = a.f64(w), b.f64(w)
        assert x.shape == y.shape and np.array_equal(x.view(np.uint64), y.view(np.uint64)), w


def _collapsing():
    """A grid with a second copy of some vertices (welded onto the first) and a sliver face
    whose corners weld together (dropped)."""
    p, f = O.grid(12, 9)
    p = np.asarray(p, np.float64).reshape(-1, 3)
    f = np.asarray(f, np.int32).reshape(-1, 3)
    n = len(p)
    dup = p[:20] + 1e-14  # within the weld tolerance of 1e-12 after rounding
    p2 = np.concatenate([p, dup])
    f2 = f.copy()
    f2[:10] = np.where(f2[:10] < 20, f2[:10] + n, f2[:10])
    sliver = np.array([[0, n, 1], [2, 2, 3]], np.int32)  # 0 and its copy weld together; a repeated index
    return p2, np.concatenate([f2, sliver])


CASES = {
    "cube6": lambda: O.cube(6),
    "uv_sphere": lambda: O.uv_sphere(48, 24),
    "torus_closed": lambda: O.torus(2.0, 0.7, 48, 24),
    "annulus": lambda: O.torus_annulus(2.0, 0.7, 64, 40),
    "grid": lambda: O.grid(32, 32),
    "cylinder": lambda: O.cylinder(1.0, 2.0, 32, 12),
    "field256_many_charts": lambda: W.height_field(256, n_sines=16, amp=0.3, seed=5),
    "collapsing_weld": _collapsing,
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_prep_matches_host(name):
    ctx = R.Context(0)
    p, f = CASES[name]()
    _same(R.prepare_mesh(p, f), R.prepare_mesh(p, f, ctx=ctx))


@pytest.mark.parametrize("angle", [-5.0, 0.0, 10.0, 89.0, 180.0])
def test_device_prep_angles(angle):
    ctx = R.Context(0)
    p, f = W.height_field(128, n_sines=16, amp=0.3, seed=9)
    _same(R.prepare_mesh(p, f, angle_min_deg=angle), R.prepare_mesh(p, f, angle_min_deg=angle, ctx=ctx))


def test_device_prep_without_weld():
    ctx = R.Context(0)
    p, f = O.grid(20, 20)
    _same(R.prepare_mesh(p, f, weld_tol=0.0), R.prepare_mesh(p, f, weld_tol=0.0, ctx=ctx))
    q, g = _collapsing()  # a face with a repeated vertex is an error without welding, on both paths
    with pytest.raises(R.RuvError):
        R.prepare_mesh(q, g, weld_tol=0.0)
    with pytest.raises(R.RuvError):
        R.prepare_mesh(q, g, weld_tol=0.0, ctx=ctx)


def test_device_prep_solves_alike():
    """The device-prepared charts unfold to the same UVs as the host-prepared ones."""
    ctx = R.Context(0)
    p, f = W.height_field(256, n_sines=16, amp=0.3, seed=5)
    a, b = R.prepare_mesh(p, f), R.prepare_mesh(p, f, ctx=ctx)
    n = int(a.i64("chart.vert_off")[-1])
    ua, _, _ = R.solve_batch(ctx, a.batch(), R.UnfoldOptions(precision=R.Precision.FP64), n)
    ub, _, _ = R.solve_batch(ctx, b.batch(), R.UnfoldOptions(precision=R.Precision.FP64), n)
    assert np.array_equal(ua, ub)


def _patch_set(meshes):
    vo, to, P, T = [0], [0], [], []
    for p, f in meshes:
        p = np.asarray(p, np.float64).reshape(-1, 3)
        f = np.asarray(f, np.int32).reshape(-1, 3)
        P.append(p)
        T.append(f)
        vo.append(vo[-1] + len(p))
        to.append(to[-1] + len(f))
    return np.array(vo), np.array(to), np.concatenate(P), np.concatenate(T).astype(np.int32)


def _welded(p, f):
    return O.Pipeline(p, f).mesh()


PATCH_CASES = {
    "disks": lambda: W.disks(96, t_min=50, t_max=20000, seed=31),
    # closed charts (anchors), two loops (cylinder strip and multi-loop), one loop
    "fixtures": lambda: _patch_set([_welded(*O.cube(6)), _welded(*O.uv_sphere(32, 16)),
                                    _welded(*O.torus(2.0, 0.7, 32, 16)), _welded(*O.torus_annulus(2.0, 0.7, 48, 24)),
                                    _welded(*O.cylinder(1.0, 2.0, 24, 10)), O.grid(17, 11)]),
}


@pytest.mark.parametrize("name", sorted(PATCH_CASES))
def test_device_patches_match_host(name):
    """ruv_prepare_patches_gpu against ruv_prepare_patches: every exported array bit for bit."""
    ctx = R.Context(0)
    vo, to, p3, tr = PATCH_CASES[name]()
    _same(R.prepare_patches(vo, to, p3, tr), R.prepare_patches(vo, to, p3, tr, ctx=ctx))


def test_device_patches_fallback_and_errors():
    """A patch of two components stays one chart on both paths (the same result); an index
    outside its patch and a vertex no triangle uses are errors on both paths."""
    ctx = R.Context(0)
    vo, to, p3, tr = W.disks(4, t_min=200, t_max=2000, seed=37)
    # patches 1 and 2 merged into one patch of two components
    merged_vo = np.array([vo[0], vo[1], vo[3], vo[4]])
    shifted = tr.copy().astype(np.int64)
    shifted[to[2]:to[3]] += vo[2] - vo[1]
    merged_to = np.array([to[0], to[1], to[3], to[4]])
    _same(R.prepare_patches(merged_vo, merged_to, p3, shifted),
          R.prepare_patches(merged_vo, merged_to, p3, shifted, ctx=ctx))
    bad = tr.copy()
    bad[to[1]] = [0, 1, vo[2] - vo[1]]  # outside patch 1
    for c in (None, ctx):
        with pytest.raises(R.RuvError) as e:
            R.prepare_patches(vo, to, p3, bad, ctx=c)
        assert e.value.status == R.Status.BAD_INPUT
    extra_vo = vo.copy()
    extra_vo[1:] += 1  # patch 0 gets one vertex no triangle uses
    extra_p3 = np.concatenate([p3[:vo[1]], [[9.0, 9.0, 9.0]], p3[vo[1]:]])
    extra_tr = tr.copy()
    for c in (None, ctx):
        with pytest.raises(R.RuvError) as e:
            R.prepare_patches(extra_vo, to, extra_p3, extra_tr, ctx=c)
        assert e.value.status == R.Status.BAD_INPUT


def test_device_patches_solve_alike():
    ctx = R.Context(0)
    vo, to, p3, tr = W.disks(64, t_min=50, t_max=20000, seed=41)
    a, b = R.prepare_patches(vo, to, p3, tr), R.prepare_patches(vo, to, p3, tr, ctx=ctx)
    n = int(vo[-1])
    ua, _, _ = R.solve_batch(ctx, a.batch(), R.UnfoldOptions(), n)
    ub, _, _ = R.solve_batch(ctx, b.batch(), R.UnfoldOptions(), n)
    assert np.array_equal(ua, ub)
