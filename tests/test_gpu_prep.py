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
