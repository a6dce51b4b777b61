"""CPU tests of the product library: the C ABI loads and exports every symbol ruv.h
declares, and the host chart stages (weld, segmentation, border loops, tangent frames,
pins) are bit-identical to the oracle restatement of the reference.  No GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

import researchuv_gb300 as R
from oracle import oracle as O
from researchuv_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "ruv.h")).read()
    declared = set(re.findall(r"^\s*(?:ruv_status|void|int32_t|int64_t|const char\*)\s+(ruv_[a-z0-9_]+)\s*\(",
                              hdr, re.M))
    assert declared, "no declarations parsed"
    L = R.lib()
    for name in declared:
        assert hasattr(L, name), f"libruv.so does not export {name}"
    assert declared <= set(R.SIGNATURES), sorted(declared - set(R.SIGNATURES))
    assert L.ruv_abi_version() == 1


def test_no_device_is_a_status_not_a_crash():
    if os.environ.get("CUDA_VISIBLE_DEVICES") is None and os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert R.lib().ruv_ctx_create(ctypes.byref(h), 0) == R.Status.NO_DEVICE
    assert R.GpuSolver.new() is None


def _compare(P, C):
    assert C.n_charts == P.n_charts
    mp, mf = P.mesh()
    assert np.array_equal(C.f64("mesh.pos").reshape(-1, 3), mp)
    assert np.array_equal(C.i64("mesh.faces").reshape(-1, 3), mf)
    for c in range(P.n_charts):
        a, b = P.chart(c), C.chart(c)
        for k in ["vertex_ids", "face_ids", "border"]:
            assert np.array_equal(a[k], b[k]), (c, k)
        assert np.array_equal(a["tris"], b["tris"]), (c, "tris")
        assert len(a["border_loops"]) == len(b["border_loops"])
        for x, y in zip(a["border_loops"], b["border_loops"]):
            assert np.array_equal(x, y), (c, "loop")
        assert a["area3d"] == b["area3d"]
        assert np.array_equal(a["p2"], b["p2"]), (c, "p2")
        pinned = np.zeros(len(a["vertex_ids"]), bool)
        pinned[a["pin_ids"]] = True
        assert np.array_equal(pinned, b["pinned"]), (c, "pin set")
        assert np.array_equal(a["pin_uv"], b["pin_uv"][a["pin_ids"]]), (c, "pin targets")


@pytest.mark.parametrize("name", ["cube", "sphere", "annulus", "torus", "grid", "cylinder"])
def test_host_stages_bitwise_vs_oracle(name):
    p, f = {"cube": lambda: O.cube(6), "sphere": lambda: O.uv_sphere(48, 24),
            "annulus": lambda: O.torus_annulus(2.0, 0.7, 64, 40), "torus": lambda: O.torus(2.0, 0.7, 64, 40),
            "grid": lambda: O.grid(32, 32), "cylinder": lambda: O.cylinder(1.0, 2.0, 32, 16)}[name]()
    _compare(O.Pipeline(p, f, lu_limit=0), R.prepare_mesh(p, f))


def test_host_stages_sharp_multichart_height_field():
    """A coarse height field with many sharp edges: hundreds of charts, multi-loop charts."""
    p, f = W.height_field(96, 8, 0.15, seed=7)
    P = O.Pipeline(p, f, lu_limit=0)
    assert P.n_charts > 10
    _compare(P, R.prepare_mesh(p, f))


def test_host_stages_thread_count_invariant():
    """pipeline.rs:369-385: results identical for 1 and many workers."""
    p, f = W.height_field(64, 8, 0.15, seed=9)
    a, b = R.prepare_mesh(p, f, threads=1), R.prepare_mesh(p, f, threads=8)
    for key in ["chart.vert_off", "chart.vertex_ids", "chart.tris", "chart.loop_ids", "chart.pinned"]:
        assert np.array_equal(a.i64(key), b.i64(key))
    for key in ["chart.p2", "chart.pin_uv", "chart.area3d"]:
        assert np.array_equal(a.f64(key), b.f64(key))


def test_patches_equal_segmentation_of_each_patch():
    vo, to, p3, tr = W.disks(24, t_min=50, t_max=3000, seed=3)
    C = R.prepare_patches(vo, to, p3, tr)
    for c in range(0, 24, 3):
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        assert P.n_charts == 1
        a, b = P.chart(0), C.chart(c)
        assert np.array_equal(a["tris"], b["tris"]) and a["area3d"] == b["area3d"]
        assert np.array_equal(a["p2"], b["p2"])
        pinned = np.zeros(len(a["vertex_ids"]), bool)
        pinned[a["pin_ids"]] = True
        assert np.array_equal(pinned, b["pinned"]) and np.array_equal(a["pin_uv"], b["pin_uv"][a["pin_ids"]])


def test_bad_inputs_are_rejected():
    p = np.zeros((3, 3))
    with pytest.raises(R.RuvError):
        R.prepare_mesh(p, np.array([[0, 1, 5]]))
    with pytest.raises(R.RuvError):
        R.prepare_patches([0, 3], [0, 1], p, np.array([[0, 1, 3]]))
    with pytest.raises(R.RuvError):  # the library implements SolverBackend::Gpu only
        R.UnfoldOptions(solver=R.SolverBackend.CPU).to_c()
    R.UnfoldOptions(keep_metric=True).to_c()  # KeepMetric runs on the GPU path (Schur complement)


@pytest.mark.parametrize("name,mesh,angle,min_faces,branch", [
    ("sphere_8x6", lambda: O.uv_sphere(8, 6), 180.0, 4, 1),
    ("sphere_24x12", lambda: O.uv_sphere(24, 12), 180.0, 8, 2),
    ("torus_closed", lambda: O.torus(2.0, 0.7, 24, 16), 180.0, 8, 1),
    ("cube_charts", lambda: O.cube(6), 30.0, 8, 1),
])
def test_seam_cut_bitwise_vs_oracle(name, mesh, angle, min_faces, branch):
    """seam.rs:167-305 (seam tree of every closed chart, charts rebuilt over the grown cut
    set) on the host: the same charts, loops, frames and pins as the oracle's restatement."""
    p, f = mesh()
    C, added = R.prepare_mesh_cut(None, p, f, angle_min_deg=angle,
                                  seam_cut=R.SeamCutOptions(enable=True, min_faces=min_faces, branch_count=branch))
    assert added == 0
    _compare(O.Pipeline(p, f, angle_deg=angle, lu_limit=0, seam_cut=(1, min_faces, branch)), C)


def test_seam_cut_opens_the_sphere():
    """seam.rs:335-357: the welded 8x6 sphere becomes one chart with one border loop."""
    p, f = O.uv_sphere(8, 6)
    C, _ = R.prepare_mesh_cut(None, p, f, angle_min_deg=180.0,
                              seam_cut=R.SeamCutOptions(enable=True, min_faces=4))
    assert C.n_charts == 1
    lo = C.i64("chart.loop_off")
    assert lo[1] - lo[0] == 1
