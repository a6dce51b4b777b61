"""Pin the oracle restatement against the reference's own known answers.

The reference is pure Rust (no toolchain here), so every assertion below is a value or
invariant taken from the reference's tests (tests/golden/reference_known_answers.json
cites file:line for each).  CPU only.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _pipe(p, f, **kw):
    return O.Pipeline(p, f, **kw)


def test_meshgen_counts(known):
    k = known["meshgen"]
    p, f = O.cube(6)
    assert (len(p), len(f)) == (k["cube6"]["verts"], k["cube6"]["faces"])
    p, f = O.uv_sphere(48, 24)
    assert (len(p), len(f)) == (k["sphere48x24_raw"]["verts"], k["sphere48x24_raw"]["faces"])
    p, f = O.torus(2.0, 0.7, 64, 40)
    assert (len(p), len(f)) == (k["torus64x40"]["verts"], k["torus64x40"]["faces"])
    p, f = O.torus_annulus(2.0, 0.7, 64, 40)
    assert (len(p), len(f)) == (k["annulus64x40"]["verts"], k["annulus64x40"]["faces"])
    p, f = O.grid(10, 8)
    assert (len(p), len(f)) == (k["grid10x8"]["verts"], k["grid10x8"]["faces"])
    assert len({tuple(q) for q in p}) == len(p)
    c = k["cylinder32x16"]
    p, f = O.cylinder(1.0, 2.0, 32, 16)
    assert len(p) == c["raw_verts"]
    P = _pipe(p, f)
    mp, mf = P.mesh()
    assert (len(mp), len(mf), P.n_charts) == (c["welded_verts"], c["faces"], c["charts"])
    assert len(P.chart(0)["border_loops"]) == c["border_loops"]


def test_cube_parity_table(known):
    k = known["parity_table"]["cube6"]
    p, f = O.cube(6)
    P = _pipe(p, f)
    mp, mf = P.mesh()
    assert (len(mp), len(mf)) == (k["welded_verts"], k["welded_faces"])
    assert P.n_charts == k["charts"]
    a = k["asserts"]
    for c in range(P.n_charts):
        ch = P.chart(c)
        assert len(ch["vertex_ids"]) == k["chart_verts"]
        assert abs(ch["area3d"] - k["area3d"]) < a["area3d_tol"]
        conf_mean, conf_max, area_ratio, flips, folds = ch["metrics"]
        assert flips == k["flips"]
        assert abs(conf_mean - k["conformal_mean"]) < a["conformal_mean_tol"]
        assert conf_max < a["conformal_max_lt"]
        assert abs(area_ratio - k["area_ratio"]) < a["area_ratio_tol"]
        ext = ch["uv"].max(0) - ch["uv"].min(0)
        assert np.all(np.abs(ext - 1.0) < 0.05)
        assert ch["iters"] == 2  # the identical re-solve on iteration 2 stops the driver
        # nf = 25 interior vertices, 24 border pins, nnz = 2 * 105 (quad diagonals dropped)
        assert (ch["free_pos"] >= 0).sum() == 25 and len(ch["pin_ids"]) == 24
        assert len(ch["csr_vals"]) == 210


def test_sphere_parity_table(known):
    k = known["parity_table"]["sphere48x24"]
    p, f = O.uv_sphere(48, 24)
    P = _pipe(p, f)
    mp, mf = P.mesh()
    assert (len(mp), len(mf), P.n_charts) == (k["welded_verts"], k["welded_faces"], k["charts"])
    ch = P.chart(0)
    assert len(ch["vertex_ids"]) == k["chart_verts"]
    assert len(ch["border_loops"]) == 0 and len(ch["border"]) == 0
    assert abs(ch["area3d"] - k["area3d"]) < k["area3d_tol"]
    conf_mean, conf_max, area_ratio, flips, _ = ch["metrics"]
    # the stored baseline table's digits, reproduced exactly by the restatement
    assert round(conf_mean, 3) == k["conformal_mean"]
    # the worst ratio sits at the antipodal singularity: solver-sensitive (parity.rs:11-15)
    assert abs(conf_max - k["conformal_max"]) / k["conformal_max"] < 1e-6
    assert round(area_ratio, 3) == k["area_ratio"]
    assert flips == 0
    lo, hi = k["asserts"]["iters_band"]
    assert lo <= ch["iters"] <= hi
    assert len(ch["pin_ids"]) == 4  # closed chart: 4 farthest-point anchors


def test_annulus_parity_table(known):
    k = known["parity_table"]["annulus64x40"]
    p, f = O.torus_annulus(2.0, 0.7, 64, 40)
    P = _pipe(p, f, lu_limit=6000)
    mp, mf = P.mesh()
    assert (len(mp), len(mf), P.n_charts) == (k["welded_verts"], k["welded_faces"], k["charts"])
    ch = P.chart(0)
    assert len(ch["border_loops"]) == k["border_loops"]
    assert len(ch["border"]) == k["island_border"]
    assert abs(ch["area3d"] - k["area3d"]) < k["area3d_tol"]
    conf_mean, conf_max, area_ratio, flips, _ = ch["metrics"]
    assert round(conf_mean, 3) == k["conformal_mean"]
    assert round(conf_max, 3) == k["conformal_max"]
    assert round(area_ratio, 3) == k["area_ratio"]
    assert flips == 0


def test_closed_torus(known):
    k = known["parity_table"]["torus64x40"]
    p, f = O.torus(2.0, 0.7, 64, 40)
    P = _pipe(p, f, lu_limit=0)  # structure only (the LU of this chart takes seconds)
    assert len(P.mesh()[1]) == k["welded_faces"] and P.n_charts == 1
    ch = P.chart(0)
    assert len(ch["border"]) == 0 and len(ch["border_loops"]) == 0
    uv = P.superlu_uv(0)
    assert np.isfinite(uv).all()
    assert P.metrics(0, uv)[3] == 0


def test_weld_cases(known):
    # two unit squares with a duplicated seam (weld.rs:69-98)
    p, f = [], []
    for quad in range(2):
        base = len(p)
        for j in range(2):
            for i in range(2):
                p.append((quad + i, j, 0.0))
        a, b, c, d = base, base + 1, base + 2, base + 3
        f += [(a, b, d), (a, d, c)]
    P = _pipe(np.array(p, float), np.array(f), weld_tol=1e-6)
    mp, mf = P.mesh()
    assert (len(mp), len(mf)) == (6, 4)
    P = _pipe(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0]], float),
              np.array([[0, 1, 2], [0, 0, 3]]))
    assert len(P.mesh()[1]) == known["weld"]["degenerate_dropped"]["faces"]
    P = _pipe(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float), np.array([[0, 1, 2]]), weld_tol=0.0)
    assert (len(P.mesh()[0]), len(P.mesh()[1])) == (3, 1)


def test_segment_cases(known):
    k = known["segment"]
    p = np.array([(i, j, 0.0) for j in range(3) for i in range(3)], float)
    f = []
    for j in range(2):
        for i in range(2):
            a = j * 3 + i
            f += [(a, a + 1, a + 4), (a, a + 4, a + 3)]
    P = _pipe(p, np.array(f))
    assert P.n_cut == 0 and P.n_charts == 1
    ch = P.chart(0)
    fg = k["flat_grid_2x2"]
    assert (len(ch["face_ids"]), len(ch["vertex_ids"]), len(ch["border"])) == (fg["faces"], fg["verts"], fg["border"])
    assert len(ch["border_loops"]) == 1 and len(ch["border_loops"][0]) == fg["loop_len"]
    P = _pipe(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float), np.array([[0, 1, 2]]))
    ch = P.chart(0)
    assert len(ch["border_loops"]) == 1 and len(ch["border_loops"][0]) == 4
    assert ch["border_loops"][0][0] == ch["border_loops"][0][3]
    tet = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], float)
    P = _pipe(tet, np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]]), angle_deg=130.0, lu_limit=0)
    assert P.n_cut == 0 and P.n_charts == 1
    assert len(P.chart(0)["border"]) == 0 and len(P.chart(0)["border_loops"]) == 0


def _coo(items):
    r = np.array([t[0] for t in items])
    c = np.array([t[1] for t in items])
    v = np.array([t[2] for t in items], float)
    return r, c, v


def _dense(n, items):
    A = np.zeros((n, n))
    for r, c, v in items:
        A[r, c] += v
    return A


@pytest.mark.parametrize("name", ["spd3", "pinned_chain"])
def test_sparse_lu_residual(known, name):
    k = known["sparse_lu"][name]
    r, c, v = _coo(k["coo"])
    x = O.sparse_solve(k["n"], r, c, v, k["b"])
    assert x is not None
    assert np.abs(_dense(k["n"], k["coo"]) @ x - np.array(k["b"])).max() < k["tol"]


def test_sparse_lu_known_solutions(known):
    k = known["sparse_lu"]
    for name in ["cache_diag", "permutation"]:
        r, c, v = _coo(k[name]["coo"])
        x = O.sparse_solve(k[name]["n"], r, c, v, k[name]["b"])
        assert np.abs(x - np.array(k[name]["x"])).max() < k[name]["tol"]
    r, c, v = _coo(k["cache_coupled"]["coo"])
    x = O.sparse_solve(2, r, c, v, k["cache_coupled"]["b"])
    assert abs(x[0] - 1.25) < 1e-12
    sp = k["spd_pivot"]
    A = _dense(3, sp["coo"])
    b = A @ np.array(sp["x"])
    r, c, v = _coo(sp["coo"])
    x = O.sparse_solve(3, r, c, v, b)
    assert np.abs(x - np.array(sp["x"])).max() < sp["tol"]
    # duplicates are summed (sparse.rs:328-333)
    r, c, v = _coo(k["duplicates"]["coo"])
    x = O.sparse_solve(1, r, c, v, [5.0])
    assert abs(x[0] - 1.0) < 1e-15
    # 5x5 Poisson (sparse.rs:356-380)
    items = []
    for i in range(25):
        rr, cc = divmod(i, 5)
        items.append((i, i, 4.0))
        for dr, dc in [(0, 1), (0, -1), (1, 0), (-1, 0)]:
            r2, c2 = rr + dr, cc + dc
            if 0 <= r2 < 5 and 0 <= c2 < 5:
                items.append((i, r2 * 5 + c2, -1.0))
    b = np.arange(25) * 0.1 + 1.0
    r, c, v = _coo(items)
    x = O.sparse_solve(25, r, c, v, b)
    assert np.abs(_dense(25, items) @ x - b).max() < 1e-8


def test_eig3(known):
    k = known["eig3"]
    w, v = O.eig3(k["diagonal"]["m"])
    assert np.abs(w - np.array(k["diagonal"]["w"])).max() < 1e-9
    m = np.array(k["known"]["m"])
    w, v = O.eig3(m)
    assert np.abs(np.sort(w) - np.array(k["known"]["w_sorted"])).max() < 1e-9
    assert np.abs(v.T @ v - np.eye(3)).max() < 1e-9
    assert np.abs(m @ v - v * w[None, :]).max() < 1e-9


def test_superlu_oracle_agrees_with_reference_lu():
    """The FP64 SuperLU oracle (large charts) and the restated reference LU agree."""
    p, f = O.grid(32, 32)
    P = _pipe(p, f, lu_limit=4000)
    ch = P.chart(0)
    uv_lu = ch["uv"]
    uv_slu = P.superlu_uv(0)
    assert O.uv_error(uv_slu, uv_lu) < 1e-12
