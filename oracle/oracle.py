"""ORACLE — test infrastructure only (it checks results; it is never the thing measured or shipped).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference
legs may import this module.  It wraps ``oracle.cpp`` — a CPU restatement of ResearchUV's
per-chart LSCM unfold path (unwrap/src/{weld,segment,lscm,lscm_eig,sparse,metrics,meshgen}.rs)
— and adds the FP64 sparse-LU oracle for systems too large for the reference's Θ(n²)
BTreeMap LU (``scipy.sparse.linalg.splu``, SuperLU, on the scalar Laplacian with the u and v
right-hand sides).

Parity pinning: the reference is pure Rust and cannot be built here; the restatement is
pinned against the known answers of the reference's own tests
(``tests/golden/reference_known_answers.json``, each item citing its file:line).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.cpp")
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile the restatement into oracle/_build/liboracle.so (plain g++, no build system),
    and the reference-kernel harness (build_ref_ptx, build_ref_cg) where it can be built."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + ".tmp"
        subprocess.check_call(["g++", *_CXXFLAGS, "-o", tmp, _SRC])
        os.replace(tmp, _LIB)
    build_ref_ptx()
    build_ref_cg()
    return _LIB


# ------------------------------------------------------------------ the reference's own GPU CG
# The reference's CG kernels (gpu/src/kernels.cu, compute_80 PTX as gpu/build.rs:41-49 builds
# them) compiled from the reference's source tree into oracle/_ref/ (not committed; built here
# where the reference is present, carried as a file elsewhere), and ref_gpu_cg.cpp, the C++
# restatement of the reference's host loop that drives them.
_REF_KERNELS = "/root/reference/crates/researchuv-gpu/src/kernels.cu"
REF_PTX = os.path.join(_HERE, "_ref", "kernels_compute80.ptx")
_REF_CG_SRC = os.path.join(_HERE, "ref_gpu_cg.cpp")
_REF_CG_LIB = os.path.join(_HERE, "_build", "libref_gpu_cg.so")
_CUDA = "/usr/local/cuda"


def build_ref_ptx() -> str:
    """nvcc -ptx -arch=compute_80 of the reference's kernels.cu into oracle/_ref/ (only where
    the reference's source tree is present; elsewhere the file built there is used)."""
    if os.path.exists(_REF_KERNELS) and (not os.path.exists(REF_PTX)
                                         or os.path.getmtime(REF_PTX) < os.path.getmtime(_REF_KERNELS)):
        os.makedirs(os.path.dirname(REF_PTX), exist_ok=True)
        nvcc = os.path.join(_CUDA, "bin", "nvcc")
        tmp = REF_PTX + ".tmp"
        subprocess.check_call([nvcc, "-ptx", "-arch=compute_80", "-o", tmp, _REF_KERNELS])
        os.replace(tmp, REF_PTX)
    return REF_PTX


def build_ref_cg() -> str | None:
    """g++ of ref_gpu_cg.cpp against the CUDA driver API (None without cuda.h)."""
    inc = os.path.join(_CUDA, "include")
    if not os.path.exists(os.path.join(inc, "cuda.h")):
        return None
    if not os.path.exists(_REF_CG_LIB) or os.path.getmtime(_REF_CG_LIB) < os.path.getmtime(_REF_CG_SRC):
        os.makedirs(os.path.dirname(_REF_CG_LIB), exist_ok=True)
        tmp = _REF_CG_LIB + ".tmp"
        libdirs = [d for d in (os.path.join(_CUDA, "lib64"), os.path.join(_CUDA, "lib64", "stubs"),
                               os.path.join(_CUDA, "targets", "sbsa-linux", "lib", "stubs"),
                               os.path.join(_CUDA, "targets", "x86_64-linux", "lib", "stubs")) if os.path.isdir(d)]
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", inc, "-o", tmp, _REF_CG_SRC,
                               *[f"-L{d}" for d in libdirs], "-lcuda"])
        os.replace(tmp, _REF_CG_LIB)
    return _REF_CG_LIB


class RefGpuCG:
    """GpuSolver::cg_solve_precond of the reference (None / Jacobi) on its own kernels."""

    def __init__(self):
        path = build_ref_cg()
        if path is None or not os.path.exists(REF_PTX):
            raise RuntimeError("reference GPU CG harness not built (needs cuda.h and oracle/_ref PTX)")
        L = ctypes.CDLL(path)
        L.rcg_init.argtypes = [ctypes.c_char_p]
        L.rcg_last_error.restype = ctypes.c_char_p
        P = ctypes.POINTER
        L.rcg_solve.argtypes = [ctypes.c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_double),
                                P(ctypes.c_double), P(ctypes.c_double), ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                P(ctypes.c_int64)]
        if L.rcg_init(REF_PTX.encode()) != 0:
            raise RuntimeError("rcg_init: " + L.rcg_last_error().decode())
        self.L = L

    def solve(self, row_ptr, cols, vals, b, max_iter, tol, jacobi=True):
        """(x, iterations) or None, as the reference returns."""
        rp = np.ascontiguousarray(row_ptr, np.int32)
        c = np.ascontiguousarray(cols, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        bb = np.ascontiguousarray(b, np.float64)
        n = len(rp) - 1
        x = np.empty(n)
        it = ctypes.c_int64(0)
        P = ctypes.POINTER
        st = self.L.rcg_solve(n, rp.ctypes.data_as(P(ctypes.c_int32)), c.ctypes.data_as(P(ctypes.c_int32)),
                              v.ctypes.data_as(P(ctypes.c_double)), bb.ctypes.data_as(P(ctypes.c_double)),
                              x.ctypes.data_as(P(ctypes.c_double)), int(max_iter), float(tol), 1 if jacobi else 0,
                              ctypes.byref(it))
        return None if st != 0 else (x, int(it.value))


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        vp, i64, f64, cp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_char_p
        P = ctypes.POINTER
        L.orc_bag_new.restype = vp
        L.orc_bag_free.argtypes = [vp]
        L.orc_len.argtypes = [vp, cp]
        L.orc_len.restype = i64
        L.orc_get_f64.argtypes = [vp, cp, P(f64)]
        L.orc_get_i64.argtypes = [vp, cp, P(i64)]
        L.orc_put_f64.argtypes = [vp, cp, P(f64), i64]
        L.orc_put_i64.argtypes = [vp, cp, P(i64), i64]
        L.orc_meshgen.argtypes = [vp, cp, i64, f64, f64, i64, i64]
        L.orc_eig3.argtypes = [P(f64), P(f64), P(f64)]
        L.orc_sparse_solve.argtypes = [i64, i64, P(i64), P(i64), P(f64), P(f64), P(f64)]
        L.orc_sparse_solve.restype = ctypes.c_int
        L.orc_pipeline.argtypes = [vp, f64, f64, f64, f64, i64, i64]
        L.orc_driver_from_solution.argtypes = [vp, i64, i64]
        L.orc_chart_metrics.argtypes = [vp, i64, P(f64), P(f64)]
        L.orc_ic0.argtypes = [vp, ctypes.c_int]
        L.orc_ic0.restype = ctypes.c_int
        L.orc_ic0_apply.argtypes = [vp, P(f64), P(f64)]
        L.orc_lscm_fixed.argtypes = [vp]
        L.orc_rectangularize.argtypes = [i64, P(f64), P(i64), P(f64), P(f64)]
        L.orc_distortion_loss.argtypes = [vp, P(f64), P(f64), P(f64), P(f64)]
        L.orc_lscm_adjoint_positions.argtypes = [vp, P(f64), P(f64), P(f64)]
        _lib = L
    return _lib


def _f64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


class Bag:
    """Owner of one oracle result set (named f64 / i64 arrays)."""

    def __init__(self):
        self.h = lib().orc_bag_new()

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_bag_free(self.h)
            self.h = None

    def has(self, name: str) -> bool:
        return lib().orc_len(self.h, name.encode()) >= 0

    def f64(self, name: str) -> np.ndarray:
        n = lib().orc_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        out = np.empty(n, np.float64)
        if lib().orc_get_f64(self.h, name.encode(), _f64p(out)) != 0:
            raise KeyError(name)
        return out

    def i64(self, name: str) -> np.ndarray:
        n = lib().orc_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        out = np.empty(n, np.int64)
        if lib().orc_get_i64(self.h, name.encode(), _i64p(out)) != 0:
            raise KeyError(name)
        return out

    def put_f64(self, name, a):
        a = np.ascontiguousarray(a, np.float64).ravel()
        lib().orc_put_f64(self.h, name.encode(), _f64p(a), a.size)

    def put_i64(self, name, a):
        a = np.ascontiguousarray(a, np.int64).ravel()
        lib().orc_put_i64(self.h, name.encode(), _i64p(a), a.size)


# ------------------------------------------------------------------ meshgen.rs fixtures
def meshgen(name: str, n: int = 0, *, r_major=0.0, r_minor=0.0, nu=0, nv=0):
    """Restated fixtures (unwrap/src/meshgen.rs:12-198). Returns (pos (V,3) f64, faces (F,3) i64)."""
    b = Bag()
    lib().orc_meshgen(b.h, name.encode(), n, r_major, r_minor, nu, nv)
    return b.f64("pos").reshape(-1, 3), b.i64("faces").reshape(-1, 3)


def cube(n):
    return meshgen("cube", n)


def uv_sphere(nu, nv):
    return meshgen("sphere", nu=nu, nv=nv)


def torus(r_major, r_minor, nu, nvt):
    return meshgen("torus", r_major=r_major, r_minor=r_minor, nu=nu, nv=nvt)


def torus_annulus(r_major, r_minor, nu, nvt):
    return meshgen("annulus", r_major=r_major, r_minor=r_minor, nu=nu, nv=nvt)


def grid(w, h):
    return meshgen("grid", nu=w, nv=h)


def cylinder(r, height, nu, nv):
    return meshgen("cylinder", r_major=r, r_minor=height, nu=nu, nv=nv)


def eig3(m):
    m = np.ascontiguousarray(m, np.float64).reshape(9)
    w = np.empty(3)
    v = np.empty(9)
    lib().orc_eig3(_f64p(m), _f64p(w), _f64p(v))
    return w, v.reshape(3, 3)


def sparse_solve(n, rows, cols, vals, b):
    """Sparse::add over the COO triples then Sparse::solve (unwrap/src/sparse.rs). None if singular."""
    r = np.ascontiguousarray(rows, np.int64)
    c = np.ascontiguousarray(cols, np.int64)
    v = np.ascontiguousarray(vals, np.float64)
    bb = np.ascontiguousarray(b, np.float64)
    x = np.empty(n)
    rc = lib().orc_sparse_solve(n, r.size, _i64p(r), _i64p(c), _f64p(v), _f64p(bb), _f64p(x))
    return None if rc != 0 else x


# ------------------------------------------------------------------ the unfold path
class Pipeline:
    """weld -> segment -> per-chart system (and, for small charts, the reference LU solve +
    damped driver) for one raw triangle soup.

    ``lu_limit``: charts whose system has at most this many unknowns (2 nf + 1) are solved by
    the restated reference LU; larger ones can be solved with :meth:`superlu_uv`.
    """

    def __init__(self, pos, faces, weld_tol=1e-12, angle_deg=30.0, angle_mix=1.0, mix_w=1.0,
                 lu_limit=4000, max_iter=100, keep_metric=False, target_area=0.0, seam_cut=None, recut=None):
        self.bag = Bag()
        self.bag.put_f64("pos", np.asarray(pos, np.float64))
        self.bag.put_i64("faces", np.asarray(faces, np.int64))
        if seam_cut is not None:  # (enable, min_faces, branch_count): seam.rs SeamCutOptions
            self.bag.put_f64("opt.seam", np.array(seam_cut, np.float64))
        if recut is not None:  # (enable, max_rounds, max_splits, fold_fraction, max_charts): recut.rs
            self.bag.put_f64("opt.recut", np.array(recut, np.float64))
        if keep_metric:  # KeepMetric's area row, solved by the reference LU every iteration
            self.bag.put_f64("opt.keep_metric", np.array([1.0]))
            self.bag.put_f64("opt.target_area", np.array([float(target_area)]))
        self.max_iter = max_iter
        lib().orc_pipeline(self.bag.h, weld_tol, angle_deg, angle_mix, mix_w, lu_limit, max_iter)
        self.n_charts = int(self.bag.i64("n_charts")[0])
        self.n_cut = int(self.bag.i64("n_cut")[0])

    def mesh(self):
        return self.bag.f64("mesh.pos").reshape(-1, 3), self.bag.i64("mesh.faces").reshape(-1, 3)

    def chart(self, c: int) -> dict:
        b = self.bag
        k = f"c{c}."
        d = {
            "face_ids": b.i64(k + "face_ids"),
            "vertex_ids": b.i64(k + "vertex_ids"),
            "tris": b.i64(k + "tris").reshape(-1, 3),
            "border": b.i64(k + "border"),
            "area3d": float(b.f64(k + "area3d")[0]),
            "p2": b.f64(k + "p2").reshape(-1, 2),
            "pin_ids": b.i64(k + "pin_ids"),
            "pin_uv": b.f64(k + "pin_uv").reshape(-1, 2),
            "free_pos": b.i64(k + "free_pos"),
            "csr_ptr": b.i64(k + "csr_ptr"),
            "csr_cols": b.i64(k + "csr_cols"),
            "csr_vals": b.f64(k + "csr_vals"),
            "rhs": b.f64(k + "rhs"),
        }
        off = b.i64(k + "loop_off")
        ids = b.i64(k + "loop_ids")
        d["border_loops"] = [ids[off[i]:off[i + 1]] for i in range(len(off) - 1)]
        if b.has(k + "uv"):
            d["uv"] = b.f64(k + "uv").reshape(-1, 2)
            d["iters"] = int(b.i64(k + "iters")[0])
            d["err_accum"] = float(b.f64(k + "err_accum")[0])
        if b.has(k + "sol"):
            d["sol"] = b.f64(k + "sol")
        if b.has(k + "metrics"):
            d["metrics"] = b.f64(k + "metrics")
        return d

    def superlu_uv(self, c: int):
        """FP64 sparse-LU oracle for chart ``c``: SuperLU (scipy) on the scalar block of the
        exported interleaved CSR (the reference's A = L (x) I2 structure), both coordinate
        right-hand sides, then the reference's damped driver update.  Returns the chart UVs."""
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla

        ch = self.chart(c)
        n2 = len(ch["csr_ptr"]) - 1
        A = sp.csr_matrix((ch["csr_vals"], ch["csr_cols"], ch["csr_ptr"]), shape=(n2, n2))
        rhs = ch["rhs"]
        if n2 == 0:
            sol = np.array([1.0])
        else:
            L = A[0::2, 0::2].tocsc()
            lu = spla.splu(L, permc_spec="COLAMD")
            B = np.stack([rhs[0:n2:2], rhs[1:n2:2]], axis=1)
            X = lu.solve(B)
            sol = np.empty(n2 + 1)
            sol[0:n2:2] = X[:, 0]
            sol[1:n2:2] = X[:, 1]
            sol[n2] = 1.0
        self.bag.put_f64(f"c{c}.sol", sol)
        lib().orc_driver_from_solution(self.bag.h, c, self.max_iter)
        return self.bag.f64(f"c{c}.uv").reshape(-1, 2)

    def metrics(self, c: int, uv):
        uv = np.ascontiguousarray(uv, np.float64).reshape(-1)
        out = np.empty(5)
        lib().orc_chart_metrics(self.bag.h, c, _f64p(uv), _f64p(out))
        return out


def uv_error(uv_test, uv_ref) -> float:
    """The reference's GPU/CPU parity measure (unwrap/src/lscm.rs:749-758):
    max_i |uv_test_i - uv_ref_i| / max_i |uv_ref_i| (Euclidean per vertex)."""
    a = np.asarray(uv_test, np.float64).reshape(-1, 2)
    b = np.asarray(uv_ref, np.float64).reshape(-1, 2)
    diff = np.sqrt(((a - b) ** 2).sum(1)).max(initial=0.0)
    scale = max(np.sqrt((b ** 2).sum(1)).max(initial=0.0), 1e-30)
    return float(diff / scale)


class Ic0:
    """IC(0) factor of a CSR matrix as the reference builds it (gpu/src/precond.rs:145-262):
    ``l_*`` (lower, diagonal last), ``lt_*`` (transpose, diagonal last), ``fwd_level`` /
    ``bwd_level`` per row; with ``colored``, of the colour-permuted matrix
    (precond.rs:49-123), with ``color``, ``to_perm``, ``to_orig`` and the permuted CSR ``p_*``.
    ``ok`` is False where the reference's factor_ic0 returns None."""

    def __init__(self, row_ptr, cols, vals, colored: bool = False):
        self.bag = Bag()
        self.bag.put_i64("a.row_ptr", np.asarray(row_ptr, dtype=np.int64))
        self.bag.put_i64("a.cols", np.asarray(cols, dtype=np.int64))
        self.bag.put_f64("a.vals", np.asarray(vals, dtype=np.float64))
        self.ok = lib().orc_ic0(self.bag.h, 1 if colored else 0) == 0
        if not self.ok:
            return
        for pre in ("l", "lt") + (("p",) if colored else ()):
            setattr(self, pre + "_ptr", self.bag.i64(pre + ".ptr"))
            setattr(self, pre + "_cols", self.bag.i64(pre + ".cols"))
            setattr(self, pre + "_vals", self.bag.f64(pre + ".vals"))
        self.fwd_level = self.bag.i64("fwd.level")
        self.bwd_level = self.bag.i64("bwd.level")
        if colored:
            self.color = self.bag.i64("color")
            self.to_perm = self.bag.i64("to_perm")
            self.to_orig = self.bag.i64("to_orig")

    def apply(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        lib().orc_ic0_apply(self.bag.h, _f64p(r), _f64p(z))
        return z


class FixedPinChart:
    """One chart's LSCM system with the pins given (unwrap/src/lscm.rs:594-676, mix_b = 0),
    solved by SuperLU in FP64, with the CPU reference gradient of a loss through the solve:
    lam = A^-1 dL/duv, then the reverse pass of the assembly (edge coefficients and corner
    cotangents differentiated by forward-mode duals)."""

    def __init__(self, p3, tris, pinned, pin_uv):
        self.p3 = np.ascontiguousarray(p3, np.float64).reshape(-1, 3)
        self.tris = np.ascontiguousarray(tris, np.int64).reshape(-1, 3)
        self.pinned = np.ascontiguousarray(pinned, np.int64).reshape(-1)
        self.pin_uv = np.ascontiguousarray(pin_uv, np.float64).reshape(-1, 2)
        self.bag = Bag()
        self.bag.put_f64("p3", self.p3.reshape(-1))
        self.bag.put_i64("tris", self.tris.reshape(-1))
        self.bag.put_i64("pinned", self.pinned)
        self.bag.put_f64("pin_uv", self.pin_uv.reshape(-1))
        lib().orc_lscm_fixed(self.bag.h)
        import scipy.sparse as sp
        self.row_of = self.bag.i64("row_of")
        nf = int((self.row_of >= 0).sum())
        self.nf = nf
        self.A = sp.csr_matrix((self.bag.f64("csr.vals"), self.bag.i64("csr.cols"), self.bag.i64("csr.ptr")),
                               shape=(nf, nf))
        self.b = self.bag.f64("b").reshape(nf, 2)
        self._lu = None

    def lu(self):
        if self._lu is None:
            import scipy.sparse.linalg as sla
            self._lu = sla.splu(self.A.tocsc(), permc_spec="MMD_AT_PLUS_A")
        return self._lu

    def solve(self, rhs=None):
        return self.lu().solve(self.b if rhs is None else rhs)

    def uv(self, x=None):
        """All-vertex UVs: the solution on free vertices, the pins elsewhere."""
        x = self.solve() if x is None else x
        out = self.pin_uv.copy()
        free = self.row_of >= 0
        out[free] = x[self.row_of[free]]
        return out

    def distortion(self, uv):
        """(loss, dL/duv (n,2), dL/dp3 (n,3), per-triangle terms)."""
        uv = np.ascontiguousarray(uv, np.float64).reshape(-1)
        n = len(self.pinned)
        loss = ctypes.c_double(0.0)
        duv = np.zeros(2 * n)
        dp3 = np.zeros(3 * n)
        lib().orc_distortion_loss(self.bag.h, _f64p(uv), ctypes.byref(loss), _f64p(duv), _f64p(dp3))
        return loss.value, duv.reshape(n, 2), dp3.reshape(n, 3), self.bag.f64("loss_t")

    def adjoint_positions(self, x, lam):
        """dp3 (n,3) of lam^T (b - A x): the position gradient through the solve."""
        n = len(self.pinned)
        dp3 = np.zeros(3 * n)
        lib().orc_lscm_adjoint_positions(self.bag.h, _f64p(np.ascontiguousarray(x, np.float64).reshape(-1)),
                                         _f64p(np.ascontiguousarray(lam, np.float64).reshape(-1)), _f64p(dp3))
        return dp3.reshape(n, 3)


def config4_loss(chart: "FixedPinChart", x, lam_l2: float, target):
    """Loss of the differentiation workload for a solution x of `chart`:
    sum_t area_t (s1/s2 - 1)^2 + lam_l2 * sum_v |uv_v - target_v|^2 over all vertices.
    Returns (loss, uv, per-triangle distortion terms)."""
    uv = chart.uv(x)
    d, _, _, lt = chart.distortion(uv)
    return d + lam_l2 * float(((uv - target) ** 2).sum()), uv, lt


def lu_adjoint_gradient(p3, tris, pinned, pin_uv, lam_l2: float, target):
    """CPU reference gradient dL/dp3 (n, 3) of config4_loss through the fixed-pin solve:
    SuperLU solve, lam = A^-1 dL/duv (free rows), reverse pass of the assembly, plus the
    explicit position gradient of the distortion term."""
    ch = FixedPinChart(p3, tris, pinned, pin_uv)
    x = ch.solve()
    uv = ch.uv(x)
    _, duv, dp_dist, _ = ch.distortion(uv)
    g = duv + 2.0 * lam_l2 * (uv - target)
    free = ch.row_of >= 0
    gf = np.zeros((ch.nf, 2))
    gf[ch.row_of[free]] = g[free]
    lam = ch.solve(gf)
    return dp_dist + ch.adjoint_positions(x, lam), uv


def fd_gradient(p3, tris, pinned, pin_uv, lam_l2: float, target, picks, h: float = 1e-6, refine: int = 0,
                reuse_base: bool = False, smooth_steps=None, edge_scale=None, richardson: bool = False):
    """Central differences of config4_loss with respect to p3[v, k] for (v, k) in picks,
    through the fixed-pin solve.  The perturbed solution is formed as x + dx with
    A' dx = (b' - b) - (A' - A) x (a right-hand side that is exactly zero away from v), and
    the loss difference term by term, so neither the solve's rounding nor the cancellation
    of two large loss totals reaches the difference quotient.

    ``reuse_base``: solve A' dx = rhs exactly with the unperturbed matrix's LU factors and a
    low-rank (Woodbury) update instead of factoring every perturbed matrix -- what makes the
    check affordable on a half-million-row chart.  A' - A is confined to the rows and
    columns S of v's neighbourhood (the coefficients of the triangles around v), so with
    M = (A' - A)[S, S] and Z = A^-1 E_S (one solve per row of S, kept per vertex),
    A'^-1 y = A^-1 y - Z M (I + Z[S] M)^-1 (A^-1 y)[S].  (Iterative refinement on the
    unperturbed factors diverges where |A^-1 (A' - A)| > 1, which an ill-conditioned chart
    reaches.)

    ``smooth_steps`` (a decreasing sequence of h): the loss is only piecewise smooth -- the
    assembly clamps every corner cotangent at 0 (lscm.rs:256-268) and drops an edge whose
    weight is <= EPS (lscm.rs:606) -- so a difference quotient across one of those kinks
    averages two one-sided derivatives.  For each pick the first h of the sequence at which
    neither v + h nor v - h moves a clamp of the triangles around v (no corner cotangent of
    them changes sign, the sparsity pattern is unchanged) is used; a pick with no such h gets
    NaN.  ``edge_scale``: each h of the sequence is first capped at edge_scale times the
    shortest edge at v, so the quotient's truncation error, which grows as (h / edge)^2,
    stays small on short edges too.  ``richardson``: each quotient D(h) is combined with
    D(h / 2) as (4 D(h / 2) - D(h)) / 3, which cancels its h^2 truncation term (next to the
    sphere's poles, where edges are ~2e-5 long, D(1e-6) alone is off by ~(h / edge)^2).
    Returns (values, h used per pick) in that case, the values alone otherwise."""
    p3 = np.ascontiguousarray(p3, np.float64).reshape(-1, 3)
    tris = np.ascontiguousarray(tris, np.int64).reshape(-1, 3)
    base = FixedPinChart(p3, tris, pinned, pin_uv)
    x = base.solve()
    uv = base.uv(x)
    _, _, _, lt = base.distortion(uv)
    free = base.row_of >= 0
    zcache = {}  # row -> column of A^-1 (solves shared by the perturbations of one vertex)
    if smooth_steps is not None:
        order = np.argsort(tris.ravel(), kind="stable")
        starts = np.searchsorted(tris.ravel()[order], np.arange(len(p3) + 1))

    def woodbury(dA, rhs):
        rows = np.unique(dA.tocoo().row[dA.tocoo().data != 0.0])
        y = base.solve(rhs)
        if len(rows) == 0:
            return y
        need = [r for r in rows if r not in zcache]
        if need:
            E = np.zeros((base.nf, len(need)))
            E[need, np.arange(len(need))] = 1.0
            Zn = base.solve(E)
            for t, r in enumerate(need):
                zcache[r] = Zn[:, t]
        Z = np.stack([zcache[r] for r in rows], axis=1)
        M = dA[rows][:, rows].toarray()
        K = np.eye(len(rows)) + Z[rows] @ M
        return y - Z @ (M @ np.linalg.solve(K, y[rows]))

    def cot_signs(q, tv):
        a, b, c = q[tv[:, 0]], q[tv[:, 1]], q[tv[:, 2]]
        out = []
        for o, u, w in ((a, b, c), (b, c, a), (c, a, b)):
            e1, e2 = u - o, w - o
            out.append(np.sign(np.einsum("ij,ij->i", e1, e2)))
        return np.stack(out, axis=1)

    def one_side(q):
        ch = FixedPinChart(q, tris, pinned, pin_uv)
        same = np.array_equal(ch.A.indptr, base.A.indptr) and np.array_equal(ch.A.indices, base.A.indices)
        return ch, same

    def diff(ch, same):
        if same:
            dA = ch.A.copy()
            dA.data = ch.A.data - base.A.data
            rhs = (ch.b - base.b) - dA @ x
            dx = woodbury(dA, rhs) if reuse_base else ch.solve(rhs)
            for _ in range(refine):  # iterative refinement of the small correction on A'
                res = rhs - ch.A @ dx
                dx = dx + (woodbury(dA, res) if reuse_base else ch.solve(res))
        else:  # an edge weight crossed the drop threshold (a clamped cotangent at 0)
            dx = ch.solve() - x
        uv2 = uv.copy()
        uv2[free] = uv[free] + dx[base.row_of[free]]
        _, _, _, lt2 = ch.distortion(uv2)
        du = uv2 - uv
        return float((lt2 - lt).sum()) + lam_l2 * float((du * (uv2 + uv - 2.0 * target)).sum())

    out, used = [], []
    last_v = None
    for v, k in picks:
        if v != last_v:
            zcache.clear()
            last_v = v
        if smooth_steps is None:
            diffs = []
            for sgn in (1.0, -1.0):
                q = p3.copy()
                q[v, k] += sgn * h
                diffs.append(diff(*one_side(q)))
            out.append((diffs[0] - diffs[1]) / (2.0 * h))
            continue
        tv = tris[order[starts[v]:starts[v + 1]] // 3]
        s0 = cot_signs(p3, tv)
        cap = float("inf")
        if edge_scale is not None:
            for a, b in ((0, 1), (1, 2), (2, 0)):
                cap = min(cap, edge_scale * float(np.linalg.norm(p3[tv[:, a]] - p3[tv[:, b]], axis=1).min()))
        val, hv = float("nan"), float("nan")
        for hh in smooth_steps:
            hh = min(hh, cap)
            sides, ok = [], True
            for sgn in (1.0, -1.0):
                q = p3.copy()
                q[v, k] += sgn * hh
                ch, same = one_side(q)
                if not same or not np.array_equal(cot_signs(q, tv), s0):
                    ok = False
                    break
                sides.append((ch, same))
            if ok:
                val = (diff(*sides[0]) - diff(*sides[1])) / (2.0 * hh)
                if richardson:
                    half = []
                    for sgn in (1.0, -1.0):
                        q = p3.copy()
                        q[v, k] += sgn * 0.5 * hh
                        half.append(diff(*one_side(q)))
                    val = (4.0 * (half[0] - half[1]) / hh - val) / 3.0
                hv = hh
                break
        out.append(val)
        used.append(hv)
    if smooth_steps is None:
        return np.array(out)
    return np.array(out), np.array(used)


def rectangularize(uv, border):
    """rectangularize (metrics.rs:147-227) of one chart: (q (n, 2), ext (2,))."""
    uv = np.ascontiguousarray(uv, np.float64).reshape(-1)
    b = np.ascontiguousarray(border, np.int64).reshape(-1)
    n = len(b)
    q = np.zeros(2 * n)
    ext = np.zeros(2)
    lib().orc_rectangularize(n, _f64p(uv), _i64p(b), _f64p(q), _f64p(ext))
    return q.reshape(n, 2), ext

