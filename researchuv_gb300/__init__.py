"""researchuv_gb300 — GB300 (sm_103a) LSCM solve path behind ResearchUV's GPU-solver boundary.

Python mirror of the reference's interface for this path (names and argument meaning as in
the reference; paths relative to its crates/, ``researchuv-`` dropped):

* :class:`CsrMatrix`, :class:`Precond`, :class:`GpuSolver` — ``gpu/src/solver.rs:14-44``,
  ``gpu/src/precond.rs:20-47``, ``GpuSolver::{global,new,cg_solve,cg_solve_precond,
  apply_ic0_for_test}`` (``solver.rs:104-565``).  Failures return ``None`` as the reference's
  ``Option`` does; the reason is in :attr:`GpuSolver.last_error`.
* :class:`UnfoldOptions`, :class:`UnfoldResult`, :class:`SolverBackend` —
  ``unwrap/src/lscm.rs:56-116``.
* :func:`prepare_mesh` / :func:`prepare_patches` + :func:`unfold_charts` — the chart stages
  and the per-chart unfold of ``unwrap/src/pipeline.rs:146-194``, all charts in one batched
  GPU solve.

Everything runs through ``libruv.so`` (C ABI in ``include/ruv.h``).  There is no CPU
fallback: importing works without a GPU, but every solve raises or returns ``None`` when
no sm_103a device is present, and a missing library raises at first use.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import os
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libruv.so")

_P = ctypes.POINTER
_i32, _i64, _f64, _u8, _vp, _cp = (ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_uint8,
                                   ctypes.c_void_p, ctypes.c_char_p)


class RuvBatch(ctypes.Structure):
    _fields_ = [("n_charts", _i64), ("vert_off", _P(_i64)), ("tri_off", _P(_i64)), ("p3", _P(_f64)),
                ("tris", _P(_i32)), ("pinned", _P(_u8)), ("pin_uv", _P(_f64)), ("p2", _P(_f64))]


class RuvUnfoldOpts(ctypes.Structure):
    _fields_ = [("angle_mix", _f64), ("mix_w", _f64), ("max_iter", _i32), ("precond", ctypes.c_int),
                ("precision", ctypes.c_int), ("tol", _f64), ("max_cg_iter", _i64)]


class RuvChartStat(ctypes.Structure):
    _fields_ = [("status", _i32), ("driver_iters", _i32), ("cg_iters", _i32), ("n_free", _i32),
                ("rel_res", _f64), ("err_accum", _f64)]


# every symbol include/ruv.h declares, with its ctypes signature
SIGNATURES = {
    "ruv_abi_version": (_i32, []),
    "ruv_status_str": (_cp, [ctypes.c_int]),
    "ruv_ctx_create": (ctypes.c_int, [_P(_vp), _i32]),
    "ruv_ctx_destroy": (None, [_vp]),
    "ruv_last_error": (_cp, [_vp]),
    "ruv_debug_fail_alloc": (ctypes.c_int, [_vp, _i64]),
    "ruv_cg_solve": (ctypes.c_int, [_vp, _i32, _P(_i32), _P(_i32), _P(_f64), _P(_f64), _P(_f64), _i64, _f64,
                                    ctypes.c_int, _P(_i64)]),
    "ruv_apply_ic0": (ctypes.c_int, [_vp, _i32, _P(_i32), _P(_i32), _P(_f64), _P(_f64), _P(_f64)]),
    "ruv_ic0_export": (ctypes.c_int, [_vp, _i32, _P(_i32), _P(_i32), _P(_f64), _i32, _i64, _P(_i64), _P(_i32),
                                      _P(_f64), _P(_i32), _P(_i64), _P(_i32), _P(_i32)]),
    "ruv_amg_export": (ctypes.c_int, [_vp, _i32, _P(_i32), _P(_i32), _P(_f64), _i32, _i32, _i64, _P(_i64),
                                      _P(_i64), _P(_i32), _P(_f64), _P(_i64), _P(_i32), _P(ctypes.c_float),
                                      _P(_i32)]),
    "ruv_unfold_opts_default": (None, [_P(RuvUnfoldOpts)]),
    "ruv_lscm_solve_batch": (ctypes.c_int, [_vp, _P(RuvBatch), _P(RuvUnfoldOpts), _P(_f64), _P(RuvChartStat)]),
    "ruv_prepare_mesh": (ctypes.c_int, [_P(_f64), _i64, _P(_i32), _i64, _f64, _f64, _i32, _P(_vp)]),
    "ruv_prepare_patches": (ctypes.c_int, [_i64, _P(_i64), _P(_i64), _P(_f64), _P(_i32), _i32, _P(_vp)]),
    "ruv_lscm_solve_batch_keep_metric": (ctypes.c_int, [_vp, _P(RuvBatch), _P(RuvUnfoldOpts), _P(_f64), _P(_f64),
                                                        _P(RuvChartStat)]),
    "ruv_cut_opts_default": (None, [_vp]),
    "ruv_prepare_mesh_cut": (ctypes.c_int, [_vp, _P(_f64), _i64, _P(_i32), _i64, _f64, _f64, _vp, _P(RuvUnfoldOpts), _i32,
                                            _P(_vp), _P(_i64)]),
    "ruv_prepare_mesh_gpu": (ctypes.c_int, [_vp, _P(_f64), _i64, _P(_i32), _i64, _f64, _f64, _i32, _P(_vp)]),
    "ruv_prepare_patches_gpu": (ctypes.c_int, [_vp, _i64, _P(_i64), _P(_i64), _P(_f64), _P(_i32), _i32, _P(_vp)]),
    "ruv_prepared_free": (None, [_vp]),
    "ruv_prepared_batch": (ctypes.c_int, [_vp, _P(RuvBatch)]),
    "ruv_prepared_get_i64": (_i64, [_vp, _cp, _P(_i64)]),
    "ruv_prepared_get_f64": (_i64, [_vp, _cp, _P(_f64)]),
    "ruv_export_chart_system": (ctypes.c_int, [_vp, _i64, _P(_i64), _P(_i64), _P(_i32), _P(_i32), _P(_f64),
                                               _P(_f64)]),
    "ruv_lscm_upload": (ctypes.c_int, [_vp, _P(RuvBatch)]),
    "ruv_lscm_solve_resident": (ctypes.c_int, [_vp, _P(RuvUnfoldOpts), _P(RuvChartStat)]),
    "ruv_lscm_download_uv": (ctypes.c_int, [_vp, _P(_f64)]),
    "ruv_lscm_forward": (ctypes.c_int, [_vp, _P(RuvBatch), _P(RuvUnfoldOpts), _P(_f64), _P(RuvChartStat)]),
    "ruv_lscm_backward": (ctypes.c_int, [_vp, _P(RuvUnfoldOpts), _P(_f64), _P(_f64), _P(RuvChartStat)]),
    "ruv_distortion_loss": (ctypes.c_int, [_vp, _P(_f64), _P(_f64), _P(_f64), _P(_f64)]),
    "ruv_chart_distortion": (ctypes.c_int, [_vp, _P(_f64), _P(_f64)]),
    "ruv_rectangularize": (ctypes.c_int, [_vp, _P(_f64), _P(_u8), _P(_f64), _P(_f64)]),
    "ruv_host_alloc": (ctypes.c_int, [_vp, _i64, _P(_vp)]),
    "ruv_host_free": (None, [_vp]),
    "ruv_selftest_fp64": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_uint64, _i64, _P(_i64), _P(_f64)]),
    "ruv_last_timings": (_i32, [_vp, _P(_f64), _i32]),
    "ruv_kernel_launches": (_i64, [_vp]),
    "ruv_cg_solve_noalloc": (ctypes.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _i64, _f64, ctypes.c_int, _P(_i64), _vp,
                                            ctypes.c_char_p, _i32]),
    "ruv_autotune": (ctypes.c_int, [_vp, ctypes.c_int, _i32, _P(_i32), _P(_i32), _P(_i32), _P(_f64)]),
    "ruv_spmv_form": (ctypes.c_int, [_vp, _P(_i32)]),
    "ruv_bench_spmv": (ctypes.c_int, [_vp, ctypes.c_int, _i32, _i32, _P(_f64), _P(_f64), _P(_f64)]),
}

_lib = None


def lib():
    """The loaded libruv.so (built by :func:`researchuv_gb300.build.build`).  Raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libruv.so not built ({LIB_PATH}); run researchuv_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class Status(enum.IntEnum):
    OK = 0
    NO_DEVICE = 1
    BAD_INPUT = 2
    OOM = 3
    NOT_CONVERGED = 4
    BREAKDOWN = 5
    TIMEOUT = 6
    LAUNCH = 7
    INTERNAL = 8


class RuvError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = Status(status)
        super().__init__(f"{self.status.name}: {msg}")


class Precond(enum.IntEnum):
    """gpu/src/precond.rs:20-47 (``None`` is spelled NONE)."""
    NONE = 0
    JACOBI = 1
    IC0 = 2
    IC0_COLOR = 3
    AMG = 4
    AMG_SA = 5

    @classmethod
    def from_env(cls) -> "Precond":
        """RESEARCHUV_GPU_PRECOND, as unwrap/src/lscm.rs:492-499 reads it (default Jacobi)."""
        return {"amgsa": cls.AMG_SA, "amg": cls.AMG, "ic0color": cls.IC0_COLOR, "ic0": cls.IC0,
                "none": cls.NONE}.get(os.environ.get("RESEARCHUV_GPU_PRECOND", ""), cls.JACOBI)


class Precision(enum.IntEnum):
    FP64 = 0
    MIXED = 1


def _ptr(a, ct):
    return a.ctypes.data_as(_P(ct)) if a is not None else None


# ------------------------------------------------------------------ GpuSolver boundary
@dataclasses.dataclass
class CsrMatrix:
    """gpu/src/solver.rs:14-44."""
    vals: np.ndarray
    cols: np.ndarray
    row_ptr: np.ndarray

    def __post_init__(self):
        self.vals = np.ascontiguousarray(self.vals, np.float64)
        self.cols = np.ascontiguousarray(self.cols, np.int32)
        self.row_ptr = np.ascontiguousarray(self.row_ptr, np.int32)

    def rows(self) -> int:
        return max(len(self.row_ptr) - 1, 0)

    def row(self, i):
        lo, hi = self.row_ptr[i], self.row_ptr[i + 1]
        return list(zip(self.cols[lo:hi].tolist(), self.vals[lo:hi].tolist()))

    def row_get(self, i, j) -> float:
        for c, v in self.row(i):
            if c == j:
                return v
        return 0.0


class Context:
    """One device context (stream + reusable device workspace).  Not thread-safe."""

    def __init__(self, device: int = 0):
        h = _vp()
        st = lib().ruv_ctx_create(ctypes.byref(h), device)
        if st != 0:
            raise RuvError(st, "ruv_ctx_create(device=%d)" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ruv_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return lib().ruv_last_error(self.h).decode()

    def check(self, st, what=""):
        if st != 0:
            raise RuvError(st, f"{what}: {self.last_error()}")


class GpuSolver:
    """gpu/src/solver.rs:49-565 — FP64 (P)CG on one SPD CSR system."""

    _global: Optional["GpuSolver"] = None
    _global_tried = False

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.last_error = ""

    @classmethod
    def new(cls, device: int = 0) -> Optional["GpuSolver"]:
        try:
            return cls(Context(device))
        except RuvError:
            return None

    @classmethod
    def global_(cls) -> Optional["GpuSolver"]:
        """GpuSolver::global (solver.rs:104-113): initialised once; None without a device."""
        if not cls._global_tried:
            cls._global_tried = True
            cls._global = cls.new()
        return cls._global

    def cg_solve_precond(self, a: CsrMatrix, b: Sequence[float], max_iter: int, tol: float,
                         precond: Precond = Precond.NONE):
        """solver.rs:284-565.  Returns (x, iters) or None."""
        b = np.ascontiguousarray(b, np.float64)
        n = a.rows()
        if n == 0 or b.size != n or a.cols.size != a.vals.size or a.row_ptr.size != n + 1:
            self.last_error = "dimension mismatch"
            return None
        x = np.empty(n, np.float64)
        iters = _i64(0)
        st = lib().ruv_cg_solve(self.ctx.h, n, _ptr(a.row_ptr, _i32), _ptr(a.cols, _i32), _ptr(a.vals, _f64),
                                _ptr(b, _f64), _ptr(x, _f64), int(max_iter), float(tol), int(precond),
                                ctypes.byref(iters))
        if st != 0:
            self.last_error = f"{Status(st).name}: {self.ctx.last_error()}"
            return None
        return x, int(iters.value)

    def cg_solve(self, a: CsrMatrix, b, max_iter: int, tol: float):
        r = self.cg_solve_precond(a, b, max_iter, tol, Precond.NONE)
        return None if r is None else r[0]

    def apply_ic0_for_test(self, a: CsrMatrix, r):
        r = np.ascontiguousarray(r, np.float64)
        if r.size != a.rows():
            return None
        z = np.empty_like(r)
        st = lib().ruv_apply_ic0(self.ctx.h, a.rows(), _ptr(a.row_ptr, _i32), _ptr(a.cols, _i32),
                                 _ptr(a.vals, _f64), _ptr(r, _f64), _ptr(z, _f64))
        if st != 0:
            self.last_error = f"{Status(st).name}: {self.ctx.last_error()}"
            return None
        return z

    def ic0_factor(self, a: CsrMatrix, colored: bool = False) -> dict:
        """The device IC(0) factor of ``a`` (natural or colour-permuted order): rows of L with
        the diagonal last, the position -> original row map, the level and colour counts."""
        n = a.rows()
        cap = int(len(a.vals))  # the factor keeps the lower pattern: at most nnz(A) entries
        ptr = np.zeros(n + 1, np.int64)
        cols = np.zeros(max(cap, 1), np.int32)
        vals = np.zeros(max(cap, 1), np.float64)
        perm = np.zeros(n, np.int32)
        nnz, lev, col = _i64(0), _i32(0), _i32(0)
        st = lib().ruv_ic0_export(self.ctx.h, n, _ptr(a.row_ptr, _i32), _ptr(a.cols, _i32), _ptr(a.vals, _f64),
                                  1 if colored else 0, cap, _ptr(ptr, _i64), _ptr(cols, _i32), _ptr(vals, _f64),
                                  _ptr(perm, _i32), ctypes.byref(nnz), ctypes.byref(lev), ctypes.byref(col))
        self.ctx.check(st, "ruv_ic0_export")
        k = nnz.value
        return {"ptr": ptr, "cols": cols[:k], "vals": vals[:k], "to_orig": perm, "levels": lev.value,
                "colours": col.value}

    def amg_level(self, a: CsrMatrix, level: int, smoothed: bool = True) -> dict:
        """Level ``level`` of the device AMG hierarchy of ``a`` (AMG-SA when ``smoothed``): the
        level operator (FP64 CSR), the prolongator to the next level and the aggregates."""
        n = a.rows()
        sizes = np.zeros(6, np.int64)
        args = (self.ctx.h, n, _ptr(a.row_ptr, _i32), _ptr(a.cols, _i32), _ptr(a.vals, _f64), 1 if smoothed else 0,
                int(level))
        nul = (None,) * 7
        self.ctx.check(lib().ruv_amg_export(*args, 0, _ptr(sizes, _i64), *nul), "ruv_amg_export")
        levels, sm, rows, nxt, annz, pnnz = (int(x) for x in sizes)
        cap = max(rows + 1, annz, pnnz, 1)
        ap, ac, av = np.zeros(cap, np.int64), np.zeros(cap, np.int32), np.zeros(cap, np.float64)
        pp, pc, pv = np.zeros(cap, np.int64), np.zeros(cap, np.int32), np.zeros(cap, np.float32)
        ag = np.zeros(cap, np.int32)
        self.ctx.check(lib().ruv_amg_export(*args, cap, _ptr(sizes, _i64), _ptr(ap, _i64), _ptr(ac, _i32),
                                            _ptr(av, _f64), _ptr(pp, _i64), _ptr(pc, _i32),
                                            _ptr(pv, ctypes.c_float), _ptr(ag, _i32)), "ruv_amg_export")
        return {"levels": levels, "smoothed": bool(sm), "rows": rows, "next_rows": nxt,
                "A": (ap[:rows + 1], ac[:annz], av[:annz]), "P": (pp[:rows + 1], pc[:pnnz], pv[:pnnz]),
                "agg": ag[:rows]}


# ------------------------------------------------------------------ unfold driver
class SolverBackend(enum.Enum):
    """unwrap/src/lscm.rs:56-72.  This library implements the GPU backend only."""
    CPU = "cpu"
    GPU = "gpu"


@dataclasses.dataclass
class UnfoldOptions:
    """unwrap/src/lscm.rs:74-101 plus the GPU solve controls (lscm.rs:471-506)."""
    max_iter: int = 100
    angle_mix: float = 1.0
    keep_metric: bool = False
    target_area: float = 0.0
    mix_w: float = 1.0
    solver: SolverBackend = SolverBackend.GPU
    precond: Precond = dataclasses.field(default_factory=Precond.from_env)
    precision: Precision = Precision.MIXED
    tol: float = 1e-12
    max_cg_iter: int = 0  # 0 = max(max_iter, 1024) * 16 (lscm.rs:501)

    def to_c(self) -> RuvUnfoldOpts:
        if self.solver != SolverBackend.GPU:
            raise RuvError(Status.BAD_INPUT, "this library implements SolverBackend::Gpu only")
        o = RuvUnfoldOpts()
        lib().ruv_unfold_opts_default(ctypes.byref(o))
        o.angle_mix = self.angle_mix
        o.mix_w = self.mix_w
        o.max_iter = self.max_iter
        o.precond = int(self.precond)
        o.precision = int(self.precision)
        o.tol = self.tol
        o.max_cg_iter = self.max_cg_iter if self.max_cg_iter > 0 else max(self.max_iter, 1024) * 16
        return o


@dataclasses.dataclass
class UnfoldResult:
    """unwrap/src/lscm.rs:103-116 plus solver statistics."""
    uv: np.ndarray
    iters: int
    err_accum: float
    target: float
    area3d: float
    status: Status = Status.OK
    cg_iters: int = 0
    n_free: int = 0
    rel_res: float = 0.0


class Charts:
    """Charts prepared on the host (weld + segment + tangent frames + pins), packed."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None):
            lib().ruv_prepared_free(self.h)
            self.h = None

    def i64(self, what: str) -> np.ndarray:
        n = lib().ruv_prepared_get_i64(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.int64)
        lib().ruv_prepared_get_i64(self.h, what.encode(), _ptr(out, _i64))
        return out

    def f64(self, what: str) -> np.ndarray:
        n = lib().ruv_prepared_get_f64(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.float64)
        lib().ruv_prepared_get_f64(self.h, what.encode(), _ptr(out, _f64))
        return out

    @property
    def n_charts(self) -> int:
        return len(self.i64("chart.vert_off")) - 1

    def batch(self) -> RuvBatch:
        v = RuvBatch()
        st = lib().ruv_prepared_batch(self.h, ctypes.byref(v))
        if st != 0:
            raise RuvError(st, "ruv_prepared_batch")
        return v

    def chart(self, c: int) -> dict:
        vo, to, bo = self.i64("chart.vert_off"), self.i64("chart.tri_off"), self.i64("chart.border_off")
        lo, ls, li = self.i64("chart.loop_off"), self.i64("chart.loop_seg"), self.i64("chart.loop_ids")
        v0, v1, t0, t1 = vo[c], vo[c + 1], to[c], to[c + 1]
        return {
            "vertex_ids": self.i64("chart.vertex_ids")[v0:v1],
            "face_ids": self.i64("chart.face_ids")[t0:t1],
            "tris": self.i64("chart.tris").reshape(-1, 3)[t0:t1],
            "border": self.i64("chart.border")[bo[c]:bo[c + 1]],
            "border_loops": [li[ls[k]:ls[k + 1]] for k in range(lo[c], lo[c + 1])],
            "area3d": float(self.f64("chart.area3d")[c]),
            "p2": self.f64("chart.p2").reshape(-1, 2)[v0:v1],
            "pinned": self.i64("chart.pinned")[v0:v1].astype(bool),
            "pin_uv": self.f64("chart.pin_uv").reshape(-1, 2)[v0:v1],
        }


def prepare_mesh(positions, faces, weld_tol: float = 1e-12, angle_min_deg: float = 30.0,
                 threads: int = 0, ctx: Optional["Context"] = None) -> Charts:
    """weld (weld.rs:19-57) + segment (segment.rs:130-331) + per-chart frames and pins.
    With a Context, the weld, edge-face lists, cut flags and chart vertex sets run on its
    device (ruv_prepare_mesh_gpu); the result is the same bit for bit."""
    p = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
    h = _vp()
    if ctx is not None:
        ctx.check(lib().ruv_prepare_mesh_gpu(ctx.h, _ptr(p, _f64), p.shape[0], _ptr(f, _i32), f.shape[0], weld_tol,
                                             angle_min_deg, threads, ctypes.byref(h)), "ruv_prepare_mesh_gpu")
        return Charts(h)
    st = lib().ruv_prepare_mesh(_ptr(p, _f64), p.shape[0], _ptr(f, _i32), f.shape[0], weld_tol, angle_min_deg,
                                threads, ctypes.byref(h))
    if st != 0:
        raise RuvError(st, "ruv_prepare_mesh")
    return Charts(h)


class RuvCutOpts(ctypes.Structure):
    _fields_ = [("seam_enable", _i32), ("seam_min_faces", _i32), ("seam_branch_count", _i32), ("recut_enable", _i32),
                ("recut_max_rounds", _i32), ("recut_max_splits", _i32), ("recut_fold_fraction", _f64),
                ("recut_max_charts", _i32)]


@dataclasses.dataclass
class SeamCutOptions:
    """unwrap/src/seam.rs:30-49."""
    enable: bool = False
    min_faces: int = 8
    branch_count: int = 1


@dataclasses.dataclass
class RecutOptions:
    """unwrap/src/recut.rs:33-59."""
    enable: bool = False
    max_rounds: int = 6
    max_splits: int = 48
    fold_fraction: float = 0.02
    max_charts: int = 64


def prepare_mesh_cut(ctx: Optional["Context"], positions, faces, weld_tol: float = 1e-12, angle_min_deg: float = 30.0,
                     seam_cut: Optional[SeamCutOptions] = None, recut: Optional[RecutOptions] = None,
                     unfold: Optional[UnfoldOptions] = None, threads: int = 0):
    """pipeline::run's chart stages with the optional seam cut and re-cutting controller
    (pipeline.rs:146-167; every controller round unfolds all charts in one batched solve on
    ctx).  Returns (Charts, cut edges added by the controller)."""
    sc, rc = seam_cut or SeamCutOptions(), recut or RecutOptions()
    o = RuvCutOpts()
    lib().ruv_cut_opts_default(ctypes.byref(o))
    o.seam_enable, o.seam_min_faces, o.seam_branch_count = int(sc.enable), sc.min_faces, sc.branch_count
    o.recut_enable, o.recut_max_rounds, o.recut_max_splits = int(rc.enable), rc.max_rounds, rc.max_splits
    o.recut_fold_fraction, o.recut_max_charts = rc.fold_fraction, rc.max_charts
    u = (unfold or UnfoldOptions()).to_c()
    p = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
    h, added = _vp(), _i64(0)
    st = lib().ruv_prepare_mesh_cut(ctx.h if ctx is not None else None, _ptr(p, _f64), p.shape[0], _ptr(f, _i32),
                                    f.shape[0], weld_tol, angle_min_deg, ctypes.byref(o), ctypes.byref(u), threads,
                                    ctypes.byref(h), ctypes.byref(added))
    if ctx is not None:
        ctx.check(st, "ruv_prepare_mesh_cut")
    elif st != 0:
        raise RuvError(st, "ruv_prepare_mesh_cut")
    return Charts(h), added.value


def prepare_patches(vert_off, tri_off, p3, tris, threads: int = 0, ctx: Optional["Context"] = None) -> Charts:
    """One chart per given patch (no weld / segmentation).  With a Context, the data-parallel
    stages run on its device (ruv_prepare_patches_gpu); the result is the same bit for bit."""
    vo = np.ascontiguousarray(vert_off, np.int64)
    to = np.ascontiguousarray(tri_off, np.int64)
    p = np.ascontiguousarray(p3, np.float64).reshape(-1)
    t = np.ascontiguousarray(tris, np.int32).reshape(-1)
    h = _vp()
    if ctx is not None:
        ctx.check(lib().ruv_prepare_patches_gpu(ctx.h, len(vo) - 1, _ptr(vo, _i64), _ptr(to, _i64), _ptr(p, _f64),
                                                _ptr(t, _i32), threads, ctypes.byref(h)), "ruv_prepare_patches_gpu")
        return Charts(h)
    st = lib().ruv_prepare_patches(len(vo) - 1, _ptr(vo, _i64), _ptr(to, _i64), _ptr(p, _f64), _ptr(t, _i32),
                                   threads, ctypes.byref(h))
    if st != 0:
        raise RuvError(st, "ruv_prepare_patches")
    return Charts(h)


def solve_batch(ctx: Context, batch: RuvBatch, opts: UnfoldOptions, n_verts: int, check: bool = True,
                area3d=None):
    """ruv_lscm_solve_batch on a packed batch.  Returns (uv (n_verts, 2), stats list, status).
    With opts.keep_metric, ruv_lscm_solve_batch_keep_metric with the per-chart targets
    (opts.target_area if > 0, else area3d[c])."""
    o = opts.to_c()
    uv = np.empty((n_verts, 2), np.float64)
    stats = (RuvChartStat * max(batch.n_charts, 1))()
    if opts.keep_metric:
        if opts.target_area > 0:
            target = np.full(batch.n_charts, float(opts.target_area))
        elif area3d is not None:
            target = np.ascontiguousarray(area3d, np.float64)
        else:
            raise RuvError(Status.BAD_INPUT, "keep_metric needs the charts' area3d (or a target_area)")
        st = lib().ruv_lscm_solve_batch_keep_metric(ctx.h, ctypes.byref(batch), ctypes.byref(o), _ptr(target, _f64),
                                                    _ptr(uv, _f64), stats)
    else:
        st = lib().ruv_lscm_solve_batch(ctx.h, ctypes.byref(batch), ctypes.byref(o), _ptr(uv, _f64), stats)
    if check and st not in (0, Status.NOT_CONVERGED):
        ctx.check(st, "ruv_lscm_solve_batch")
    return uv, [stats[i] for i in range(batch.n_charts)], Status(st)


def unfold_charts(ctx: Context, charts: Charts, opts: Optional[UnfoldOptions] = None) -> List[UnfoldResult]:
    """unfold_chart (lscm.rs:512-727) for every chart, in one batched GPU solve."""
    opts = opts or UnfoldOptions()
    vo = charts.i64("chart.vert_off")
    area = charts.f64("chart.area3d")
    uv, stats, _ = solve_batch(ctx, charts.batch(), opts, int(vo[-1]), area3d=area)
    out = []
    for c, s in enumerate(stats):
        out.append(UnfoldResult(uv=uv[vo[c]:vo[c + 1]].copy(), iters=s.driver_iters, err_accum=s.err_accum,
                                target=opts.target_area if opts.target_area > 0 else float(area[c]),
                                area3d=float(area[c]), status=Status(s.status), cg_iters=s.cg_iters,
                                n_free=s.n_free, rel_res=s.rel_res))
    return out


# ------------------------------------------------------------------ page-locked host arrays
class _PinnedOwner:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if self.ptr:
            lib().ruv_host_free(self.ptr)
            self.ptr = None


def pinned_empty(ctx: Context, shape, dtype) -> np.ndarray:
    """A numpy array in page-locked host memory (ruv_host_alloc); freed with the array."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    nbytes = max(n * dtype.itemsize, 1)
    ptr = _vp()
    ctx.check(lib().ruv_host_alloc(ctx.h, nbytes, ctypes.byref(ptr)), "ruv_host_alloc")
    buf = (ctypes.c_char * nbytes).from_address(ptr.value)
    buf._owner = _PinnedOwner(ptr.value)  # the array keeps `buf` (its base), `buf` keeps the memory
    return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)


def pinned_batch(ctx: Context, charts: "Charts"):
    """A copy of a prepared batch in page-locked host memory: (RuvBatch, the arrays that own it)."""
    b = charts.batch()
    nc = b.n_charts
    vo = np.ctypeslib.as_array(b.vert_off, shape=(nc + 1,))
    to = np.ctypeslib.as_array(b.tri_off, shape=(nc + 1,))
    nv, nt = int(vo[-1]), int(to[-1])
    srcs = {"vert_off": (vo, _i64), "tri_off": (to, _i64),
            "p3": (np.ctypeslib.as_array(b.p3, shape=(max(3 * nv, 1),))[:3 * nv], _f64),
            "tris": (np.ctypeslib.as_array(b.tris, shape=(max(3 * nt, 1),))[:3 * nt], _i32),
            "pinned": (np.ctypeslib.as_array(b.pinned, shape=(max(nv, 1),))[:nv], _u8),
            "pin_uv": (np.ctypeslib.as_array(b.pin_uv, shape=(max(2 * nv, 1),))[:2 * nv], _f64),
            "p2": (np.ctypeslib.as_array(b.p2, shape=(max(2 * nv, 1),))[:2 * nv], _f64)}
    keep = {}
    out = RuvBatch()
    out.n_charts = nc
    for name, (src, ct) in srcs.items():
        a = pinned_empty(ctx, src.shape, src.dtype)
        a[...] = src
        keep[name] = a
        setattr(out, name, _ptr(a, ct))
    return out, keep


# ------------------------------------------------------------------ differentiation
def lscm_forward(ctx: Context, batch: RuvBatch, opts: UnfoldOptions, n_verts: int):
    """Forward half of the differentiable unfold (ruv_lscm_forward): the batched solve; the
    batch and its solution stay on the context.  Returns (uv (n_verts, 2), stats)."""
    o = opts.to_c()
    uv = np.empty((n_verts, 2), np.float64)
    stats = (RuvChartStat * max(batch.n_charts, 1))()
    ctx.check(lib().ruv_lscm_forward(ctx.h, ctypes.byref(batch), ctypes.byref(o), _ptr(uv, _f64), stats),
              "ruv_lscm_forward")
    return uv, [stats[i] for i in range(batch.n_charts)]


def lscm_backward(ctx: Context, dl_duv, opts: UnfoldOptions, n_charts: int):
    """Backward half (ruv_lscm_backward): dL/dp3 (n_verts, 3) of the last forward solve from
    dL/duv (n_verts, 2), pins held at their targets.  Returns (dL/dp3, adjoint-solve stats)."""
    g = np.ascontiguousarray(dl_duv, np.float64).reshape(-1, 2)
    dp = np.empty((g.shape[0], 3), np.float64)
    o = opts.to_c()
    stats = (RuvChartStat * max(n_charts, 1))()
    ctx.check(lib().ruv_lscm_backward(ctx.h, ctypes.byref(o), _ptr(g, _f64), _ptr(dp, _f64), stats),
              "ruv_lscm_backward")
    return dp, [stats[i] for i in range(n_charts)]


def distortion_loss(ctx: Context, uv, n_charts: int, grad: bool = True):
    """sum_t area_t (s1/s2 - 1)^2 per chart of the resident batch (ruv_distortion_loss).
    Returns (loss (n_charts,), dL/duv (n, 2) or None, dL/dp3 (n, 3) or None)."""
    u = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    loss = np.empty(max(n_charts, 1), np.float64)
    duv = np.empty_like(u) if grad else None
    dp = np.empty((u.shape[0], 3), np.float64) if grad else None
    ctx.check(lib().ruv_distortion_loss(ctx.h, _ptr(u, _f64), _ptr(loss, _f64), _ptr(duv, _f64), _ptr(dp, _f64)),
              "ruv_distortion_loss")
    return loss[:n_charts], duv, dp


def chart_distortion(ctx: Context, uv, n_charts: int) -> np.ndarray:
    """chart_distortion (metrics.rs:73-141) per chart of the resident batch: rows of
    [conformal mean, conformal max, area-ratio mean, flips, folds]."""
    u = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    out = np.empty((max(n_charts, 1), 5), np.float64)
    ctx.check(lib().ruv_chart_distortion(ctx.h, _ptr(u, _f64), _ptr(out, _f64)), "ruv_chart_distortion")
    return out[:n_charts]


def border_flags(charts: "Charts") -> np.ndarray:
    """One flag per packed vertex: the vertex is in its chart's border set (segment.rs)."""
    vo, bo = charts.i64("chart.vert_off"), charts.i64("chart.border_off")
    vid, bd = charts.i64("chart.vertex_ids"), charts.i64("chart.border")
    out = np.zeros(int(vo[-1]), np.uint8)
    for c in range(len(vo) - 1):
        ids = vid[vo[c]:vo[c + 1]]  # sorted source ids
        b = bd[bo[c]:bo[c + 1]]
        out[vo[c] + np.searchsorted(ids, b)] = 1
    return out


def rectangularize(ctx: Context, uv, border, n_charts: int):
    """rectangularize (metrics.rs:147-227) of every chart of the resident batch.  Returns
    (rectified UVs (n, 2), extents (n_charts, 2))."""
    u = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    b = np.ascontiguousarray(border, np.uint8).reshape(-1)
    q = np.empty_like(u)
    ext = np.empty((max(n_charts, 1), 2), np.float64)
    ctx.check(lib().ruv_rectangularize(ctx.h, _ptr(u, _f64), _ptr(b, _u8), _ptr(q, _f64), _ptr(ext, _f64)),
              "ruv_rectangularize")
    return q, ext[:n_charts]


def selftest_fp64(ctx: Context, mode: int, seed: int, n: int):
    """Bitwise comparison of the assembly's FP64 division / square root (integer and FP32
    pipes) with the hardware operations on n seeded inputs of class `mode` (0-5).  Returns
    (mismatches, (a, b, got, want) of the first)."""
    bad = _i64(0)
    first = np.zeros(4, np.float64)
    ctx.check(lib().ruv_selftest_fp64(ctx.h, int(mode), ctypes.c_uint64(seed), int(n), ctypes.byref(bad),
                                      _ptr(first, _f64)), "ruv_selftest_fp64")
    return bad.value, tuple(first)


def export_chart_system(ctx: Context, chart: int):
    """Interleaved CSR (Sparse::to_csr(2 nf), sparse.rs:69-84) + rhs of a chart of the last batch."""
    nf, nnz = _i64(0), _i64(0)
    ctx.check(lib().ruv_export_chart_system(ctx.h, chart, ctypes.byref(nf), ctypes.byref(nnz), None, None, None,
                                            None), "export")
    rp = np.empty(2 * nf.value + 1, np.int32)
    cols = np.empty(nnz.value, np.int32)
    vals = np.empty(nnz.value, np.float64)
    rhs = np.empty(2 * nf.value, np.float64)
    ctx.check(lib().ruv_export_chart_system(ctx.h, chart, ctypes.byref(nf), ctypes.byref(nnz), _ptr(rp, _i32),
                                            _ptr(cols, _i32), _ptr(vals, _f64), _ptr(rhs, _f64)), "export")
    return rp, cols, vals, rhs


def last_timings(ctx: Context):
    """Device ms of [assembly, batched PCG, driver, preconditioner set-up within PCG] of the
    last resident solve."""
    out = (_f64 * 4)()
    n = lib().ruv_last_timings(ctx.h, out, 4)
    return [out[i] for i in range(n)]


def bench_spmv(ctx: Context, precision: Precision = Precision.MIXED, reps: int = 20, n_buffers: int = 2):
    """(ms per launch, algorithmic bytes per launch, stream bytes per launch) of the batched SpMV
    on the last assembled batch: algorithmic bytes count 32-bit column indices, stream bytes
    the 16-bit ones the kernel reads where the operator has them."""
    ms, by, sb = _f64(0), _f64(0), _f64(0)
    ctx.check(lib().ruv_bench_spmv(ctx.h, int(precision), reps, n_buffers, ctypes.byref(ms), ctypes.byref(by),
                                   ctypes.byref(sb)), "ruv_bench_spmv")
    return ms.value, by.value, sb.value


def autotune(ctx: Context, precision: Precision = Precision.MIXED, reps: int = 10):
    """Pick the fastest SpMV launch shape and form on the last assembled batch; returns
    (lanes_per_row, rows_in_flight, tile_rows, ms of that SpMV plus the CG iteration's other
    tile kernels); the form: spmv_form(ctx)."""
    l, u, t, ms = _i32(0), _i32(0), _i32(0), _f64(0)
    ctx.check(lib().ruv_autotune(ctx.h, int(precision), reps, ctypes.byref(l), ctypes.byref(u), ctypes.byref(t),
                                 ctypes.byref(ms)), "ruv_autotune")
    return l.value, u.value, t.value, ms.value


def spmv_form(ctx: Context) -> int:
    """1 when this context's solves use the bulk-copy staged SpMV, 0 for the CSR-vector one."""
    b = _i32(0)
    ctx.check(lib().ruv_spmv_form(ctx.h, ctypes.byref(b)), "ruv_spmv_form")
    return b.value
