"""The allocation-free CG entry point (ruv_cg_solve_noalloc) against ruv_cg_solve.

ruv_cg_solve_noalloc exists for callers that cannot call cudaMalloc — host applications
that own all device memory through their own allocator or pool, or that must not trigger an
allocation mid-frame.  It takes device pointers and keeps its scratch in a fixed array
compiled into the library.  This file is collected last so that a run stopping at the first
failure has run every other test; it passes alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

import researchuv_gb300 as R

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-10  # FP64 CG vs FP64 CG: relative max-abs, as the other FP64 parity tests
MAX_ROWS = 262144  # RUV_NOALLOC_MAX_ROWS in include/ruv.h


def _lap1d(n):
    i = np.arange(n)
    rows = np.concatenate([i[1:], i, i[:-1]])
    cols = np.concatenate([i[1:] - 1, i, i[:-1] + 1])
    vals = np.concatenate([np.full(n - 1, -1.0), np.full(n, 2.0), np.full(n - 1, -1.0)])
    order = np.lexsort((cols, rows))
    rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))])
    b = np.zeros(n)
    b[0] = b[-1] = 1.0
    return R.CsrMatrix(vals[order], cols[order], rp), b


def _poisson(side):
    n = side * side
    r, c = np.divmod(np.arange(n), side)
    rows, cols, vals = [np.arange(n)], [np.arange(n)], [np.where(np.arange(n) % 11 == 0, 4.05, 4.0)]
    for dr, dc in [(-1, 0), (1, 0), (0, -1), (0, 1)]:
        ok = (r + dr >= 0) & (r + dr < side) & (c + dc >= 0) & (c + dc < side)
        rows.append(np.arange(n)[ok])
        cols.append(((r + dr) * side + (c + dc))[ok])
        vals.append(np.full(ok.sum(), -1.0))
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    order = np.lexsort((cols, rows))
    rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))])
    return R.CsrMatrix(vals[order], cols[order], rp), (np.arange(n) % 97) * 0.01 + 1.0


def _noalloc(a: R.CsrMatrix, b, max_iter, tol, pc, stream=None):
    """One call through the C ABI; returns (status, x, iters, message, free device bytes
    before the call, free device bytes after it)."""
    n = a.rows()
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(a.row_ptr).to(dev)
    d_c = torch.from_numpy(a.cols).to(dev)
    d_v = torch.from_numpy(a.vals).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(b, np.float64)).to(dev)
    d_x = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)  # poisoned output
    torch.cuda.synchronize()
    msg = ctypes.create_string_buffer(256)
    iters = ctypes.c_int64(-1)
    free_before = torch.cuda.mem_get_info(dev)[0]
    st = R.lib().ruv_cg_solve_noalloc(n, d_rp.data_ptr(), d_c.data_ptr(), d_v.data_ptr(), d_b.data_ptr(),
                                      d_x.data_ptr(), max_iter, tol, int(pc), ctypes.byref(iters),
                                      None if stream is None else stream.cuda_stream, msg, 256)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info(dev)[0]
    return st, d_x.cpu().numpy(), iters.value, msg.value.decode(), free_before, free_after


@pytest.mark.parametrize("case", ["lap1d_jacobi", "poisson_none", "lap1d_jacobi_stream"])
def test_noalloc_matches_cg_solve_on_two_calls(case):
    if case.startswith("lap1d_jacobi"):
        a, b = _lap1d(4096)
        pc, max_iter, tol = R.Precond.JACOBI, 20_000, 1e-12
    else:
        a, b = _poisson(400)
        pc, max_iter, tol = R.Precond.NONE, 100_000, 1e-10
    stream = torch.cuda.Stream() if case.endswith("_stream") else None
    ref = R.GpuSolver.new().cg_solve_precond(a, b, max_iter, tol, pc)
    assert ref is not None
    x_ref, it_ref = ref
    scale = max(1.0, np.abs(x_ref).max())
    for call in range(2):  # the shared scratch keeps the previous call's contents
        st, x, iters, msg, free_before, free_after = _noalloc(a, b, max_iter, tol, pc, stream)
        assert st == R.Status.OK, f"call {call}: {R.Status(st).name}: {msg}"
        assert np.abs(x - x_ref).max() <= TOL * scale, f"call {call}: differs from ruv_cg_solve"
        assert iters == it_ref
        if call == 1:  # warm: the module (and its scratch array) is loaded; nothing is allocated
            assert free_after == free_before, f"a warm call changed free device memory by {free_before - free_after} B"
    if case.startswith("lap1d_jacobi"):
        assert np.abs(x - 1.0).max() < 1e-8  # gpu/src/solver.rs:768-779 known answer


def test_noalloc_rejects_sizes_beyond_the_maximum():
    a, b = _lap1d(8)
    dev = torch.device("cuda", 0)
    d = torch.zeros(16, dtype=torch.float64, device=dev)
    msg = ctypes.create_string_buffer(256)
    st = R.lib().ruv_cg_solve_noalloc(MAX_ROWS + 1, d.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                      d.data_ptr(), 10, 1e-10, int(R.Precond.NONE), None, None, msg, 256)
    assert st == R.Status.BAD_INPUT
    assert "maximum" in msg.value.decode()
