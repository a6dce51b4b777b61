#!/usr/bin/env python
"""Benchmark of the batched LSCM solve (one JSON line on rank 0).

Workload (default): 4096 disk charts, triangle counts log-uniform in [50, 50 000] (seeded
synthetic meshes, researchuv_gb300/workloads.py), one chart per disk, Dirichlet border pins
(the reference's border-rectangle pass).  A step = one batched unfold of every chart: GPU
assembly of the cotangent systems with the pins eliminated, the smoothed-aggregation AMG
hierarchy set-up on the GPU (--precond amg: tentative prolongators instead), one batched
mixed-precision AMG-PCG over the packed block-diagonal operator to rel-res 1e-12 per chart
(double-float refinement), and the damped driver update.

* value  — unknowns/s (sum over charts of 2 * free vertices per step time), inputs resident
           in HBM (ruv_lscm_upload once), step time = device time of the three phases
           (CUDA events on the library's stream).  Inputs (~1 GB operator) exceed L2.
* e2e    — the same metric through ruv_lscm_solve_batch with host buffers (page-locked,
           ruv_host_alloc): H2D of the batch and D2H of the UVs inside the timed region
           (wall clock; the call is synchronous).
* roofline — the batched SpMV kernel (the dominant kernel) timed alone with CUDA events on
           the same operator: algorithmic bytes per launch / mean launch time vs the
           measured HBM copy bandwidth.
* cpu_baseline — the reference CPU algorithm (the oracle port of unfold_chart + the BTreeMap
           sparse LU) on a bounded size-stratified sample of the same charts, 1 core,
           extrapolated by chart to the whole workload; its UVs also give the UV error of the
           GPU result on those charts (plus FP64 SuperLU on the six largest charts).
* cpu_superlu_whole_workload — every chart through the oracle and FP64 SuperLU, all cores.

--impl reference runs that CPU port on all host cores for the whole workload (a per-chart
cost model calibrated on a stratified sample, the reference's par_map schedule; see
run_reference).  `config` holds only the keys that describe the workload and is the same in
both arms.

--workload hf1024 / hf2048 (the single-large-chart workloads) add the UV error of every chart
against FP64 SuperLU; --compare ic0_color,amg solves the resident workload once per named
preconditioner.  --workload sphere512 is the differentiation workload (gradient against the
CPU LU adjoint and FP64 central differences on 64 vertices of the full sphere).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "batched LSCM unknowns/s at <=1e-6 UV err vs FP64 LU"
UNIT = "unknowns/s"
L2_BYTES = 129 * 1024 * 1024
L2_NOTE = "inputs larger than L2 (operator and vectors of a step ~1 GB or more)"
# DRAM bytes (read + write) per algorithmic byte of the batched SpMV kernel, from one ncu
# capture of its first launch on the 1024-disk operator with the 16-bit column stream
# (198.6 MB of traffic for 256.9 MB of algorithmic bytes).
# The disk workloads scale by count, so the traffic of a launch on the 4096-disk operator is
# this ratio times its algorithmic bytes.
SPMV_DRAM_PER_ALG_BYTE = 0.773


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="disks4096",
                    help="disks<N> (N disk charts, the default 4096 is the headline), hf1024, hf2048, "
                         "sphere<L> (the differentiation workload on an L x 2L sphere; sphere512 at full size)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--precond", default="amg_sa", choices=["jacobi", "amg", "amg_sa", "none"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-single-chart", action="store_true")
    ap.add_argument("--single-chart-sample", type=int, default=192)
    ap.add_argument("--no-superlu-baseline", action="store_true",
                    help="skip the whole-workload FP64 SuperLU leg of the disks workloads")
    ap.add_argument("--compare", default="",
                    help="comma-separated preconditioners (ic0, ic0_color, amg, amg_sa, jacobi; amg+k2 / amg_sa+k2: "
                         "with the K-cycle on the top 2 levels) solved once each on the resident workload after the "
                         "timed steps, for iterations and time")
    ap.add_argument("--kcycle", type=int, default=0,
                    help="AMG levels in the K-form for the timed steps (0: V(1,1) cycle)")
    ap.add_argument("--ncu-step", action="store_true",
                    help="for profiler launch lists: upload, one warm-up solve, then one solve of the workload "
                         "(launch shape from RUV_LPR / RUV_UNROLL / RUV_TILE_ROWS); prints the kernel count "
                         "before the last solve to stderr and nothing else")
    ap.add_argument("--e2e-sweep", default="",
                    help="semicolon-separated settings of the one-call entry's copy knobs, each a comma-separated "
                         "list of NAME=VALUE environment variables (RUV_UPLOAD_PARTS, RUV_H2D_GRID, RUV_D2H_GRID, "
                         "RUV_H2D_KERNEL): the e2e call timed --steps times per setting after --warmup untimed "
                         "calls, one JSON line per setting, then the device-resident solve; nothing else runs")
    ap.add_argument("--no-autotune", action="store_true",
                    help="with --step-sweep: keep the context's SpMV shape (RUV_LPR / RUV_UNROLL / RUV_TILE_ROWS or "
                         "the default) instead of autotuning it first")
    ap.add_argument("--step-sweep", default="",
                    help="the same form of settings (any RUV_* variable the library reads per call): the "
                         "device-resident solve timed --steps times per setting after --warmup untimed solves, one "
                         "JSON line per setting (step, phases, CG iterations); nothing else runs")
    return ap.parse_args()


def sweep_settings(text):
    """The settings of --e2e-sweep / --step-sweep: settings separated by ';', each a
    comma-separated list of NAME=VALUE environment variables (values may hold '/', not ',')."""
    out = []
    for setting in text.split(";"):
        if not setting.strip():
            continue
        env = {}
        for kv in setting.split(","):
            if not kv.strip():
                continue
            if "=" not in kv:
                raise ValueError(f"sweep setting {kv!r} is not NAME=VALUE")
            k, v = kv.split("=", 1)
            env[k.strip()] = v.strip()
        out.append(env)
    return out


def step_sweep(args, local):
    """The device-resident solve under each setting of the library's environment variables:
    device time per step from the call's CUDA events (median, mean), its phases and the CG
    iterations, and whether the UVs equal those of the first setting."""
    import ctypes

    import researchuv_gb300 as R

    cfg, src = workload_config(args.workload)
    ctx = R.Context(local)
    prepare(src, ctx)
    charts, _ = prepare(src, ctx)
    L = R.lib()
    nv = int(charts.i64("chart.vert_off")[-1])
    prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
    pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA,
          "none": R.Precond.NONE}[args.precond]
    opts = R.UnfoldOptions(precision=prec, precond=pc)
    copts = opts.to_c()
    batch = charts.batch()
    stats = (R.RuvChartStat * max(batch.n_charts, 1))()
    for _ in range(2):
        R.solve_batch(ctx, batch, opts, nv)
    tuned = None if args.no_autotune else R.autotune(ctx, prec, reps=5)
    print(json.dumps({"spmv_shape_autotuned": list(tuned) if tuned else None,
                      "bulk_copy_staging": bool(R.spmv_form(ctx))}), flush=True)
    ctx.check(L.ruv_lscm_upload(ctx.h, ctypes.byref(batch)), "upload")
    uv = np.empty((nv, 2), np.float64)
    first = None
    for env in sweep_settings(args.step_sweep):
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        for _ in range(max(args.warmup, 1)):
            ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "warm-up")
        dev, ph = [], np.zeros(4)
        for _ in range(args.steps):
            ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")
            t = R.last_timings(ctx)
            dev.append(sum(t[:3]))
            ph += np.array(t)
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        ctx.check(L.ruv_lscm_download_uv(ctx.h, uv.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "download")
        if first is None:
            first = uv.copy()
        its = np.array([stats[c].cg_iters for c in range(batch.n_charts)])
        ph /= max(args.steps, 1)
        print(json.dumps({"setting": env, "step_ms_median": round(statistics.median(dev), 3),
                          "step_ms_mean": round(statistics.mean(dev), 3),
                          "phase_ms": {"assembly": round(ph[0], 3), "pcg": round(ph[1], 3), "driver": round(ph[2], 3),
                                       "precond_setup_in_pcg": round(ph[3], 3)},
                          "cg_iters_max": int(its.max()), "cg_iters_mean": round(float(its.mean()), 2),
                          "uv_max_abs_diff_to_first": float(np.abs(uv - first).max())}), flush=True)


def e2e_sweep(args, local):
    """The one-call entry on page-locked buffers under each setting of its copy knobs (read by
    the library on every call): wall time per call on the host, the call's device and assembly
    times from its CUDA events, and whether the UVs equal those of the first setting."""
    import ctypes

    import researchuv_gb300 as R

    cfg, src = workload_config(args.workload)
    ctx = R.Context(local)
    prepare(src, ctx)
    charts, _ = prepare(src, ctx)
    L = R.lib()
    nv = int(charts.i64("chart.vert_off")[-1])
    prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
    pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA,
          "none": R.Precond.NONE}[args.precond]
    opts = R.UnfoldOptions(precision=prec, precond=pc)
    copts = opts.to_c()
    batch = charts.batch()
    stats = (R.RuvChartStat * max(batch.n_charts, 1))()
    for _ in range(2):
        R.solve_batch(ctx, batch, opts, nv)
    R.autotune(ctx, prec, reps=5)
    pb, _keep = R.pinned_batch(ctx, charts)
    uv = R.pinned_empty(ctx, (nv, 2), np.float64)
    ptr = uv.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    first = None
    for env in sweep_settings(args.e2e_sweep):
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        for _ in range(max(args.warmup, 1)):
            ctx.check(L.ruv_lscm_solve_batch(ctx.h, ctypes.byref(pb), ctypes.byref(copts), ptr, stats), "warm-up")
        wall, dev, asm = [], [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            st = L.ruv_lscm_solve_batch(ctx.h, ctypes.byref(pb), ctypes.byref(copts), ptr, stats)
            wall.append(1000.0 * (time.perf_counter() - t0))
            ctx.check(st, "e2e")
            t = R.last_timings(ctx)
            dev.append(sum(t[:3]))
            asm.append(t[0])
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        if first is None:
            first = uv.copy()
        print(json.dumps({"setting": env, "wall_ms_mean": round(statistics.mean(wall), 2),
                          "wall_ms_median": round(statistics.median(wall), 2), "wall_ms_min": round(min(wall), 2),
                          "device_ms_median": round(statistics.median(dev), 2),
                          "assembly_ms_median": round(statistics.median(asm), 2),
                          "uv_equal_to_first": bool(np.array_equal(first, uv))}), flush=True)
    ctx.check(L.ruv_lscm_upload(ctx.h, ctypes.byref(batch)), "upload")
    dev, asm = [], []
    for _ in range(args.steps):
        ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")
        t = R.last_timings(ctx)
        dev.append(sum(t[:3]))
        asm.append(t[0])
    print(json.dumps({"resident_device_ms_median": round(statistics.median(dev), 2),
                      "resident_assembly_ms_median": round(statistics.median(asm), 2)}), flush=True)


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as tdist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo", rank=rank, world_size=world)
        pg = tdist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def workload_config(name):
    """Generate a workload (numpy only, no library call) and its config: the keys that
    describe the workload, identical in both arms.  Returns (cfg, src)."""
    from researchuv_gb300 import workloads as W

    if name.startswith("disks"):
        n = int(name[5:])
        vo, to, p3, tr = W.disks(n, 50, 50_000, seed=3)
        cfg = {"workload": f"{n} displaced polar-disk charts, triangles log-uniform [50, 50000], seed 3",
               "charts": n, "triangles": int(to[-1]), "vertices": int(vo[-1]),
               "unknowns": W.disk_unknowns(vo, to, tr), "l2": L2_NOTE}
        return cfg, ("patches", vo, to, p3, tr)
    n, ns, amp = (1024, 8, 0.15) if name == "hf1024" else (2048, 16, 0.3)
    p, f = W.height_field(n, ns, amp, seed=2)
    cfg = {"workload": f"{n}x{n} height field, {ns} sines, amplitude {amp}, seed 2",
           "triangles": int(f.shape[0]), "vertices": int(p.shape[0]), "l2": L2_NOTE}
    return cfg, ("mesh", p, f)


def prepare(src, ctx=None):
    """The chart stages (weld + segment + frames + pins), timed; with a context their
    data-parallel parts run on its device (the same charts bit for bit)."""
    import researchuv_gb300 as R

    t0 = time.time()
    if src[0] == "patches":
        charts = R.prepare_patches(*src[1:], ctx=ctx)
    else:
        charts = R.prepare_mesh(*src[1:], ctx=ctx)
    return charts, round(time.time() - t0, 3)


def host_info():
    """nproc, uname -m and the CPU model of the host the CPU legs run on."""
    import platform

    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"nproc": os.cpu_count(), "uname_m": platform.machine(), "cpu_model": model or "unknown"}


class Clocks:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU (oracle) legs
def _oracle_chart(args):
    """One chart through the reference CPU algorithm (oracle port): weld(0) + segment +
    unfold_chart with the BTreeMap LU.  Returns (uv, unknowns, seconds, charts found)."""
    p, f = args
    from oracle import oracle as O

    t0 = time.perf_counter()
    P = O.Pipeline(p, f, weld_tol=0.0, lu_limit=1 << 40)
    dt = time.perf_counter() - t0
    ch = P.chart(0)
    return ch.get("uv"), 2 * int((ch["free_pos"] >= 0).sum()), dt, P.n_charts


def _oracle_chart_timed(args):
    """(chart id, seconds) of one chart through the reference CPU algorithm."""
    c, p, f = args
    _, _, dt, _ = _oracle_chart((p, f))
    return c, dt


def _superlu_chart(args):
    """One chart through the oracle's chart stages and the FP64 SuperLU direct solve (the
    practical CPU direct solve): (chart id, unknowns, seconds, UVs)."""
    c, p, f = args
    from oracle import oracle as O

    t0 = time.perf_counter()
    P = O.Pipeline(p, f, weld_tol=0.0, lu_limit=0)
    uv = P.superlu_uv(0) if P.n_charts == 1 else None
    dt = time.perf_counter() - t0
    return c, 2 * int((P.chart(0)["free_pos"] >= 0).sum()), dt, uv


def parmap_wall(t, workers):
    """Wall time of core::exec::par_map (core/src/exec.rs:28-60) over items costing t, in
    order: contiguous chunks of ceil(n / workers) items, one per worker thread."""
    t = np.asarray(t, np.float64)
    if workers <= 1 or len(t) <= 1:
        return float(t.sum())
    workers = min(workers, len(t))
    chunk = -(-len(t) // workers)
    return float(max(t[i:i + chunk].sum() for i in range(0, len(t), chunk)))


def stratified_charts(nv, cap, per_stratum=2, strata=24, seed=13):
    """Chart ids of a sample stratified by size: `strata` log-spaced vertex-count bins over the
    whole range, up to `per_stratum` seeded picks from each bin, charts above `cap` vertices
    left out (the reference LU is Theta(n^2) per chart)."""
    nv = np.asarray(nv)
    edges = np.geomspace(nv.min(), nv.max() + 1, strata + 1)
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for s in range(strata):
        idx = np.nonzero((nv >= edges[s]) & (nv < edges[s + 1]) & (nv <= cap))[0]
        if len(idx):
            out.extend(int(i) for i in rng.choice(idx, min(per_stratum, len(idx)), replace=False))
    return sorted(out, key=lambda c: nv[c])


class ChartCostModel:
    """Seconds of the reference CPU algorithm per chart, from timed charts of a stratified
    sample: each chart costs its nearest timed chart's time (in log vertex count) scaled by
    (nv / nv_timed)^beta, beta fitted over the timed charts of at least 400 vertices.  Charts
    larger than the largest timed one scale from the mean of the four largest timed charts
    with the exponent min(beta, 2): the reference LU's triangular solves are Theta(n^2), and
    a fit over small charts can be steeper than the large charts' growth (measured on one
    host: 6k -> 12k vertices grew as n^1.84), so the cap keeps the extrapolation in the CPU's
    favour."""

    def __init__(self, nv_timed, t_timed):
        self.nv = np.asarray(nv_timed, np.float64)
        self.t = np.asarray(t_timed, np.float64)
        big = self.nv >= 400
        if big.sum() >= 3:
            self.beta = float(np.polyfit(np.log(self.nv[big]), np.log(self.t[big]), 1)[0])
        else:
            self.beta = 2.0
        order = np.argsort(self.nv)
        self.nv, self.t = self.nv[order], self.t[order]

    def __call__(self, nv):
        nv = np.asarray(nv, np.float64)
        ln, lt = np.log(self.nv), np.log(nv)
        near = np.abs(lt[:, None] - ln[None, :]).argmin(1)
        est = self.t[near] * (nv / self.nv[near]) ** self.beta
        top = slice(max(0, len(self.nv) - 4), len(self.nv))
        beyond = nv > self.nv[-1]
        if beyond.any():
            b = min(self.beta, 2.0)
            est[beyond] = np.mean(self.t[top][None, :] * (nv[beyond][:, None] / self.nv[top][None, :]) ** b, 1)
        return est


def _time_charts(pool, src, ids):
    _, vo, to, p3, tr = src
    tasks = [(int(c), p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]]) for c in sorted(ids, key=lambda c: -(vo[c + 1] - vo[c]))]
    out = dict(pool.imap_unordered(_oracle_chart_timed, tasks, chunksize=1))
    return np.array([out[c] for c in ids])


def reference_model(src, cores, cap):
    """Calibrate the per-chart cost model on `cores` processes: a stratified sample of charts
    up to `cap` vertices, each timed once through the reference CPU algorithm."""
    import multiprocessing as mp

    _, vo, to, _, _ = src
    nv = np.diff(vo)
    ids = stratified_charts(nv, cap)
    with mp.get_context("spawn").Pool(cores) as pool:
        t0 = time.perf_counter()
        t = _time_charts(pool, src, ids)
        wall = time.perf_counter() - t0
    return ChartCostModel(nv[ids], t), ids, t, wall


def cpu_baseline(src, uv_gpu, budget_s, unknowns):
    """1-core baseline: the reference CPU algorithm (oracle port) timed on a stratified sample
    of charts of at most 1500 vertices (a bounded ~10-30 s of work), extrapolated by chart over
    the whole workload with the fitted per-chart cost model; its UVs also give the GPU
    result's error on those charts, plus FP64 SuperLU on the six largest charts."""
    from oracle import oracle as O

    _, vo, to, p3, tr = src
    nv = np.diff(vo)
    ids = stratified_charts(nv, 1500, per_stratum=3)
    t_used, errs, used, ts = 0.0, [], [], []
    for c in ids:
        if t_used > budget_s:
            break
        uv, _, dt, nch = _oracle_chart((p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]]))
        t_used += dt
        used.append(c)
        ts.append(dt)
        if uv is not None and nch == 1:
            errs.append(O.uv_error(uv_gpu[vo[c]:vo[c + 1]], uv))
    model = ChartCostModel(nv[used], ts)
    total = float(model(nv).sum())
    big = np.argsort(-nv)[:6]
    for c in big:
        P = O.Pipeline(p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]], weld_tol=0.0, lu_limit=0)
        if P.n_charts == 1:
            errs.append(O.uv_error(uv_gpu[vo[c]:vo[c + 1]], P.superlu_uv(0)))
    return {"value": unknowns / total, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{len(used)} charts of <= 1500 vertices, stratified by size over the whole range, "
                      f"{t_used:.1f} s on 1 core (weld + segment + unfold_chart + BTreeMap LU per chart); "
                      f"extrapolated by chart to all {len(nv)} charts ({total:.0f} s) with a per-chart cost "
                      f"~ nv^{model.beta:.2f}",
            "host": host_info()}, (max(errs) if errs else None), len(errs)


def superlu_baseline(src, cores):
    """The practical FP64 CPU direct solve over the WHOLE workload: every chart through the
    oracle's chart stages and SuperLU (scipy splu, COLAMD) on the scalar Laplacian with the u
    and v right-hand sides, one process per core."""
    import multiprocessing as mp

    _, vo, to, p3, tr = src
    n = len(vo) - 1
    order = np.argsort(-np.diff(vo))
    tasks = [(int(c), p3[vo[c]:vo[c + 1]], tr[to[c]:to[c + 1]]) for c in order]
    with mp.get_context("spawn").Pool(cores) as pool:
        t0 = time.perf_counter()
        res = list(pool.imap_unordered(_superlu_chart, tasks, chunksize=4))
        wall = time.perf_counter() - t0
    unk = sum(r[1] for r in res)
    cpu_s = sum(r[2] for r in res)
    return {"value": unk / wall, "unit": UNIT, "cores": cores, "wall_s": round(wall, 2),
            "cpu_s_sum": round(cpu_s, 2), "single_core_value": unk / cpu_s, "charts": n,
            "what": "every chart: oracle chart stages + FP64 SuperLU (scipy splu, COLAMD) on the scalar Laplacian, "
                    "2 right-hand sides; process pool over charts, largest first"}


def run_reference(args, rank):
    """Reference arm: the reference CPU algorithm (oracle port of weld + segment +
    unfold_chart with the BTreeMap LU) over the whole workload on all host cores, as the
    reference's par_map runs it (pipeline.rs:192-194).  The Theta(n^2) LU of the largest
    charts runs for many minutes each, so a run calibrates a per-chart cost model once (a
    stratified sample up to 4000 vertices, timed on all cores); each step then times a
    bounded stratified sample again and scales the model's whole-workload par_map wall time
    by the ratio of measured to modelled time on that sample.  No GPU and no part of this
    repository's library is used."""
    if rank != 0:
        return
    import multiprocessing as mp

    cfg, src = workload_config(args.workload)
    if src[0] != "patches":
        print(json.dumps({"impl": "reference", "metric": METRIC, "value": None, "unit": UNIT,
                          "unavailable": "the reference LU is Theta(n^2) per chart: a single 1M-vertex chart is "
                                         "infeasible (extrapolated days); run the disks workload"}))
        return
    _, vo, to, p3, tr = src
    nv = np.diff(vo)
    cores = os.cpu_count() or 1
    model, cal_ids, cal_t, cal_wall = reference_model(src, cores, cap=4000)
    t_model = model(nv)
    wall_model = parmap_wall(t_model, cores)
    # the per-step sample: calibration charts in ascending size while the sample's modelled
    # work stays within ~6 s on all cores and no chart exceeds ~4 s
    step_ids = []
    acc = 0.0
    for c in cal_ids:
        tc = float(model(np.array([nv[c]]))[0])
        if tc > 4.0 or (acc + tc) / cores > 6.0:
            break
        step_ids.append(c)
        acc += tc
    step_pred = float(model(nv[step_ids]).sum())
    with mp.get_context("spawn").Pool(cores) as pool:
        for _ in range(args.warmup):
            _time_charts(pool, src, step_ids)
        walls, extrap = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ts = _time_charts(pool, src, step_ids)
            walls.append(time.perf_counter() - t0)
            extrap.append(wall_model * float(ts.sum()) / step_pred)
    unknowns = cfg["unknowns"]
    whole_s = statistics.mean(extrap)
    value = unknowns / whole_s
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(walls), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"whole workload ({len(nv)} charts, {unknowns} unknowns) by chart: "
                                       f"per-chart cost model calibrated on {len(cal_ids)} size-stratified charts "
                                       f"up to 4000 vertices ({cal_wall:.0f} s on {cores} cores, cost ~ nv^"
                                       f"{model.beta:.2f}); each step times {len(step_ids)} of them again and scales "
                                       "the modelled whole-workload wall time by measured / modelled",
                             "host": host_info()},
            "value_from": "unknowns of the whole workload / its extrapolated wall time under the reference's par_map "
                          "(contiguous chunks, one per core, core/src/exec.rs:28-60); ms_per_step is the wall time of "
                          "each step's timed sample",
            "extrapolated_s_per_workload": whole_s,
            "modelled_cpu_s_per_workload": float(t_model.sum()),
            "calibration": {"charts": len(cal_ids), "max_vertices": int(nv[cal_ids].max()),
                            "max_chart_s": float(cal_t.max()), "beta": model.beta,
                            "largest_chart_vertices": int(nv.max()),
                            "largest_chart_modelled_s": float(model(np.array([nv.max()]))[0])},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def single_chart_baseline(ctx, vo, unknowns, batched_ms, n_sample, precond_name="JACOBI"):
    """The measuring stick of the batched solve: plain single-chart FP64 GPU PCG, i.e. one
    GpuSolver::cg_solve_precond call (FP64, tol 1e-12; Jacobi is the reference's default,
    lscm.rs:492-501, IC(0) its strongest single-level preconditioner) per chart on that
    chart's interleaved CSR, sequentially, as the reference's per-chart unfold would.  Timed
    on a size-stratified sample of charts and scaled to the whole workload by unknowns
    (larger charts need more iterations per unknown, so the scaling understates the full
    sequential time)."""
    import researchuv_gb300 as R

    pc = getattr(R.Precond, precond_name)

    sizes = np.diff(vo)
    order = np.argsort(sizes)
    idx = order[np.linspace(0, len(order) - 1, min(n_sample, len(order))).astype(int)]
    systems = []
    for c in idx:
        rp, cols, vals, rhs = R.export_chart_system(ctx, int(c))
        if len(rp) > 1:
            systems.append((R.CsrMatrix(vals, cols, rp), rhs))
    solver = R.GpuSolver.new()
    for a, rhs in systems[:4]:  # warm-up
        solver.cg_solve_precond(a, rhs, 16384, 1e-12, pc)
    t0 = time.perf_counter()
    unk, iters, fails = 0, 0, 0
    for a, rhs in systems:
        r = solver.cg_solve_precond(a, rhs, 16384, 1e-12, pc)
        unk += a.rows()
        if r is None:
            fails += 1
        else:
            iters += r[1]
    dt = time.perf_counter() - t0
    full_ms = 1000.0 * dt * unknowns / max(unk, 1)
    return {"ms_per_step_extrapolated": full_ms, "sample_charts": len(systems), "sample_unknowns": unk,
            "sample_s": round(dt, 3), "sample_iters": iters, "failed": fails,
            "batched_speedup": full_ms / batched_ms,
            "what": f"sequential ruv_cg_solve per chart (FP64 {precond_name.lower()} PCG, host CSR in / x out), "
                    "size-stratified sample scaled by unknowns"}


def field_parity(src, uv_gpu, charts):
    """UV error of the GPU result on EVERY chart of a height field against the FP64 sparse-LU
    oracle (oracle chart stages, SuperLU on the scalar Laplacian with both right-hand sides,
    the reference's damped driver), normalised as unwrap/src/lscm.rs:749-758; the oracle's
    time is the practical 1-core FP64 direct solve of the same workload."""
    from oracle import oracle as O

    _, p, f = src
    t0 = time.perf_counter()
    P = O.Pipeline(p, f, lu_limit=0)
    t_prep = time.perf_counter() - t0
    vo = charts.i64("chart.vert_off")
    assert P.n_charts == len(vo) - 1, (P.n_charts, len(vo) - 1)
    worst, worst_chart, checked, unk, t_lu = 0.0, -1, 0, 0, 0.0
    for c in range(P.n_charts):
        ch = P.chart(c)
        nf = int((ch["free_pos"] >= 0).sum())
        t1 = time.perf_counter()
        uv_lu = P.superlu_uv(c)
        t_lu += time.perf_counter() - t1
        unk += 2 * nf
        err = O.uv_error(uv_gpu[vo[c]:vo[c + 1]], uv_lu)
        checked += 1
        if err > worst:
            worst, worst_chart = err, c
    return {"uv_err_max_vs_lu": worst, "uv_err_charts_checked": checked,
            "uv_err_worst_chart": {"chart": worst_chart, "vertices": int(vo[worst_chart + 1] - vo[worst_chart])},
            "cpu_direct": {"value": unk / (t_prep + t_lu), "unit": UNIT, "cores": 1, "kind": "port",
                           "oracle_prep_s": round(t_prep, 2), "superlu_s": round(t_lu, 2), "host": host_info(),
                           "what": "whole workload, 1 core: oracle weld + segment + assembly, then FP64 SuperLU "
                                   "(scipy splu, COLAMD) per chart with 2 right-hand sides and the damped driver"}}


def compare_preconds(ctx, args, stats, names):
    """One solve of the resident workload per preconditioner: device time of the phases and
    CG iterations (the AMG-against-IC(0) comparison of the large-chart workload)."""
    import ctypes

    import researchuv_gb300 as R

    L = R.lib()
    prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
    out = {}
    for name in names:
        base, _, kc = name.partition("+k")  # "amg_sa+k2": the K-cycle on the top 2 levels
        pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA, "ic0": R.Precond.IC0,
              "ic0_color": R.Precond.IC0_COLOR}[base]
        copts = R.UnfoldOptions(precision=prec, precond=pc).to_c()
        old_k = os.environ.get("RUV_AMG_KCYCLE")
        if kc:
            os.environ["RUV_AMG_KCYCLE"] = kc
        st = L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats)
        if kc:
            if old_k is None:
                del os.environ["RUV_AMG_KCYCLE"]
            else:
                os.environ["RUV_AMG_KCYCLE"] = old_k
        t = R.last_timings(ctx)
        it = [stats[i].cg_iters for i in range(len(stats))]
        out[name] = {"status": R.Status(st).name, "ms": round(sum(t[:3]), 3), "pcg_ms": round(t[1], 3),
                     "setup_ms": round(t[3], 3), "cg_iters_max": int(max(it)),
                     # the iterations of the slowest chart set the batch's pace
                     "ms_per_iteration": round((t[1] - t[3]) / max(max(it), 1), 4),
                     "charts_not_ok": int(sum(1 for i in range(len(stats)) if stats[i].status != 0))}
    return out


def single_chart_reference(ctx, vo, unknowns, batched_ms, n_sample):
    """The measuring stick of the >= 5x target as the reference builds it: its own CG kernels
    (gpu/src/kernels.cu, compute_80 PTX JIT-loaded) under the oracle's restatement of its host
    loop (gpu/src/solver.rs:284-565: per-call uploads, a host-summed dot product after every
    kernel that needs one), FP64 Jacobi PCG (the reference's default, lscm.rs:492-501), tol
    1e-12, 16384 iterations, one chart after another on its interleaved CSR.  Timed on the
    size-stratified sample of single_chart_baseline, scaled to the workload by unknowns."""
    import researchuv_gb300 as R
    from oracle import oracle as O

    try:
        ref = O.RefGpuCG()
    except Exception as e:  # no PTX (built only where the reference's source is present)
        return {"unavailable": str(e)}
    sizes = np.diff(vo)
    order = np.argsort(sizes)
    idx = order[np.linspace(0, len(order) - 1, min(n_sample, len(order))).astype(int)]
    systems = []
    for c in idx:
        rp, cols, vals, rhs = R.export_chart_system(ctx, int(c))
        if len(rp) > 1:
            systems.append((rp, cols, vals, rhs))
    for rp, cols, vals, rhs in systems[:4]:  # warm-up (module JIT, first allocations)
        ref.solve(rp, cols, vals, rhs, 16384, 1e-12, jacobi=True)
    t0 = time.perf_counter()
    unk, iters, fails = 0, 0, 0
    for rp, cols, vals, rhs in systems:
        r = ref.solve(rp, cols, vals, rhs, 16384, 1e-12, jacobi=True)
        unk += len(rp) - 1
        if r is None:
            fails += 1
        else:
            iters += r[1]
    dt = time.perf_counter() - t0
    full_ms = 1000.0 * dt * unknowns / max(unk, 1)
    return {"ms_per_step_extrapolated": full_ms, "sample_charts": len(systems), "sample_unknowns": unk,
            "sample_s": round(dt, 3), "sample_iters": iters, "failed": fails, "batched_speedup": full_ms / batched_ms,
            "what": "the reference's CG kernels (kernels.cu, compute_80 PTX) under the restated host loop of "
                    "solver.rs:284-565, FP64 Jacobi PCG per chart, size-stratified sample scaled by unknowns"}


FD_STEPS = (1e-6, 1e-7, 1e-8, 1e-9)
FD_EDGE_SCALE = None  # (a cap of h at a multiple of the vertex's shortest edge: off)
FD_REFINE = 0  # refinement steps of each perturbed solve (two changed nothing on the full-size sphere)


def _fd_worker(args):
    from oracle import oracle as O

    p3, tris, pinned, pin_uv, lam, target, picks = args
    return O.fd_gradient(p3, tris, pinned, pin_uv, lam, target, picks, reuse_base=True, smooth_steps=FD_STEPS,
                         edge_scale=FD_EDGE_SCALE, refine=FD_REFINE)


def fd_parallel(p3, tris, pinned, pin_uv, lam, target, picks, workers):
    """oracle.fd_gradient over `picks` split across `workers` spawned processes (each factors
    the unperturbed system once): (values, h used per pick -- the largest of FD_STEPS at which
    the perturbation moves no clamp of the assembly around the vertex)."""
    import multiprocessing as mp

    chunks = [picks[i::workers] for i in range(workers)]
    with mp.get_context("spawn").Pool(workers) as pool:
        parts = pool.map(_fd_worker, [(p3, tris, pinned, pin_uv, lam, target, c) for c in chunks if c])
    out = {}
    for c, (vals, hs) in zip([c for c in chunks if c], parts):
        for pk, v, hv in zip(c, vals, hs):
            out[pk] = (v, hv)
    return np.array([out[pk][0] for pk in picks]), np.array([out[pk][1] for pk in picks])


# ------------------------------------------------------------------ GPU arm
def run_adjoint(args, rank, world, local, pg):
    """Differentiation workload: an n_lat x 2 n_lat spherical-harmonic sphere cut into one disk
    chart; a step = forward solve + distortion loss with gradients + backward (adjoint solve
    and the assembly's reverse pass) through the host-buffer API, giving d(loss)/d(positions)
    for loss = sum_t area_t (s1/s2 - 1)^2 + lam |uv - target|^2.  Checks the gradient
    against the CPU LU adjoint and against FP64 central differences (h = 1e-6, or smaller where
    +-1e-6 would move a clamp of the assembly) on 64 random vertices, both on the full-size
    sphere."""
    import researchuv_gb300 as R
    from oracle import oracle as O
    from researchuv_gb300 import workloads as W

    n_lat = int(args.workload[6:])
    t0 = time.time()
    p, f = W.sh_sphere(n_lat, 2 * n_lat, seed=4)
    charts = R.prepare_patches(np.array([0, len(p)]), np.array([0, len(f)]), p, f)
    ch = charts.chart(0)
    prep = time.time() - t0
    n = len(p)
    rng = np.random.Generator(np.random.PCG64(11))
    target = ch["p2"] + 0.01 * rng.standard_normal(ch["p2"].shape)
    lam = 1.0 / n
    ctx = R.Context(local)
    prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
    pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA,
          "none": R.Precond.NONE}[args.precond]
    opts = R.UnfoldOptions(precision=prec, precond=pc)
    batch = charts.batch()

    def step():
        uv, st = R.lscm_forward(ctx, batch, opts, n)
        loss, duv, dp_dist = R.distortion_loss(ctx, uv, 1)
        dp_solve, st_b = R.lscm_backward(ctx, duv + 2.0 * lam * (uv - target), opts, 1)
        total = float(loss[0]) + lam * float(((uv - target) ** 2).sum())
        return dp_dist + dp_solve, total, st[0], st_b[0]

    for _ in range(max(args.warmup, 1)):
        grad, total, st_f, st_b = step()
    L = R.lib()
    l0 = L.ruv_kernel_launches(ctx.h)
    clk = Clocks(local)
    barrier(pg)
    clk.start()
    times = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        grad, total, st_f, st_b = step()
        times.append(1000.0 * (time.perf_counter() - t1))
    barrier(pg)
    clock_info = clk.stop()
    launches = (L.ruv_kernel_launches(ctx.h) - l0) // max(args.steps, 1)
    ms = allmax(pg, statistics.mean(times))
    unknowns = int(2 * st_f.n_free)
    line = {
        "metric": "LSCM adjoint d(loss)/d(positions): unknowns/s (forward + loss + backward)",
        "value": world * unknowns / (ms / 1000.0), "unit": "unknowns/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 loss/adjoint, " + args.precision + " solves",
        "data": "synthetic",
        "config": {"workload": f"{n_lat}x{2 * n_lat} sphere, radius 1 + 0.05 * 8 seeded real harmonics "
                               f"(degree <= 6), cut at one meridian and both poles, seed 4",
                   "vertices": n, "triangles": int(len(f)), "unknowns": unknowns, "host_prep_s": round(prep, 3),
                   "precond": args.precond, "precision": args.precision, "lam": lam,
                   "forward_cg_iters": int(st_f.cg_iters), "adjoint_cg_iters": int(st_b.cg_iters),
                   "timing": "wall clock of the host-buffer calls (H2D/D2H inside)"},
        "e2e": {"value": world * unknowns / (ms / 1000.0), "unit": "unknowns/s",
                "h2d_bytes_per_step": int(8 * (3 * n + 2 * n + 2 * n + 2 * n) + 12 * len(f) + n),
                "d2h_bytes_per_step": int(8 * (2 * n + 2 * n + 3 * n + 3 * n)), "ms_per_step": ms},
        "gpu_launches": int(launches), "clocks": clock_info, "loss": total,
    }
    if rank == 0 and not args.no_cpu_baseline:
        t1 = time.time()
        ref, _ = O.lu_adjoint_gradient(p, ch["tris"], ch["pinned"].astype(np.int64), ch["pin_uv"], lam, target)
        cpu_s = time.time() - t1
        line["cpu_baseline"] = {"value": unknowns / cpu_s, "unit": "unknowns/s", "cores": 1, "kind": "port",
                                "sample": "the whole workload once: oracle fixed-pin assembly, SuperLU factor, "
                                          "forward + adjoint solves, reverse pass (FP64)"}
        line["grad_rel_err_vs_lu_adjoint"] = float(np.linalg.norm(grad - ref) / np.linalg.norm(ref))
        # central differences on 64 random vertices of the same sphere, 3 coordinates each
        picks = [(int(v), k) for v in np.random.Generator(np.random.PCG64(5)).choice(n, 64, replace=False)
                 for k in range(3)]
        t1 = time.time()
        fd, fd_h = fd_parallel(p, ch["tris"], ch["pinned"].astype(np.int64), ch["pin_uv"], lam, target, picks,
                               min(os.cpu_count() or 1, 16))
        ad = np.array([grad[v, k] for v, k in picks])
        ok = np.isfinite(fd)
        a_, f_ = ad[ok], fd[ok]
        e_ = np.abs(a_ - f_)
        floor = 1e-3 * np.abs(f_).max() if ok.any() else 0.0
        line["fd_check"] = {
            "instance": f"the {n_lat}x{2 * n_lat} sphere itself", "picks": len(picks),
            "what": "FP64 central differences of the loss through the fixed-pin SuperLU solve (perturbed systems "
                    "by a low-rank update of the unperturbed factors)",
            "h": "per pick, the largest of 1e-6, 1e-7, 1e-8, 1e-9 at which neither +h nor -h moves a clamp of "
                 "the assembly around the vertex (a corner cotangent's clamp at 0, an edge weight's drop "
                 "threshold): the loss is piecewise smooth, and a quotient across a kink averages two one-sided "
                 "derivatives",
            "h_counts": {"1e-6": int((fd_h == 1e-6).sum()), "below 1e-6": int((fd_h < 1e-6).sum())},
            "h_min": float(np.nanmin(fd_h)) if np.isfinite(fd_h).any() else None,
            "picks_without_smooth_h": int((~ok).sum()),
            "components": int(ok.sum()),
            "rel_err_norm": float(np.linalg.norm(a_ - f_) / np.linalg.norm(f_)) if ok.any() else None,
            "per_component_rel_err_max": float((e_ / np.maximum(np.abs(f_), floor)).max()) if ok.any() else None,
            "per_component_floor": "|fd| floored at 1e-3 max|fd|",
            "components_below_floor": int((np.abs(f_) < floor).sum()),
            "cpu_s": round(time.time() - t1, 1)}
        # the same split by the vertex's shortest incident edge: next to the poles (edges down to
        # ~2e-5) no step gives a clean quotient -- h = 1e-6 is 5% of an edge (truncation), and the
        # smaller steps that avoid the clamps leave differences of entries ~1e9 (rounding)
        tri = np.asarray(ch["tris"], np.int64)
        emin = np.full(n, np.inf)
        for a, b in ((0, 1), (1, 2), (2, 0)):
            el = np.linalg.norm(p[tri[:, a]] - p[tri[:, b]], axis=1)
            np.minimum.at(emin, tri[:, a], el)
            np.minimum.at(emin, tri[:, b], el)
        far = np.array([emin[v] >= 1e-3 for v, _ in picks]) & ok
        if far.any():
            a2, f2 = ad[far], fd[far]
            fl2 = 1e-3 * np.abs(f2).max()
            line["fd_check"]["away_from_poles"] = {
                "criterion": "shortest incident edge >= 1e-3 (h <= 1e-3 x the edge)", "components": int(far.sum()),
                "rel_err_norm": float(np.linalg.norm(a2 - f2) / np.linalg.norm(f2)),
                "per_component_rel_err_max": float((np.abs(a2 - f2) / np.maximum(np.abs(f2), fl2)).max())}
            line["fd_check"]["next_to_poles_vertices"] = sorted({int(v) for (v, _), r in zip(picks, far) if not r})
    if rank == 0:
        print(json.dumps(line))
    barrier(pg)


def main():
    args = parse()
    if args.kcycle > 0:
        os.environ["RUV_AMG_KCYCLE"] = str(args.kcycle)
    rank, world, local, pg = dist()
    if args.impl == "reference":
        run_reference(args, rank)
        barrier(pg)
        return
    if args.workload.startswith("sphere"):
        run_adjoint(args, rank, world, local, pg)
        return
    if args.e2e_sweep:
        e2e_sweep(args, local)
        return
    if args.step_sweep:
        step_sweep(args, local)
        return
    if args.ncu_step:
        import ctypes

        import researchuv_gb300 as R

        charts, _ = prepare(workload_config(args.workload)[1])
        ctx = R.Context(local)
        L = R.lib()
        pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA,
              "none": R.Precond.NONE}[args.precond]
        prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
        copts = R.UnfoldOptions(precision=prec, precond=pc).to_c()
        batch = charts.batch()
        stats = (R.RuvChartStat * max(batch.n_charts, 1))()
        ctx.check(L.ruv_lscm_upload(ctx.h, ctypes.byref(batch)), "upload")
        ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")
        sys.stderr.write(f"kernels before the profiled solve: {L.ruv_kernel_launches(ctx.h)}\n")
        ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")
        sys.stderr.write(f"kernels after the profiled solve: {L.ruv_kernel_launches(ctx.h)}\n")
        return
    import ctypes

    import researchuv_gb300 as R

    cfg, src = workload_config(args.workload)
    ctx = R.Context(local)
    prepare(src, ctx)  # warm (the first device preparation allocates its workspace)
    charts, prep_s = prepare(src, ctx)
    L = R.lib()
    batch = charts.batch()
    vo = charts.i64("chart.vert_off")
    nv = int(vo[-1])
    prec = R.Precision.MIXED if args.precision == "mixed" else R.Precision.FP64
    pc = {"jacobi": R.Precond.JACOBI, "amg": R.Precond.AMG, "amg_sa": R.Precond.AMG_SA,
          "none": R.Precond.NONE}[args.precond]
    opts = R.UnfoldOptions(precision=prec, precond=pc)
    copts = opts.to_c()
    stats = (R.RuvChartStat * max(batch.n_charts, 1))()

    # warm-up (also the first e2e solve: allocates the workspace)
    for _ in range(max(args.warmup, 1)):
        uv, st, status = R.solve_batch(ctx, batch, opts, nv)
    n_free = np.array([s.n_free for s in st])
    unknowns = int(2 * n_free.sum())
    if "unknowns" in cfg:
        assert unknowns == cfg["unknowns"], (unknowns, cfg["unknowns"])
    else:
        cfg = {**cfg, "charts": int(batch.n_charts), "unknowns": unknowns}
    statuses = np.array([s.status for s in st])
    cg_iters = np.array([s.cg_iters for s in st])

    # launch-shape autotuning on the assembled operator (outside the timed region)
    tuned = R.autotune(ctx, prec, reps=5)

    # device-resident timed region
    ctx.check(L.ruv_lscm_upload(ctx.h, ctypes.byref(batch)), "upload")
    ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")  # warm
    clk = Clocks(local)
    barrier(pg)
    clk.start()
    l0 = L.ruv_kernel_launches(ctx.h)
    dev_ms = []
    phases = np.zeros(4)
    for _ in range(args.steps):
        ctx.check(L.ruv_lscm_solve_resident(ctx.h, ctypes.byref(copts), stats), "solve")
        t = R.last_timings(ctx)  # assembly, PCG (incl. preconditioner set-up), driver, set-up
        phases += np.array(t)
        dev_ms.append(sum(t[:3]))
    launches = (L.ruv_kernel_launches(ctx.h) - l0) // max(args.steps, 1)
    barrier(pg)
    # the clock record covers the device-timed region; the sampler's driver queries would
    # otherwise stall the host-buffer copies timed next
    clock_info = clk.stop()
    # end-to-end through the host-buffer call, inputs and outputs in page-locked host memory
    e2e_ms = []
    pbatch, _keep = R.pinned_batch(ctx, charts)
    uv = R.pinned_empty(ctx, (nv, 2), np.float64)
    for _ in range(max(args.warmup, 1)):  # untimed, as for the device-timed loop
        ctx.check(L.ruv_lscm_solve_batch(ctx.h, ctypes.byref(pbatch), ctypes.byref(copts),
                                         uv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), stats), "e2e warm-up")
    e2e_dev, e2e_asm = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st_ = L.ruv_lscm_solve_batch(ctx.h, ctypes.byref(pbatch), ctypes.byref(copts),
                                     uv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), stats)
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
        ctx.check(st_, "e2e")
        tt = R.last_timings(ctx)
        e2e_dev.append(sum(tt[:3]))
        e2e_asm.append(tt[0])
    barrier(pg)
    ms = allmax(pg, statistics.mean(dev_ms))
    ems = allmax(pg, statistics.mean(e2e_ms))
    phases /= max(args.steps, 1)

    # dominant kernel (batched SpMV) timed alone on the same operator
    spmv_ms, spmv_bytes, spmv_stream = R.bench_spmv(ctx, prec, reps=30, n_buffers=2)
    peak, peak_src = peaks()
    achieved = spmv_bytes / (spmv_ms * 1e-3) / 1e9 if spmv_ms > 0 else 0.0
    streamed = spmv_stream / (spmv_ms * 1e-3) / 1e9 if spmv_ms > 0 else 0.0

    h2d = sum(int(x) for x in [
        8 * (batch.n_charts + 1) * 2, 3 * 8 * nv, 3 * 4 * int(charts.i64("chart.tri_off")[-1]), nv, 2 * 8 * nv,
        2 * 8 * nv])
    d2h = 2 * 8 * nv

    line = {
        "metric": METRIC, "value": world * unknowns / (ms / 1000.0), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if prec == R.Precision.MIXED else "f64",
        "data": "synthetic",
        "config": cfg,
        "solver": {"precision": args.precision, "precond": args.precond, "tol": 1e-12,
                   "prep_s": prep_s, "prep": "chart stages with their data-parallel parts on the device "
                                             "(ruv_prepare_patches_gpu / ruv_prepare_mesh_gpu), untimed",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "phase_ms": {"assembly": round(phases[0], 3), "pcg": round(phases[1], 3),
                                "driver": round(phases[2], 3), "precond_setup_in_pcg": round(phases[3], 3)},
                   "cg_iters_max": int(cg_iters.max()), "cg_iters_mean": float(cg_iters.mean()),
                   "spmv_shape": {"lanes_per_row": tuned[0], "rows_in_flight": tuned[1], "tile_rows": tuned[2],
                                  "bulk_copy_staging": bool(R.spmv_form(ctx))},
                   "charts_not_ok": int((statuses != 0).sum())},
        "e2e": {"value": world * unknowns / (ems / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": ems,
                "ms_median": statistics.median(e2e_ms), "ms_min": min(e2e_ms),
                "per_call_ms": [round(x, 2) for x in e2e_ms],
                "per_call_device_ms": [round(x, 2) for x in e2e_dev],
                "per_call_assembly_ms": [round(x, 2) for x in e2e_asm]},
        "roofline": {"bound": "hbm", "kernel": "k_spmv_pq (batched CSR-vector SpMV + p.q)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src,
                     "traffic": (SPMV_DRAM_PER_ALG_BYTE * spmv_bytes if args.workload.startswith("disks") else None),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the "
                                       "1024-disk operator, scaled by algorithmic bytes",
                     "ms_per_launch": spmv_ms, "algorithmic_bytes": spmv_bytes,
                     "algorithmic_bytes_what": "FP32 values + 32-bit columns per entry, row pointers, p read once, "
                                               "q written (the canonical scalar-pattern SpMV)",
                     "stream_bytes": spmv_stream, "stream_gbs": streamed, "stream_frac": streamed / peak,
                     "stream_bytes_what": "the same with the 16-bit column stream the kernel reads (offsets "
                                          "from the chart's first row, or from the row itself in charts of "
                                          "more than 65536 rows)"},
        "gpu_launches": int(launches),
        "clocks": clock_info,
    }
    if rank == 0 and not args.no_single_chart:
        line["single_chart_reference_kernels"] = single_chart_reference(ctx, vo, unknowns, ms,
                                                                        args.single_chart_sample)
        line["single_chart_fp64_pcg"] = single_chart_baseline(ctx, vo, unknowns, ms, args.single_chart_sample)
        line["single_chart_fp64_pcg_ic0"] = single_chart_baseline(ctx, vo, unknowns, ms,
                                                                  max(args.single_chart_sample // 4, 1), "IC0")
    if rank == 0 and args.compare:
        line["compare"] = compare_preconds(ctx, args, stats, [x for x in args.compare.split(",") if x])
    if rank == 0 and not args.no_cpu_baseline and src[0] == "patches":
        base, err, n_err = cpu_baseline(src, uv, args.cpu_budget, unknowns)
        line["cpu_baseline"] = base
        line["uv_err_max_vs_lu"] = err
        line["uv_err_charts_checked"] = n_err
        if not args.no_superlu_baseline:
            line["cpu_superlu_whole_workload"] = superlu_baseline(src, os.cpu_count() or 1)
    if rank == 0 and not args.no_cpu_baseline and src[0] == "mesh":
        line.update(field_parity(src, np.array(uv), charts))
    if rank == 0:
        print(json.dumps(line))
    barrier(pg)


if __name__ == "__main__":
    main()
