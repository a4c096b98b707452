"""Benchmark: right-hand sides per second of the HODLR3D matvec and GMRES solve
at N = 64^3 (1/r with the quadrature diagonal, ACA tol 1e-10, leaf 64).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one matvec of 32 right-hand sides in the mixed form (FP32 factors
and near field, FP64 accumulation across tiles) with the inputs resident in
HBM.  `e2e` is the same product through the C-ABI host entry point
(hodlr3d_matvec_host: host buffers, copies inside the timed region).  The
FP64 form at one right-hand side and the GMRES solves are reported beside it.
`--impl reference` times the reference algorithm on the host cores (the CPU
oracle port of it: the reference's sources do not travel with this package):
it assembles the whole operator, then every step is one complete FP64 matvec.  For N > 1 (torchrun) every
rank runs an independent replica; value = all ranks' right-hand sides / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RHS/sec (matvec, GMRES) at N=64^3, 1/r, 1e-6 err: mixed+batched vs FP64 GPU"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(os.environ.get("HODLR3D_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"hodlr3d_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if os.environ.get("H3D_BACKEND") != "gloo" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"  # gloo reduces host tensors
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------
def cpu_full_product(pts, tol_pow, steps, warmup, threads, qchoice=16, diag=float("nan")):
    """Times the reference algorithm on the host cores: the CPU oracle (the
    reference's CUR form, src/ACA.cpp:127-238, with the kernel entries of Ac,
    Ar and the near-field blocks re-evaluated at every product as
    src/HODLR3DTree.cpp:1660-1755 does) assembles the whole operator, then
    every step is one complete FP64 matvec (all boxes of every level and the
    whole near field, one right-hand side), timed by the wall clock.
    Returns (seconds per step for the timed steps, assembly seconds)."""
    from oracle import oracle as orc
    orc.set_threads(threads)
    # lean: pivots and the r x r L, R per pair, as the reference stores them
    o = orc.Oracle(pts, 4, 1.0, tol_pow, qchoice, diag, lean=True)
    t = time.perf_counter()
    o.assemble()
    t_aca = time.perf_counter() - t
    x = np.random.default_rng(5).standard_normal(o.N)
    out = []
    for it in range(warmup + steps):
        t = time.perf_counter()
        o.matvec(x)
        dt = time.perf_counter() - t
        if it >= warmup:
            out.append(dt)
    return out, t_aca


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    from hodlr3d_gb300.workloads import grid_cell_centres
    pts = grid_cell_centres(args.n)
    threads = os.cpu_count() or 1
    secs, t_aca = cpu_full_product(pts, args.tol_pow, args.steps, args.warmup, threads,
                                   qchoice=args.qchoice, diag=args.diag)
    s = float(np.mean(secs))
    v = 1.0 / s
    desc = (f"the whole {args.n}^3 operator: every step one complete FP64 matvec of one right-hand "
            f"side (all levels, all boxes, near field; entries re-evaluated as the reference does), "
            f"wall clock; CPU oracle, {threads} threads ({cpu_model()}); assembly {t_aca:.1f} s "
            f"beforehand, untimed")
    line = {
        "metric": METRIC, "value": v, "unit": "RHS/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": config(args),
        "cpu_baseline": {"value": v, "unit": "RHS/s", "cores": threads, "kind": "port",
                         "sample": desc, "extrapolated": False},
        "e2e": {"value": v, "unit": "RHS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "assembly_seconds": t_aca,
        "step_seconds": secs,
    }
    print(json.dumps(line), flush=True)


def config(args):
    kern = ("kernel 1/r with quadrature diagonal (Qchoice 16)" if args.qchoice == 16 and args.diag != args.diag
            else f"kernel Qchoice {args.qchoice}" + ("" if args.diag != args.diag else f", diagonal {args.diag:g}"))
    return {"workload": f"HODLR3D matvec, {args.n}^3 grid cell centres on [-1,1]^3, leaf 64 "
                        f"(nP1D 4), {kern}, ACA tol 1e-{args.tol_pow}, {args.nrhs} right-hand "
                        f"sides N(0,1)",
            "N": args.n ** 3, "nrhs": args.nrhs, "precision": "mixed (FP32 factors and near field, "
            "FP64 accumulation across tiles)", "tol_pow": args.tol_pow,
            "l2": "inputs larger than L2 (the FP32 factors alone exceed 129 MB by two orders)"}


# ----------------------------------------------------------------------------
def measured_traffic(kernel, args):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu
    summary (profiles/traffic.json), when it covers this workload; else None."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "traffic.json")
    try:
        with open(path) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return None
    e = rec.get(kernel)
    if (not e or e.get("n") != args.n or e.get("nrhs") != args.nrhs or e.get("tol_pow") != args.tol_pow
            or e.get("qchoice") != args.qchoice or args.diag == args.diag):
        return None
    return e["bytes_per_launch"]


def pair_sizes(H):
    """Per compressed pair (level, target box, source box): its rank and the
    populations n of the target box and m of the source box."""
    P = H.pairs()
    R = H.ranks().astype(np.int64)
    off = H.leaf_offsets()
    d = int(P[:, 0].max()) if len(P) else 0

    def sizes(level, boxes):
        sh = 3 * (d - level)
        return off[(boxes + 1) << sh] - off[boxes << sh]

    n = np.zeros(len(P), np.int64)
    m = np.zeros(len(P), np.int64)
    for j in range(1, d + 1):
        sel = P[:, 0] == j
        n[sel] = sizes(j, P[sel, 1].astype(np.int64))
        m[sel] = sizes(j, P[sel, 2].astype(np.int64))
    return P, R, n, m, d, off


# FP64 arithmetic rate for the assembly's fraction: GB300's nominal dense FP64
ASSEMBLY_PEAK_GFLOPS = 1250.0
# FP64 FMAs per second at that nominal rate
FP64_FMA_PEAK = ASSEMBLY_PEAK_GFLOPS * 1e9 / 2


def aca_work(H):
    """Work of the partially pivoted ACA (src/ACA.cpp:127-238) at the ranks it
    produced.  Iteration k of a pair evaluates one residual row (m kernel
    entries) and one residual column (n), subtracts the k earlier terms from
    each (k (n + m) FMAs) and updates the norm estimate with k cross terms
    (k (n + m) FMAs); one more row and column end the loop.  Evaluations
    E = sum (r + 1)(n + m); FP64 flops = 9 E (an entry: 3 subtractions, 3 for
    r^2, square root and division counted as 1, the scale, the diagonal
    select) + sum 2 r (r - 1)(n + m)."""
    _, R, n, m, _, _ = pair_sizes(H)
    nm = n + m
    evals = int(((R + 1) * nm).sum())
    flops = 9 * evals + int((2 * R * (R - 1) * nm).sum())
    return evals, flops


# few-column engine chunking (hodlr3d_gb300/csrc/matvec.h): V-stack columns
# per forward work item, U rows per transposed work item
GEMV_COLS = 1024
GEMV_ROWS_T = 256


def engine_of(kernels) -> str:
    """The matvec engine whose kernels a profile report names."""
    if "uy64" in kernels or "vy64" in kernels:
        return "f64"
    if "leaf_rows" in kernels:
        return "tc"
    if "uy" in kernels or "vy" in kernels:
        return "gemv"
    return "simt"


def level_bytes(H, nr_pad, s, engine):
    """Algorithmic bytes per launch of each kernel (see level_bytes_engine);
    the FP64 streaming engine ("f64") is the few-column engine's stages on
    8-byte factors and near-field blocks, one column."""
    if engine == "f64":
        gv = level_bytes_engine(H, 1, 8, "gemv", near_bytes=8)
        return {k + "64": v for k, v in gv.items()}
    return level_bytes_engine(H, nr_pad, s, engine)


def level_bytes_engine(H, nr_pad, s, engine, near_bytes=4):
    """Algorithmic bytes per launch of each kernel of one matvec engine
    ("simt", "tc" or "gemv"), keyed by the names its profiler spans carry: the
    factor entries it streams (s bytes each), plus its right-hand-side,
    intermediate (T, slice or chunk partials) and output traffic counted once;
    the tensor-core leaf kernel and the few-column output kernels also stream
    the FP32 near-field blocks."""
    P, R, n, m, d, off = pair_sizes(H)
    N = H.N
    leaf = P[:, 0] == d
    up = ~leaf
    above = P[:, 0] < d - 1
    nslices = 8 ** np.maximum(d - 1 - P[:, 0], 0)
    xb = N * nr_pad * s                       # right-hand sides in tree order
    t_up = int(R[up].sum()) * nr_pad * s      # T of the non-leaf pairs
    t_leaf = int(R[leaf].sum()) * nr_pad * s  # T of the leaf pairs
    parts = int((R[above] * nslices[above]).sum()) * nr_pad * s
    u_up, v_up = int((R[up] * n[up]).sum()) * s, int((R[up] * m[up]).sum()) * s
    u_leaf, v_leaf = int((R[leaf] * n[leaf]).sum()) * s, int((R[leaf] * m[leaf]).sum()) * s
    ynl = N * nr_pad * 8
    y = N * min(nr_pad, 64) * 8
    gather = y + xb
    if engine == "simt":
        return {"gather": gather,
                "vtx": v_up + xb + t_up + parts,
                "tred": parts + t_up,
                "ut": u_up + t_up + ynl,
                "leaf": u_leaf + v_leaf + xb + ynl + y}
    # FP32 near-field blocks (tensor-core and few-column engines): every leaf
    # with itself and its face / edge neighbours (vertex neighbours are
    # compressed pairs)
    nl = len(off) - 1
    cnt = np.diff(off)
    cnt4 = (cnt + 3) // 4 * 4
    nb = H.neighbors(d) if d >= 1 else np.full((nl, 26), -1, np.int32)
    vertex = np.array([abs(dx) + abs(dy) + abs(dz) == 3 for dz in (-1, 0, 1) for dy in (-1, 0, 1)
                       for dx in (-1, 0, 1) if (dx, dy, dz) != (0, 0, 0)])
    nbn = np.where((nb >= 0) & ~vertex[None, :], cnt4[np.maximum(nb, 0)], 0).sum(axis=1)
    near = int((cnt * (cnt4 + nbn)).sum()) * near_bytes
    if engine == "tc":
        # the leaf level as dense FP32 blocks (leaf rows): every leaf-level
        # pair's n x round4(m) block next to the near-field blocks
        far_leaf = int((n[leaf] * ((m[leaf] + 3) // 4 * 4)).sum()) * 4
        return {"gather": gather,
                "ta_slice": v_up + xb + t_up + parts,
                "tred": parts + t_up,
                "ut_tc": u_up + t_up + ynl,
                "leaf_rows": near + far_leaf + xb + ynl + y}
    # few-column engine: chunk partials of the V stacks wider than GEMV_COLS
    # (forward) and of the U blocks taller than GEMV_ROWS_T (transpose), each
    # read once and reduced into the pair's rows of T
    nch = -(-((m + 3) // 4 * 4) // GEMV_COLS)
    ncht = -(-n // GEMV_ROWS_T)
    r4 = (R + 3) // 4 * 4
    tred = int((R * (nch + 1))[nch > 1].sum()) * nr_pad * s
    tred_t = int((r4 * ncht + R)[ncht > 1].sum()) * nr_pad * s
    return {"gather": gather,
            "vt": v_up + v_leaf + xb + t_up + t_leaf,
            "tred": tred,
            "uy": u_up + u_leaf + near + t_up + t_leaf + xb + y,
            "ut": u_up + u_leaf + xb + t_up + t_leaf,
            "tred_t": tred_t,
            "vy": v_up + v_leaf + near + t_up + t_leaf + xb + y}


def run_ours(args):
    import torch

    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import charges_normal, charges_uniform, grid_cell_centres

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pts = grid_cell_centres(args.n)
    N = len(pts)
    t = time.perf_counter()
    H = HODLR3D(4, 1.0, args.tol_pow, args.qchoice, pts, device=local, diag_override=args.diag)
    H.assemble()
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t
    st = H.stats()
    aca_evals, aca_flops = aca_work(H)
    nrhs = args.nrhs
    X = torch.tensor(charges_normal(N, nrhs, seed=11), device=dev).reshape(N, nrhs)
    x1 = X[:, 0].contiguous()
    stream = torch.cuda.current_stream()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        barrier(ws)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        return e0.elapsed_time(e1) / steps

    # accuracy against the dense FP64 product on sampled rows
    rows = np.sort(np.random.default_rng(3).choice(N, 512, replace=False))
    Yd = H.dense_rows(rows, X)
    ridx = torch.as_tensor(rows, device=dev)

    def col_err(Y):
        D = Yd.reshape(len(rows), -1)
        return float((torch.linalg.norm(Y.reshape(N, -1)[ridx] - D, dim=0) /
                      torch.linalg.norm(D, dim=0)).max().item())

    err_mixed = col_err(H.matvec(X, "mixed"))
    err_fp64 = col_err(H.matvec(X, "fp64"))

    # ---- headline: mixed, nrhs columns, device resident ------------------
    launches0 = H.launch_count()
    clk = ClockSampler(local)
    clk.start()
    ms = timed(lambda: H.matvec(X, "mixed"), args.steps, args.warmup)
    clocks = clk.stop()
    # the library's own kernel launches: per step, and inside the timed
    # region (the steps after the warm-up ones)
    launches_step = (H.launch_count() - launches0) // (args.steps + args.warmup)
    launches = launches_step * args.steps
    ms_max = max_over_ranks(ws, ms)
    value = ws * nrhs / (ms_max * 1e-3)

    # ---- FP64 form, one right-hand side: the FP64 streaming engine (the
    # automatic choice), and the CUDA-core FP64 kernels beside it -----------
    ms64 = timed(lambda: H.matvec(x1, "fp64"), max(3, args.steps // 2), 2)
    H.set_engine("simt")
    ms64_simt = timed(lambda: H.matvec(x1, "fp64"), max(3, args.steps // 4), 2)
    H.set_engine("auto")

    # ---- per-kernel times (events between launches) -> roofline ----------
    H.set_profiling(True)
    nprof = max(3, args.steps // 2)
    for _ in range(nprof):
        H.matvec(X, "mixed")
    torch.cuda.synchronize()
    rep = H.profile_report()
    H.set_profiling(False)
    kern_ms = {k: v[1] / v[0] for k, v in rep.items()}
    nr_pad = 1 << (nrhs - 1).bit_length()
    alg = level_bytes(H, nr_pad, 4, engine_of(kern_ms))
    top = max(kern_ms, key=kern_ms.get)
    hbm, peak_kind = peaks()
    achieved = alg[top] / (kern_ms[top] * 1e-3) / 1e9
    ran = {k: alg[k] for k in kern_ms}
    roof = {"bound": "hbm", "kernel": f"k_{top}", "achieved": achieved, "peak": hbm,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": measured_traffic(f"k_{top}", args), "kernel_ms": kern_ms,
            "algorithmic_bytes": ran,
            "whole_matvec_GBps": sum(ran.values()) / (ms * 1e-3) / 1e9}

    # ---- one right-hand side in the mixed form (few-column engine) --------
    def kernel_split(fn):
        H.set_profiling(True)
        for _ in range(nprof):
            fn()
        torch.cuda.synchronize()
        r = H.profile_report()
        H.set_profiling(False)
        return {k: v[1] / v[0] for k, v in r.items()}

    one = {}
    for name, tr in (("forward", False), ("transpose", True)):
        ms1 = timed(lambda: H.matvec(x1, "mixed", transpose=tr), max(3, args.steps // 2), 3)
        k1 = kernel_split(lambda: H.matvec(x1, "mixed", transpose=tr))
        a1 = level_bytes(H, 1, 4, engine_of(k1))
        t1 = max(k1, key=k1.get)
        ach = a1[t1] / (k1[t1] * 1e-3) / 1e9
        one[name] = {"ms": ms1, "rhs_per_s": 1e3 / ms1, "kernel_ms": k1,
                     "top_kernel": f"k_{t1}", "top_achieved_GBps": ach, "top_frac": ach / hbm,
                     "whole_GBps": sum(a1[k] for k in k1) / (ms1 * 1e-3) / 1e9}
    d1 = Yd.reshape(len(rows), -1)[:, 0]
    y1 = H.matvec(x1, "mixed")[ridx]
    one["forward"]["error_vs_dense_fp64"] = float((torch.linalg.norm(y1 - d1) / torch.linalg.norm(d1)).item())
    one["speedup_vs_fp64_1rhs"] = ms64 / one["forward"]["ms"]

    # FP64 streaming engine: bytes against HBM, FMAs against GB300's FP64 rate
    k64 = kernel_split(lambda: H.matvec(x1, "fp64"))
    a64 = level_bytes(H, 1, 8, engine_of(k64))
    fp64_entries = st["factor_entries"] + st["near_entries"]
    fp64 = {"rhs_per_s": 1e3 / ms64, "ms": ms64, "engine": engine_of(k64), "kernel_ms": k64,
            "whole_GBps": sum(a64[k] for k in k64 if k in a64) / (ms64 * 1e-3) / 1e9,
            "fma_per_s": fp64_entries / (ms64 * 1e-3),
            "fma_peak_nominal": FP64_FMA_PEAK, "fma_frac_nominal": fp64_entries / (ms64 * 1e-3) / FP64_FMA_PEAK,
            "cuda_core_fp64_ms": ms64_simt, "speedup_vs_cuda_core_fp64": ms64_simt / ms64}

    # ---- FP64-accurate products in FP32-pair arithmetic (fp64x) ----------
    msx = timed(lambda: H.matvec(x1, "fp64x"), max(3, args.steps // 2), 3)
    kx = kernel_split(lambda: H.matvec(x1, "fp64x"))
    y64, yx = H.matvec(x1, "fp64"), H.matvec(x1, "fp64x")
    fp64x = {"ms": msx, "rhs_per_s": 1e3 / msx, "kernel_ms": kx,
             "whole_GBps": 2 * sum(level_bytes(H, 1, 4, engine_of(kx))[k] for k in kx)
             / (msx * 1e-3) / 1e9,
             "rel_diff_vs_fp64": float((torch.linalg.norm(yx - y64) / torch.linalg.norm(y64)).item()),
             "speedup_vs_fp64_1rhs": ms64 / msx}

    # ---- GMRES: b = A x_true, x_true U[0,1) ------------------------------
    xt = torch.tensor(charges_uniform(N, nrhs, seed=21), device=dev).reshape(N, nrhs)
    B = H.matvec(xt, "fp64")
    torch.cuda.synchronize()
    t = time.perf_counter()
    Xs, info = H.gmres(B, maxit=300, tol=1e-10, restart=30, precision="mixed")
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t
    fwd_mixed = float((torch.linalg.norm(Xs - xt, dim=0) / torch.linalg.norm(xt, dim=0)).max())
    b1 = B[:, 0].contiguous()
    t = time.perf_counter()
    x64, info64 = H.gmres(b1, maxit=400, tol=1e-10, restart=0, precision="fp64")
    torch.cuda.synchronize()
    t_fp64 = time.perf_counter() - t
    t = time.perf_counter()
    x1m, info1 = H.gmres(b1, maxit=300, tol=1e-10, restart=30, precision="mixed")
    torch.cuda.synchronize()
    t_mixed1 = time.perf_counter() - t
    gmres = {"mixed_rhs_per_s": nrhs / t_mixed, "mixed_seconds": t_mixed,
             "mixed_iterations": info["iterations"], "mixed_outer": info["outer"],
             "mixed_rel_residual": info["rel_residual"], "mixed_forward_err": fwd_mixed,
             "fp64_rhs_per_s": 1.0 / t_fp64, "fp64_seconds": t_fp64,
             "fp64_iterations": info64["iterations"], "fp64_rel_residual": info64["rel_residual"],
             "speedup_mixed_batched_vs_fp64": (nrhs / t_mixed) / (1.0 / t_fp64),
             "mixed_1rhs_seconds": t_mixed1, "mixed_1rhs_iterations": info1["iterations"],
             "mixed_1rhs_rel_residual": info1["rel_residual"],
             "speedup_mixed_1rhs_vs_fp64": t_fp64 / t_mixed1}

    # ---- e2e through the C ABI with host buffers -------------------------
    # host arrays of the caller, (N, nrhs) by rows; each step copies them in
    # and the result out (hodlr3d_matvec_host_rows)
    Xh = np.ascontiguousarray(X.cpu().numpy())
    Yh = np.empty_like(Xh)
    for _ in range(2):
        H.MatVecProduct(Xh, "mixed", out=Yh)
    t = time.perf_counter()
    ke = max(3, args.steps // 2)
    for _ in range(ke):
        H.MatVecProduct(Xh, "mixed", out=Yh)
    t_e2e = (time.perf_counter() - t) / ke
    t_e2e = max_over_ranks(ws, t_e2e)
    e2e = {"value": ws * nrhs / t_e2e, "unit": "RHS/s", "h2d_bytes_per_step": int(Xh.nbytes),
           "d2h_bytes_per_step": int(Xh.nbytes), "ms_per_step": t_e2e * 1e3,
           "entry": "hodlr3d_matvec_host_rows"}

    # ---- the same product replayed from a CUDA graph (captured once; last of
    # the GPU measurements, so that its private memory pool cannot perturb
    # the others) ---------------------------------------------------------------
    graph = None
    try:
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            H.matvec(X, "mixed")
        stream.wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            Yg = H.matvec(X, "mixed")
        msg = timed(g.replay, args.steps, args.warmup)
        graph = {"ms": msg, "rhs_per_s": nrhs / (msg * 1e-3),
                 "matches_eager": bool(torch.equal(Yg, H.matvec(X, "mixed")))}
        del g
    except RuntimeError as e:  # capture refused by the runtime: report, keep going
        graph = {"error": str(e)[:200]}

    # ---- the engine autotuner over this operator (after the timed
    # measurements; the automatic choice returns to the rules afterwards) -----
    tune = None
    if not args.no_autotune:
        t = time.perf_counter()
        tune_rows = H.autotune(reps=3)
        ch = H.tuning()
        launch = H.launch_tuning()
        H.autotune(reps=0)
        counts = (1, 2, 4, 8, 16, 32, 64)
        tune = {"seconds": time.perf_counter() - t,
                "forward": {n: ch["forward"][n - 1] for n in counts},
                "transpose": {n: ch["transpose"][n - 1] for n in counts},
                "ms": {f"{'AT' if tr else 'A'}_{n}_{e}": round(ms, 3) for tr, n, e, ms in tune_rows},
                "ta_split_ms": {k: round(v, 3) for k, v in launch["ta_split"].items()},
                "ta_split_chosen": launch["ta_split_chosen"]}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the whole operator assembled by the CPU oracle, then complete FP64
        # products timed (after the GPU measurements: the host threads would
        # perturb their launches)
        threads = os.cpu_count() or 1
        secs, t_aca = cpu_full_product(pts, args.tol_pow, 2, 1, threads, qchoice=args.qchoice,
                                       diag=args.diag)
        cpu = {"value": 1.0 / float(np.mean(secs)), "unit": "RHS/s", "cores": threads,
               "kind": "port", "extrapolated": False,
               "sample": f"two complete FP64 matvecs of the whole {args.n}^3 operator (one right-hand "
                         f"side each, entries re-evaluated as the reference does) after one untimed, "
                         f"wall clock, {threads} threads ({cpu_model()}); CPU assembly {t_aca:.1f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "RHS/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "gpu_launches_per_step": int(launches_step),
            "clocks": clocks,
            "fp64_1rhs": fp64,
            "cuda_graph": graph,
            "autotune": tune,
            "mixed_1rhs": one,
            "fp64x_1rhs": fp64x,
            "speedup_mixed_batched_vs_fp64": value / ws / (1e3 / ms64),
            "error_vs_dense_fp64": {"mixed_max_col_rel": err_mixed, "fp64_max_col_rel": err_fp64,
                                    "rows_sampled": len(rows)},
            "gmres": gmres, "setup_seconds": t_setup,
            "assembly": {"seconds": st["assemble_seconds"], "tree_seconds": st["tree_seconds"],
                         "pairs": st["n_pairs"], "max_rank": st["max_rank"],
                         "factor_bytes_fp32": st["factor_bytes_fp32"],
                         "factor_bytes_fp64": st["factor_bytes_fp64"],
                         "aca_batches": st["aca_batches"],
                         "aca_kernel_seconds": st["aca_kernel_seconds"],
                         "finish_seconds": st["finish_seconds"],
                         "roofline": {"bound": "fp64", "entry_evaluations": aca_evals,
                                      "flops": aca_flops,
                                      "achieved": aca_flops / st["assemble_seconds"] / 1e9,
                                      "peak": ASSEMBLY_PEAK_GFLOPS, "unit": "GFLOP/s",
                                      "peak_kind": "nominal",
                                      "frac": aca_flops / st["assemble_seconds"] / 1e9
                                      / ASSEMBLY_PEAK_GFLOPS}},
        }
        print(json.dumps(line), flush=True)
    H.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--nrhs", type=int, default=32)
    ap.add_argument("--tol-pow", type=int, default=10)
    ap.add_argument("--qchoice", type=int, default=16, help="kernel (the reference's Qchoice)")
    ap.add_argument("--diag", type=float, default=float("nan"),
                    help="diagonal value override (e.g. 1 for exp(-r), Qchoice 1)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="skip the engine autotuner's table")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
