"""Benchmark: time to relative residual 1e-8 on the 128^3 graph Laplacian with IC(0).

Workload (one "step" = one full solve from x0 = 0):
  128^3 7-point Laplacian, edge weights lognormal(0, 0.5), + 1e-3 I (n = 2,097,152,
  nnz = 14,581,760), b ~ U[-1,1] (seed 1002), IC(0), tol 1e-8 relative to ||b||.
  value  = mixed-precision solve time, precision=2: FP64 Krylov recurrence
           (x, r, p, q, alpha, beta) around the FP32 SpMV and the FP32 IC(0)
           triangular solves, with FP64 residual replacement; device-resident
           inputs, CUDA events on the solver stream;
  fp64   = the plain FP64 device PCG on the same system (the comparator the
           metric names);
  fp32_krylov = precision=1: FP32 Krylov vectors, SpMV and IC(0) inside FP64
           iterative refinement (reported beside; needs ~1.75x the iterations);
  e2e    = the same mixed solve through gb_pcg_solve_host from pinned host
           buffers (b, x0 in; x out), copies inside the timed region.
  parity = every GPU solve against the reference's CPU PCG on the same
           inputs at full size (IC(0) and GS_std, k = 1): its iteration count
           and the relative distance of x from the reference's x.
  cpu_baseline = one full FP64 IC(0)-PCG solve by the reference's algorithm
           (the oracle's C restatement of LAP's serial path) on one host core,
           measured, not extrapolated.
Inputs (matrix 175 MB FP64 + 117 MB FP32 copy + factors) exceed the 129 MB L2,
so no explicit L2 flush is done between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU algorithm on this host: the
oracle's restatement of LAP's OpenMP backend (SpMV on a team of 16 threads as
openmp_blas.c:37 fixes it, dot on all host threads, serial triangular
solves).  Each timed step is one full solve; warm-up steps are short samples.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to rel-res 1e-8, mixed-prec IC0-PCG on 128^3 Laplacian (1 GB300)"
MIXED = 2  # the headline mixed-precision mode (gb_pcg_opts.precision)
UNIT = "ms"
WORKLOAD = "grid3d_lognormal_128 (n=2097152, nnz=14581760), IC0, tol 1e-8"


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of each kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9
                          for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(nside):
    from lap_gb300 import gen

    return gen.grid3d_lognormal(nside, seed=1002)


def host_info():
    """Host cores, CPU model and OMP_NUM_THREADS of the machine the CPU legs ran on."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None and os.path.exists("/proc/cpuinfo"):
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
    return {"nproc": os.cpu_count(), "cpu_model": model, "machine": os.uname().machine,
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}


def reference_solve(A, b, prec, tol, kind="serial", max_iters_run=0):
    """The reference's CPU PCG (the oracle: LAP's serial path restated, or its
    OpenMP backend mirror) on the full system, from x0 = 0."""
    import oracle

    return oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, tol, 20000, kind=kind, max_iters_run=max_iters_run)


def cpu_baseline(ref):
    """Measured time of one full serial solve (cg() only, as LAP's Time line)."""
    return dict(value=round(ref["solve_s"] * 1e3, 1), unit=UNIT, cores=1, kind="port",
                sample=f"one full FP64 IC0-PCG solve of the 128^3 system ({ref['iters']} iterations) by the "
                       f"oracle's restatement of LAP's serial path on 1 host core; cg() only, as LAP's Time "
                       f"line; IC0 setup {ref['setup_s']:.2f} s excluded",
                host=host_info())


def parity_entry(ref, x, r):
    """A GPU solve against the reference's: iterations and distance of x."""
    xr = ref["x"]
    err = float(np.linalg.norm(x.cpu().numpy() - xr) / np.linalg.norm(xr))
    slack = max(1, int(np.ceil(0.02 * ref["iters"])))
    return {"iters": r["iters"], "x_rel_err_vs_reference": err, "rel_true_res": r["rel_true_res"],
            "iters_within_2pct": abs(r["iters"] - ref["iters"]) <= slack, "x_within_1e-6": err <= 1e-6}


def run_reference(args, world, rank):
    """The reference's CPU PCG (oracle restatement, OpenMP mirror) timed on host cores."""
    if rank != 0:
        return
    import oracle

    A, b = make_workload(args.size)
    t0 = time.time()
    for _ in range(args.warmup):  # untimed: page in the matrix, start the thread team
        reference_solve(A, b, "ichol", args.tol, kind="omp", max_iters_run=3)
    times, iters = [], []
    for _ in range(args.steps):  # each timed step: one full solve
        r = reference_solve(A, b, "ichol", args.tol, kind="omp")
        times.append(r["solve_s"] * 1e3)
        iters.append(r["iters"])
    v = statistics.mean(times)
    L = oracle.lib("omp")
    spmv_t, dot_t = L.orc_spmv_threads(), L.orc_num_threads()
    line = {"metric": METRIC, "value": round(v, 1), "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD + " (reference: FP64 IC0-PCG, CPU)", "iterations": iters[-1],
                       "flag": r["flag"], "steps_ms": [round(t, 1) for t in times]},
            "cpu_baseline": {"value": round(v, 1), "unit": UNIT, "cores": max(spmv_t, dot_t), "kind": "port",
                             "sample": f"one full solve per step ({iters[-1]} iterations, cg() only as LAP's "
                                       f"Time line); restatement of LAP's OpenMP backend: SpMV on {spmv_t} "
                                       f"threads (openmp_blas.c:37), dot on {dot_t}, serial triangular solves",
                             "host": host_info()},
            "e2e": {"value": round(v, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(time.time() - t0, 1)}
    print(json.dumps(line), flush=True)


def run_kernels_only(args, local):
    """Per-kernel device times of PCG iterations run eagerly (no graph), for
    each precision mode -- the launches a profiler can attribute one by one."""
    import torch

    import lap_gb300 as gb

    torch.cuda.set_device(local)
    A, b = make_workload(args.size)
    sysm = gb.System.from_csr(A, "ichol")
    db = torch.from_numpy(b).cuda()
    precs = [int(t) for t in args.profile_precisions.split(",")]
    out = {p: [(k["name"], round(k["ms"], 5)) for k in sysm.profile(db, precision=p, iters=args.profile_iters)]
           for p in precs}
    print(json.dumps({"kernels_only": out, "n": A.n, "nnz": A.nnz}), flush=True)


def _timed_solves(fn, steps):
    import torch

    out = []
    for _ in range(steps):
        torch.cuda.synchronize()
        out.append(fn())
    return out


def _edge_positions(A, ei, ej):
    """CSR positions of each edge's two entries and of every diagonal, and the
    index of each edge among A's strict-lower entries (row-major)."""
    rows = np.repeat(np.arange(A.n), np.diff(A.ia))
    key = rows.astype(np.int64) * A.n + A.ja
    lo, hi = np.minimum(ei, ej), np.maximum(ei, ej)
    strict_lower = np.nonzero(A.ja < rows)[0]
    p_lh = np.searchsorted(key, lo * A.n + hi)
    p_hl = np.searchsorted(key, hi * A.n + lo)
    diag = np.searchsorted(key, np.arange(A.n, dtype=np.int64) * (A.n + 1))
    return lo, hi, p_lh, p_hl, diag, np.searchsorted(strict_lower, p_hl)


def run_workload(args, local):
    """The other configurations at full size (256^2 Jacobi, Chung-Lu, the
    kNN batch, multi-RHS, the adjoint, the Matrix Market read; parity cases
    beside the headline bench line): one JSON line each with times and
    accuracy."""
    import torch

    import lap_gb300 as gb
    from lap_gb300 import gen

    torch.cuda.set_device(local)
    wl = args.workload
    line = {"workload": wl, "data": "synthetic (seeded generator)"}
    t0 = time.time()
    if wl == "jacobi256":
        import oracle

        A, b = gen.grid2d_unit(256, seed=1001)
        line["config"] = "256^2 unit 5-point + 1e-2 I, line_jacobi, tol 1e-8, maxit 10000 (FP64)"
        sysm = gb.System.from_csr(A, "line_jacobi")
        db = torch.from_numpy(b).cuda()
        for _ in range(3):
            sysm.solve(db, tol=1e-8, maxit=10000)
        res = _timed_solves(lambda: sysm.solve(db, tol=1e-8, maxit=10000), 5)
        x, r = res[-1]
        ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, "line_jacobi", 1e-8, 10000)
        line.update(ms=statistics.mean(rr["device_ms"] for _, rr in res), iters=r["iters"],
                    ref_iters=ref["iters"], rel_true_res=r["rel_true_res"],
                    x_rel_err_vs_reference=float(np.linalg.norm(x.cpu().numpy() - ref["x"]) /
                                                 np.linalg.norm(ref["x"])),
                    cpu_reference_ms=ref["solve_s"] * 1e3, cpu_cores=1)
    elif wl == "mmread128":
        import ctypes as C
        import tempfile

        A, _ = gen.grid3d_lognormal(128, seed=1002)
        line["config"] = ("128^3 lognormal Laplacian written as 'coordinate real symmetric' (lower triangle, "
                          "%.17g values), read into CSR: host read_mm_file + coo_to_csr vs gb_mm_read_csr")
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "g128.mtx")
            tw = time.time()
            gen.write_mm(path, A)
            line["file_bytes"] = os.path.getsize(path)
            line["write_s"] = round(time.time() - tw, 1)
            L = gb.lib()
            gb.read_mm_device(path)  # warm-up (module load, first allocations)
            runs = []
            for _ in range(3):
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                ia, ja, a, info = gb.read_mm_device(path)
                runs.append((time.perf_counter() - t1, info))
            wall, info = min(runs, key=lambda t: t[0])
            line["device"] = {"wall_ms": round(wall * 1e3, 1), "read_ms": round(info["read_ms"], 1),
                              "h2d_ms": round(info["h2d_ms"], 2), "device_ms": round(info["device_ms"], 2),
                              "device_gbs_of_file": round(line["file_bytes"] / info["device_ms"] / 1e6, 1),
                              "host_parsed": info["host_parsed"], "nnz": info["nnz"]}
            M = gb.MMatrix()
            t1 = time.perf_counter()
            L.read_mm_file(path.encode(), C.byref(M))
            L.coo_to_csr(C.byref(M))
            line["host_reader_ms"] = round((time.perf_counter() - t1) * 1e3, 1)
            hia = np.ctypeslib.as_array(M.csr_ia, (M.n + 1,)).copy()
            hja = np.ctypeslib.as_array(M.csr_ja, (M.nnz_unpacked,)).copy()
            ha = np.ctypeslib.as_array(M.csr_vals, (M.nnz_unpacked,)).copy()
            libc = C.CDLL(None)
            for q in (M.csr_ia, M.csr_ja, M.csr_vals):
                libc.free(C.cast(q, C.c_void_p))
            line["identical_to_host_reader"] = bool(
                np.array_equal(ia.cpu().numpy(), hia) and np.array_equal(ja.cpu().numpy(), hja)
                and np.array_equal(a.cpu().numpy().view(np.int64), ha.view(np.int64)))
            line["identical_to_generator"] = bool(
                np.array_equal(hia, A.ia) and np.array_equal(hja, A.ja) and np.array_equal(ha, A.a))
            line["speedup_vs_host_reader"] = round(line["host_reader_ms"] / (wall * 1e3), 1)
    elif wl == "chunglu4m":
        A, b = gen.chung_lu(1 << 22, seed=1003)
        line["config"] = f"Chung-Lu n={A.n} nnz={A.nnz}, A=1.001 D - W, ichol, tol 1e-10"
        line["generate_s"] = round(time.time() - t0, 1)
        t1 = time.time()
        sysm = gb.System.from_csr(A, "ichol")
        line["setup_s"] = round(time.time() - t1, 1)
        line["levels"] = sysm.info()
        db = torch.from_numpy(b).cuda()
        kw = dict(tol=1e-10, maxit=20000)
        x64, r64 = sysm.solve(db, precision=0, **kw)
        for p in (0, 1, 2):
            sysm.solve(db, precision=p, **kw)
            x, r = sysm.solve(db, precision=p, **kw)
            line[f"precision{p}"] = {"ms": round(r["device_ms"], 2), "iters": r["iters"], "outer": r["outer"],
                                     "flag": r["flag"], "rel_true_res": r["rel_true_res"],
                                     "rel_err_vs_fp64": float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64))}
        # the mode chosen by timing (gb_pcg_autotune_precision), then a solve in it
        tune = sysm.autotune_precision(db, **kw)
        sysm.solve(db, precision=-1, **kw)
        res = _timed_solves(lambda: sysm.solve(db, precision=-1, **kw), 3)
        x, r = res[-1]
        line["autotune_precision"] = {"best": tune["best"], "ms_per_mode": [round(v, 2) for v in tune["ms"]],
                                      "solve_ms": round(statistics.mean(rr["device_ms"] for _, rr in res), 2),
                                      "iters": r["iters"],
                                      "rel_err_vs_fp64": float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64))}
    elif wl == "batch512":
        mats, rhs = gen.knn_batch(512, seed=1004)
        line["config"] = (f"512 kNN(k=8) Laplacians, n log-uniform 1k-200k (sum n = {sum(A.n for A in mats)}, "
                          f"sum nnz = {sum(A.nnz for A in mats)}), line_jacobi, tol 1e-8, one graph launch")
        line["generate_s"] = round(time.time() - t0, 1)
        bt = gb.Batch(mats, "line_jacobi")
        db = torch.from_numpy(np.concatenate(rhs)).cuda()
        x64, i64, f64, r64 = bt.solve(db, tol=1e-8, maxit=20000, precision=0)
        for p in (0, 2):
            bt.solve(db, tol=1e-8, maxit=20000, precision=p)
            res = _timed_solves(lambda: bt.solve(db, tol=1e-8, maxit=20000, precision=p), 3)
            x, its, fl, r = res[-1]
            line[f"precision{p}"] = {"ms": round(statistics.mean(rr["device_ms"] for *_, rr in res), 2),
                                     "max_iters": int(its.max()), "all_converged": bool((fl == 0).all()),
                                     "rel_true_res_max": r["rel_true_res"],
                                     "rel_err_vs_fp64": float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64))}
        # the autotuner's plan for this batch, then the same solves on it
        tune = bt.autotune(db, iters=16)
        line["autotune"] = dict(tune)
        for p in (0, 2):
            bt.solve(db, tol=1e-8, maxit=20000, precision=p)
            res = _timed_solves(lambda: bt.solve(db, tol=1e-8, maxit=20000, precision=p), 3)
            x, its, fl, r = res[-1]
            line["autotune"][f"precision{p}_ms"] = round(statistics.mean(rr["device_ms"] for *_, rr in res), 2)
            line["autotune"][f"precision{p}_all_converged"] = bool((fl == 0).all())
            line["autotune"][f"precision{p}_rel_err_vs_fp64"] = float(torch.linalg.norm(x - x64) /
                                                                      torch.linalg.norm(x64))
        t2 = time.time()  # the same systems one by one with the single-system solver
        ms = 0.0
        for A, b in zip(mats, rhs):
            sg = gb.System.from_csr(A, "line_jacobi")
            _, rs = sg.solve(torch.from_numpy(b).cuda(), tol=1e-8, maxit=20000)
            ms += rs["device_ms"]
            sg.close()
        line["one_by_one_device_ms"] = round(ms, 2)
        line["one_by_one_wall_s"] = round(time.time() - t2, 1)
    elif wl in ("multirhs32", "multirhs64"):
        nr = int(wl[len("multirhs"):])
        A, _ = gen.grid3d_lognormal(128, seed=1002)
        Bm = torch.from_numpy(gen.multi_rhs(A.n, nr, seed=1005)).cuda()
        line["config"] = (f"128^3 lognormal Laplacian, {nr} RHS, line_jacobi, tol 1e-8, "
                          + ("one graph launch" if nr <= 32 else "chunks of 32 RHS, one graph launch each"))
        sysm = gb.System.from_csr(A, "line_jacobi")
        X64, i64, _ = gb.solve_multi(sysm, Bm, tol=1e-8, maxit=20000, precision=0)
        forms = [("", None)] + ([("blocks_", "blocks")] if nr > 32 else [])
        for tag, form in forms:
            if form:  # every column in one launch on concatenated vectors
                os.environ["GBLAP_MULTI_FORM"] = form
            for p in (0, 2):
                gb.solve_multi(sysm, Bm, tol=1e-8, maxit=20000, precision=p)
                X, its, r = gb.solve_multi(sysm, Bm, tol=1e-8, maxit=20000, precision=p)
                line[f"{tag}precision{p}"] = {
                    "ms": round(r["device_ms"], 2), "max_iters": int(its.max()), "flag": r["flag"],
                    "rel_true_res_max": r["rel_true_res"],
                    "rel_err_vs_fp64": float(torch.linalg.norm(X - X64) / torch.linalg.norm(X64))}
            os.environ.pop("GBLAP_MULTI_FORM", None)
        tune = gb.autotune_multi(sysm, Bm, iters=16)  # columns per interleaved chunk, by timing
        line["autotune"] = dict(tune)
        for p in (0, 2):
            gb.solve_multi(sysm, Bm, tol=1e-8, maxit=20000, precision=p)
            X, its, r = gb.solve_multi(sysm, Bm, tol=1e-8, maxit=20000, precision=p)
            line["autotune"][f"precision{p}_ms"] = round(r["device_ms"], 2)
            line["autotune"][f"precision{p}_rel_err_vs_fp64"] = float(torch.linalg.norm(X - X64) /
                                                                      torch.linalg.norm(X64))
        ms = 0.0
        for k in range(Bm.shape[0]):
            _, rs = sysm.solve(Bm[k], tol=1e-8, maxit=20000)
            ms += rs["device_ms"]
        line["one_by_one_device_ms"] = round(ms, 2)
    elif wl == "adjoint1024":
        nside = 1024
        ei, ej, w = gen.grid2d_aniso_edges(nside, seed=1006)
        A = gen.laplacian_from_edges(nside * nside, ei, ej, w, shift=1e-2)
        rng = np.random.default_rng(1006)
        xs = torch.from_numpy(rng.standard_normal(A.n)).cuda()
        b = torch.from_numpy(rng.uniform(-1, 1, A.n)).cuda()
        line["config"] = ("1024^2 anisotropic lognormal grid + 1e-2 I, ichol, loss 0.5||x-x*||^2; forward and "
                          "adjoint in split precision (tol 1e-10); central differences h=1e-6 (FP64, tol 1e-13) "
                          "and the reference CPU PCG's own adjoint (FP64 IC(0), tol 1e-10) on the same random edges")
        sysm = gb.System.from_csr(A, "ichol")
        kw = dict(tol=1e-10, maxit=20000, precision=2)
        sysm.solve(b, **kw)
        x, rf = sysm.solve(b, **kw)
        lam, G, eg, ra = sysm.adjoint(x, (x - xs).contiguous(), **kw)
        line["forward_ms"], line["adjoint_ms"] = round(rf["device_ms"], 2), round(ra["device_ms"], 2)
        line["iters"] = [rf["iters"], ra["iters"]]
        lo, hi, p_lh, p_hl, diag, t_of_edge = _edge_positions(A, ei, ej)
        a0 = torch.from_numpy(A.a).cuda()
        edges = np.random.default_rng(1007).choice(len(w), args.fd_edges, replace=False)
        fds, ads = [], []
        for e in edges:
            vals = []
            for sgn in (1.0, -1.0):
                a = a0.clone()
                d = sgn * 1e-6
                a[int(p_lh[e])] -= d
                a[int(p_hl[e])] -= d
                a[int(diag[lo[e]])] += d
                a[int(diag[hi[e]])] += d
                sysm.set_values(a)
                xe, _ = sysm.solve(b, tol=1e-13, maxit=50000, precision=0)
                vals.append(0.5 * float(torch.sum((xe - xs) ** 2)))
            fds.append((vals[0] - vals[1]) / 2e-6)
            ads.append(float(eg[int(t_of_edge[e])]))
        sysm.set_values(a0)
        fds, ads = np.array(fds), np.array(ads)
        line["fd_edges"] = int(args.fd_edges)
        line["fd_abs_err_max_over_max_grad"] = float(np.abs(fds - ads).max() / np.abs(ads).max())
        line["fd_rel_err_median"] = float(np.median(np.abs(fds - ads) / np.abs(ads)))
        # the reference's CPU PCG (the oracle, FP64 IC(0)) for the forward and
        # the adjoint solve; its gradient on the same edges and its dL/db
        import oracle

        t2 = time.time()
        bn, xsn = b.cpu().numpy(), xs.cpu().numpy()
        ref_f = oracle.solve(A.n, A.ia, A.ja, A.a, bn, "ichol", 1e-10, 20000)
        ref_a = oracle.solve(A.n, A.ia, A.ja, A.a, ref_f["x"] - xsn, "ichol", 1e-10, 20000)
        xr, lr = ref_f["x"], ref_a["x"]
        g_ref = np.array([-(lr[lo[e]] - lr[hi[e]]) * (xr[lo[e]] - xr[hi[e]]) for e in edges])
        lam_np = lam.cpu().numpy()
        line["reference_adjoint"] = {
            "iters": [ref_f["iters"], ref_a["iters"]], "cpu_s": round(time.time() - t2, 1),
            "grad_abs_err_max_over_max_grad": float(np.abs(ads - g_ref).max() / np.abs(g_ref).max()),
            "grad_rel_err_median": float(np.median(np.abs(ads - g_ref) / np.abs(g_ref))),
            "dL_db_rel_err": float(np.linalg.norm(lam_np - lr) / np.linalg.norm(lr)),
            "fd_vs_reference_grad_max_over_max_grad": float(np.abs(fds - g_ref).max() / np.abs(g_ref).max())}
    else:
        raise SystemExit(f"unknown workload {wl}")
    line["wall_s"] = round(time.time() - t0, 1)
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch

    import lap_gb300 as gb

    torch.cuda.set_device(local)
    A, b = make_workload(args.size)
    n, nnz = A.n, A.nnz
    sysm = gb.System.from_csr(A, "ichol")
    info = sysm.info()
    db = torch.from_numpy(b).cuda()
    kw = dict(tol=args.tol, maxit=20000)

    # warm-up: graphs captured, clocks up
    for _ in range(args.warmup):
        sysm.solve(db, precision=MIXED, **kw)
        sysm.solve(db, precision=0, **kw)
    sysm.solve(db, precision=1, **kw)

    def timed(precision, steps):
        ms, res = [], None
        barrier(world)
        torch.cuda.synchronize()
        for _ in range(steps):
            x, res = sysm.solve(db, precision=precision, **kw)
            ms.append(res["device_ms"])
        torch.cuda.synchronize()
        barrier(world)
        return ms, res, x

    with ClockSampler(local) as clk:
        t0 = time.time()
        ms_mixed, r_mixed, x_mixed = timed(MIXED, args.steps)
        wall = time.time() - t0
    ms_fp64, r_fp64, x_fp64 = timed(0, max(2, args.steps // 2))
    ms_f32k, r_f32k, x_f32k = timed(1, 2)
    err_vs_fp64 = float(torch.linalg.norm(x_mixed - x_fp64) / torch.linalg.norm(x_fp64))

    # end to end from pinned host buffers
    bh = torch.from_numpy(b).pin_memory()
    xh = torch.zeros(n, dtype=torch.float64).pin_memory()
    e2e = []
    for _ in range(args.steps):
        xh.zero_()
        r = gb.PcgResult()
        o = gb.opts(precision=MIXED, **kw)
        gb.check(gb.lib().gb_pcg_solve_host(sysm.h, bh.data_ptr(), xh.data_ptr(), gb.C.byref(o),
                                            gb.C.byref(r)), "gb_pcg_solve_host")
        e2e.append(r.device_ms)

    # per-kernel device time of one iteration (CUDA events on the solver stream)
    peak, peak_kind = measured_peak()
    pname = {0: "fp64", 1: "fp32-krylov", 2: "split"}
    prof = {p: sysm.profile(db, precision=p, iters=20) for p in (0, 1, 2)}
    traffic = ncu_traffic()
    kernels = []
    for p, lst in prof.items():
        for k in lst:
            gbs = k["bytes"] / (k["ms"] * 1e-3) / 1e9 if k["ms"] > 0 else 0.0
            kernels.append({"kernel": k["name"], "precision": pname[p],
                            "ms": round(k["ms"], 5), "bytes": k["bytes"], "gbs": round(gbs, 1),
                            "frac": round(gbs / peak, 4)})
    src = f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s"

    def roof(k):
        return {"bound": "hbm", "kernel": k["kernel"], "precision": k["precision"],
                "achieved": k["gbs"], "peak": peak, "unit": "GB/s", "frac": k["frac"],
                "traffic": traffic.get(f"{k['kernel']}:{k['precision']}"), "peak_source": src}

    mixed_k = [k for k in kernels if k["precision"] == pname[MIXED]]
    dom = max(mixed_k, key=lambda k: k["ms"])  # a triangular solve: dependency-latency bound
    roofline = roof(dom)
    # the bandwidth-bound kernels of the same iteration (SpMV + fused vector updates)
    bw = {k["kernel"]: roof(k) for k in kernels
          if k["precision"] in ("fp64", pname[MIXED]) and k["kernel"] in ("spmv_pq", "spmv_pq_split", "update")}

    v = allmax(world, statistics.mean(ms_mixed))
    v64 = allmax(world, statistics.mean(ms_fp64))
    v32k = allmax(world, statistics.mean(ms_f32k))
    ve2e = allmax(world, statistics.mean(e2e))
    if rank != 0:
        return
    it_in, outer = r_mixed["iters"], r_mixed["outer"]
    # our kernels per split-precision solve: first outer residual 1, prologue 4
    # (residual, sentinel fill, lower, upper), 4 per iteration (one graph body:
    # spmv_pq_split, update, lower, upper), an outer residual after each of the
    # `outer` pauses, 4 per resume (resume, fill, lower, upper; all pauses but
    # the last), final true residual 1
    # our kernels per split solve: the first FP64 residual; the prologue
    # (residual, sentinel fill, the two triangular solves, r'w); 5 per
    # iteration (SpMV, update, the two solves, r'w); per replacement its
    # FP64 residual and, unless it ends the solve, the resume (state reset,
    # sentinel fill, solves, r'w); the final true residual
    launches_mixed = 1 + 5 + 5 * it_in + outer + 5 * max(outer - 1, 0) + 1
    line = {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 SpMV + IC0 solves / f64 Krylov recurrence", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": WORKLOAD, "n": n, "nnz": nnz, "preconditioner": "ichol",
                       "precision": "FP64 PCG recurrence around FP32 SpMV and FP32 IC(0) triangular "
                                    "solves, FP64 residual replacement (gb_pcg_opts.precision=2)",
                       "l2": "inputs larger than L2 (no flush)",
                       "lower_levels": info["lower_levels"], "upper_levels": info["upper_levels"],
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "mixed": {"ms": round(v, 4), "iters": it_in, "replacements": outer,
                      "rel_true_res": r_mixed["rel_true_res"], "rel_err_vs_fp64_solution": err_vs_fp64},
            "fp64": {"ms": round(v64, 4), "iters": r_fp64["iters"], "rel_true_res": r_fp64["rel_true_res"]},
            "fp32_krylov": {"ms": round(v32k, 4), "iters": r_f32k["iters"], "outer": r_f32k["outer"],
                            "rel_true_res": r_f32k["rel_true_res"]},
            "speedup_mixed_vs_fp64": round(v64 / v, 3),
            "solves_per_s_all_gpus": round(world * 1e3 / v, 3),
            "e2e": {"value": round(ve2e, 4), "unit": UNIT, "steps_ms": [round(v, 2) for v in e2e],
                    "h2d_bytes_per_step": 2 * 8 * n,
                    "d2h_bytes_per_step": 8 * n},
            "roofline": roofline, "roofline_bandwidth_kernels": bw, "kernels": kernels,
            "gpu_launches": launches_mixed * args.steps,
            "clocks": clk.summary(), "wall_s_timed": round(wall, 3)}
    if world == 1 and not args.no_cpu_baseline:
        # the reference's CPU PCG on the same system: the measured CPU
        # baseline, and what every GPU solve's x and iteration count are
        # checked against
        ref = reference_solve(A, b, "ichol", args.tol)
        line["cpu_baseline"] = cpu_baseline(ref)
        line["parity"] = {
            "reference": "oracle: C restatement of LAP's serial PCG (cg.c, simple_blas.c), pinned bit for bit "
                         "to LAP's own compiled code on the golden fixtures; same system, b, tol, x0 = 0",
            "bar": "x within 1e-6 relative of the reference's x; iterations within +-2% (GS / IC0)",
            "ichol": {"ref_iters": ref["iters"], "ref_flag": ref["flag"],
                      "fp64": parity_entry(ref, x_fp64, r_fp64),
                      "mixed": parity_entry(ref, x_mixed, r_mixed),
                      "fp32_krylov": parity_entry(ref, x_f32k, r_f32k)}}
        if not args.no_gs_parity:
            line["parity"]["GS_std"] = gs_parity(A, b, db, args.tol)
    print(json.dumps(line), flush=True)


def gs_parity(A, b, db, tol):
    """GS_std (M = K = 1) on the headline system in the three precision modes,
    against the reference's CPU GS_std-PCG."""
    import lap_gb300 as gb

    sg = gb.System.from_csr(A, "GS_std")
    res = {}
    for p in (0, 1, 2):
        sg.solve(db, precision=p, tol=tol, maxit=20000)  # graph capture
        res[p] = sg.solve(db, precision=p, tol=tol, maxit=20000)
    sg.close()
    ref = reference_solve(A, b, "GS_std", tol)
    out = {"ref_iters": ref["iters"], "ref_flag": ref["flag"], "ref_cpu_ms_1core": round(ref["solve_s"] * 1e3, 1)}
    for p, name in ((0, "fp64"), (2, "mixed"), (1, "fp32_krylov")):
        x, r = res[p]
        out[name] = dict(parity_entry(ref, x, r), ms=round(r["device_ms"], 3))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU reference solves (baseline and parity)")
    ap.add_argument("--no-gs-parity", action="store_true", help="skip the GS_std parity solves")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only the eager per-kernel profile of each precision mode (for ncu)")
    ap.add_argument("--profile-iters", type=int, default=3)
    ap.add_argument("--workload", default="ichol128",
                    choices=["ichol128", "jacobi256", "chunglu4m", "batch512", "multirhs32", "multirhs64", "adjoint1024",
                             "mmread128"],
                    help="ichol128 is the headline line; the others are the remaining configurations")
    ap.add_argument("--fd-edges", type=int, default=64)
    ap.add_argument("--profile-precisions", default="0,1,2",
                    help="--kernels-only: precision modes to run (comma list of 0, 1, 2)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.kernels_only:
        run_kernels_only(args, local)
    elif args.workload != "ichol128":
        run_workload(args, local)
    else:
        import __graft_entry__

        __graft_entry__.build() if not os.path.exists(os.path.join(ROOT, "lap_gb300", "libgblap.so")) else None
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
