#!/usr/bin/env python3
"""Time-to-1e-4 relative KKT of the restarted Halpern PDHG solve on GB300.

Workload (default): the 20M-nnz power-law LP -- m = 1,000,000 constraints,
n = 2,000,000 variables, column degrees rank-Zipf(1.2) capped at 50,000, rows
uniform within a column, values N(0,1) with 5% +-1, feasible bounds from
x0 ~ U[0,1] (30% equality rows), 0 <= x <= 10, c ~ U[-1,1], seed 1.  Solved
to eps 1e-4 with the reference defaults (Ruiz 10, Pock-Chambolle 1,
evaluation every 200 iterations), presolve off: FP32 PDHG with FP64
refinement (the headline), and plain FP64 beside it.

One step = one full solve (GPU rescaling, power method, PDHG loop, result).
  value : seconds per solve with the LP already resident in HBM
          (CUDA events on the solve's stream, mean over the timed steps)
  e2e   : seconds per solve through solve_lp_problem() from host arrays
          (upload, transpose and result copy-back inside the timed region)
The matrices (480 MB) and vectors exceed the 129 MB L2, so no flush is
needed between steps.

--impl reference times the reference's own single-GPU FP64 solve (its
cuSPARSE/cuBLAS code built from its sources for sm_103a) on the same seeded
LP through its solve_lp_problem, one full solve per step; the FP64 oracle on
the host cores is reported as cpu_baseline.
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
sys.path.insert(0, os.path.join(ROOT, "d-pdlp_gb300"))

METRIC = "time-to-1e-4 rel KKT (FP32+refine vs FP64); batched LPs/s; p50/p99 latency"

WORKLOADS = {
    "powerlaw_m1M_n2M_nnz20M_seed1": {
        "kind": "powerlaw", "args": (1000000, 2000000, 20000000, 1.2, 50000, 1),
        "desc": "power-law LP m=1,000,000 n=2,000,000 nnz~20M Zipf(1.2) cap 50,000, seed 1",
    },
    "transport_2000x5000_seed2": {
        "kind": "transport", "args": (2000, 5000, 2),
        "desc": "transportation LP 2,000 sources x 5,000 sinks (n=10M, m=7,000, nnz=20M), seed 2",
    },
    "random_m2k_n5k_nnz20k_seed0": {
        "kind": "random", "args": (2000, 5000, 20000, 0),
        "desc": "random LP m=2,000 n=5,000 nnz=20,000, seed 0",
    },
}
DEFAULT_WORKLOAD = "powerlaw_m1M_n2M_nnz20M_seed1"

# Many independent LPs: each generated as the random LP above, with m
# log-uniform in [1,000, 100,000], n = 2.5 m and 10 non-zeros per column.
BATCH_WORKLOADS = {
    "batch_random_512_seed100": {
        "lps": 512, "seed0": 100,
        "desc": "512 random LPs (seeds 100..611), m log-uniform in [1e3, 1e5], n = 2.5 m, "
                "10 nnz per column, FP64, eps 1e-4",
    },
}
# Open-loop serving: Poisson arrivals; each request is drawn from a seeded
# pool of LPs with the batch distribution, 10% of them large (m = 200,000,
# n = 500,000, nnz = 5M).
SERVE_WORKLOADS = {
    "serve_poisson_seed7": {
        "seed": 7, "rate": 200.0, "duration": 60.0, "pool_small": 2000, "pool_large": 50,
        "queue_bytes": 4 << 30,
        "desc": "Poisson arrivals at 200/s for 60 s (seed 7); each request an LP from the "
                "batch distribution (m log-uniform in [1e3, 1e5], n = 2.5 m, 10 nnz per "
                "column), 10% of them large (m=200,000 n=500,000 nnz=5M), eps 1e-4",
    },
}

def C_byref(obj):
    import ctypes
    return ctypes.byref(obj)


def gpu_visible() -> bool:
    """A CUDA GPU is visible to this process (nvidia-smi lists one)."""
    try:
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=30)
    except (OSError, subprocess.SubprocessError):
        return False
    return r.returncode == 0 and "GPU" in r.stdout


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def visible_device_for_rank(local: int, visible: str | None) -> str:
    """The one GPU a replica rank uses: entry `local` of CUDA_VISIBLE_DEVICES
    (or of 0..63 when unset); the solver library then sees it as device 0."""
    devs = visible.split(",") if visible else [str(i) for i in range(64)]
    return devs[local]


def max_over_ranks(values: list[float]) -> list[float]:
    """Element-wise max over all ranks of the default process group (NCCL on
    GPUs, gloo on CPU); returns `values` unchanged without a process group."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(values, dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def make_problem(cp, name):
    w = WORKLOADS[name]
    return cp.Problem.generated(w["kind"], *w["args"])


def make_oracle_problem(name):
    """The same seeded LP from the oracle library's copy of the generators,
    for the baseline arms (they load nothing of the product library)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    w = WORKLOADS[name]
    return oracle_lib.OracleProblem(w["kind"], *w["args"])


def single_config(name, m, n, nnz, eps, world):
    """`config` of a single-LP line, identical in both arms."""
    return {"workload": name, "description": WORKLOADS[name]["desc"], "m": m, "n": n,
            "nnz": nnz, "eps": eps,
            "termination": "relative primal and dual residuals and gap below eps, FP64 KKT "
                           "of the original LP",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "inputs (A and A^T, 480 MB at 20M nnz) larger than L2; no flush needed"}


def params_for(cp, eps=1e-4):
    p = cp.default_parameters()
    p.presolve = False
    p.termination_criteria.eps_optimal_relative = eps
    p.termination_criteria.eps_feasible_relative = eps
    return p


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names[1:], parts[5:9]):
                    if v.lower() in ("active", "1", "yes"):
                        reasons.add(nm)
        os.unlink(self.path)
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def kernel_bytes(m, n, nnz, s=8):
    """Algorithmic bytes per launch of the two iteration kernels (values and
    vectors of s bytes, int32 indices, each vector touched once)."""
    primal = (s + 4) * nnz + 4 * (n + 1) + s * m + 7 * s * n   # A^T stream, gather y, 5 reads + 2 writes of n
    dual = (s + 4) * nnz + 4 * (m + 1) + s * n + 5 * s * m     # A stream, gather x_ref, 4 reads + 1 write of m
    return primal, dual


def load_traffic(workload, precision, kernel):
    """DRAM bytes per launch of a step kernel from one ncu capture
    (profiles/ncu_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            d = json.load(f)
        e = d.get(workload, {}).get(precision, {}).get(kernel)
        return None if e is None else float(e["dram_bytes_per_launch"])
    except (ValueError, KeyError, TypeError):
        return None


def cpu_sample(name, params, iters_total, power_total, loop_iters=300, power_iters=10):
    """CPU baseline: the FP64 oracle (OpenMP on every host core) on the same
    seeded LP, generated by the oracle library.  Measured: rescaling and
    transpose once, `power_iters` power-method iterations and `loop_iters`
    iterations of the driver loop (evaluations, restarts and all) on the full
    LP; the solve time is projected from them to `iters_total` iterations (the
    count the GPU arm measured: the oracle runs the same schedule, and its
    counts equal the GPU's and the reference's on the configured LPs).  A
    workload that the oracle solves within a few seconds is solved to the end
    instead.  Returns (seconds, description, parts)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import ctypes as C

    import cupdlpx as cpy  # ctypes structures only; the product library is not loaded
    import oracle_lib
    O = oracle_lib.load()
    prob = make_oracle_problem(name)
    if WORKLOADS[name]["kind"] == "random":
        t0 = time.perf_counter()
        r, _ = oracle_lib.oracle_solve(O, prob, params)
        el = time.perf_counter() - t0
        return el, (f"full FP64 oracle solve of the LP ({r['total_count']} iterations, "
                    f"{r['status']})"), {"iterations": r["total_count"], "measured": True}
    O.oracle_session_create.restype = C.c_void_p
    O.oracle_session_create.argtypes = [C.POINTER(cpy.LpProblem), C.POINTER(cpy.PdhgParameters),
                                        C.c_int, cpy._dp]
    O.oracle_session_power.restype = C.c_double
    O.oracle_session_power.argtypes = [C.c_void_p, C.c_int]
    O.oracle_session_iterate.restype = C.c_double
    O.oracle_session_iterate.argtypes = [C.c_void_p, C.c_int]
    O.oracle_session_free.argtypes = [C.c_void_p]
    setup = C.c_double()
    sess = O.oracle_session_create(prob.ptr, C.byref(params), 0, C.byref(setup))
    try:
        pw = O.oracle_session_power(sess, power_iters) / power_iters
        it = O.oracle_session_iterate(sess, loop_iters) / loop_iters
    finally:
        O.oracle_session_free(sess)
        prob.free()
    total = setup.value + pw * power_total + it * iters_total
    desc = (f"measured on the full LP: rescaling + transpose {setup.value:.2f} s, "
            f"{power_iters} power iterations ({pw * 1e3:.2f} ms each), {loop_iters} "
            f"iterations of the driver loop ({it * 1e3:.2f} ms each); value = projection to "
            f"{iters_total} iterations and {power_total} power iterations, not a full run")
    return total, desc, {"setup_s": round(setup.value, 3), "power_ms": round(pw * 1e3, 3),
                         "iter_ms": round(it * 1e3, 3), "measured_iterations": loop_iters,
                         "projected_iterations": iters_total, "measured": False}


def run_ours(args, cp, rank, world, local):
    L = cp.lib()
    name = args.workload
    prob = make_problem(cp, name)
    a = prob.arrays()
    m, n, nnz = a["m"], a["n"], a["nnz"]
    params = params_for(cp, args.eps)
    prec = {"fp32": cp.PRECISION_FP32_REFINE, "fp32m": cp.PRECISION_FP32_MATRIX,
            "fp64": cp.PRECISION_FP64}[args.precision]
    dp = cp.DeviceProblem(prob)
    first_info = {}
    for i in range(args.warmup):
        out = dp.solve(params, precision=prec)
        if i == 0:
            first_info = out.info
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    dev_s, wall_s, launches, last = [], [], 0, None
    live = [0.0, 0.0, 0]  # in-loop primal ms x chunks, dual ms x chunks, chunks
    fp64 = None
    with ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0])
                      if world > 1 else 0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = dp.solve(params, precision=prec)
            wall_s.append(time.perf_counter() - t0)
            dev_s.append(out.info["device_seconds"])
            launches += out.info["kernel_launches"]
            k = out.info["timed_chunks"]
            live[0] += out.info["primal_step_ms"] * k
            live[1] += out.info["dual_step_ms"] * k
            live[2] += k
            last = out
        # end-to-end through the public C API from host arrays
        e2e_s = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            eo = cp.solve(prob, params, precision=prec)
            e2e_s.append(time.perf_counter() - t0)
        if prec != cp.PRECISION_FP64 and args.fp64_steps > 0:
            # the plain FP64 solve of the same LP, for the FP32-vs-FP64 half of the metric
            f_dev, f_last = [], None
            for i in range(args.fp64_steps + 1):
                fo = dp.solve(params, precision=cp.PRECISION_FP64)
                if i:
                    f_dev.append(fo.info["device_seconds"])
                    f_last = fo
            fp64 = {"value": round(statistics.mean(f_dev), 4), "unit": "s", "steps": len(f_dev),
                    "warmup": 1, "iterations": f_last.result["total_count"],
                    "status": f_last.result["status"],
                    "primal_obj": f_last.result["primal_objective_value"],
                    "us_per_iteration": round(f_last.info["loop_seconds"] /
                                              max(1, f_last.result["total_count"]) * 1e6, 2),
                    "speedup_of_headline": round(statistics.mean(f_dev) / statistics.mean(dev_s),
                                                 3)}
            # error of the headline result against the FP64 solve (whose
            # iterates equal the reference's on the configured LPs)
            a, b = last.result, f_last.result
            rel = lambda u, v: abs(u - v) / (1.0 + abs(v))
            vrel = lambda u, v: float(abs(u - v).max() / (1.0 + abs(v).max())) if len(v) else 0.0
            err = lambda a, b: {
                "primal_obj_rel": rel(a["primal_objective_value"], b["primal_objective_value"]),
                "dual_obj_rel": rel(a["dual_objective_value"], b["dual_objective_value"]),
                "x_rel_max": vrel(a["x"], b["x"]), "y_rel_max": vrel(a["y"], b["y"])}
            fp64["error_of_headline_vs_fp64"] = err(a, b)
            if args.fp64_oracle_eps:
                # untimed FP64 solve to a tighter tolerance: the FP64 oracle
                # of the result (the configured mixed-precision comparison)
                op = params_for(cp, args.fp64_oracle_eps)
                oo = dp.solve(op, precision=cp.PRECISION_FP64)
                fp64["oracle"] = {
                    "eps": args.fp64_oracle_eps, "status": oo.result["status"],
                    "iterations": oo.result["total_count"],
                    "seconds": round(oo.info["device_seconds"], 3),
                    "error_of_headline": err(a, oo.result),
                    "error_of_fp64": err(b, oo.result)}
    clocks = clk.summary()
    value, e2e_mean = max_over_ranks([statistics.mean(dev_s), statistics.mean(e2e_s)])
    r = last.result
    ms = dp.time_kernels(params, reps=args.kernel_reps, precision=prec)
    pb, db = kernel_bytes(m, n, nnz, 8)
    if prec == cp.PRECISION_FP32_REFINE:
        pb, db = kernel_bytes(m, n, nnz, 4)
    elif prec == cp.PRECISION_FP32_MATRIX:  # 4-byte values, 8-byte vectors
        pb -= 4 * nnz
        db -= 4 * nnz
    if live[2] > 0:
        # CUDA events on the solve's stream inside the timed solves
        kernels = {"primal_step": (live[0] / live[2], pb), "dual_step": (live[1] / live[2], db)}
        timing = (f"CUDA events inside the {args.steps} timed solves on the solver's stream: one "
                  f"ordinary primal and dual launch per 100-iteration chunk, {live[2]} chunks")
    else:
        kernels = {"primal_step": (ms[0], pb), "dual_step": (ms[1], db)}
        timing = f"CUDA events on the solver's stream over {args.kernel_reps} isolated launches"
    dom = max(kernels, key=lambda k: kernels[k][0])
    peak, peak_kind = load_peaks()
    ach = kernels[dom][1] / (kernels[dom][0] * 1e-3) / 1e9
    iters, pm_iters = r["total_count"], last.info["power_iterations"]
    # uploaded by solve_lp_problem: A and A^T (CSR), c, bounds, power start vector
    h2d = 4 * (m + 1) + 4 * (n + 1) + 24 * nnz + 24 * n + 16 * m + 8 * m
    d2h = 8 * (2 * n + m)  # primal, reduced cost, dual
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value * 1e3, 2),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {cp.PRECISION_FP32_REFINE: "f32 iterates + f64 KKT/refinement",
                  cp.PRECISION_FP32_MATRIX: "f32 matrix/SpMV + f64 iterates/KKT/refinement",
                  cp.PRECISION_FP64: "f64"}[prec],
        "data": "synthetic (seeded generator, no dataset)",
        "config": single_config(name, m, n, nnz, args.eps, world),
        "precision": {
            cp.PRECISION_FP32_REFINE: "FP32 PDHG + FP64 iterative refinement",
            cp.PRECISION_FP32_MATRIX: "FP32 matrix and SpMVs, FP64 iterates + FP64 iterative "
                                      "refinement",
            cp.PRECISION_FP64: "FP64 plain PDHG"}[prec],
        "e2e": {"value": round(e2e_mean, 4), "unit": "s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "api": "solve_lp_problem (pageable host arrays)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(ach / peak, 4),
                     "traffic": load_traffic(name, args.precision, dom),
                     "peak_source": f"{peak_kind} hbm_gbs (STREAM copy; the only HBM figure "
                                    "measured)",
                     "algorithmic_bytes_per_launch": kernels[dom][1],
                     "ms_per_launch": round(kernels[dom][0], 4),
                     "other_kernels": {k: {"ms": round(v[0], 4), "bytes": v[1],
                                           "gbs": round(v[1] / (v[0] * 1e-3) / 1e9, 1)}
                                       for k, v in kernels.items()},
                     "timing": timing,
                     "isolated_ms": {"primal_step": round(ms[0], 4), "dual_step": round(ms[1], 4),
                                     "eval_A": round(ms[2], 4), "eval_AT": round(ms[3], 4)}},
        "spmv_kernels": {"A": ["fused", "pipelined"][out.info["spmv_kernel_A"]],
                         "A^T": ["fused", "pipelined"][out.info["spmv_kernel_AT"]],
                         "chosen_by": "timing both on the step kernels at the problem's first "
                                      "solve (ms per launch: A fused, A pipelined, A^T fused, "
                                      "A^T pipelined)",
                         "tune_ms": [round(v, 4) for v in first_info.get("tune_ms", [])]},
        "solve": {"status": r["status"], "iterations": iters, "power_iterations": pm_iters,
                  "rel_primal": r["relative_primal_residual"],
                  "rel_dual": r["relative_dual_residual"], "rel_gap": r["relative_objective_gap"],
                  "primal_obj": r["primal_objective_value"], "dual_obj": r["dual_objective_value"],
                  "wall_s_per_step": round(statistics.mean(wall_s), 4),
                  "loop_s": round(last.info["loop_seconds"], 4),
                  "setup_s": round(last.info["setup_seconds"], 4),
                  "power_s": round(last.info["power_seconds"], 4),
                  "us_per_iteration": round(last.info["loop_seconds"] / max(iters, 1) * 1e6, 2)},
        "clocks": clocks,
    }
    if fp64 is not None:
        line["fp64"] = fp64
    if prec != cp.PRECISION_FP64:
        line["solve"]["refinement_rounds"] = last.info["refinement_rounds"]
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU oracle runs the FP64 algorithm: extrapolate with the FP64 iteration count
        f_iters = fp64["iterations"] if fp64 is not None else iters
        cpu_v, desc, parts = cpu_sample(name, params, f_iters, pm_iters)
        line["cpu_baseline"] = {"value": round(cpu_v, 2), "unit": "s", "cores": os.cpu_count(),
                                "kind": "port", "sample": desc, "parts": parts}
    dp.free()
    return line


def run_kernels_only(args, cp):
    """Upload the workload and time the four iteration-kernel kinds alone
    (CUDA events over --kernel-reps launches each): a short command with few
    launches, for profilers."""
    prob = make_problem(cp, args.workload)
    params = params_for(cp, args.eps)
    prec = {"fp32": cp.PRECISION_FP32_REFINE, "fp32m": cp.PRECISION_FP32_MATRIX,
            "fp64": cp.PRECISION_FP64}[args.precision]
    dp = cp.DeviceProblem(prob)
    ms = dp.time_kernels(params, reps=args.kernel_reps, precision=prec)
    dp.free()
    print(json.dumps({"workload": args.workload, "precision": args.precision,
                      "kernel_reps": args.kernel_reps,
                      "ms_per_launch": {"primal_step": ms[0], "dual_step": ms[1],
                                        "eval_A": ms[2], "eval_AT": ms[3]}}))


PRECISIONS = {"fp32": 1, "fp32m": 2, "fp64": 0}
DTYPES = {"fp32": "f32 iterates + f64 KKT/refinement",
          "fp32m": "f32 matrix/SpMV + f64 iterates/KKT/refinement", "fp64": "f64"}


def batch_shapes(count, seed0):
    """(m, n, nnz, seed) of the batch workload's LPs."""
    import numpy as np
    rng = np.random.default_rng(seed0)
    out = []
    for i in range(count):
        m = int(np.exp(rng.uniform(np.log(1e3), np.log(1e5))))
        n = int(2.5 * m)
        out.append((m, n, 10 * n, seed0 + i))
    return out


def generate_parallel(cp, shapes, threads=None):
    """Generate random LPs on host threads (the generator releases the GIL)."""
    import concurrent.futures as cf
    threads = threads or min(32, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(threads) as ex:
        return list(ex.map(lambda sh: cp.Problem.generated("random", *sh), shapes))


def run_batch(args, cp):
    """Batched LPs/s of pdlp_batch_solve against the same LPs solved one after
    another through solve_lp_problem."""
    w = BATCH_WORKLOADS[args.workload]
    count = args.batch_lps or w["lps"]
    shapes = batch_shapes(count, w["seed0"])
    lps = generate_parallel(cp, shapes)
    nnz_total = sum(sh[2] for sh in shapes)
    params = params_for(cp, args.eps)
    prec = PRECISIONS[args.precision]
    for _ in range(args.warmup):
        cp.batch_solve(lps, params, precision=prec, workers=args.workers)
    vals, iters = [], 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            res, info = cp.batch_solve(lps, params, precision=prec, workers=args.workers)
            vals.append(info["lps_per_second"])
            iters = info["iterations"]
            failed = info["failed"]
    clocks = clk.summary()
    statuses = sorted({r["status"] for r in res if r is not None})
    worst = max(max(r["relative_primal_residual"], r["relative_dual_residual"],
                    r["relative_objective_gap"]) for r in res if r is not None)
    fp64_batch = None
    if prec != cp.PRECISION_FP64:
        r64, i64 = cp.batch_solve(lps, params, workers=args.workers)
        fp64_batch = {"lps_per_second": round(i64["lps_per_second"], 2),
                      "iterations": i64["iterations"]}
    # the same LPs one after another (our FP64 path, one stream)
    t0 = time.perf_counter()
    seq = [cp.solve(lp, params).result for lp in lps]
    t_seq = time.perf_counter() - t0
    if prec == cp.PRECISION_FP64:
        same = all(a is not None and a["total_count"] == b["total_count"]
                   for a, b in zip(res, seq))
    else:  # FP32 + refinement against the FP64 solves: objectives within eps
        same = all(a is not None and abs(a["primal_objective_value"] - b["primal_objective_value"])
                   <= 10 * args.eps * (1 + abs(b["primal_objective_value"]))
                   for a, b in zip(res, seq))
    value = statistics.mean(vals)
    # work done: non-zeros x iterations summed over the LPs (one iteration
    # is one pass over A and one over A^T), as a rate against each path's time
    nnz_it = sum(sh[2] * r["total_count"] for sh, r in zip(shapes, res) if r is not None)
    nnz_it_seq = sum(sh[2] * r["total_count"] for sh, r in zip(shapes, seq) if r is not None)
    # the reference's own single-GPU FP64 solve, LP after LP in batch order
    # (a fresh process each), for about a minute: sequential LPs/s
    ref_seq = None
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    if oracle_lib.ref_gpu_available() and gpu_visible() and args.ref_seconds > 0:
        t0, k, solve_s = time.perf_counter(), 0, 0.0
        try:
            while k < count and time.perf_counter() - t0 < args.ref_seconds:
                solve_s += oracle_lib.ref_gpu_solve(lps[k], eps=args.eps, timeout=600)["wall_s"]
                k += 1
            el = time.perf_counter() - t0
            ref_seq = {"lps_per_second": round(k / solve_s, 3), "lps": k,
                       "solve_seconds": round(solve_s, 2), "process_seconds": round(el, 2),
                       "api": "the reference's solve_lp_problem (single-GPU FP64 build), one "
                              "process per LP, the first LPs of the batch in order; LPs/s "
                              "over the solve_lp_problem calls alone (process start and CUDA "
                              "context creation excluded)"}
        except (RuntimeError, OSError) as e:
            ref_seq = {"unavailable": str(e)[:200]}
    cpu = None
    if not args.no_cpu_baseline:
        # the FP64 oracle on every host core, LPs in batch order for ~15 s
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib
        O = oracle_lib.load()
        t0, k = time.perf_counter(), 0
        while k < count and time.perf_counter() - t0 < 15.0:
            oracle_lib.oracle_solve(O, lps[k], params)
            k += 1
        el = time.perf_counter() - t0
        cpu = {"value": round(k / el, 3), "unit": "LPs/s", "cores": os.cpu_count(),
               "kind": "port", "sample": f"the first {k} LPs of the batch solved by the FP64 "
                                         f"oracle in {el:.1f} s"}
    line = {
        "metric": "batched LPs/s", "value": round(value, 2), "unit": "LPs/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(count / value * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": args.workload, "description": w["desc"], "lps": count,
                   "precision": args.precision,
                   "nnz_total": nnz_total, "workers": args.workers, "eps": args.eps,
                   "l2": "inputs larger than L2; no flush needed"},
        "e2e": {"value": round(value, 2), "unit": "LPs/s",
                "h2d_bytes_per_step": int(sum(24 * sh[2] + 32 * sh[1] + 20 * sh[0]
                                              for sh in shapes)),
                "d2h_bytes_per_step": int(sum(8 * (2 * sh[1] + sh[0]) for sh in shapes)),
                "api": "pdlp_batch_solve from host arrays (upload, solve, copy-back per LP)"},
        "sequential": {"lps_per_second": round(count / t_seq, 2), "seconds": round(t_seq, 2),
                       "nnz_iterations": nnz_it_seq,
                       "g_nnz_iterations_per_s": round(nnz_it_seq / t_seq / 1e9, 2),
                       "api": "solve_lp_problem, one LP after another"},
        "reference_sequential": ref_seq,
        "batch": {"iterations": iters, "nnz_iterations": nnz_it,
                  "g_nnz_iterations_per_s": round(nnz_it * value / count / 1e9, 2),
                  "failed": failed, "max_concurrent": info["max_concurrent"],
                  "statuses": statuses, "worst_relative_kkt": worst,
                  "results_match_sequential": same},
        "fp64_batched": fp64_batch,
        "clocks": clocks,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))


def run_serve(args, cp):
    """Open-loop serving: requests arrive by a Poisson process at the
    configured rate for the configured window; latency runs from the
    scheduled arrival to the result on the host.  The server's queue is
    bounded in host memory, so under a load above the GPU's capacity the
    backlog stays bounded and the requests it cannot take are refused and
    counted.  Each request is drawn from a pool of distinct seeded LPs
    generated before the run (new LPs at 200/s cannot be generated on the
    host's cores while it serves)."""
    import numpy as np
    w = SERVE_WORKLOADS[args.workload]
    rate = args.rate or w["rate"]
    duration = args.duration or w["duration"]
    rng = np.random.default_rng(w["seed"])
    shapes = batch_shapes(w["pool_small"], 7000)
    shapes += [(200000, 500000, 5000000, 8000 + i) for i in range(w["pool_large"])]
    tg = time.perf_counter()
    pool = generate_parallel(cp, shapes)
    gen_s = time.perf_counter() - tg
    arrivals, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        large = rng.random() < 0.1
        idx = (w["pool_small"] + int(rng.integers(w["pool_large"]))) if large else \
            int(rng.integers(w["pool_small"]))
        arrivals.append((t, idx))
    params = params_for(cp, args.eps)
    prec = PRECISIONS[args.precision]
    import threading
    lat, done_t = [None] * len(arrivals), [None] * len(arrivals)
    with cp.Server(params, precision=prec, workers=args.workers) as srv:
        srv.set_queue_limit(w["queue_bytes"])
        ids = [None] * len(arrivals)
        t0 = time.perf_counter()

        def collect():
            for k in range(len(arrivals)):
                while ids[k] is None:
                    time.sleep(0.0005)
                if ids[k] < 0:
                    continue
                srv.wait(ids[k])
                done_t[k] = time.perf_counter() - t0
                lat[k] = done_t[k] - arrivals[k][0]

        th = threading.Thread(target=collect)
        with ClockSampler(0) as clk:
            th.start()
            for k, (ta, idx) in enumerate(arrivals):
                d = ta - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                ids[k] = srv.submit(pool[idx])
            th.join()
        st = srv.stats()
    clocks = clk.summary()
    served = [k for k in range(len(arrivals)) if lat[k] is not None]
    total = max(done_t[k] for k in served)
    lat_ms = np.array([lat[k] for k in served]) * 1e3
    large_ms = np.array([lat[k] for k in served if arrivals[k][1] >= w["pool_small"]]) * 1e3
    line = {
        "metric": "served LPs/s; p50/p99 latency", "value": round(len(served) / total, 2),
        "unit": "LPs/s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": round(total * 1e3, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": args.workload, "description": w["desc"], "rate_per_s": rate,
                   "precision": args.precision, "duration_s": duration,
                   "requests": len(arrivals), "workers": args.workers,
                   "pool": f"{w['pool_small']} + {w['pool_large']} distinct LPs generated "
                           f"before the run ({gen_s:.1f} s)",
                   "queue_bound_host_bytes": w["queue_bytes"], "eps": args.eps},
        "latency_ms": {"p50": round(float(np.percentile(lat_ms, 50)), 2),
                       "p99": round(float(np.percentile(lat_ms, 99)), 2),
                       "mean": round(float(lat_ms.mean()), 2),
                       "max": round(float(lat_ms.max()), 2),
                       "large_p50": round(float(np.percentile(large_ms, 50)), 2)
                       if len(large_ms) else None},
        "requests": {"arrived": len(arrivals), "served": len(served),
                     "refused_by_queue_bound": int(st["rejected"]),
                     "offered_rate_per_s": round(len(arrivals) / duration, 1)},
        "e2e": {"value": round(len(served) / total, 2), "unit": "LPs/s",
                "api": "pdlp_server_submit / pdlp_server_wait from host arrays"},
        "server": {"completed": st["completed"], "failed": st["failed"],
                   "max_in_flight": st["max_in_flight"], "iterations": st["iterations"]},
        "clocks": clocks,
    }
    print(json.dumps(line))


def run_reference(args, rank):
    """The reference's own single-GPU FP64 solve (cuSPARSE/cuBLAS, built from
    its sources by `make -C oracle refgpu`) on the same seeded LP: one full
    solve per step, each in a fresh process (the reference draws its
    power-method start from a process-global generator), timed around
    solve_lp_problem from host arrays -- host rescaling, upload, transpose,
    power method, loop and result copy -- the scope of our arm's `e2e`.
    Where that build is absent, the FP64 oracle on the host cores stands in
    (complete solves where they take seconds, else a measured sample)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cupdlpx as cpy  # ctypes structures only; the product library is not loaded
    import oracle_lib
    name = args.workload
    O = oracle_lib.load()
    params = cpy.PdhgParameters()
    O.oracle_default_parameters(C_byref(params))
    params.presolve = False
    params.termination_criteria.eps_optimal_relative = args.eps
    params.termination_criteria.eps_feasible_relative = args.eps
    prob = make_oracle_problem(name)
    a = prob.arrays()
    m, n, nnz = a["m"], a["n"], a["nnz"]
    del a
    base = {"metric": METRIC, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, no dataset)",
            "config": single_config(name, m, n, nnz, args.eps, 1), "impl": "reference",
            "precision": "FP64 (the reference's only arithmetic)"}
    if oracle_lib.ref_gpu_available() and gpu_visible():
        fd, lp_file = tempfile.mkstemp(suffix=".lp")
        os.close(fd)
        try:
            oracle_lib.write_lp_file(prob, lp_file)
            prob.free()
            walls, last = [], None
            with ClockSampler(0) as clk:
                for i in range(args.warmup + args.steps):
                    r = oracle_lib.ref_gpu_solve(None, eps=args.eps, lp_file=lp_file,
                                                 timeout=3600)
                    if i >= args.warmup:
                        walls.append(r["wall_s"])
                        last = r
        finally:
            os.unlink(lp_file)
        value = statistics.mean(walls)
        line = dict(base)
        line.update({
            "value": round(value, 4), "unit": "s", "ms_per_step": round(value * 1e3, 1),
            "solve": {"status": last["status"], "iterations": last["total_count"],
                      "primal_obj": last["primal_objective_value"],
                      "dual_obj": last["dual_objective_value"],
                      "rel_primal": last["relative_primal_residual"],
                      "rel_dual": last["relative_dual_residual"],
                      "rel_gap": last["relative_objective_gap"],
                      "loop_cpu_s": last["cumulative_time_sec"],
                      "host_rescaling_s": last["rescaling_time_sec"],
                      "wall_s_per_step": [round(w, 4) for w in walls]},
            "cpu_baseline": {"value": round(value, 4), "unit": "s", "cores": 1,
                             "kind": "reference",
                             "sample": "the reference's single-GPU solve (src/solver.cu "
                                       "optimize via solve_lp_problem, cuSPARSE CSR_ALG2 SpMV, "
                                       "FP64) on the GB300, full solve per step; its host "
                                       "rescaling runs on one core"},
            "e2e": {"value": round(value, 4), "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0,
                    "api": "the reference's solve_lp_problem from host arrays"},
            "clocks": clk.summary(),
        })
        print(json.dumps(line))
        return
    # no reference build: the FP64 oracle on the host cores, a complete solve
    # where it takes seconds, else the measured time per driver-loop iteration
    vals, desc, unit = [], "", "s"
    for i in range(args.warmup + args.steps):
        if WORKLOADS[name]["kind"] == "random":
            v, desc, _ = cpu_sample(name, params, 0, 0)
        else:
            _, desc, parts = cpu_sample(name, params, 0, 0, loop_iters=100, power_iters=2)
            v, unit = parts["iter_ms"], "ms/iteration"
            desc = "FP64 oracle, 100 driver-loop iterations of the full LP per step (measured)"
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    line = dict(base)
    line.update({"value": round(value, 4), "unit": unit, "ms_per_step": None,
                 "cpu_baseline": {"value": round(value, 4), "unit": unit,
                                  "cores": os.cpu_count(), "kind": "port", "sample": desc},
                 "e2e": {"value": round(value, 4), "unit": unit, "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0},
                 "note": "the reference's single-GPU build is absent here; the FP64 oracle "
                         "stands in"})
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) +
                    sorted(SERVE_WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--workers", type=int, default=8,
                    help="batch / serving workload: worker threads (one CUDA stream each)")
    ap.add_argument("--batch-lps", type=int, default=0,
                    help="batch workload: number of LPs (0: the workload's 512)")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="serving workload: arrivals per second (0: the workload's 200)")
    ap.add_argument("--duration", type=float, default=0.0,
                    help="serving workload: arrival window in seconds (0: the workload's 60)")
    ap.add_argument("--eps", type=float, default=1e-4)
    ap.add_argument("--ref-seconds", type=float, default=60.0,
                    help="batch workload: seconds of sequential solves by the reference's "
                         "own GPU build")
    ap.add_argument("--kernel-reps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["fp32", "fp32m", "fp64"], default=None,
                    help="fp32: FP32 iterates + FP64 refinement; fp32m: FP32 matrix "
                         "and SpMVs with FP64 iterates + FP64 refinement; fp64: plain FP64 "
                         "(default: fp32, the metric's headline; single solves report the "
                         "FP64 solve beside it)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="time the iteration kernels alone and exit (a short command for "
                         "profilers; prints no bench line)")
    ap.add_argument("--fp64-oracle-eps", type=float, default=0.0,
                    help="also solve the LP in FP64 to this tolerance (untimed) and report "
                         "the error of the headline and FP64 results against it")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="timed FP64 solves reported beside an FP32 run (0: skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.precision is None:
        # the metric is FP32 + FP64 refinement against FP64: the headline is
        # the FP32 + refinement solve, with the FP64 solve beside it
        args.precision = "fp32"
    os.environ.setdefault("PDLP_QUIET", "1")
    rank, world, local = rank_info()
    if world > 1:
        # one GPU per rank: the solver library uses device 0 of what it sees
        os.environ["CUDA_VISIBLE_DEVICES"] = visible_device_for_rank(
            local, os.environ.get("CUDA_VISIBLE_DEVICES"))
    import cupdlpx as cp
    if args.kernels_only:
        if rank == 0:
            run_kernels_only(args, cp)
        return
    if args.workload in BATCH_WORKLOADS or args.workload in SERVE_WORKLOADS:
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable":
                                  "batched and served workloads have no CPU reference arm; "
                                  "the sequential line is in the bench output"}))
            return
        if rank == 0:
            (run_batch if args.workload in BATCH_WORKLOADS else run_serve)(args, cp)
        return
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    line = run_ours(args, cp, rank, world, local)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
