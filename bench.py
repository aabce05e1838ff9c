#!/usr/bin/env python
"""Benchmark of the GB300 Krylov solver core.

Metric: time to a 1e-8 residual of the T-FlowS solvers, mixed precision
against FP64, as whole-job solves/s (higher is better), with the HBM
bandwidth the solver kernel achieves.

Headline workload (the metric's own configuration): the 256^3 perturbed-hex
variable-density pressure-correction system (density ratio 7), CG with
IC(0) preconditioning, mixed precision -- FP32 SpMV and vectors, BF16
off-diagonal IC factors with FP32 pivots, exact triangular sweeps -- inside
FP64 iterative refinement, to the reference's test ||r|| < 1e-8*||b||,
x0 = 0.  The same line carries the like-for-like comparison: the same method
and preconditioner on the fastest FP64 build (fused multiply-adds), the
reference-arithmetic FP64 build, and the diagonal and Jacobi-sweep IC
variants, each with its iteration count and its error against a tight FP64
solve (||r|| <= 1e-12*||b||).  Synthetic seeded data (mesh.py documents it;
the reference uses no public dataset); the 2 GB of matrix and vectors exceed
the 129 MB L2, so no flush is needed between steps.

A "step" is one complete solve.  `value` times K solves on data resident in
HBM (device API); `e2e` times K calls of the Fortran-facing C ABI (tflows_cg
with the mixed-precision options set) with the matrix, x and b in pinned
host memory, host<->device copies inside each call.  The CPU baseline is the
oracle (the reference's algorithm restated in C) on the host cores: a full
256^3 IC(0) solve takes tens of minutes on one core, so each sample times
the solve's set-up and a few whole iterations and scales them by the
iteration count of one committed full run (oracle/cfg3_256cube_full_solve.json).

Multi-GPU: the solves are independent replicas (one per rank, no
collective); value = total solves / max-over-ranks time.

--impl reference: the reference algorithm (oracle port, FP64, serial per
solve as in the reference) on every host core, one solve per core at a time,
on the same workload, scaled the same way.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CG/BiCG time-to-1e-8 residual & HBM GB/s: mixed-prec vs FP64, 1 GB300"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel, workload, method, prec):
    """DRAM bytes per launch of this kernel on this workload from the committed
    ncu summary (profiles/traffic.json), or None when it was not captured."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(f"{kernel}|{workload}|{method}|{prec}")
    except Exception:
        return None


def profiled_limiter(kernel, workload, method, prec):
    """What the committed ncu summary shows bounding this kernel on this
    workload (profiles/traffic.json, "limiters"), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get("limiters", {}).get(f"{kernel}|{workload}|{method}|{prec}")
    except Exception:
        return None


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(v, world, device):
    """The slowest rank's time (every rank gets it); the identity for one
    rank.  Works with any process-group backend (NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [v.strip() for v in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        finally:
            os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference_throughput(s, method, prec, threads, seconds_budget):
    """Oracle solves of the same system on `threads` host threads, one solve
    per thread at a time, for about `seconds_budget`; returns (solves/s,
    solves done, iterations)."""
    import oracle
    oracle.build()
    done = [0] * threads
    its = [0]
    stop = time.perf_counter() + seconds_budget

    def work(t):
        while True:
            _, _, it, _, _ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                          s.Ab, s.x, s.b, prec, 200, s.tol)
            its[0] = it
            done[t] += 1
            if time.perf_counter() >= stop:
                break

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    el = time.perf_counter() - t0
    return sum(done) / el, sum(done), its[0], el


FULL_RUN = os.path.join(ROOT, "oracle", "cfg3_256cube_full_solve.json")


def oracle_full_iterations(s, method, prec):
    """Iterations of the committed full oracle solve of this workload, or
    None when no committed run matches it."""
    try:
        with open(FULL_RUN) as f:
            d = json.load(f)
        if d["workload"] == s.name and d["method"] == method and d["prec"] == prec:
            return int(d["iterations"])
    except Exception:
        pass
    return None


class OracleSampler:
    """The oracle on `threads` host threads, each running the same solve
    concurrently (one per core, as the reference runs one solve per MPI
    rank).  A sample times the set-up (Prec1, ||b||, Resid) and `iters` whole
    iterations; the time of a full solve is the set-up plus the full run's
    iteration count times the measured time per iteration."""

    def __init__(self, s, method, prec, threads, iters, fallback_iterations=None):
        import oracle
        oracle.build()
        self.s, self.method, self.prec, self.threads, self.iters = s, method, prec, threads, iters
        self.full_it = oracle_full_iterations(s, method, prec)
        self.full_it_source = "committed full oracle run"
        if self.full_it is None and (s.N <= 300000 or not fallback_iterations):
            # small workloads (tests): one full solve gives the count
            _, _, self.full_it, _, _ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow,
                                                    s.Adia, s.Ab, s.x, s.b, prec, 20000, s.tol)
            self.full_it_source = "full oracle solve in this run"
        elif self.full_it is None:
            # the reference-arithmetic GPU solve runs the same algorithm
            self.full_it = int(fallback_iterations)
            self.full_it_source = "iterations of the reference-arithmetic GPU solve"
        self.t_setup = self.run(0)

    def run(self, iters):
        import oracle
        s = self.s

        def work():
            oracle.solve(self.method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x,
                         s.b, self.prec, iters, s.tol)

        ths = [threading.Thread(target=work) for _ in range(self.threads)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        return time.perf_counter() - t0

    def sample(self):
        """One sample: (solves/s over all threads, seconds of the sample,
        estimated seconds of one full solve)."""
        t = self.run(self.iters)
        t_iter = max(t - self.t_setup, 1e-9) / max(self.iters, 1)
        t_full = self.t_setup + self.full_it * t_iter
        return self.threads / t_full, t, t_full

    def describe(self, elapsed):
        return (f"{self.threads} concurrent oracle solves of the workload (one per thread), "
                f"each timed over its set-up ({self.t_setup:.2f} s) and {self.iters} whole "
                f"iterations, scaled to {self.full_it} iterations ({self.full_it_source}); "
                f"{elapsed:.1f} s of sampling")


def run_reference(args):
    import __graft_entry__ as ge
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pkg = ge.load_package()
    s = make_workload(pkg, args.workload, args.scale)
    method, prec = args.method, args.prec
    cores = os.cpu_count() or 1
    sampler = OracleSampler(s, method, prec, cores, args.oracle_iters)
    for _ in range(args.warmup):
        sampler.sample()
    t0 = time.perf_counter()
    vals = []
    t_full = 0.0
    for _ in range(args.steps):
        v, _, t_full = sampler.sample()
        vals.append(v)
    el = time.perf_counter() - t0
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(s, method, prec),
        "arithmetic": "FP64 as the reference (oracle C restatement, no fused multiply-adds)",
        "full_solve_seconds_per_core": t_full,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": sampler.describe(el)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(s, method, prec, precision=None):
    c = {"workload": f"{s.name}: {method} solve to 1e-8*||b|| (absolute test as the "
                     f"reference), x0=0, prec {prec}",
         "n": s.N, "nnz": s.nnz, "method": method, "prec": prec,
         "l2": "inputs larger than L2 (no flush)"}
    if precision:
        c["precision"] = precision
    return c


ARITHMETIC = {"fp64": "FP64, reference arithmetic (separate rounded products and sums)",
              "fp64_fma": "FP64 with fused multiply-adds and a reciprocal diagonal",
              "mixed": "FP32 inner solves (FP32 SpMV in difference form and FP32 vectors), "
                       "FP64 residual and refinement"}


def make_workload(pkg, name, scale):
    idx = {"cfg1": 1, "cfg2": 2, "cfg3": 3, "cfg5": 5}[name]
    return pkg.mesh.config_system(idx, scale=scale)


def device_solves(pkg, topo, val, b, x, method, prec, tol, opts, steps, warmup, barrier=None):
    """Warm-up, then `steps` timed solves with CUDA events on the current
    stream; returns (elapsed seconds, list of result records)."""
    import torch
    for _ in range(warmup):
        x.zero_()
        res = topo.solve(val, b, x, method, prec, 20000, tol, opts=opts)
        if res["status"] != pkg.OK:
            raise RuntimeError(f"solve failed: {res}")
    if barrier:
        barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = []
    e0.record()
    for _ in range(steps):
        x.zero_()
        out.append(topo.solve(val, b, x, method, prec, 20000, tol, opts=opts))
    e1.record()
    torch.cuda.synchronize()
    if barrier:
        barrier()
    return e0.elapsed_time(e1) * 1e-3, out


# The like-for-like rows of the config-3 comparison: (label, precision,
# prec, IC options).  Mixed rows use BF16 factor entries; each mixed row has
# an FP64 row with the same preconditioner on the fastest FP64 build.
CFG3_ROWS = (("fp64_fma_ic_exact", "fp64_fma", 2, {}),
             ("fp64_ic_exact", "fp64", 2, {}),
             ("mixed_diag", "mixed", 1, {}),
             ("fp64_fma_diag", "fp64_fma", 1, {}),
             ("mixed_ic_jacobi1_bf16", "mixed", 2, {"ic_sweeps": 1, "ic_bf16": 1}),
             ("fp64_fma_ic_jacobi1", "fp64_fma", 2, {"ic_sweeps": 1}),
             ("mixed_ic_jacobi2_bf16", "mixed", 2, {"ic_sweeps": 2, "ic_bf16": 1}),
             ("fp64_fma_ic_jacobi2", "fp64_fma", 2, {"ic_sweeps": 2}))
PAIRS = (("ic_exact", "mixed_ic_exact_bf16", "fp64_fma_ic_exact", "fp64_ic_exact"),
         ("diag", "mixed_diag", "fp64_fma_diag", None),
         ("ic_jacobi1", "mixed_ic_jacobi1_bf16", "fp64_fma_ic_jacobi1", None),
         ("ic_jacobi2", "mixed_ic_jacobi2_bf16", "fp64_fma_ic_jacobi2", None))


def precision_mode(pkg, name):
    return {"fp64": pkg.FP64, "fp64_fma": pkg.FP64_FMA, "mixed": pkg.MIXED}[name]


def cfg3_comparison(pkg, dev, topo, s, val, b, headline, x_head, reps=1):
    """Every row of CFG3_ROWS on the headline system (each with its own tuned
    launch shape, tuned on a first untimed solve), the headline's own result,
    and for each the relative error max|x - x*| / max|x*| against a tight FP64
    solve x* (FP64-FMA, exact IC, ||r|| <= 1e-12*||b||); speed-ups of each
    mixed row over its FP64 rows with the same preconditioner."""
    import torch
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    tight = pkg.options(precision=pkg.FP64_FMA, tol_mode=pkg.TOL_RELATIVE, autotune=1)
    res = topo.solve(val, b, x, "cg", 2, 20000, 1e-12, opts=tight)
    x_star = x.clone()
    scale = float(x_star.abs().max())
    out = {"tight_reference": {"what": "FP64-FMA CG + exact IC(0) to ||r|| <= 1e-12*||b||",
                               "iterations": res["iterations"], "status": res["status"]}}

    def err(xv):
        return float((xv - x_star).abs().max()) / scale

    head = dict(headline)
    head["rel_err_vs_tight_fp64"] = err(x_head)
    out["mixed_ic_exact_bf16"] = head
    for label, prec_name, prec, ic in CFG3_ROWS:
        opts = pkg.options(precision=precision_mode(pkg, prec_name), autotune=1, **ic)
        el, rr = device_solves(pkg, topo, val, b, x, "cg", prec, s.tol, opts, reps, 1)
        r = rr[-1]
        out[label] = {"ms": 1e3 * el / reps, "iterations": r["iterations"],
                      "inner_iterations": r["inner_iterations"], "refinements": r["refinements"],
                      "fin_res": r["fin_res"], "status": r["status"],
                      "gbs": r["bytes"] / r["seconds"] / 1e9, "block_size": r["block_size"],
                      "grid_blocks": r["grid_blocks"], "rel_err_vs_tight_fp64": err(x)}
    speed = {}
    for kind, mixed, fma, ref in PAIRS:
        if mixed in out and fma in out:
            speed[kind] = {"vs_fp64_fma": out[fma]["ms"] / out[mixed]["ms"],
                           "mixed_over_fp64_iterations":
                               out[mixed]["inner_iterations"] / max(1, out[fma]["iterations"])}
            if ref and ref in out:
                speed[kind]["vs_fp64_reference_arithmetic"] = out[ref]["ms"] / out[mixed]["ms"]
    out["speedups"] = speed
    return out


def batched_cfg4(pkg, dev, reps, count=48, autotune=True):
    """48 independent systems of uneven size (log-uniform 16^3..160^3 cells),
    odd ones variable-density pressure (CG + IC), even ones scalar transport
    (BiCG + diagonal), mixed precision with FP64 refinement to 1e-8 relative,
    solved by one graph-captured persistent launch per replay.  The IC(0)
    systems run with BF16 factor entries and either exact triangular sweeps
    or one Jacobi sweep per triangle; the faster plan is the block's result,
    both are reported."""
    import torch
    shapes = pkg.mesh.batch_sizes(count)
    systems = []
    for k, (nx, ny, nz) in enumerate(shapes):
        if k % 2:
            systems.append((pkg.mesh.pressure_system(nx, ny, nz, perturb=0.2, seed=100 + k,
                                                     variable_density=True), "cg", 2))
        else:
            systems.append((pkg.mesh.convection_diffusion_system(nx, ny, nz, perturb=0.2,
                                                                 seed=100 + k), "bicg", 1))
    topos = [pkg.Topology.from_system(s) for s, _, _ in systems]
    vals = [torch.from_numpy(s.A[:-1].copy()).to(dev) for s, _, _ in systems]
    bs = [torch.from_numpy(s.b.copy()).to(dev) for s, _, _ in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device=dev) for s, _, _ in systems]
    rows = sum(s.N for s, _, _ in systems)
    # each system's tight FP64 solution (FP64-FMA, ||r|| <= 1e-12*||b||)
    tight = pkg.options(precision=pkg.FP64_FMA, tol_mode=pkg.TOL_RELATIVE)
    x_star, tight_ok = [], 0
    for (sy, m, p), tp, v, bb in zip(systems, topos, vals, bs):
        xt = torch.zeros(sy.N, dtype=torch.float64, device=dev)
        r = tp.solve(v, bb, xt, m, p, 20000, 1e-12, opts=tight, raise_on_error=False)
        tight_ok += r["status"] == pkg.OK
        x_star.append(xt)
    variants = {}
    for label, ic in (("ic_exact_bf16", {"ic_bf16": 1}),
                      ("ic_jacobi1_bf16", {"ic_bf16": 1, "ic_sweeps": 1})):
        opts = pkg.options(precision=pkg.MIXED, tol_mode=pkg.TOL_RELATIVE,
                           autotune=int(autotune), **ic)
        for x in xs:
            x.zero_()  # the plan tunes on x0 = 0, as every replay starts
        plan = pkg.Plan(topos, vals, bs, xs, [m for _, m, _ in systems],
                        [p for _, _, p in systems], [20000] * count, [1e-8] * count, opts)
        tuning = plan.tuning()
        plan.launch()
        plan.results()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            for x in xs:
                x.zero_()
            plan.launch()
        e1.record()
        res = plan.results()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        byts = sum(r["bytes"] for r in res)
        errs = [float((xk - xs_k).abs().max() / xs_k.abs().max()) for xk, xs_k in zip(xs, x_star)]
        variants[label] = {
            "ms_per_batch": ms, "systems_per_s": count * 1e3 / ms,
            "converged": sum(1 for r in res if r["status"] == pkg.OK),
            "max_iterations": max(r["iterations"] for r in res),
            "iterations": [r["iterations"] for r in res],
            "rel_err_vs_tight_fp64": errs, "max_rel_err_vs_tight_fp64": max(errs),
            "gbs": byts / (ms * 1e-3) / 1e9, "tuning": tuning,
            "group_blocks": [r["grid_blocks"] for r in res]}
        plan.close()
    best = min(variants, key=lambda k: variants[k]["ms_per_batch"])
    out = {"workload": f"{count} systems, sizes {min(s.N for s, _, _ in systems)}.."
                       f"{max(s.N for s, _, _ in systems)} rows (total {rows}), odd: CG+IC "
                       "pressure, even: BiCG+diag transport, mixed precision, tol 1e-8 relative, "
                       "one graph-captured cooperative launch",
           "variant": best, **variants[best]}
    out["all_variants"] = {k: {kk: vv for kk, vv in v.items()
                               if kk not in ("group_blocks", "iterations", "rel_err_vs_tight_fp64")}
                           for k, v in variants.items()}
    out["tight_fp64_converged"] = tight_ok
    out["cpu_baseline"] = cfg4_cpu_estimate(pkg, dev, systems, topos, vals, bs)
    for tp in topos:
        tp.close()
    return out


def lpt_makespan(times, cores):
    """Wall time of independent jobs run one per core, longest first, each
    on the core that frees up first."""
    loads = [0.0] * max(1, cores)
    for t in sorted(times, reverse=True):
        k = loads.index(min(loads))
        loads[k] += t
    return max(loads)


def cfg4_cpu_estimate(pkg, dev, systems, topos, vals, bs, iters=2):
    """The oracle on the batch, one solve per host core.  Each system's
    oracle solve is its set-up (an oracle run with no iterations) plus
    `iters` whole iterations, scaled to the iteration count of the
    reference-arithmetic GPU solve of the same system at the same tolerance
    (the same algorithm; its counts match the oracle's within 1); the
    estimates are then placed longest first on the least-loaded core."""
    import numpy as np
    import torch
    import oracle
    ref = pkg.options(precision=pkg.FP64, tol_mode=pkg.TOL_RELATIVE)
    est, its = [], []
    for (sy, m, p), tp, v, bb in zip(systems, topos, vals, bs):
        xt = torch.zeros(sy.N, dtype=torch.float64, device=dev)
        r = tp.solve(v, bb, xt, m, p, 20000, 1e-8, opts=ref, raise_on_error=False)
        tol = 1e-8 * float(np.linalg.norm(sy.b))
        t0 = time.perf_counter()
        oracle.solve(m, sy.N, sy.NB, sy.NONZ, sy.A, sy.Acol, sy.Arow, sy.Adia, sy.Ab, sy.x, sy.b,
                     p, 0, tol)
        t1 = time.perf_counter()
        oracle.solve(m, sy.N, sy.NB, sy.NONZ, sy.A, sy.Acol, sy.Arow, sy.Adia, sy.Ab, sy.x, sy.b,
                     p, iters, tol)
        t2 = time.perf_counter()
        t_it = max((t2 - t1) - (t1 - t0), 0.0) / iters
        its.append(r["iterations"])
        est.append((t1 - t0) + r["iterations"] * t_it)
    cores = os.cpu_count() or 1
    span = lpt_makespan(est, cores)
    return {"seconds_per_batch": span, "systems_per_s": len(est) / span,
            "one_core_seconds": sum(est), "cores": cores, "kind": "port",
            "sample": f"per system the oracle's set-up and {iters} whole iterations, scaled to the "
                      "iteration count of the reference-arithmetic GPU solve at 1e-8 relative; "
                      f"the {len(est)} solves placed longest first on {cores} host cores",
            "iterations_fp64": its}


def spmv_block(topo, s, val, peak, dev, repeat=20):
    """The standalone product y = A x on the workload's own system, FP64
    (reference-arithmetic sums) and FP32 (difference form), SELL-32 slices
    with one-byte column patterns when the mesh has few stencils.
    Algorithmic bytes per product: the values and column data once, the
    slice offsets, x read once and y written once.  Time per product from
    CUDA events over `repeat` back-to-back products after one untimed call;
    the matrix is several times larger than L2, so it streams from HBM every
    product."""
    import torch
    x = torch.rand(s.N, dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    slices = (s.N + 31) // 32
    cols_per = s.N if topo.patterns else None  # one byte per row with patterns
    out = {"workload": f"{s.name}: y = A x", "n": s.N, "nnz": s.nnz,
           "column_patterns": topo.patterns}
    ref = s.scipy() @ x.cpu().numpy()
    for label, fp32, sv in (("fp64", False, 8), ("fp32", True, 4)):
        topo.spmv(val, x, y, repeat=1, fp32=fp32)
        err = float(abs(y.cpu().numpy() - ref).max() / abs(ref).max())
        sec = topo.spmv(val, x, y, repeat=repeat, fp32=fp32)
        cols = cols_per if cols_per is not None else 4 * s.nnz
        byts = sv * s.nnz + cols + 8 * (slices + 1) + 2 * s.N * sv
        out[label] = {"us_per_product": 1e6 * sec, "algorithmic_bytes": byts,
                      "gbs": byts / sec / 1e9, "frac": byts / sec / 1e9 / peak,
                      "max_rel_diff_vs_host_product": err}
    return out


def legacy_e2e(pkg, s, method, prec, opts_kw, steps, warmup):
    """Seconds of `steps` calls of the Fortran-facing C ABI (tflows_cg /
    _bicg / _cgs) with A, x and b in pinned host memory and the given
    options set process-wide; host<->device copies are inside each call."""
    import torch
    A_h = torch.from_numpy(s.A.copy()).pin_memory().numpy()
    x_h = torch.zeros(s.NB + s.N + 1, dtype=torch.float64).pin_memory().numpy()
    r_h = torch.zeros(s.N, dtype=torch.float64).pin_memory().numpy()
    pkg.set_options(**opts_kw)
    legacy = {"cg": pkg.cg, "bicg": pkg.bicg, "cgs": pkg.cgs}[method]
    t = 0.0
    out = None
    for k in range(warmup + steps):
        x_h[:] = 0.0
        r_h[:] = s.b
        t0 = time.perf_counter()
        out = legacy(s.N, s.NB, s.NONZ, A_h, s.Acol, s.Arow, s.Adia, s.Ab, x_h, r_h, prec, 20000,
                     s.tol)
        t1 = time.perf_counter()
        if k >= warmup:
            t += t1 - t0
    pkg.set_options()
    if out.status != pkg.OK:
        raise RuntimeError(f"e2e solve failed: {out}")
    return t, {"h2d_bytes_per_step": int(8 * s.nnz + 16 * s.N), "d2h_bytes_per_step": int(16 * s.N)}


def cfg2_block(pkg, dev, peak, reps=10, cpu_seconds=10.0):
    """Config 2: the 128^3 perturbed convection-diffusion system (momentum /
    scalar transport), BiCG + diagonal in FP64 with fused multiply-adds,
    device-resident and through tflows_bicg with host buffers, the other
    config-2 solvers, the GPU answer against the oracle and the one-core
    oracle throughput."""
    import numpy as np
    import torch
    import oracle
    s = make_workload(pkg, "cfg2", None)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    tuning = topo.autotune(val, b, "bicg", 1, opts=pkg.options(precision=pkg.FP64_FMA))
    opts = pkg.options(precision=pkg.FP64_FMA, autotune=1)
    el, res = device_solves(pkg, topo, val, b, x, "bicg", 1, s.tol, opts, reps, 3)
    kern_s = sum(r["seconds"] for r in res)
    kern_b = sum(r["bytes"] for r in res)
    out = {"workload": workload_config(s, "bicg", 1, "fp64_fma")["workload"], "n": s.N,
           "solves_per_s": reps / el, "ms_per_solve": 1e3 * el / reps,
           "iterations": res[-1]["iterations"], "launch": tuning,
           "roofline": {"bound": "hbm", "achieved": kern_b / kern_s / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": kern_b / kern_s / 1e9 / peak,
                        "kernel": "fma::krylov_kernel<double,0>"}}
    x_gpu = x.cpu().numpy()
    t, io = legacy_e2e(pkg, s, "bicg", 1, {"precision": pkg.FP64_FMA, "autotune": 1}, reps, 2)
    out["e2e"] = {"value": reps / t, "unit": "solves/s", **io}
    out["methods"] = cfg2_methods(pkg, dev, topo, s, val, b)
    topo.close()
    xo, _, it_o, _, _ = oracle.solve("bicg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                     s.x, s.b, 1, 20000, s.tol)
    xo = xo[s.NB + 1:]
    out["rel_err_vs_oracle"] = float(np.abs(x_gpu - xo).max() / np.abs(xo).max())
    out["oracle_iterations"] = int(it_o)
    v, n, it, el_c = cpu_reference_throughput(s, "bicg", 1, 1, cpu_seconds)
    out["cpu_oracle_1core"] = {"solves_per_s": v, "solves": n, "seconds": el_c}
    return out


def cfg2_methods(pkg, dev, topo, s, val, b, reps=3):
    """The config-2 solvers on the same 128^3 system besides the headline:
    BiCG and CGS in reference arithmetic (TFLOWS_FP64) and with fused
    multiply-adds (TFLOWS_FP64_FMA), the true-BiCG extension (shadow sequence
    with A^T) and BiCG in mixed precision, each to the same absolute
    tolerance from x0 = 0."""
    import torch
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    out = {}
    for label, method, precision in (("bicg_fp64", "bicg", pkg.FP64),
                                     ("bicg_fp64_fma", "bicg", pkg.FP64_FMA),
                                     ("cgs_fp64", "cgs", pkg.FP64),
                                     ("cgs_fp64_fma", "cgs", pkg.FP64_FMA),
                                     ("bicg_true_fp64_fma", "bicg_true", pkg.FP64_FMA),
                                     ("bicg_mixed", "bicg", pkg.MIXED)):
        opts = pkg.options(precision=precision, autotune=1)
        el, res = device_solves(pkg, topo, val, b, x, method, 1, s.tol, opts, reps, 1)
        r = res[-1]
        out[label] = {"ms": 1e3 * el / reps, "solves_per_s": reps / el,
                      "iterations": r["iterations"], "status": r["status"],
                      "gbs": r["bytes"] / r["seconds"] / 1e9, "fin_res": r["fin_res"],
                      "block_size": r["block_size"], "grid_blocks": r["grid_blocks"]}
    return out


def cfg1_latency(pkg, dev, reps=20):
    """Config 1: the 32^3 Jacobi-CG system (32,768 rows), FP64 in reference
    arithmetic and with fused multiply-adds, device-resident and through the
    Fortran-facing C ABI, against the one-core oracle.  Its 2.8 MB of values
    fit in L2, so a solve is bound by the latency of its grid barriers, not by
    HBM: reported per solve and per iteration, not against the roofline."""
    import numpy as np
    import torch
    import oracle
    s = make_workload(pkg, "cfg1", None)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    out = {"workload": f"{s.name}: CG + diagonal to 1e-8*||b|| (absolute), x0=0", "n": s.N}
    for label, precision in (("fp64", pkg.FP64), ("fp64_fma", pkg.FP64_FMA)):
        opts = pkg.options(precision=precision, autotune=1)
        el, res = device_solves(pkg, topo, val, b, x, "cg", 1, s.tol, opts, reps, 3)
        r = res[-1]
        out[label] = {"us_per_solve": 1e6 * el / reps, "iterations": r["iterations"],
                      "us_per_iteration": 1e6 * el / reps / max(r["iterations"], 1),
                      "status": r["status"], "block_size": r["block_size"],
                      "grid_blocks": r["grid_blocks"]}
    pkg.set_options(precision=pkg.FP64)
    xh, rh = s.x.copy(), s.b.copy()
    pkg.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, xh, rh, 1, 20000, s.tol)
    t0 = time.perf_counter()
    for _ in range(reps):
        xh, rh = s.x.copy(), s.b.copy()
        pkg.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, xh, rh, 1, 20000, s.tol)
    out["c_abi_us_per_solve"] = 1e6 * (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    xo, _, ito, _, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                    s.x, s.b, 1, 20000, s.tol)
    out["cpu_oracle_us_per_solve"] = 1e6 * (time.perf_counter() - t0)
    out["cpu_cores"] = 1
    out["oracle_iterations"] = ito
    out["rel_err_vs_oracle"] = float(np.abs(xh - xo).max() / np.abs(xo).max())
    pkg.set_options()
    topo.close()
    return out


def ic_block(pkg, dev, n=128, iters=0, precisions=("fp64", "fp64_fma", "mixed"), tiled=(0, 1),
             reps=2, blocks=(0,), restart=None):
    """IC(0)-preconditioned CG on the config-3 variable-density pressure
    system at n^3: per precision and per sweep kind (tiled / level-ordered),
    the time per iteration of the persistent solve (capped at `iters`
    iterations, 0 = to the tolerance) and one standalone IC apply (pivots +
    forward + backward, tflows_ic_apply_device) for the FP64 builds."""
    import torch
    s = make_workload(pkg, "cfg3", n)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    z = torch.empty_like(x)
    maxit = iters if iters > 0 else 20000
    mode = {"fp64": pkg.FP64, "fp64_fma": pkg.FP64_FMA, "mixed": pkg.MIXED}
    out = {"workload": f"{s.name}: CG + IC(0), tol 1e-8*||b|| (absolute), x0=0"
                       + (f", capped at {iters} iterations" if iters else ""), "n": s.N}
    for label, t, blk in ((p, t, k) for p in precisions for t in tiled for k in blocks):
        if True:
            kw = {"ic_bf16": 1} if label == "mixed" else {}
            if label == "mixed" and restart is not None:
                kw["refine_restart"] = restart
            opts = pkg.options(precision=mode[label], ic_tiled=t, block_size=blk, **kw)
            x.zero_()
            topo.solve(val, b, x, "cg", 2, maxit, s.tol, opts=opts, raise_on_error=False)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                x.zero_()
                r = topo.solve(val, b, x, "cg", 2, maxit, s.tol, opts=opts, raise_on_error=False)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            it = max(1, r["inner_iterations"] if label == "mixed" else r["iterations"])
            rec = {"ms": ms, "iterations": it, "us_per_iteration": 1e3 * ms / it,
                   "status": r["status"], "gbs": r["bytes"] / r["seconds"] / 1e9,
                   "refinements": r["refinements"]}
            if label != "mixed":
                topo.ic_apply(val, b, z, opts=opts)
                torch.cuda.synchronize()
                e0.record()
                for _ in range(reps):
                    topo.ic_apply(val, b, z, opts=opts)
                e1.record()
                torch.cuda.synchronize()
                rec["pivots_plus_apply_ms"] = e0.elapsed_time(e1) / reps
            rec["block_size"] = r["block_size"]
            out[f"{label}_{'tiled' if t else 'level'}" + (f"_b{blk}" if blk else "")] = rec
    topo.close()
    return out


def adjoint_cfg5(pkg, dev, reps=3):
    """Config 5: 64^3 variable-density pressure assembled differentiably from
    its float32 face coefficients, loss 0.5||x - x_t||^2, one forward solve
    and one backward (transposed) solve per step; gradients with respect to
    b (float64) and the coefficients (float32)."""
    import numpy as np
    import torch
    from tflows_gb300 import autograd as ag
    s = pkg.mesh.pressure_system(64, 64, 64, perturb=0.2, seed=0, variable_density=True,
                                 keep_faces=True)
    solver = ag.DifferentiableSolver.from_system(s, method="cg", prec=1, rtol=1e-10)
    asm = ag.FaceAssembly(s, device=dev)
    xt = torch.as_tensor(np.random.default_rng(100).uniform(-1, 1, s.N), device=dev)
    coef = torch.tensor(s.face_coef, dtype=torch.float32, device=dev, requires_grad=True)
    b = torch.tensor(s.b, dtype=torch.float64, device=dev, requires_grad=True)

    def step():
        coef.grad = None
        b.grad = None
        x = solver(asm(coef), b)
        loss = 0.5 * ((x - xt) ** 2).sum()
        loss.backward()
        return loss

    for _ in range(2):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    fw, bw = solver.last_forward, solver.last_adjoint
    solver.topo.close()
    # CPU baseline: the oracle's forward solve and its adjoint solve (the
    # system is symmetric, so the transposed solve is a CG on A with the
    # loss gradient as right-hand side), one host core each, timed whole
    import oracle
    t0 = time.perf_counter()
    xo, _, it_f, _, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                     s.x, s.b, 1, 20000, 1e-10 * float(np.linalg.norm(s.b)))
    t1 = time.perf_counter()
    g = xo[s.NB + 1:] - xt.cpu().numpy()
    _, _, it_a, _, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                    s.x, g, 1, 20000, 1e-10 * float(np.linalg.norm(g)))
    t2 = time.perf_counter()
    return {"workload": f"{s.name} differentiable CG + diagonal, rtol 1e-10, loss 0.5||x-x_t||^2",
            "n": s.N, "ms_per_forward_backward": ms,
            "forward": {"iterations": fw["iterations"], "ms": 1e3 * fw["seconds"]},
            "adjoint": {"iterations": bw["iterations"], "ms": 1e3 * bw["seconds"]},
            "grad_b_norm": float(b.grad.norm()), "grad_coef_norm": float(coef.grad.norm()),
            "cpu_oracle_1core": {"forward_ms": 1e3 * (t1 - t0), "forward_iterations": it_f,
                                 "adjoint_ms": 1e3 * (t2 - t1), "adjoint_iterations": it_a}}


def simple_step(pkg, dev, n=128, reps=3, autotune=True):
    """The five solves of one SIMPLE outer iteration on one 128^3 mesh (one
    topology): mixture fraction (cg, Process/CalcZmix.f90:394), three momentum
    components (bicg, NewUVW.f90:506) and the pressure correction (cg,
    CalcPS.f90:217), FP64 with diagonal preconditioning, each to 1e-8*||b||
    absolute; one graph-captured persistent launch per step against five
    consecutive single-system solves."""
    import numpy as np
    import torch
    cd = pkg.mesh.convection_diffusion_system(n, n, n, perturb=0.2, seed=21)
    zm = pkg.mesh.convection_diffusion_system(n, n, n, perturb=0.2, seed=22)
    pr = pkg.mesh.pressure_system(n, n, n, perturb=0.2, seed=23, variable_density=True)
    assert np.array_equal(cd.Arow, pr.Arow) and np.array_equal(cd.Acol, pr.Acol)
    topo = pkg.Topology.from_system(pr)
    rng = np.random.default_rng(24)
    mom = [torch.from_numpy(cd.b * (1.0 + 0.1 * k) + rng.uniform(-0.1, 0.1, cd.N)).to(dev)
           for k in range(3)]
    systems = [(zm, torch.from_numpy(zm.b.copy()).to(dev), "cg")] + \
              [(cd, bk, "bicg") for bk in mom] + \
              [(pr, torch.from_numpy(pr.b.copy()).to(dev), "cg")]
    vals = {id(m): torch.from_numpy(m.A[:-1].copy()).to(dev) for m in (cd, zm, pr)}
    vs = [vals[id(m)] for m, _, _ in systems]
    bs = [bk for _, bk, _ in systems]
    tols = [1e-8 * float(bk.norm()) for bk in bs]
    xs = [torch.zeros(pr.N, dtype=torch.float64, device=dev) for _ in systems]
    opts = pkg.options(autotune=int(autotune))
    plan = pkg.Plan([topo] * 5, vs, bs, xs, [m for _, _, m in systems], [1] * 5, [20000] * 5,
                    tols, opts)
    tuning = plan.tuning()
    plan.launch()
    plan.results()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        for x in xs:
            x.zero_()
        plan.launch()
    e1.record()
    res = plan.results()
    torch.cuda.synchronize()
    plan_ms = e0.elapsed_time(e1) / reps
    seq = pkg.options()
    x = torch.zeros(pr.N, dtype=torch.float64, device=dev)
    for _ in range(1):
        for (m, bk, meth), v, tl in zip(systems, vs, tols):
            x.zero_()
            topo.solve(v, bk, x, meth, 1, 20000, tl, opts=seq)
    torch.cuda.synchronize()
    e0.record()
    seq_res = []
    for _ in range(reps):
        for (m, bk, meth), v, tl in zip(systems, vs, tols):
            x.zero_()
            seq_res.append(topo.solve(v, bk, x, meth, 1, 20000, tl, opts=seq))
    e1.record()
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1) / reps
    plan.close()
    topo.close()
    return {"workload": f"SIMPLE step on {n}^3 (one topology): Zmix cg, 3x momentum bicg, "
                        "pressure cg, prec 1, FP64, tol 1e-8*||b||",
            "plan_ms": plan_ms, "sequential_ms": seq_ms, "speedup": seq_ms / plan_ms,
            "iterations": [r["iterations"] for r in res],
            "converged": sum(1 for r in res if r["status"] == pkg.OK),
            "group_blocks": [r["grid_blocks"] for r in res], "tuning": tuning}


def assembly_block(pkg, dev, n=128, reps=5):
    """The pressure-correction assembly (Process/CalcPS.f90:49-202) of an
    n^3 perturbed box on the GPU: inflow on x-min, outflow on x-max, walls
    elsewhere, seeded fields.  Reports the device time, the algorithmic bytes
    (every input read once, every output written once) against the HBM peak,
    and the host->device copy of Aval and b it makes unnecessary when the
    fields live on the GPU; the CPU restatement (one core) beside it."""
    import numpy as np
    import torch
    import oracle
    msh = pkg.mesh.box_faces(n, n, n, perturb=0.2, seed=7)
    NC, NbC, NS = msh["NC"], msh["NbC"], msh["NS"]
    NONZ = int(msh["Acol"][-1])
    rng = np.random.default_rng(8)
    m = NbC + NC + 1
    tb = np.full(m, 2, np.int32)
    tb[NbC:] = 0
    ny = nz = n
    tb[NbC - np.arange(1, ny * nz + 1)] = 1           # x-min walls: inflow (cells -1..)
    tb[NbC - np.arange(ny * nz + 1, 2 * ny * nz + 1)] = 3  # x-max: outflow
    cpu = {"volume": msh["volume"], "Asave": rng.uniform(1.0, 2.0, m)}
    for k in ("rho_n", "rho_o", "rho_oo"):
        cpu[k] = rng.uniform(0.5, 1.5, m)
    for k in ("U", "V", "W", "P", "Px", "Py", "Pz"):
        cpu[k] = rng.uniform(-1.0, 1.0, m)
    asm = pkg.Assembly.from_faces(msh, tb)
    key = {"rho_n": "rho_n", "rho_o": "rho_o", "rho_oo": "rho_oo", "u": "U", "v": "V", "w": "W",
           "p": "P", "px": "Px", "py": "Py", "pz": "Pz", "asave": "Asave"}
    fields = {k: torch.from_numpy(cpu[v]).to(dev) for k, v in key.items()}
    aval = torch.empty(NONZ, dtype=torch.float64, device=dev)
    b = torch.empty(NC, dtype=torch.float64, device=dev)
    abou = torch.zeros(NbC, dtype=torch.float64, device=dev)
    flux = torch.empty(NS, dtype=torch.float64, device=dev)
    secs = []
    for _ in range(reps + 2):
        secs.append(asm.calcps(fields, aval, b, abou, flux, Nmat=1, dt=0.01)["seconds"])
    sec = min(secs[2:])
    # what the assembly reads and writes once: geometry 7 doubles + 4 ints per
    # face, 12 cell arrays + TypeBC + Adia, outputs Aval, b, Flux
    byts = NS * (7 * 8 + 4 * 4) + m * (12 * 8 + 4) + NC * 4 + 8 * (NONZ + NC + NS)
    # the copy it replaces: Aval and b from pinned host memory
    h = torch.empty(NONZ + NC, dtype=torch.float64).pin_memory()
    dd = torch.empty_like(h, device=dev)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    dd.copy_(h, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    h2d = e0.elapsed_time(e1) * 1e-3
    gpu_aval = aval.cpu().numpy()
    t0 = time.perf_counter()
    ref = oracle.calcps_assembly(NC, NbC, NS, NONZ, 1, 0.01, msh["SideC"], msh["SidAij"],
                                 msh["Adia"], tb, {k: msh[k] for k in oracle.FACE_GEOM},
                                 {k: cpu[k] for k in oracle.CELL_FIELDS})
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(gpu_aval.view(np.uint64), ref[0].view(np.uint64)))
    asm.close()
    peak, _ = load_peaks()
    return {"workload": f"CalcPS assembly, {n}^3 perturbed box ({NC} cells, {NS} faces), "
                        "inflow/outflow/walls, Nmat 1",
            "ms": sec * 1e3, "gbs": byts / sec / 1e9, "frac": byts / sec / 1e9 / peak,
            "algorithmic_bytes": byts, "h2d_aval_b_ms": h2d * 1e3,
            "cpu_oracle_ms": cpu_s * 1e3, "cpu_cores": 1, "aval_bitwise_vs_oracle": same}


def momentum_block(pkg, dev, n=128, reps=5):
    """The momentum assembly (Process/NewUVW.f90:138-499) of component U on
    an n^3 perturbed box on the GPU: SMART blending (ConvScheme with the
    CalMinMax bounds), upwind sums, implicit diffusion, two time levels;
    inflow on x-min, outflow on x-max, walls elsewhere; seeded fields.  Device
    time, algorithmic bytes (every input read once, every output written
    once) against the HBM peak, the one-core CPU restatement beside it."""
    import numpy as np
    import torch
    import oracle
    msh = pkg.mesh.box_faces(n, n, n, perturb=0.2, seed=7)
    NC, NbC, NS = msh["NC"], msh["NbC"], msh["NS"]
    NONZ = int(msh["Acol"][-1])
    rng = np.random.default_rng(9)
    m = NbC + NC + 1
    tb = np.full(m, 2, np.int32)
    tb[NbC:] = 0
    tb[NbC - np.arange(1, n * n + 1)] = 1
    tb[NbC - np.arange(n * n + 1, 2 * n * n + 1)] = 3
    cpu = {}
    for k in ("rho_n", "rho_o", "rho_oo"):
        cpu[k] = rng.uniform(0.5, 1.5, m)
    for k in oracle.MOMENTUM_CELL_FIELDS[3:]:
        cpu[k] = rng.uniform(-1.0, 1.0, m)
    for k in ("flux_u", "flux"):
        cpu[k] = rng.uniform(-1.0, 1.0, NS)
    cpu["ff"] = msh["f"].copy()
    cpu["scoef"] = ((msh["Sx"] * msh["Sx"] + msh["Sy"] * msh["Sy"] + msh["Sz"] * msh["Sz"])
                    / (msh["Dx"] * msh["Sx"] + msh["Dy"] * msh["Sy"] + msh["Dz"] * msh["Sz"]))
    material = np.ones(m, np.int32)
    smart, yes = oracle.SCHEME["smart"], oracle.SCHEME["yes"]
    opts = dict(visc=1e-2, dt=0.01, urf=0.7)
    asm = pkg.Assembly.from_faces(msh, tb)
    fields = {("source" if k == "ui_source" else k): torch.from_numpy(cpu[k]).to(dev)
              for k in oracle.MOMENTUM_CELL_FIELDS + oracle.MOMENTUM_FACE_FIELDS}
    fields.update(material=torch.from_numpy(material).to(dev),
                  blend=torch.tensor([smart], dtype=torch.int32, device=dev),
                  blend_tem=torch.tensor([yes], dtype=torch.int32, device=dev),
                  urfc=torch.tensor([0.9], dtype=torch.float64, device=dev))
    aval = torch.empty(NONZ, dtype=torch.float64, device=dev)
    b = torch.empty(NC, dtype=torch.float64, device=dev)
    abou = torch.zeros(NbC, dtype=torch.float64, device=dev)
    asave = torch.empty(NC, dtype=torch.float64, device=dev)
    rhoui = torch.empty(m, dtype=torch.float64, device=dev)
    secs = []
    for _ in range(reps + 2):
        secs.append(asm.newuvw(1, fields, aval, b, abou, asave, rhoui, **opts)["seconds"])
    sec = min(secs[2:])
    # inputs once: 12 doubles + c1, c2, SidAij per face; 15 cell fields,
    # material, TypeBC, volume per cell; Adia; outputs Aval, b, Asave, rhoUi, Abou
    byts = (NS * (12 * 8 + 4 * 4) + m * (15 * 8 + 4 + 4 + 8) + NC * 4
            + 8 * (NONZ + 2 * NC + m + NbC))
    gpu_aval, gpu_b = aval.cpu().numpy(), b.cpu().numpy()
    asm.close()
    geom = {k: msh[k] for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f")}
    geom["volume"] = msh["volume"]
    t0 = time.perf_counter()
    ref = oracle.momentum_assembly(NC, NbC, NS, NONZ, msh["SideC"], msh["SidAij"], msh["Adia"],
                                   tb, material, geom, cpu, 1, 1, np.array([smart], np.int32),
                                   np.array([yes], np.int32), np.array([0.9]), **opts)
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(gpu_aval.view(np.uint64), ref[0].view(np.uint64))
                and np.array_equal(gpu_b.view(np.uint64), ref[1].view(np.uint64)))
    peak, _ = load_peaks()
    return {"workload": f"NewUVW momentum assembly (U), {n}^3 perturbed box ({NC} cells, "
                        f"{NS} faces), SMART blending, inflow/outflow/walls",
            "ms": sec * 1e3, "gbs": byts / sec / 1e9, "frac": byts / sec / 1e9 / peak,
            "algorithmic_bytes": byts, "cpu_oracle_ms": cpu_s * 1e3, "cpu_cores": 1,
            "aval_b_bitwise_vs_oracle": same}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg3", choices=["cfg1", "cfg2", "cfg3", "cfg5"])
    ap.add_argument("--scale", type=int, default=None, help="box edge (default: the config's)")
    ap.add_argument("--method", default="cg")
    ap.add_argument("--prec", type=int, default=2)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "fp64_fma", "mixed"],
                    help="fp64: reference arithmetic; fp64_fma: FP64 with fused multiply-adds "
                         "(within 1e-8 of the reference); mixed: FP32 inner + FP64 refinement")
    ap.add_argument("--ic-sweeps", type=int, default=0,
                    help="prec 2: Jacobi sweeps per triangle (0 = exact triangular sweeps)")
    ap.add_argument("--ic-factors", default="bf16", choices=["bf16", "fp32"],
                    help="mixed + prec 2: precision of the off-diagonal IC factor entries")
    ap.add_argument("--oracle-iters", type=int, default=2,
                    help="CPU legs: whole oracle iterations timed per sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the config-3 comparison rows")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched (cfg4) block")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the config-1/2/5, SIMPLE-step and assembly blocks")
    ap.add_argument("--no-autotune", action="store_true",
                    help="fixed launch shape (256 threads, one slice per warp)")
    ap.add_argument("--block", default=None,
                    choices=["calcps", "newuvw", "cfg1", "cfg2", "ic", "spmv"],
                    help="run only this block (an assembly on a --scale^3 box, default 128, "
                         "the config-1 latency block, the config-2 block, IC(0) CG on the "
                         "config-3 system at --scale^3, or the standalone product on the "
                         "config-3 system at --scale^3, default 256), print its JSON and exit")
    ap.add_argument("--ic-iters", type=int, default=0,
                    help="--block ic: iteration cap of each solve (0 = to the tolerance)")
    ap.add_argument("--ic-tiled", type=int, default=-1,
                    help="--block ic: 1 tiled sweeps only, 0 level-ordered only, -1 both")
    ap.add_argument("--ic-precisions", default="fp64,fp64_fma,mixed",
                    help="--block ic: comma-separated precisions to time")
    ap.add_argument("--ic-restart", type=int, default=None,
                    help="--block ic: mixed refinement, 1 restarted, 0 reliable updates")
    ap.add_argument("--ic-blocks", default="0",
                    help="--block ic: comma-separated threads per block (0 = default)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.block:
        import torch
        import __graft_entry__ as ge
        pkg = ge.load_package()
        pkg.load_library()
        dev = torch.device("cuda", 0)
        if args.block == "cfg1":
            print(json.dumps(cfg1_latency(pkg, dev)), flush=True)
            return
        if args.block == "cfg2":
            print(json.dumps(cfg2_block(pkg, dev, load_peaks()[0])), flush=True)
            return
        if args.block == "spmv":
            s = make_workload(pkg, "cfg3", args.scale)
            topo = pkg.Topology.from_system(s)
            val = torch.from_numpy(s.A[:-1].copy()).to(dev)
            print(json.dumps(spmv_block(topo, s, val, load_peaks()[0], dev)), flush=True)
            topo.close()
            return
        if args.block == "ic":
            tiled = (0, 1) if args.ic_tiled < 0 else (args.ic_tiled,)
            print(json.dumps(ic_block(pkg, dev, n=args.scale or 128, iters=args.ic_iters,
                                      precisions=tuple(args.ic_precisions.split(",")),
                                      tiled=tiled, reps=1 if args.ic_iters else 2,
                                      blocks=tuple(int(b) for b in args.ic_blocks.split(",")),
                                      restart=args.ic_restart)),
                  flush=True)
            return
        fn = {"calcps": assembly_block, "newuvw": momentum_block}[args.block]
        print(json.dumps(fn(pkg, dev, n=args.scale or 128)), flush=True)
        return

    import torch
    import torch.distributed as dist

    import __graft_entry__ as ge
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    pkg = ge.load_package()
    pkg.load_library()
    peak, peak_kind = load_peaks()

    s = make_workload(pkg, args.workload, args.scale)
    method, prec = args.method, args.prec
    dev = torch.device("cuda", local)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    prec_mode = precision_mode(pkg, args.precision)
    ic = {}
    if prec == 2:
        ic["ic_sweeps"] = args.ic_sweeps
        if args.precision == "mixed" and args.ic_factors == "bf16":
            ic["ic_bf16"] = 1
    opts = pkg.options(precision=prec_mode, autotune=int(not args.no_autotune), **ic)
    tuning = None
    if not args.no_autotune:
        # launch shape (threads per block, rows per warp) timed on this
        # system before the timed region; every timed solve uses it
        tuning = topo.autotune(val, b, method, prec, opts=pkg.options(precision=prec_mode, **ic))

    def barrier():
        if world > 1:
            dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    el, results = device_solves(pkg, topo, val, b, x, method, prec, s.tol, opts, args.steps,
                                args.warmup, barrier)
    clk = clocks.stop()
    el = max_over_ranks(el, world, dev)
    value = world * args.steps / el
    kern_s = sum(r["seconds"] for r in results)
    kern_b = sum(r["bytes"] for r in results)
    last = results[-1]
    mixed = args.precision == "mixed"
    dtype = {"fp64": "f64", "fp64_fma": "f64"}.get(args.precision,
                                                   "f32+bf16+f64" if ic.get("ic_bf16") else "f32+f64")
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": dtype, "data": "synthetic",
        "config": workload_config(s, method, prec, args.precision),
        "arithmetic": ARITHMETIC[args.precision] +
                      (f"; IC(0) factor entries {args.ic_factors.upper()}, "
                       + ("exact triangular sweeps" if not args.ic_sweeps
                          else f"{args.ic_sweeps} Jacobi sweeps per triangle")
                       if prec == 2 else ""),
        "launch": ({"autotuned": True, **tuning} if tuning else
                   {"autotuned": False, "block_size": 256}),
        "iterations": last["inner_iterations"] if mixed else last["iterations"],
        "refinements": last["refinements"] if mixed else None,
        "fin_res": last["fin_res"], "tol": s.tol,
        "time_to_tol_ms": 1e3 * el / args.steps,
    }
    line["config"]["workload"] = (f"{s.name}: {method} + " +
                                  ({2: "IC(0)", 1: "diagonal"}.get(prec, "no") + " preconditioning")
                                  + f", {ARITHMETIC[args.precision]}, to ||r|| < 1e-8*||b|| "
                                    "(the reference's absolute test), x0 = 0")
    achieved = kern_b / kern_s / 1e9
    kname = {"fp64": "krylov_kernel_fp64", "fp64_fma": "krylov_kernel_fp64_fma",
             "mixed": "mixed_kernel"}[args.precision]
    line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak,
                        "traffic": profiled_traffic(kname, s.name, method, prec),
                        "kernel": {"fp64": "ref::krylov_kernel<double>",
                                   "fp64_fma": "fma::krylov_kernel<double>",
                                   "mixed": "fma::mixed_kernel"}[args.precision]
                                  + " (one persistent launch per solve)",
                        "limiter": profiled_limiter(kname, s.name, method, prec),
                        "peak_kind": peak_kind}

    if not args.no_e2e:
        t, io = legacy_e2e(pkg, s, method, prec,
                           {"precision": prec_mode, "autotune": int(not args.no_autotune), **ic},
                           args.steps, args.warmup)
        t = max_over_ranks(t, world, dev)
        line["e2e"] = {"value": world * args.steps / t, "unit": "solves/s",
                       "via": f"tflows_{method} (Fortran-facing C ABI), pinned host buffers", **io}
    line["clocks"] = clk
    line["gpu_launches"] = 2 * args.steps
    if rank == 0 and args.workload == "cfg3" and not args.no_compare:
        headline = {"ms": 1e3 * el / args.steps, "iterations": last["iterations"],
                    "inner_iterations": last["inner_iterations"],
                    "refinements": last["refinements"], "fin_res": last["fin_res"],
                    "status": last["status"], "gbs": achieved,
                    "block_size": last["block_size"], "grid_blocks": last["grid_blocks"]}
        line["comparison"] = cfg3_comparison(pkg, dev, topo, s, val, b, headline, x.clone())
        line["rel_err_vs_tight_fp64"] = line["comparison"]["mixed_ic_exact_bf16"]["rel_err_vs_tight_fp64"]
        line["speedups"] = line["comparison"]["speedups"]
    if rank == 0 and not args.no_extras:
        line["spmv"] = spmv_block(topo, s, val, peak, dev)
    topo.close()
    del val, b, x
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_cpu_baseline:
        ref_it = (line.get("comparison", {}).get("fp64_ic_exact", {}).get("iterations")
                  if prec == 2 else None)
        sampler = OracleSampler(s, method, prec, 1, args.oracle_iters, ref_it)
        t0 = time.perf_counter()
        v, _, t_full = sampler.sample()
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": sampler.describe(time.perf_counter() - t0),
                                "full_solve_seconds": t_full,
                                "oracle_full_run_iterations": sampler.full_it}
    if rank == 0 and not args.no_extras:
        line["cfg2"] = cfg2_block(pkg, dev, peak, cpu_seconds=5.0)
        torch.cuda.empty_cache()
        line["cfg1_latency"] = cfg1_latency(pkg, dev)
        line["adjoint_cfg5"] = adjoint_cfg5(pkg, dev)
        torch.cuda.empty_cache()
        line["simple_step"] = simple_step(pkg, dev, autotune=not args.no_autotune)
        torch.cuda.empty_cache()
        line["assembly_calcps"] = assembly_block(pkg, dev)
        line["assembly_newuvw"] = momentum_block(pkg, dev)
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_batch:
        line["batched_cfg4"] = batched_cfg4(pkg, dev, 2, autotune=not args.no_autotune)
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
