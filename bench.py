#!/usr/bin/env python
"""Benchmark of the GB300 Krylov solver core.

Metric: time to a 1e-8 relative residual of the T-FlowS solvers, reported as
whole-job solves/s (higher is better), with the HBM bandwidth the solver
kernel achieves.  Default workload: 128^3 perturbed-hex convection-diffusion
system (momentum / scalar transport), BiCG with diagonal preconditioning in
FP64 with fused multiply-adds (--precision fp64 for the reference's own
arithmetic), the reference's convergence test (absolute tolerance
1e-8*||b||), x0 = 0.  Synthetic data (seeded); the matrix and vectors
(~260 MB) exceed the 129 MB L2, so no flush is needed between steps.

A "step" is one complete solve.  `value` times K solves on data resident in
HBM (device API); `e2e` times K calls of the Fortran-facing C ABI
(tflows_bicg) with the matrix, x and b in pinned host memory, host<->device
copies inside each call.  The CPU baseline is the oracle (the reference's
algorithm restated in C) on the host cores.

Multi-GPU: the solves are independent replicas (one per rank, no
collective); value = total solves / max-over-ranks time.

--impl reference: the reference algorithm (oracle port, FP64, serial per
solve as in the reference) on the host cores, one solve per core at a time.
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


def run_reference(args):
    import __graft_entry__ as ge
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pkg = ge.load_package()
    s = pkg.mesh.config_system(2)
    cores = os.cpu_count() or 1
    # W warm-up steps and K timed steps; each step is one round of
    # concurrent solves (one per core).
    import oracle
    oracle.build()
    for _ in range(args.warmup):
        cpu_reference_throughput(s, "bicg", 1, cores, 0.0)
    t0 = time.perf_counter()
    total = 0
    it = 0
    for _ in range(args.steps):
        _, n, it, _ = cpu_reference_throughput(s, "bicg", 1, cores, 0.0)
        total += n
    el = time.perf_counter() - t0
    value = total / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(s, "bicg", 1),
        "arithmetic": "FP64 as the reference (oracle C restatement, no fused multiply-adds)",
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent full BiCG solves per step "
                                   f"({it} iterations each), oracle C restatement, 1 thread each"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(s, method, prec):
    return {"workload": f"{s.name}: {method} solve to 1e-8*||b|| (absolute test as the "
                        f"reference), x0=0, prec {prec}",
            "n": s.N, "nnz": s.nnz, "method": method, "prec": prec,
            "l2": "inputs larger than L2 (no flush)"}


ARITHMETIC = {"fp64": "FP64, reference arithmetic (separate rounded products and sums)",
              "fp64_fma": "FP64 with fused multiply-adds and a reciprocal diagonal",
              "mixed": "FP32 inner solves, FP64 refinement"}


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


IC_VARIANTS = (("exact_fp32", {}), ("exact_bf16", {"ic_bf16": 1}),
               ("jacobi1_bf16", {"ic_sweeps": 1, "ic_bf16": 1}),
               ("jacobi2_bf16", {"ic_sweeps": 2, "ic_bf16": 1}),
               ("jacobi2_fp32", {"ic_sweeps": 2}),
               ("jacobi4_bf16", {"ic_sweeps": 4, "ic_bf16": 1}))


def mixed_vs_fp64(pkg, dev, scale, precs, reps):
    """The variable-density pressure system (cfg3): CG with each given
    preconditioner in FP64 (reference arithmetic) and in mixed precision
    (FP32 inner solves, FP64 refinement), same absolute tolerance.  With
    IC(0) the mixed solve is run with each factor variant (FP32 or BF16
    factor entries, exact triangular solves or k Jacobi sweeps)."""
    import torch
    s = make_workload(pkg, "cfg3", scale)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)

    def run(prec, opts):
        # every variant runs with its own tuned launch shape (tuned on the
        # first, untimed solve)
        opts.autotune = 1
        el, out = device_solves(pkg, topo, val, b, x, "cg", prec, s.tol, opts, reps, 1)
        r = out[-1]
        return {"ms": 1e3 * el / reps, "iterations": r["iterations"],
                "refinements": r["refinements"], "fin_res": r["fin_res"],
                "gbs": r["bytes"] / r["seconds"] / 1e9, "status": r["status"],
                "block_size": r["block_size"], "grid_blocks": r["grid_blocks"]}, x.clone()

    result = {}
    for prec in precs:
        fp, x64 = run(prec, pkg.options(precision=pkg.FP64))
        fpf, _ = run(prec, pkg.options(precision=pkg.FP64_FMA))
        variants = IC_VARIANTS if prec == 2 else (("jacobi_fp32", {}),)
        mixed = {}
        for label, kw in variants:
            rec, xm = run(prec, pkg.options(precision=pkg.MIXED, **kw))
            rec["rel_diff_vs_fp64"] = float((xm - x64).abs().max() / x64.abs().max())
            mixed[label] = rec
        ok = [k for k in mixed if mixed[k]["status"] == pkg.OK] or list(mixed)
        best = min(ok, key=lambda k: mixed[k]["ms"])
        result[prec] = {"workload": f"{s.name}, CG prec {prec}, tol 1e-8*||b|| absolute",
                        "n": s.N, "fp64": fp, "fp64_fma": fpf, "mixed": mixed[best],
                        "mixed_variant": best,
                        "speedup": fp["ms"] / mixed[best]["ms"],
                        "speedup_vs_fp64_fma": fpf["ms"] / mixed[best]["ms"],
                        "mixed_rel_diff_vs_fp64": mixed[best]["rel_diff_vs_fp64"]}
        if len(mixed) > 1:
            result[prec]["all_mixed_variants"] = mixed
    topo.close()
    return result


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
        variants[label] = {
            "ms_per_batch": ms, "systems_per_s": count * 1e3 / ms,
            "converged": sum(1 for r in res if r["status"] == pkg.OK),
            "max_iterations": max(r["iterations"] for r in res),
            "gbs": byts / (ms * 1e-3) / 1e9, "tuning": tuning,
            "group_blocks": [r["grid_blocks"] for r in res]}
        plan.close()
    best = min(variants, key=lambda k: variants[k]["ms_per_batch"])
    out = {"workload": f"{count} systems, sizes {min(s.N for s, _, _ in systems)}.."
                       f"{max(s.N for s, _, _ in systems)} rows (total {rows}), odd: CG+IC "
                       "pressure, even: BiCG+diag transport, mixed precision, tol 1e-8 relative, "
                       "one graph-captured cooperative launch",
           "variant": best, **variants[best]}
    out["all_variants"] = {k: {kk: vv for kk, vv in v.items() if kk != "group_blocks"}
                           for k, v in variants.items()}
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
    return {"workload": f"{s.name} differentiable CG + diagonal, rtol 1e-10, loss 0.5||x-x_t||^2",
            "n": s.N, "ms_per_forward_backward": ms,
            "forward": {"iterations": fw["iterations"], "ms": 1e3 * fw["seconds"]},
            "adjoint": {"iterations": bw["iterations"], "ms": 1e3 * bw["seconds"]},
            "grad_b_norm": float(b.grad.norm()), "grad_coef_norm": float(coef.grad.norm())}


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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg5"])
    ap.add_argument("--scale", type=int, default=None, help="box edge (default: the config's)")
    ap.add_argument("--method", default="bicg")
    ap.add_argument("--prec", type=int, default=1)
    ap.add_argument("--precision", default="fp64_fma", choices=["fp64", "fp64_fma", "mixed"],
                    help="fp64: reference arithmetic; fp64_fma: FP64 with fused multiply-adds "
                         "(within 1e-8 of the reference); mixed: FP32 inner + FP64 refinement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--compare-scale", type=int, default=256,
                    help="edge of the cfg3 mixed-vs-FP64 comparison (0 = skip)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched (cfg4) block")
    ap.add_argument("--ic-sweeps", type=int, default=0,
                    help="mixed + prec 2: Jacobi sweeps per triangle (0 = exact sweeps)")
    ap.add_argument("--ic-bf16", action="store_true", help="mixed + prec 2: BF16 factor entries")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the config-2 method, config-5 adjoint and SIMPLE-step blocks")
    ap.add_argument("--no-autotune", action="store_true",
                    help="fixed launch shape (256 threads, one slice per warp)")
    ap.add_argument("--ic-compare-scale", type=int, default=256,
                    help="edge of the IC mixed-vs-FP64 comparison (0 = skip)")
    ap.add_argument("--block", default=None, choices=["calcps", "newuvw", "cfg1", "ic"],
                    help="run only this block (an assembly on a --scale^3 box, default 128, "
                         "the config-1 latency block, or IC(0) CG on the config-3 system at "
                         "--scale^3), print its JSON and exit")
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

    import numpy as np
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
    tol = s.tol
    dev = torch.device("cuda", local)
    topo = pkg.Topology.from_system(s)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    prec_mode = {"fp64": pkg.FP64, "fp64_fma": pkg.FP64_FMA, "mixed": pkg.MIXED}[args.precision]
    ic = {"ic_sweeps": args.ic_sweeps, "ic_bf16": int(args.ic_bf16)}
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
    el, results = device_solves(pkg, topo, val, b, x, method, prec, tol, opts, args.steps,
                                args.warmup, barrier)
    clk = clocks.stop()
    el = max_over_ranks(el, world, dev)
    value = world * args.steps / el
    kern_s = sum(r["seconds"] for r in results)
    kern_b = sum(r["bytes"] for r in results)
    iters = [r["iterations"] for r in results]

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": workload_config(s, method, prec),
        "arithmetic": ARITHMETIC[args.precision],
        "launch": ({"autotuned": True, **tuning} if tuning else
                   {"autotuned": False, "block_size": 256}),
        "iterations": int(statistics.median(iters)),
        "time_to_tol_ms": 1e3 * el / args.steps,
    }
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
        # e2e through the Fortran-facing C ABI, inputs in pinned host memory.
        A_h = torch.from_numpy(s.A.copy()).pin_memory().numpy()
        x_h = torch.zeros(s.NB + s.N + 1, dtype=torch.float64).pin_memory().numpy()
        r_h = torch.zeros(s.N, dtype=torch.float64).pin_memory().numpy()
        pkg.set_options(precision=prec_mode, autotune=int(not args.no_autotune))
        legacy = {"cg": pkg.cg, "bicg": pkg.bicg, "cgs": pkg.cgs}[method]
        e2e_t = 0.0
        for k in range(args.warmup + args.steps):
            x_h[:] = 0.0
            r_h[:] = s.b
            t0 = time.perf_counter()
            out = legacy(s.N, s.NB, s.NONZ, A_h, s.Acol, s.Arow, s.Adia, s.Ab, x_h, r_h, prec,
                         20000, tol)
            t1 = time.perf_counter()
            if k >= args.warmup:
                e2e_t += t1 - t0
        pkg.set_options()
        if out.status != pkg.OK:
            raise RuntimeError(f"e2e solve failed: {out}")
        e2e_t = max_over_ranks(e2e_t, world, dev)
        line["e2e"] = {"value": world * args.steps / e2e_t, "unit": "solves/s",
                       "h2d_bytes_per_step": int(8 * s.nnz + 16 * s.N),
                       "d2h_bytes_per_step": int(16 * s.N)}

    # standalone SELL products (FP64 and FP32) for the SpMV roofline
    y = torch.empty_like(x)
    xs = torch.rand(s.N, dtype=torch.float64, device=dev)
    sl = (s.N + 31) // 32
    for tag, fp32, sv in (("spmv_fp64", False, 8), ("spmv_fp32", True, 4)):
        sec = topo.spmv(val, xs, y, repeat=20, fp32=fp32)
        idx = s.N if topo.patterns else 4.0 * s.nnz  # pattern id per row, or a column per entry
        byts = s.nnz * sv + idx + 8.0 * (sl + 1) + 2.0 * s.N * sv
        line[tag] = {"gbs": byts / sec / 1e9, "frac": byts / sec / 1e9 / peak, "us": sec * 1e6,
                     "bytes": byts}
    line["clocks"] = clk
    line["gpu_launches"] = 2 * args.steps
    x_gpu = x.cpu().numpy()
    if rank == 0 and not args.no_extras:
        line["cfg2_methods"] = cfg2_methods(pkg, dev, topo, s, val, b)
    topo.close()
    del val, b, x, y, xs
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_extras:
        line["cfg1_latency"] = cfg1_latency(pkg, dev)
        line["adjoint_cfg5"] = adjoint_cfg5(pkg, dev)
        torch.cuda.empty_cache()
        line["simple_step"] = simple_step(pkg, dev, autotune=not args.no_autotune)
        torch.cuda.empty_cache()
        line["assembly_calcps"] = assembly_block(pkg, dev)
        line["assembly_newuvw"] = momentum_block(pkg, dev)
        torch.cuda.empty_cache()

    if rank == 0 and (args.compare_scale or args.ic_compare_scale):
        # cfg3 at the comparison scale: diagonal and IC(0) preconditioning
        same = args.compare_scale == args.ic_compare_scale
        if args.compare_scale:
            cmp = mixed_vs_fp64(pkg, dev, args.compare_scale, (1, 2) if same else (1,), 1)
            line["mixed_vs_fp64"] = cmp[1]
            if same:
                line["mixed_vs_fp64_ic"] = cmp[2]
            torch.cuda.empty_cache()
        if args.ic_compare_scale and not same:
            line["mixed_vs_fp64_ic"] = mixed_vs_fp64(pkg, dev, args.ic_compare_scale, (2,), 1)[2]
            torch.cuda.empty_cache()
    if rank == 0 and not args.no_batch:
        line["batched_cfg4"] = batched_cfg4(pkg, dev, 2, autotune=not args.no_autotune)
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_cpu_baseline:
        v, n, it, el_c = cpu_reference_throughput(s, method, prec, 1, args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": f"{n} full {method} solves ({it} iterations) of the "
                                          f"same system, oracle C restatement, 1 thread, "
                                          f"{el_c:.1f} s"}
        # the GPU answer against the CPU restatement of the reference
        import oracle
        xo, _, it_o, _, _ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                         s.Ab, s.x, s.b, prec, 20000, tol)
        xo = xo[s.NB + 1:]
        line["rel_err_vs_oracle"] = float(np.abs(x_gpu - xo).max() / np.abs(xo).max())
        line["oracle_iterations"] = int(it_o)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
