"""One full oracle solve of a benchmark system (test infrastructure).

Runs the C restatement of the reference solver (oracle/krylov_oracle.c) on
one of the benchmark workloads to the benchmark tolerance and prints one JSON
line: iterations, IniRes, FinRes and wall time on one host core.  The
benchmark's CPU legs time bounded samples of oracle iterations and scale them
by the iteration count of such a run, because a full 256^3 IC(0) solve takes
many minutes on one core.

    python oracle/full_solve.py --config 3 --scale 256 --method cg --prec 2
"""
import argparse
import json
import os
import platform
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--scale", type=int, default=None)
    ap.add_argument("--method", default="cg")
    ap.add_argument("--prec", type=int, default=2)
    ap.add_argument("--maxiter", type=int, default=20000)
    a = ap.parse_args()
    import __graft_entry__ as ge
    import oracle
    oracle.build()
    pkg = ge.load_package()
    t0 = time.perf_counter()
    s = pkg.mesh.config_system(a.config, scale=a.scale)
    t_mesh = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, _, it, ini, fin = oracle.solve(a.method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                      s.Ab, s.x, s.b, a.prec, a.maxiter, s.tol)
    el = time.perf_counter() - t0
    print(json.dumps({"workload": s.name, "method": a.method, "prec": a.prec, "n": s.N,
                      "tol": s.tol, "iterations": it, "ini_res": ini, "fin_res": fin,
                      "seconds": el, "mesh_seconds": t_mesh, "cores": 1,
                      "host": platform.processor() or platform.machine()}), flush=True)


if __name__ == "__main__":
    main()
