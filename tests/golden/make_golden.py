"""Generate the golden fixtures by executing the reference's own source text.

Reads Process/{CG,BiCG,CGS,Prec1,Resid}.f90 from a T-FlowS checkout (default
the path given as the first argument or in TFLOWS_REFERENCE), translates them
with fortran_subset.py, runs a fixed list of small cases through the
translated subroutines and writes one .npz per case into this directory:
inputs (the Fortran-layout arrays and scalars) and outputs (x, r1, niter,
IniRes, FinRes, and the module variable `error` after the call; D for Prec1,
r1 for Resid).  Cases that chain calls (to pin the module state carried
between calls) store every call of the chain.

Run:  python tests/golden/make_golden.py [/path/to/T-FlowS]
"""
from __future__ import annotations

import os
import sys
import time
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

from fortran_subset import FArr, Module, load_subroutines  # noqa: E402

FILES = ("CG.f90", "BiCG.f90", "CGS.f90", "Prec1.f90", "Resid.f90")
MODULE_ARRAYS = "d p1 p2 q1 q2 r2 u1 u2 v1 v2 nbbs nbbe bufind".split()
MODULE_SCALARS = "alfa beta rho rhoold bnrm2 sum1 sum2 error i j k iter sub npro".split()


def _mesh():
    import importlib.util
    pkg = os.path.join(REPO, "t-flows-old-compressible_gb300", "mesh.py")
    spec = importlib.util.spec_from_file_location("_golden_mesh", pkg)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def reference_subroutines(root):
    texts = [open(os.path.join(root, "Process", f)).read() for f in FILES]
    names = {n: "array" for n in MODULE_ARRAYS}
    names.update({n: "scalar" for n in MODULE_SCALARS})
    subs, _ = load_subroutines(texts, names, {"tiny": "1e-64"})
    return subs


def new_module(N, NB):
    """sol_mod / par_mod state as Process/GeoAloc.f90:40-49 allocates it
    (zero-filled), single domain (Npro = 0)."""
    z = lambda lo, hi: FArr([np.float64(0.0)] * (hi - lo + 1), 0, lo)  # noqa: E731
    M = Module(npro=0, nbbs=FArr([0], 0, 1), nbbe=FArr([0], 0, 1), bufind=FArr([0], 0, 1))
    M.d = z(1, N)
    M.p1, M.p2 = z(-NB, N), z(-NB, N)
    for n in ("q1", "q2", "r2", "u1", "u2", "v1", "v2"):
        setattr(M, n, z(1, N))
    for n in ("alfa", "beta", "rho", "rhoold", "bnrm2", "sum1", "sum2", "error"):
        setattr(M, n, np.float64(0.0))
    for n in ("i", "j", "k", "iter", "sub"):
        setattr(M, n, 0)
    return M


def _reals(a):
    return [np.float64(v) for v in np.asarray(a, dtype=np.float64)]


def run_solver(subs, M, method, s, x, r1, prec, niter, tol, ini=np.nan, fin=np.nan):
    A = FArr(_reals(s.A))
    Acol = FArr([int(v) for v in s.Acol])
    Arow = FArr([int(v) for v in s.Arow])
    Adia = FArr([int(v) for v in s.Adia])
    Ab = FArr(_reals(s.Ab) or [np.float64(0.0)])
    xb = _reals(x)
    rb = _reals(r1)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        out = subs[method](M, s.N, s.NB, s.NONZ, A, Acol, Arow, Adia, Ab, FArr(xb), FArr(rb),
                           prec, niter, np.float64(tol), np.float64(ini), np.float64(fin))
    return (np.array(xb), np.array(rb), int(out["niter"]), float(out["inires"]),
            float(out["finres"]), float(M.error))


def small_systems(mesh):
    return {
        "p543": mesh.pressure_system(5, 4, 3, perturb=0.0, seed=1),
        "pvd444": mesh.pressure_system(4, 4, 4, perturb=0.2, seed=2, variable_density=True),
        "cd453": mesh.convection_diffusion_system(4, 5, 3, perturb=0.2, seed=3),
        "cd333": mesh.convection_diffusion_system(3, 3, 3, perturb=0.2, seed=4, dt=10.0),
        "p1": mesh.pressure_system(1, 1, 1, seed=5),
        "p311": mesh.pressure_system(3, 1, 1, seed=6),
        "pvd876": mesh.pressure_system(8, 7, 6, perturb=0.2, seed=8, variable_density=True),
        "cd765": mesh.convection_diffusion_system(7, 6, 5, perturb=0.2, seed=9, dt=1.0),
    }


def cases(mesh):
    """(name, system key, [calls]); each call = (method, prec, niter, rel_tol,
    x0 kind).  Calls of one case share the module state."""
    return [
        ("cg_p543_prec0", "p543", [("cg", 0, 400, 1e-10, "zero")]),
        ("cg_p543_prec1", "p543", [("cg", 1, 400, 1e-10, "zero")]),
        ("cg_p543_prec2", "p543", [("cg", 2, 400, 1e-10, "zero")]),
        ("cg_pvd444_prec2_warm", "pvd444", [("cg", 2, 400, 1e-9, "rand")]),
        ("cg_pvd444_prec1_maxiter", "pvd444", [("cg", 1, 5, 1e-12, "zero")]),
        ("cg_cd453_nonsym_prec1", "cd453", [("cg", 1, 50, 1e-8, "zero")]),
        ("bicg_cd453_prec1", "cd453", [("bicg", 1, 200, 1e-10, "zero")]),
        ("bicg_cd453_prec2", "cd453", [("bicg", 2, 200, 1e-10, "rand")]),
        ("bicg_cd333_prec0", "cd333", [("bicg", 0, 200, 1e-10, "zero")]),
        ("cgs_cd453_prec0", "cd453", [("cgs", 0, 200, 1e-10, "zero")]),
        ("cgs_cd453_prec1", "cd453", [("cgs", 1, 200, 1e-10, "rand")]),
        ("cgs_cd453_prec2", "cd453", [("cgs", 2, 200, 1e-10, "zero")]),
        ("cgs_p543_prec2_maxiter", "p543", [("cgs", 2, 3, 1e-14, "zero")]),
        ("cg_p1_single_cell", "p1", [("cg", 1, 10, 1e-12, "rhs_one")]),
        # b = 0 with tol = 0: nothing exits early, alfa = 0/0 and NaN runs
        # to the iteration limit (niter_in + 1, FinRes NaN).
        ("cg_p1_zero_rhs_zero_tol_nan", "p1", [("cg", 1, 4, 0.0, "zero")]),
        ("cg_p311_prec2", "p311", [("cg", 2, 10, 1e-12, "zero")]),
        ("cg_pvd876_prec2", "pvd876", [("cg", 2, 800, 1e-10, "zero")]),
        ("cg_pvd876_prec1", "pvd876", [("cg", 1, 800, 1e-10, "rand")]),
        ("bicg_cd765_prec2", "cd765", [("bicg", 2, 200, 1e-12, "zero")]),
        ("cgs_cd765_prec1", "cd765", [("cgs", 1, 200, 1e-12, "rand")]),
        ("cgs_cd765_prec2", "cd765", [("cgs", 2, 200, 1e-12, "zero")]),
        # Module state: a zero RHS exits on ||b|| < tol and reports the
        # previous call's `error` as FinRes; IniRes is left untouched.
        ("chain_cg_then_zero_rhs", "p543", [("cg", 1, 400, 1e-10, "zero"),
                                             ("cg", 1, 400, 1e-10, "zero_rhs"),
                                             ("bicg", 2, 400, 1e-10, "zero_rhs")]),
        # Warm start at the solution: exits on IniRes < tol with iter = 0.
        ("chain_cg_restart_at_solution", "p543", [("cg", 2, 400, 1e-10, "zero"),
                                                   ("cg", 2, 400, 1e-6, "previous")]),
    ]


def main(root):
    mesh = _mesh()
    subs = reference_subroutines(root)
    systems = small_systems(mesh)
    for name, key, calls in cases(mesh):
        s = systems[key]
        M = new_module(s.N, s.NB)
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        rec = dict(N=s.N, NB=s.NB, NONZ=s.NONZ, A=s.A, Acol=s.Acol, Arow=s.Arow, Adia=s.Adia,
                   Ab=s.Ab, ncalls=len(calls))
        prev_x = None
        t0 = time.time()
        for ci, (method, prec, niter, rel, x0kind) in enumerate(calls):
            x = s.x.copy()
            b = s.b.copy()
            if x0kind == "rand":
                x[s.NB + 1:] = rng.uniform(-1.0, 1.0, s.N)
            elif x0kind == "previous":
                x = prev_x.copy()
            elif x0kind == "zero_rhs":
                b[:] = 0.0
            elif x0kind == "rhs_one":
                b[:] = 1.0
            tol = rel * float(np.sqrt(np.dot(b, b))) if x0kind != "zero_rhs" else \
                rel * float(np.sqrt(np.dot(s.b, s.b)))
            ini_in = -1.0 - ci
            fin_in = -2.0 - ci
            xo, ro, it, ini, fin, err = run_solver(subs, M, method, s, x, b, prec, niter, tol,
                                                   ini_in, fin_in)
            prev_x = xo
            p = f"c{ci}_"
            rec.update({p + "method": method, p + "prec": prec, p + "niter_in": niter,
                        p + "tol": tol, p + "x_in": x, p + "r1_in": b, p + "IniRes_in": ini_in,
                        p + "FinRes_in": fin_in, p + "x_out": xo, p + "r1_out": ro,
                        p + "niter_out": it, p + "IniRes_out": ini, p + "FinRes_out": fin,
                        p + "error_state": err})
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(f"{name:34s} N={s.N:4d} calls={len(calls)} "
              f"niter_out={[int(rec[f'c{i}_niter_out']) for i in range(len(calls))]} "
              f"({time.time() - t0:.1f}s)")

    # Prec1 and Resid on their own, all three preconditioner settings.
    for key in ("cd453", "pvd444"):
        s = systems[key]
        rec = dict(N=s.N, NB=s.NB, NONZ=s.NONZ, A=s.A, Acol=s.Acol, Arow=s.Arow, Adia=s.Adia,
                   Ab=s.Ab)
        for prec in (0, 1, 2):
            D = FArr([np.float64(0.0)] * s.N)
            subs["prec1"](None, s.N, s.NONZ, FArr(_reals(s.A)),
                          FArr(list(map(int, s.Acol))), FArr(list(map(int, s.Arow))),
                          FArr(list(map(int, s.Adia))), D, prec)
            rec[f"D_prec{prec}"] = np.array(D.buf)
        rng = np.random.default_rng(7)
        x = rng.uniform(-1, 1, s.NB + s.N + 1)
        r = FArr(_reals(s.b))
        M = new_module(s.N, s.NB)
        subs["resid"](M, s.N, s.NB, s.NONZ, FArr(_reals(s.A)),
                      FArr(list(map(int, s.Acol))), FArr(list(map(int, s.Arow))),
                      FArr(_reals(s.Ab) or [np.float64(0.0)]), FArr(_reals(x)), r)
        rec.update(resid_x=x, resid_r1_in=s.b, resid_r1_out=np.array(r.buf))
        np.savez_compressed(os.path.join(HERE, f"prec1_resid_{key}.npz"), **rec)
        print(f"prec1_resid_{key}")



def reference_root():
    """The T-FlowS checkout to read: the first argument, else the
    TFLOWS_REFERENCE environment variable; one of them is required."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TFLOWS_REFERENCE")
    if not root:
        sys.exit(f"usage: {os.path.basename(sys.argv[0])} PATH_TO_T-FLOWS_CHECKOUT "
                 "(or set TFLOWS_REFERENCE)")
    return root

if __name__ == "__main__":
    main(reference_root())
