"""ORACLE -- test infrastructure only (see krylov_oracle.c).

ctypes access to the C restatement of the reference's Krylov solver path.
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs import this package, as the reference the GPU results are
compared with or as the timed CPU baseline; the product library never loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkrylov_oracle.so")
_lib = None
_lock = threading.Lock()

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with make (gcc, -O3 -ffp-contract=off)."""
    srcs = ("krylov_oracle.c", "assembly_oracle.c")
    if force or not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, f)) for f in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            solver_args = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _I, _I, _I, _D, _D,
                           _D, ctypes.c_int, _I, ctypes.c_double, _D, _D]
            for name in ("oracle_cg", "oracle_bicg", "oracle_cgs"):
                fn = getattr(L, name)
                fn.argtypes = solver_args
                fn.restype = None
            L.oracle_prec1.argtypes = [ctypes.c_int, ctypes.c_int, _D, _I, _I, _I, _D, ctypes.c_int]
            L.oracle_prec1.restype = None
            L.oracle_resid.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _I, _I, _D,
                                       _D, _D]
            L.oracle_resid.restype = None
            L.oracle_topolm.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _I, _I, _I]
            L.oracle_topolm.restype = ctypes.c_int
            L.oracle_reset_state.argtypes = []
            L.oracle_reset_state.restype = None
            L.oracle_error_state.argtypes = []
            L.oracle_error_state.restype = ctypes.c_double
            L.oracle_calcps_assembly.argtypes = (
                [ctypes.c_int] * 5 + [ctypes.c_double] + [_I] * 4 + [_D] * 24)
            L.oracle_calcps_assembly.restype = None
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def reset_state():
    lib().oracle_reset_state()


def error_state() -> float:
    return lib().oracle_error_state()


def solve(method, N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1, prec, niter, tol,
          IniRes=float("nan"), FinRes=float("nan")):
    """Call oracle_<method> on copies; returns (x, r1, niter, IniRes, FinRes).

    ``x`` is the full x(-NB:N) array, ``Ab`` is Ab(-NB:-1) (length NB).
    """
    fn = {"cg": lib().oracle_cg, "bicg": lib().oracle_bicg, "cgs": lib().oracle_cgs}[method]
    A, Ab = _f64(A), _f64(Ab) if NB > 0 else np.zeros(1)
    Acol, Arow, Adia = _i32(Acol), _i32(Arow), _i32(Adia)
    xo, ro = _f64(x).copy(), _f64(r1).copy()
    it = ctypes.c_int(int(niter))
    ini, fin = ctypes.c_double(IniRes), ctypes.c_double(FinRes)
    fn(int(N), int(NB), int(NONZ), _dp(A), _ip(Acol), _ip(Arow), _ip(Adia), _dp(Ab), _dp(xo),
       _dp(ro), int(prec), ctypes.byref(it), float(tol), ctypes.byref(ini), ctypes.byref(fin))
    return xo, ro, it.value, ini.value, fin.value


def solve_system(method, sysm, prec, niter=1000, tol=None, x=None, b=None):
    """Convenience wrapper over a mesh.System."""
    return solve(method, sysm.N, sysm.NB, sysm.NONZ, sysm.A, sysm.Acol, sysm.Arow, sysm.Adia,
                 sysm.Ab, sysm.x if x is None else x, sysm.b if b is None else b, prec, niter,
                 sysm.tol if tol is None else tol)


def prec1(N, NONZ, A, Acol, Arow, Adia, prec):
    D = np.zeros(N)
    lib().oracle_prec1(int(N), int(NONZ), _dp(_f64(A)), _ip(_i32(Acol)), _ip(_i32(Arow)),
                       _ip(_i32(Adia)), _dp(D), int(prec))
    return D


def resid(N, NB, NONZ, A, Acol, Arow, Ab, x, r1):
    r = _f64(r1).copy()
    Abv = _f64(Ab) if NB > 0 else np.zeros(1)
    lib().oracle_resid(int(N), int(NB), int(NONZ), _dp(_f64(A)), _ip(_i32(Acol)),
                       _ip(_i32(Arow)), _dp(Abv), _dp(_f64(x)), _dp(r))
    return r


def topolm(NC, side_c):
    """Process/TopolM.f90 restated: SideC (NS, 2) 1-based -> (Acol, Arow, Adia, SidAij)."""
    sc = _i32(side_c)
    NS = sc.shape[0]
    ninterior = int((sc[:, 1] > 0).sum())
    nnz = NC + 2 * ninterior
    Acol = np.zeros(NC + 1, np.int32)
    Arow = np.zeros(nnz + 1, np.int32)
    Adia = np.zeros(NC, np.int32)
    sid = np.zeros((NS, 2), np.int32)
    nonz = lib().oracle_topolm(int(NC), int(NS), _ip(sc), _ip(Acol), _ip(Arow), _ip(Adia),
                               _ip(sid))
    assert nonz == nnz + 1
    return Acol, Arow, Adia, sid


CELL_FIELDS = ("volume", "Asave", "rho_n", "rho_o", "rho_oo", "U", "V", "W", "P", "Px", "Py",
               "Pz")
FACE_GEOM = ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f")


def calcps_assembly(NC, NbC, NS, NONZ, Nmat, dt, SideC, SidAij, Adia, TypeBC, geom, fields):
    """Process/CalcPS.f90:49-202 restated (assembly_oracle.c).

    SideC: (NS, 3) int array = SideC(0:2, NS) in memory order; SidAij (NS, 2);
    Adia (NC,) 1-based; TypeBC and every entry of ``fields`` (CELL_FIELDS)
    span cells -NbC..NC (index c + NbC); ``geom`` holds the FACE_GEOM arrays.
    Returns (Aval[NONZ], b[NC], Abou[NbC] (cells -NbC..-1), Flux[NS], errmax).
    """
    Aval, b = np.zeros(NONZ), np.zeros(NC)
    Abou, Flux = np.zeros(max(NbC, 1)), np.zeros(NS)
    em = ctypes.c_double()
    keep = [_i32(SideC), _i32(SidAij), _i32(Adia), _i32(TypeBC)]
    g = [_f64(geom[k]) for k in FACE_GEOM]
    fl = [_f64(fields[k]) for k in CELL_FIELDS]
    lib().oracle_calcps_assembly(int(NC), int(NbC), int(NS), int(NONZ), int(Nmat), float(dt),
                                 *[_ip(a) for a in keep], *[_dp(a) for a in g],
                                 *[_dp(a) for a in fl], _dp(Aval), _dp(b), _dp(Abou), _dp(Flux),
                                 ctypes.byref(em))
    return Aval, b, Abou[:NbC], Flux, em.value
