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
EXCHANGE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, _D, ctypes.c_int)
GLOSUM_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, _D)


def build(force: bool = False) -> str:
    """Compile the oracle with make (gcc, -O3 -ffp-contract=off)."""
    srcs = ("krylov_oracle.c", "assembly_oracle.c", "momentum_oracle.c")
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
            L.oracle_set_halo.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _I, EXCHANGE_FN,
                                          GLOSUM_FN, ctypes.c_void_p]
            L.oracle_set_halo.restype = None
            L.oracle_clear_halo.argtypes = []
            L.oracle_clear_halo.restype = None
            L.oracle_halo_failed.argtypes = []
            L.oracle_halo_failed.restype = ctypes.c_int
            L.oracle_reset_state.argtypes = []
            L.oracle_reset_state.restype = None
            L.oracle_error_state.argtypes = []
            L.oracle_error_state.restype = ctypes.c_double
            L.oracle_calcps_assembly.argtypes = (
                [ctypes.c_int] * 5 + [ctypes.c_double] + [_I] * 4 + [_D] * 24)
            L.oracle_calcps_assembly.restype = None
            _PP = ctypes.POINTER(_D)
            L.oracle_newuvw_assembly.argtypes = (
                [ctypes.c_int] * 4 + [_I, _D] + [_I] * 7 + [_D] * 3 + [_PP] * 3 + [_D] * 5
                + [_I])
            L.oracle_newuvw_assembly.restype = None
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


class halo:
    """Context manager: the oracle's subdomain run on the calling thread
    (oracle_set_halo).  ``NBBs``/``NBBe``: NBBs(sub), NBBe(sub) for
    sub = 1..Npro; ``BufInd``: BufInd(-NB:-1).  ``exchange(phi)`` swaps the
    neighbours' segments of PHI(-NB:-1) (``phi[NB + k]`` = PHI(k)) in place;
    ``glosum(v)`` returns the sum of ``v`` over the ranks.  Raises on exit
    when a callback failed."""

    def __init__(self, Npro, NB, NBBs, NBBe, BufInd, exchange, glosum):
        self.args = (_i32(NBBs), _i32(NBBe), _i32(BufInd if NB > 0 else np.zeros(1)))
        self.Npro, self.NB = int(Npro), int(NB)

        def _ex(user, phi, nb):
            try:
                exchange(np.ctypeslib.as_array(phi, shape=(nb,)))
                return 0
            except Exception:
                return 1

        def _gs(user, v):
            try:
                v[0] = float(glosum(float(v[0])))
                return 0
            except Exception:
                return 1

        self._ex, self._gs = EXCHANGE_FN(_ex), GLOSUM_FN(_gs)

    def __enter__(self):
        bs, be, bi = self.args
        lib().oracle_set_halo(self.Npro, self.NB, _ip(bs), _ip(be), _ip(bi), self._ex, self._gs,
                              None)
        return self

    def __exit__(self, exc_type, exc, tb):
        failed = lib().oracle_halo_failed()
        lib().oracle_clear_halo()
        if failed and exc_type is None:
            raise RuntimeError("oracle halo: an exchange or global-sum callback failed")
        return False


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


MOMENTUM_CELL_FIELDS = ("rho_n", "rho_o", "rho_oo", "ui_n", "ui_o", "ui_oo", "duidi", "duidj",
                        "duidk", "dujdi", "dukdi", "dujdj", "dukdk", "pi", "ui_source")
MOMENTUM_FACE_FIELDS = ("flux_u", "flux", "ff", "scoef")
# Processor.f90:314-340: the face vectors (Si, Sj, Sk, Di, Dj, Dk) per component
MOMENTUM_FACE_VECTORS = {1: ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz"),
                         2: ("Sy", "Sx", "Sz", "Dy", "Dx", "Dz"),
                         3: ("Sz", "Sx", "Sy", "Dz", "Dx", "Dy")}
# Process/IniPar.f90:22-49
SCHEME = {"ab": 1, "cn": 2, "fi": 3, "lin": 4, "par": 5, "yes": 10, "no": 11, "cds": 20,
          "quick": 21, "luds": 22, "minmod": 23, "smart": 24, "avl_smart": 25, "superbee": 26,
          "gamma": 27}


def momentum_assembly(NC, NbC, NS, NONZ, SideC, SidAij, Adia, TypeBC, material, geom, fields,
                      Nmat, var, blend, blend_tem, urfc, visc, dt, urf, convec=3, cross=3,
                      diffus=3, inert=4, moin_problem=0):
    """Process/NewUVW.f90:138-499 with ConvScheme.f90 and CalMinMax.f90
    restated (momentum_oracle.c), for momentum component ``var``.

    ``geom``: Sx..Dz, f (faces) and volume (cells -NbC..NC); ``fields``: the
    MOMENTUM_CELL_FIELDS over cells -NbC..NC and MOMENTUM_FACE_FIELDS over
    faces; material over cells -NbC..NC; blend, blend_tem, urfc per material.
    Returns (Aval[NONZ], b[NC], Abou[NbC], Asave[NC], rhoUi[NbC+NC+1],
    status); status 1 = undefined blending, 2 = material out of range.
    """
    Aval, b, Asave = np.zeros(NONZ), np.zeros(NC), np.zeros(NC)
    Abou, rhoUi = np.zeros(max(NbC, 1)), np.zeros(NbC + NC + 1)
    st = ctypes.c_int()
    iopt = _i32([Nmat, var, moin_problem, convec, cross, diffus, inert])
    dopt = _f64([visc, dt, urf])
    ints = [_i32(SideC), _i32(SidAij), _i32(Adia), _i32(TypeBC), _i32(material), _i32(blend),
            _i32(blend_tem)]
    dbl = [_f64(urfc), _f64(geom["f"]), _f64(geom["volume"])]
    fv = [_f64(geom[k]) for k in MOMENTUM_FACE_VECTORS[var]]
    ff = [_f64(fields[k]) for k in MOMENTUM_FACE_FIELDS]
    cf = [_f64(fields[k]) for k in MOMENTUM_CELL_FIELDS]
    ptrs = [(_D * len(g))(*[_dp(a) for a in g]) for g in (fv, ff, cf)]
    lib().oracle_newuvw_assembly(int(NC), int(NbC), int(NS), int(NONZ), _ip(iopt), _dp(dopt),
                                 *[_ip(a) for a in ints], *[_dp(a) for a in dbl], *ptrs,
                                 _dp(Aval), _dp(b), _dp(Abou), _dp(Asave), _dp(rhoUi),
                                 ctypes.byref(st))
    return Aval, b, Abou[:NbC], Asave, rhoUi, st.value
