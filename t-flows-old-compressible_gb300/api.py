"""Python mirror of the reference's solver interface over the C ABI.

``cg``, ``bicg``, ``cgs``, ``prec1`` and ``resid`` take the same arguments
as the Fortran subroutines (Process/CG.f90:2-34, BiCG.f90, CGS.f90,
Prec1.f90:2-18, Resid.f90:2-16) as numpy arrays in the same layout: 1-based
``Acol``/``Arow``/``Adia``, ``x`` holding x(-NB:N), ``Ab`` holding
Ab(-NB:-1).  Like the Fortran dummies, ``x`` and ``r1`` (and ``D``) are
updated in place; the scalar outputs (niter, IniRes, FinRes) are returned.
Every call goes through libtflows_krylov.so on the GPU; there is no CPU path.

``Topology`` is the device-array interface used by the PyTorch binding: a
registered compressed-row pattern whose solves take torch CUDA tensors and
run on torch's current stream.
"""
from __future__ import annotations

import ctypes
import os
from typing import NamedTuple

import numpy as np

from . import _native

(OK, NOT_CONVERGED, BREAKDOWN, NONFINITE, TIMEOUT, BAD_INPUT, CUDA_ERROR, NO_DEVICE, UNSUPPORTED,
 HALO_ERROR) = range(10)
CG, BICG, CGS, BICG_TRUE = 0, 1, 2, 3
FP64, MIXED, FP64_FMA = 0, 1, 2
TOL_ABSOLUTE, TOL_RELATIVE = 0, 1
METHODS = {"cg": CG, "bicg": BICG, "cgs": CGS, "bicg_true": BICG_TRUE}


class SolverError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{status_string(status)}: {message}")
        self.status = status


class SolveOutput(NamedTuple):
    niter: int
    IniRes: float
    FinRes: float
    status: int


def lib():
    return _native.load()


def status_string(st: int) -> str:
    return lib().tflows_status_string(int(st)).decode()


def last_status() -> int:
    return lib().tflows_last_status()


def last_error() -> str:
    return lib().tflows_last_error().decode()


def last_result() -> dict:
    r = _native.Result()
    lib().tflows_last_result(ctypes.byref(r))
    return r.as_dict()


def options(**kw) -> _native.Options:
    o = _native.Options()
    lib().tflows_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def set_options(**kw) -> None:
    lib().tflows_set_options(ctypes.byref(options(**kw)))


def finalize() -> None:
    lib().tflows_finalize()


def forget_topologies() -> None:
    """tflows_forget_topologies: drop the legacy calls' cached device
    patterns (after the caller rewrote Acol/Arow/Adia in place)."""
    lib().tflows_forget_topologies()


def autotune_clear() -> None:
    """Forget every tuned launch shape of this process."""
    lib().tflows_autotune_clear()


def _ci(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _cd(a, writable=False):
    if writable:
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
            raise TypeError("in/out arrays must be C-contiguous float64 numpy arrays")
    else:
        a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _byref_i(v):
    return ctypes.c_int(int(v))


def solve_ex(method, N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1, prec, niter, tol,
             IniRes=0.0, FinRes=0.0, opts=None, raise_on_error=True):
    """tflows_solve_ex: one of the reference solvers with options.  ``x``
    (length NB+N+1) and ``r1`` (length N) are updated in place."""
    m = METHODS.get(method, method)
    A_, pA = _cd(A)
    Acol_, pAcol = _ci(Acol)
    Arow_, pArow = _ci(Arow)
    Adia_, pAdia = _ci(Adia)
    Ab_, pAb = _cd(Ab if NB > 0 else np.zeros(1))
    _, px = _cd(x, writable=True)
    _, pr = _cd(r1, writable=True)
    cN, cNB, cNZ, cp, cit = (_byref_i(N), _byref_i(NB), _byref_i(NONZ), _byref_i(prec),
                             _byref_i(niter))
    ctol, cini, cfin = ctypes.c_double(tol), ctypes.c_double(IniRes), ctypes.c_double(FinRes)
    res = _native.Result()
    st = lib().tflows_solve_ex(int(m), ctypes.byref(cN), ctypes.byref(cNB), ctypes.byref(cNZ),
                               pA, pAcol, pArow, pAdia, pAb, px, pr, ctypes.byref(cp),
                               ctypes.byref(cit), ctypes.byref(ctol), ctypes.byref(cini),
                               ctypes.byref(cfin), ctypes.byref(opts) if opts else None,
                               ctypes.byref(res))
    if raise_on_error and st in (BAD_INPUT, CUDA_ERROR, NO_DEVICE, UNSUPPORTED, TIMEOUT):
        raise SolverError(st, last_error())
    return SolveOutput(cit.value, cini.value, cfin.value, st)


def _legacy(method):
    def fn(N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1, prec, niter, tol, IniRes=0.0,
           FinRes=0.0):
        return solve_ex(method, N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1, prec, niter, tol,
                        IniRes, FinRes, opts=None)
    fn.__name__ = method
    fn.__doc__ = (f"The reference's `{method}` (Process/{ {'cg': 'CG', 'bicg': 'BiCG', 'cgs': 'CGS'}[method]}.f90) "
                  "on the GPU: x and r1 updated in place; returns (niter, IniRes, FinRes, status).")
    return fn


_halo_keep = None


def set_halo(Npro, NB, NBBs, NBBe, BufInd, exchange, glosum):
    """tflows_set_halo: register this rank's subdomain halo for the
    Fortran-facing entry points (the reference's Npro > 0 run).

    ``NBBs``, ``NBBe``: Npro entries, NBBs(sub) and NBBe(sub) for sub = 1..Npro
    as Parallel/Double/BufLoa.f90 leaves them; ``BufInd``: BufInd(-NB:-1)
    (length NB).  ``exchange(phi)`` receives the float64 array PHI(-NB:-1)
    (``phi[NB + k]`` = PHI(k)) whose buffer cells hold the values of the
    cells they mirror and must swap each neighbour's segment
    PHI(NBBe(sub):NBBs(sub)) with rank sub-1 in place; ``glosum(v)`` returns
    the sum of ``v`` over the ranks.  An exception in either ends the solve
    with HALO_ERROR."""
    global _halo_keep
    bs = np.ascontiguousarray(NBBs, dtype=np.int32)
    be = np.ascontiguousarray(NBBe, dtype=np.int32)
    bi = np.ascontiguousarray(BufInd if NB > 0 else np.zeros(1), dtype=np.int32)

    def _ex(user, phi, nb):
        try:
            exchange(np.ctypeslib.as_array(phi, shape=(nb,)))
            return 0
        except Exception:  # reported to the solver as a failed exchange
            return 1

    def _gs(user, v):
        try:
            v[0] = float(glosum(float(v[0])))
            return 0
        except Exception:  # reported to the solver as a failed sum
            return 1

    ex, gs = _native.EXCHANGE_FN(_ex), _native.GLOSUM_FN(_gs)
    ip = ctypes.POINTER(ctypes.c_int)
    st = lib().tflows_set_halo(int(Npro), int(NB), bs.ctypes.data_as(ip), be.ctypes.data_as(ip),
                               bi.ctypes.data_as(ip), ex, gs, None)
    if st != OK:
        raise SolverError(st, last_error())
    _halo_keep = (ex, gs)  # the library calls them until the halo is cleared


def clear_halo():
    """tflows_clear_halo: back to the one-domain run (Ab not read)."""
    global _halo_keep
    lib().tflows_clear_halo()
    _halo_keep = None


cg = _legacy("cg")
bicg = _legacy("bicg")
cgs = _legacy("cgs")


def prec1(N, NONZ, A, Acol, Arow, Adia, D, prec):
    """Process/Prec1.f90: fills D (length N, float64) in place."""
    _, pA = _cd(A)
    _, pAcol = _ci(Acol)
    _, pArow = _ci(Arow)
    _, pAdia = _ci(Adia)
    _, pD = _cd(D, writable=True)
    lib().tflows_prec1(ctypes.byref(_byref_i(N)), ctypes.byref(_byref_i(NONZ)), pA, pAcol,
                       pArow, pAdia, pD, ctypes.byref(_byref_i(prec)))
    st = last_status()
    if st != OK:
        raise SolverError(st, last_error())


def resid(N, NB, NONZ, A, Acol, Arow, Ab, x, r1):
    """Process/Resid.f90: r1 <- r1 - A x, r1 updated in place."""
    _, pA = _cd(A)
    _, pAcol = _ci(Acol)
    _, pArow = _ci(Arow)
    _, pAb = _cd(Ab if NB > 0 else np.zeros(1))
    _, px = _cd(x)
    _, pr = _cd(r1, writable=True)
    lib().tflows_resid(ctypes.byref(_byref_i(N)), ctypes.byref(_byref_i(NB)),
                       ctypes.byref(_byref_i(NONZ)), pA, pAcol, pArow, pAb, px, pr)
    st = last_status()
    if st != OK:
        raise SolverError(st, last_error())


def solve_system(method, s, prec, niter=1000, tol=None, x=None, b=None, opts=None):
    """Convenience: solve a mesh.System; returns (x(-NB:N), r1, SolveOutput, result dict)."""
    xo = (s.x if x is None else x).astype(np.float64, copy=True)
    ro = (s.b if b is None else b).astype(np.float64, copy=True)
    out = solve_ex(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, xo, ro, prec,
                   niter, s.tol if tol is None else tol, opts=opts)
    return xo, ro, out, last_result()


# ---- device-array interface -------------------------------------------------------

def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Topology:
    """A compressed-row pattern registered on the current CUDA device.

    ``rowptr``, ``col``, ``diag`` are int32 arrays (numpy or torch, host or
    CUDA) with the given index base.  Solves take torch CUDA tensors.
    """

    def __init__(self, n, rowptr, col, diag, index_base=0):
        import torch
        self.n = int(n)
        self.nnz = int(len(col))
        self._h = ctypes.c_void_p()
        on_dev = 0
        keep = []
        arrs = []
        for a in (rowptr, col, diag):
            if isinstance(a, torch.Tensor):
                a = a.to(torch.int32).contiguous()
                on_dev = 1 if a.is_cuda else on_dev
                keep.append(a)
                arrs.append(ctypes.c_void_p(a.data_ptr()))
            else:
                a = np.ascontiguousarray(a, dtype=np.int32)
                keep.append(a)
                arrs.append(ctypes.c_void_p(a.ctypes.data))
        st = lib().tflows_topology_create(ctypes.byref(self._h), self.n, self.nnz, *arrs,
                                          int(index_base), on_dev)
        if st != OK:
            raise SolverError(st, last_error())

    @classmethod
    def from_system(cls, s):
        return cls(s.N, s.Acol, s.Arow[:-1], s.Adia, index_base=1)

    def close(self):
        if self._h:
            lib().tflows_topology_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def patterns(self):
        """Distinct column patterns the products read (0: explicit columns)."""
        return int(lib().tflows_topology_patterns(self._h))

    def transpose_map(self):
        """Device pointer of the transposed-entry map (int32, nnz)."""
        p = lib().tflows_topology_transpose_map(self._h)
        if not p:
            raise SolverError(CUDA_ERROR, last_error())
        return p

    def solve(self, val, b, x, method="cg", prec=1, maxiter=1000, tol=1e-8, r_out=None,
              opts=None, raise_on_error=True):
        """Solve in place on torch CUDA float64 tensors (x: initial guess in,
        solution out).  Returns the result record as a dict."""
        for t in (val, b, x):
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
                raise TypeError("val, b, x must be contiguous CUDA float64 tensors")
        res = _native.Result()
        st = lib().tflows_solve_device(self._h, int(METHODS.get(method, method)), int(prec),
                                       ctypes.byref(opts) if opts else None, _ptr(val), _ptr(b),
                                       _ptr(x), _ptr(r_out) if r_out is not None else None,
                                       int(maxiter), float(tol), _stream(), ctypes.byref(res))
        if raise_on_error and st in (BAD_INPUT, CUDA_ERROR, NO_DEVICE, UNSUPPORTED, TIMEOUT):
            raise SolverError(st, last_error())
        return res.as_dict()

    def autotune(self, val, b, method="cg", prec=1, opts=None):
        """Time candidate launch shapes on these device values and
        right-hand side (tflows_autotune) and return the chosen one as a
        dict; later solves of this class with ``autotune=1`` use it."""
        for t in (val, b):
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
                raise TypeError("val, b must be contiguous CUDA float64 tensors")
        out = _native.Tuning()
        st = lib().tflows_autotune(self._h, int(METHODS.get(method, method)), int(prec),
                                   ctypes.byref(opts) if opts else None, _ptr(val), _ptr(b),
                                   _stream(), ctypes.byref(out))
        if st != OK:
            raise SolverError(st, last_error())
        return out.as_dict()

    def ic_apply(self, val, r, z, opts=None):
        """IC(0) pivots and z = M^-1 r (tflows_ic_apply_device) on torch CUDA
        float64 tensors; returns the result record as a dict."""
        for t in (val, r, z):
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
                raise TypeError("val, r, z must be contiguous CUDA float64 tensors")
        res = _native.Result()
        st = lib().tflows_ic_apply_device(self._h, ctypes.byref(opts) if opts else None,
                                          _ptr(val), _ptr(r), _ptr(z), _stream(),
                                          ctypes.byref(res))
        if st != OK:
            raise SolverError(st, last_error())
        return res.as_dict()

    def spmv(self, val, x, y, repeat=1, fp32=False):
        sec = ctypes.c_double()
        st = lib().tflows_spmv_device(self._h, _ptr(val), _ptr(x), _ptr(y), int(repeat),
                                      int(bool(fp32)), _stream(), ctypes.byref(sec))
        if st != OK:
            raise SolverError(st, last_error())
        return sec.value

    def pattern_outer(self, lam, x, grad):
        st = lib().tflows_pattern_outer(self._h, _ptr(lam), _ptr(x), _ptr(grad), _stream())
        if st != OK:
            raise SolverError(st, last_error())
        return grad


def solve_batched(topos, vals, bs, xs, methods, precs, maxiters, tols, opts=None,
                  raise_on_error=True):
    """All systems in one persistent cooperative launch (tflows_solve_batched_device).

    Lists of equal length: Topology objects (a pattern may repeat), CUDA
    float64 tensors for values, right-hand sides and solutions (x updated in
    place), method names or codes, preconditioners, iteration caps and
    tolerances.  Returns one result record (dict) per system.
    """
    n = len(topos)
    arrs = [vals, bs, xs, methods, precs, maxiters, tols]
    if any(len(a) != n for a in arrs):
        raise ValueError("all per-system lists must have the same length")
    VP = ctypes.c_void_p * n
    h = VP(*[t.handle.value for t in topos])
    pv = VP(*[v.data_ptr() for v in vals])
    pb = VP(*[v.data_ptr() for v in bs])
    px = VP(*[v.data_ptr() for v in xs])
    for t in list(vals) + list(bs) + list(xs):
        if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
            raise TypeError("vals, bs, xs must be contiguous CUDA float64 tensors")
    m = (ctypes.c_int * n)(*[int(METHODS.get(x, x)) for x in methods])
    pr = (ctypes.c_int * n)(*[int(x) for x in precs])
    mi = (ctypes.c_int * n)(*[int(x) for x in maxiters])
    tl = (ctypes.c_double * n)(*[float(x) for x in tols])
    res = (_native.Result * n)()
    st = lib().tflows_solve_batched_device(n, h, m, pr, ctypes.byref(opts) if opts else None, pv,
                                           pb, px, mi, tl, _stream(), res)
    if raise_on_error and st in (BAD_INPUT, CUDA_ERROR, NO_DEVICE, UNSUPPORTED, TIMEOUT):
        raise SolverError(st, last_error())
    return [r.as_dict() for r in res]


class Plan:
    """A batched solve recorded once into a CUDA graph (tflows_plan_*).

    The tensors passed here are bound by address: change their contents
    (new matrix values, right-hand sides, initial guesses) and call
    ``launch()`` again; ``results()`` waits and returns one record per
    system."""

    def __init__(self, topos, vals, bs, xs, methods, precs, maxiters, tols, opts=None):
        n = len(topos)
        VP = ctypes.c_void_p * n
        self._keep = (topos, vals, bs, xs)
        self._n = n
        self._h = ctypes.c_void_p()
        st = lib().tflows_plan_create(
            ctypes.byref(self._h), n, VP(*[t.handle.value for t in topos]),
            (ctypes.c_int * n)(*[int(METHODS.get(m, m)) for m in methods]),
            (ctypes.c_int * n)(*[int(p) for p in precs]), ctypes.byref(opts) if opts else None,
            VP(*[v.data_ptr() for v in vals]), VP(*[v.data_ptr() for v in bs]),
            VP(*[v.data_ptr() for v in xs]), (ctypes.c_int * n)(*[int(m) for m in maxiters]),
            (ctypes.c_double * n)(*[float(t) for t in tols]))
        if st != OK:
            raise SolverError(st, last_error())

    def launch(self):
        st = lib().tflows_plan_launch(self._h, _stream())
        if st != OK:
            raise SolverError(st, last_error())

    def results(self):
        res = (_native.Result * self._n)()
        lib().tflows_plan_results(self._h, res)
        return [r.as_dict() for r in res]

    def tuning(self):
        """Block size and group-balance timing the plan chose at creation
        (options.autotune = 1); runs = 0 when it was not tuned."""
        out = _native.BatchTuning()
        st = lib().tflows_plan_tuning(self._h, ctypes.byref(out))
        if st != OK:
            raise SolverError(st, last_error())
        return out.as_dict()

    def close(self):
        if self._h:
            lib().tflows_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Assembly:
    """The pressure-correction assembly of Process/CalcPS.f90:49-202 and the
    momentum assembly of Process/NewUVW.f90:138-499 on the GPU
    (tflows_assembly_create / tflows_calcps_assemble_device /
    tflows_newuvw_assemble_device).

    Mesh arrays as the reference holds them: SideC (NS, 3) = SideC(0:2, NS),
    SidAij (NS, 2), Adia 1-based, TypeBC and volume over cells -NbC..NC,
    face geometry Sx, Sy, Sz, Dx, Dy, Dz, f.  ``mesh.box_faces`` builds them
    for a box."""

    GEOM = ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f")
    FIELDS = ("rho_n", "rho_o", "rho_oo", "u", "v", "w", "p", "px", "py", "pz", "asave")

    def __init__(self, NC, NbC, NS, NONZ, SideC, SidAij, Adia, TypeBC, geom, volume, device=-1):
        self.NC, self.NbC, self.NS, self.NONZ = int(NC), int(NbC), int(NS), int(NONZ)
        ints = [np.ascontiguousarray(a, dtype=np.int32) for a in (SideC, SidAij, Adia, TypeBC)]
        dbls = [np.ascontiguousarray(geom[k], dtype=np.float64) for k in self.GEOM]
        dbls.append(np.ascontiguousarray(volume, dtype=np.float64))
        self._h = ctypes.c_void_p()
        st = lib().tflows_assembly_create(ctypes.byref(self._h), self.NC, self.NbC, self.NS,
                                          self.NONZ, *[a.ctypes.data for a in ints],
                                          *[a.ctypes.data for a in dbls], int(device))
        if st != OK:
            raise SolverError(st, last_error())

    @classmethod
    def from_faces(cls, msh, TypeBC, device=-1):
        return cls(msh["NC"], msh["NbC"], msh["NS"], int(msh["Acol"][-1]), msh["SideC"],
                   msh["SidAij"], msh["Adia"], TypeBC, msh, msh["volume"], device)

    def calcps(self, fields, aval, b, abou, flux, Nmat=1, dt=1.0, errmax=True):
        """Fill aval (NONZ), b (NC), abou (NbC, cells -NbC..-1) and flux (NS)
        from the cell fields (CUDA float64 tensors over cells -NbC..NC,
        keys FIELDS) on torch's current stream.  Returns {errmax, seconds}."""
        for t in list(fields.values()) + [aval, b, abou, flux]:
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
                raise TypeError("fields and outputs must be contiguous CUDA float64 tensors")
        F = _native.CalcpsFields(**{k: fields[k].data_ptr() for k in self.FIELDS})
        em, sec = ctypes.c_double(), ctypes.c_double()
        st = lib().tflows_calcps_assemble_device(self._h, int(Nmat), float(dt), ctypes.byref(F),
                                                 _ptr(aval), _ptr(b), _ptr(abou), _ptr(flux),
                                                 ctypes.byref(em) if errmax else None,
                                                 _stream(), ctypes.byref(sec))
        if st != OK:
            raise SolverError(st, last_error())
        return {"errmax": em.value if errmax else None, "seconds": sec.value}

    # Process/IniPar.f90:22-49
    CODES = {"ab": 1, "cn": 2, "fi": 3, "lin": 4, "par": 5, "yes": 10, "no": 11, "cds": 20,
             "quick": 21, "luds": 22, "minmod": 23, "smart": 24, "avl_smart": 25,
             "superbee": 26, "gamma": 27}

    def newuvw(self, var, fields, aval, b, abou, asave=None, rhoui=None, *, nmat=1, visc,
               dt, urf, convec=3, cross=3, diffus=3, inert=4, moin_problem=0):
        """Momentum assembly of component ``var`` (1, 2, 3) into aval (NONZ),
        b (NC), abou (NbC, cells -NbC..-1), asave (NC, var 1 only; optional)
        and rhoui (cells -NbC..NC; optional) on torch's current stream.
        ``fields``: CUDA tensors keyed as tflows_newuvw_fields -- int32
        material (cells), blend and blend_tem (materials); float64 cell fields
        over -NbC..NC, face fields over 1..NS, urfc over materials; ``scoef``
        may be absent (|S|^2/(S.d) of the mesh); rho_oo and ui_oo only for
        inert == PAR (5).  Returns {seconds}."""
        ptrs = {}
        for k in _native.NEWUVW_FIELDS:
            t = fields.get(k)
            if t is None:
                ptrs[k] = None
                continue
            want = 4 if k in ("material", "blend", "blend_tem") else 8
            if not (t.is_cuda and t.dtype.itemsize == want and t.is_contiguous()):
                raise TypeError(f"field {k!r} must be a contiguous CUDA "
                                f"{'int32' if want == 4 else 'float64'} tensor")
            ptrs[k] = t.data_ptr()
        outs = [aval, b, abou] + [t for t in (asave, rhoui) if t is not None]
        for t in outs:
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous()):
                raise TypeError("outputs must be contiguous CUDA float64 tensors")
        F = _native.NewuvwFields(**ptrs)
        P = _native.NewuvwParams(var=int(var), nmat=int(nmat), moin_problem=int(moin_problem),
                                 convec=int(convec), cross=int(cross), diffus=int(diffus),
                                 inert=int(inert), visc=float(visc), dt=float(dt),
                                 urf=float(urf))
        sec = ctypes.c_double()
        st = lib().tflows_newuvw_assemble_device(
            self._h, ctypes.byref(P), ctypes.byref(F), _ptr(aval), _ptr(b), _ptr(abou),
            _ptr(asave) if asave is not None else None,
            _ptr(rhoui) if rhoui is not None else None, _stream(), ctypes.byref(sec))
        if st != OK:
            raise SolverError(st, last_error())
        return {"seconds": sec.value}

    def close(self):
        if self._h:
            lib().tflows_assembly_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_mesh(cns_path, geo_path=None):
    """Load NAME.cns (and NAME.geo) as Process/CnsLoa.f90 and
    Library/GeoLoa.f90 read them (tflows_mesh_read).  Returns a dict of numpy
    copies: sizes NC, NbC, NS, NSsh, Nmat; SideC (NS, 3) = SideC(0:2, NS);
    material, xc, yc, zc over cells -NbC..NC; bcmark, CopyC over -NbC..-1;
    volume, delta, WallDs over 1..NC; face arrays Sx..zsp over 1..NS."""
    p = ctypes.POINTER(_native.Mesh)()
    st = lib().tflows_mesh_read(os.fsencode(cns_path),
                                os.fsencode(geo_path) if geo_path else None, ctypes.byref(p))
    if st != OK:
        raise SolverError(st, last_error())
    m = p.contents
    NC, NbC, NS = m.NC, m.NbC, m.NS
    out = {"NC": NC, "NbC": NbC, "NS": NS, "NSsh": m.NSsh, "Nmat": m.Nmat}

    def take(ptr, n):
        return np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].copy()

    out["material"] = take(m.material, NbC + NC + 1)
    out["SideC"] = take(m.SideC, 3 * NS).reshape(NS, 3)
    out["bcmark"] = take(m.bcmark, NbC)
    out["CopyC"] = take(m.CopyC, NbC)
    if geo_path:
        for k in ("xc", "yc", "zc"):
            out[k] = take(getattr(m, k), NbC + NC + 1)
        for k in ("volume", "delta", "WallDs"):
            out[k] = take(getattr(m, k), NC)
        for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "xsp", "ysp", "zsp"):
            out[k] = take(getattr(m, k), NS)
    lib().tflows_mesh_free(p)
    return out


def topolm(NC, SideC):
    """The solver's compressed-row layout of a face list (tflows_topolm,
    Process/TopolM.f90:24-98): 1-based (Acol, Arow, Adia, SidAij (NS, 2))
    with Arow of length NONZ = stored entries + 1."""
    sc = np.ascontiguousarray(SideC, dtype=np.int32)
    NS = sc.shape[0]
    nz = ctypes.c_int()
    st = lib().tflows_topolm(int(NC), NS, sc.ctypes.data, None, None, None, None,
                             ctypes.byref(nz))
    if st != OK:
        raise SolverError(st, last_error())
    Acol = np.zeros(NC + 1, np.int32)
    Arow = np.zeros(nz.value, np.int32)
    Adia = np.zeros(NC, np.int32)
    sid = np.zeros((NS, 2), np.int32)
    st = lib().tflows_topolm(int(NC), NS, sc.ctypes.data, Acol.ctypes.data, Arow.ctypes.data,
                             Adia.ctypes.data, sid.ctypes.data, ctypes.byref(nz))
    if st != OK:
        raise SolverError(st, last_error())
    return Acol, Arow, Adia, sid
