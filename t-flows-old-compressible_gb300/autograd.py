"""Differentiable solves: a hand-written adjoint behind torch.autograd.Function.

Forward: x = A^-1 b with the GPU Krylov solver.  Backward, for an upstream
gradient g = dL/dx: one transposed solve A^T lam = g through the same
kernels (A^T has A's pattern; its stored values are A's values permuted by
the transpose map, entry (i,j) <- entry (j,i)), then

    dL/db        = lam
    dL/dA_ij     = -lam_i x_j   over the stored pattern (tflows_pattern_outer)

Gradients with respect to anything that produced the matrix values (for
example face coefficients through `FaceAssembly`) follow from torch's chain
rule.  The pattern must be structurally symmetric (every finite-volume
matrix of the reference is: entries come in (c1,c2)/(c2,c1) pairs,
Process/TopolM.f90:81-94).
"""
from __future__ import annotations

import numpy as np
import torch

from . import api


def transpose_index(rowptr, col):
    """For each stored entry k = (i, j) the position of (j, i), as int64.
    Raises if the pattern is not structurally symmetric."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    n = rowptr.shape[0] - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    key = rows * n + col
    order = np.argsort(key, kind="stable")
    skey = key[order]
    tkey = col * n + rows
    pos = np.searchsorted(skey, tkey)
    pos = np.minimum(pos, skey.shape[0] - 1)
    if not np.array_equal(skey[pos], tkey):
        raise ValueError("pattern is not structurally symmetric")
    return order[pos]


class _Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, val, b, solver):
        x = torch.zeros(b.shape[0], dtype=torch.float64, device=b.device)
        v64 = val.detach().to(torch.float64).contiguous()
        b64 = b.detach().to(torch.float64).contiguous()
        res = solver.topo.solve(v64, b64, x, solver.method, solver.prec, solver.maxiter,
                                solver.rtol, opts=solver.opts)
        if res["status"] != api.OK:
            raise api.SolverError(res["status"], f"forward solve: {res}")
        solver.last_forward = res
        ctx.solver = solver
        ctx.val_dtype, ctx.b_dtype = val.dtype, b.dtype
        ctx.save_for_backward(v64, x)
        return x

    @staticmethod
    def backward(ctx, gx):
        solver = ctx.solver
        v64, x = ctx.saved_tensors
        g = gx.detach().to(torch.float64).contiguous()
        lam = torch.zeros_like(x)
        if float(g.abs().max()) > 0.0:
            vt = v64[solver.tindex].contiguous()
            res = solver.topo.solve(vt, g, lam, solver.adjoint_method, solver.prec,
                                    solver.maxiter, solver.rtol, opts=solver.opts)
            if res["status"] != api.OK:
                raise api.SolverError(res["status"], f"adjoint solve: {res}")
            solver.last_adjoint = res
        grad_val = None
        if ctx.needs_input_grad[0]:
            gv = torch.empty_like(v64)
            solver.topo.pattern_outer(lam, x, gv)
            grad_val = gv.to(ctx.val_dtype)
        grad_b = lam.to(ctx.b_dtype) if ctx.needs_input_grad[1] else None
        return grad_val, grad_b, None


class DifferentiableSolver:
    """x = solve(val, b), differentiable in the stored values and in b.

    ``rtol`` is relative to ||b|| (and to ||dL/dx|| for the adjoint solve);
    ``method`` defaults to CG for a symmetric pattern of values, and the
    adjoint uses the same method on A^T.
    """

    def __init__(self, topo: "api.Topology", rowptr0, col0, method="cg", prec=1, rtol=1e-12,
                 maxiter=20000, precision=api.FP64, device="cuda"):
        self.topo = topo
        self.method = method
        self.adjoint_method = method
        self.prec = prec
        self.rtol = rtol
        self.maxiter = maxiter
        self.opts = api.options(precision=precision, tol_mode=api.TOL_RELATIVE)
        self.tindex = torch.as_tensor(transpose_index(rowptr0, col0), device=device)
        self.last_forward = None
        self.last_adjoint = None

    @classmethod
    def from_system(cls, s, **kw):
        topo = api.Topology.from_system(s)
        return cls(topo, s.Acol - 1, s.Arow[:-1] - 1, **kw)

    def __call__(self, val, b):
        return _Solve.apply(val, b, self)


class FaceAssembly:
    """Pressure-type assembly from face coefficients, differentiable in torch:
    entries (c1,c2) and (c2,c1) get -coef, both diagonals get +coef, plus a
    fixed diagonal part (the pattern of Process/CalcPS.f90:87-102).  Faces in
    `mesh.interior_faces` order; `s` must come from
    `mesh.pressure_system(..., keep_faces=True)`."""

    def __init__(self, s, device="cuda"):
        from . import mesh
        c1, c2, p12, p21 = mesh.interior_faces(*s.shape)
        dia = s.Adia.astype(np.int64) - 1
        self.p12 = torch.as_tensor(p12, device=device)
        self.p21 = torch.as_tensor(p21, device=device)
        self.d1 = torch.as_tensor(dia[c1], device=device)
        self.d2 = torch.as_tensor(dia[c2], device=device)
        fixed = np.zeros(s.nnz)
        fixed[dia] = s.fixed_diag
        self.fixed = torch.as_tensor(fixed, device=device)
        self.c1, self.c2 = c1, c2

    def __call__(self, coef):
        c = coef.to(torch.float64)
        val = self.fixed.clone()
        val = val.index_add(0, self.p12, -c).index_add(0, self.p21, -c)
        val = val.index_add(0, self.d1, c).index_add(0, self.d2, c)
        return val
