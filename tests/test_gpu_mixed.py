"""Mixed precision (FP32 inner Krylov + FP64 iterative refinement) on the GPU.

The outer loop recomputes the true residual b - A x in FP64 with the FP64
matrix and stops on the reference's test ||r|| < tol, so the returned FinRes
is the true FP64 residual norm; the solution must agree with the FP64 oracle
solve to the accuracy the tolerance implies.
"""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _mixed(s, method, prec, rel_tol, **kw):
    opts = tflows.options(precision=tflows.MIXED, **kw)
    x, r = s.x.copy(), s.b.copy()
    tol = rel_tol * float(np.linalg.norm(s.b))
    out = tflows.solve_ex(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r,
                          prec, 5000, tol, opts=opts)
    return x, r, out, tol, tflows.last_result()


@pytest.mark.parametrize("method,prec", [("cg", 1), ("cg", 2), ("cg", 0), ("bicg", 1),
                                         ("cgs", 1), ("cgs", 2)])
def test_mixed_reaches_fp64_tolerance(method, prec):
    if method == "cg":
        s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    else:
        s = mesh.convection_diffusion_system(24, 20, 18, perturb=0.2, seed=5)
    x, r, out, tol, res = _mixed(s, method, prec, 1e-10)
    assert out.status == tflows.OK, (out, res)
    A = s.scipy()
    true_r = s.b - A @ x[s.NB + 1:]
    assert np.linalg.norm(true_r) < tol
    # FinRes is the true FP64 residual norm and r1 the true residual
    assert abs(np.linalg.norm(true_r) - out.FinRes) <= 1e-3 * out.FinRes + 1e-14 * out.IniRes
    assert np.abs(r - true_r).max() <= 1e-12 * np.abs(s.b).max()
    xo, *_ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x,
                          s.b, prec, 5000, tol)
    rel = np.abs(x - xo).max() / np.abs(xo).max()
    assert rel < 1e-6, rel
    assert res["refinements"] >= 1 and res["inner_iterations"] >= res["refinements"]


def test_mixed_early_exits_match_reference_conventions():
    s = mesh.pressure_system(8, 8, 8, seed=3)
    opts = tflows.options(precision=tflows.MIXED)
    x, r = s.x.copy(), np.zeros(s.N)
    out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1,
                          100, 1e-8, IniRes=-3.0, opts=opts)
    assert out.niter == 0 and out.IniRes == -3.0 and not x.any()


def test_mixed_relative_tolerance_mode():
    s = mesh.convection_diffusion_system(16, 16, 16, perturb=0.2, seed=2)
    opts = tflows.options(precision=tflows.MIXED, tol_mode=tflows.TOL_RELATIVE)
    x, r = s.x.copy(), s.b.copy()
    out = tflows.solve_ex("bicg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1,
                          500, 1e-9, opts=opts)
    assert out.status == tflows.OK
    assert out.FinRes < 1e-9 * np.linalg.norm(s.b)


def test_mixed_divergent_inner_solve_is_rejected():
    """CG run on a strongly nonsymmetric system (what the reference's bicg
    does) can diverge in FP32; the refinement loop must not return a worse
    x than it started from."""
    s = mesh.convection_diffusion_system(24, 20, 18, perturb=0.2, seed=5, dt=1.0)
    x, r, out, tol, res = _mixed(s, "bicg", 1, 1e-10)
    assert out.status in (tflows.OK, tflows.NOT_CONVERGED, tflows.NONFINITE)
    if out.status != tflows.OK:
        assert np.isfinite(out.FinRes) and out.FinRes <= out.IniRes * 1.0001
