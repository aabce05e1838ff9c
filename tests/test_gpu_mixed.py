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


@pytest.mark.parametrize("method", ["cg", "cgs"])
@pytest.mark.parametrize("sweeps,bf16", [(0, 1), (1, 0), (2, 1), (3, 0)])
def test_mixed_ic_variants_reach_fp64_tolerance(method, sweeps, bf16):
    """IC(0) in the FP32 inner solves with BF16 factor entries and/or Jacobi
    sweeps in place of the exact triangular solves: a different (cheaper)
    preconditioner, the same FP64 answer."""
    if method == "cg":
        s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    else:
        s = mesh.convection_diffusion_system(24, 20, 18, perturb=0.2, seed=5)
    x, r, out, tol, res = _mixed(s, method, 2, 1e-10, ic_sweeps=sweeps, ic_bf16=bf16)
    assert out.status == tflows.OK, (out, res)
    true_r = s.b - s.scipy() @ x[s.NB + 1:]
    assert np.linalg.norm(true_r) < tol
    xo, *_ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x,
                          s.b, 2, 5000, tol)
    assert np.abs(x - xo).max() / np.abs(xo).max() < 1e-6


def test_ic_jacobi_sweeps_tend_to_the_exact_apply():
    """With at least as many Jacobi sweeps as the triangles have wavefront
    levels the sweeps reproduce the exact triangular solves (up to FP32
    rounding), so the inner iteration count matches the exact apply's; with
    fewer sweeps the preconditioner is weaker but still converges."""
    s = mesh.pressure_system(6, 5, 4, perturb=0.2, seed=8, variable_density=True)
    levels = 6 + 5 + 4 - 2  # a box's IC wavefronts: nx + ny + nz - 2
    runs = {}
    for k in (0, levels + 1, 1):
        x, r, out, tol, res = _mixed(s, "cg", 2, 1e-11, ic_sweeps=k, inner_rtol=1e-6,
                                     refine_restart=1)
        assert out.status == tflows.OK, (k, out, res)
        runs[k] = res["inner_iterations"]
    assert abs(runs[levels + 1] - runs[0]) <= 1, runs
    assert runs[1] >= runs[0], runs
