"""Subdomain (halo-coupled) solves on the CPU: two or three ranks as gloo
processes, each running the oracle's restatement of the reference's coupled
loops (Exchng after every product, the Ab halo terms, glosum after every
inner product; CG.f90:200-208, Resid.f90:36-42) on its part of a system
split by mesh.partition.  With the diagonal or no preconditioner the coupled
iteration is the one-domain iteration up to the order of the global sums,
so iteration counts and solutions must match the one-domain oracle solve;
with IC(0) each rank preconditions its own block (the reference's
subdomain-local sweeps), so only the converged solution must match.  The
partition itself must reproduce the global residual row by row."""
import numpy as np
import pytest

import oracle
from conftest import tflows
from halo_ranks import exchange, glosum, run_ranks

mesh = tflows.mesh


def _system():
    return mesh.pressure_system(10, 9, 12, perturb=0.2, seed=7, variable_density=True)


def _convdiff():
    return mesh.convection_diffusion_system(10, 9, 12, perturb=0.2, seed=8)


def _solve_rank(rank, world, kind, method, prec, tol_rel):
    s = _system() if kind == "pressure" else _convdiff()
    sd = mesh.partition(s, world)[rank]
    tol = tol_rel * float(np.linalg.norm(s.b))
    with oracle.halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum()):
        x, r, it, ini, fin = oracle.solve(method, sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow,
                                          sd.Adia, sd.Ab, sd.x, sd.b, prec, 5000, tol)
    return sd.rows, x[sd.NB + 1:], it, ini, fin


def _resid_rank(rank, world):
    s = _system()
    sd = mesh.partition(s, world)[rank]
    xg = np.random.default_rng(3).uniform(-1, 1, s.N)
    x = sd.x.copy()
    x[sd.NB + 1:] = xg[sd.rows]
    # the caller's exchange of x before Resid (Exchng.f90:36-43, then the swap)
    phi = x[:sd.NB].copy()
    for k in range(-sd.NB, 0):
        if sd.BufInd[sd.NB + k] > 0:
            phi[sd.NB + k] = x[sd.NB + sd.BufInd[sd.NB + k]]
    exchange(sd)(phi)
    x[:sd.NB] = phi
    with oracle.halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum()):
        r = oracle.resid(sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Ab, x, sd.b)
    return sd.rows, r, (s.b - s.scipy() @ xg)[sd.rows]


@pytest.mark.parametrize("world", [2, 3])
def test_partitioned_resid_matches_global_rows(world):
    for rows, r, ref in run_ranks(_resid_rank, world):
        assert np.abs(r - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("kind,method,prec", [("pressure", "cg", 1), ("pressure", "cg", 0),
                                              ("convdiff", "bicg", 1), ("convdiff", "cgs", 1)])
def test_coupled_solve_matches_one_domain(kind, method, prec):
    s = _system() if kind == "pressure" else _convdiff()
    tol = 1e-10 * float(np.linalg.norm(s.b))
    xo, _, ito, inio, _ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                       s.Ab, s.x, s.b, prec, 5000, tol)
    xo = xo[s.NB + 1:]
    out = run_ranks(_solve_rank, 2, kind, method, prec, 1e-10)
    x = np.zeros(s.N)
    for rows, xl, it, ini, fin in out:
        x[rows] = xl
        assert abs(it - ito) <= 1, (it, ito)
        assert abs(ini - inio) <= 1e-12 * inio
        assert fin < tol
    assert len({o[2] for o in out}) == 1  # every rank took the same exit
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()


@pytest.mark.parametrize("method", ["cg", "cgs"])
def test_coupled_ic_solve_converges_to_one_domain_solution(method):
    """IC(0) per subdomain (block IC, as the reference's sweeps stop at the
    subdomain's rows): a different preconditioner, the same solution."""
    s = _system()
    tol = 1e-10 * float(np.linalg.norm(s.b))
    xo, *_ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x,
                          s.b, 2, 5000, 1e-3 * tol)
    xo = xo[s.NB + 1:]
    out = run_ranks(_solve_rank, 3, "pressure", method, 2, 1e-10)
    x = np.zeros(s.N)
    for rows, xl, it, ini, fin in out:
        x[rows] = xl
        assert fin < tol and it < 5000
    assert np.abs(x - xo).max() <= 1e-6 * np.abs(xo).max()
