"""Subdomain (halo-coupled) solves on the GPU through the Fortran-facing
entry points: two ranks as processes sharing the one GPU, coupled on the
host by gloo (no kernel waits on another rank).  Each rank registers its
par_mod maps with tflows_set_halo, solves its subdomain on the device, then
runs the oracle's restatement of the same coupled loops (CG.f90:200-208,
BiCG.f90:202-211, CGS.f90:201-208 and :301-308, Resid.f90:36-42) with the
same exchange and sums; both must agree, and the assembled solution must
match the one-domain oracle solve."""
import numpy as np
import pytest

import oracle
from conftest import tflows
from halo_ranks import exchange, glosum, run_ranks

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _make(kind):
    if kind == "pressure":
        return mesh.pressure_system(12, 10, 14, perturb=0.2, seed=17, variable_density=True)
    return mesh.convection_diffusion_system(12, 10, 14, perturb=0.2, seed=18)


def _rank_solve(rank, world, kind, method, prec):
    import torch
    torch.cuda.set_device(0)
    s = _make(kind)
    sd = mesh.partition(s, world)[rank]
    tol = 1e-10 * float(np.linalg.norm(s.b))
    x, r = sd.x.copy(), sd.b.copy()
    # physical boundary cells x(-2:-1) and x(0): markers the solver must not
    # change; buffer cells hold x0 = 0, the neighbours' values of x0 = 0, as
    # Resid reads them
    x[sd.NB - 2:sd.NB] = (7.5, 8.5)
    x[sd.NB] = -2.0
    x_in = x.copy()
    tflows.set_halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum())
    try:
        out = tflows.solve_ex(method, sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Adia,
                              sd.Ab, x, r, prec, 5000, tol)
        # a second call reuses the kept buffers (and IC pattern): same answer
        x2, r2 = x_in.copy(), sd.b.copy()
        out2 = tflows.solve_ex(method, sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Adia,
                               sd.Ab, x2, r2, prec, 5000, tol)
        assert out2.niter == out.niter and np.array_equal(x2, x) and np.array_equal(r2, r)
    finally:
        tflows.clear_halo()
    with oracle.halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum()):
        xo, ro, ito, inio, fino = oracle.solve(method, sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol,
                                               sd.Arow, sd.Adia, sd.Ab, x_in, sd.b, prec, 5000,
                                               tol)
    return dict(status=out.status, it=out.niter, ini=out.IniRes, fin=out.FinRes, x=x, r=r,
                x_in=x_in, NB=sd.NB, rows=sd.rows, ito=ito, inio=inio, xo=xo, ro=ro, tol=tol)


@pytest.mark.parametrize("kind,method,prec", [
    ("pressure", "cg", 1), ("pressure", "cg", 2), ("pressure", "cg", 0),
    ("convdiff", "bicg", 1), ("convdiff", "cgs", 1), ("pressure", "cgs", 2)])
def test_halo_solve_matches_coupled_oracle(kind, method, prec):
    out = run_ranks(_rank_solve, 2, kind, method, prec)
    s = _make(kind)
    xg = np.zeros(s.N)
    for o in out:
        NB = o["NB"]
        assert o["status"] == tflows.OK, o["status"]
        assert abs(o["it"] - o["ito"]) <= (1 if method != "cgs" else 2), (o["it"], o["ito"])
        assert abs(o["ini"] - o["inio"]) <= 1e-12 * o["inio"]
        assert o["fin"] < o["tol"]
        xl, xo = o["x"][NB + 1:], o["xo"][NB + 1:]
        assert np.abs(xl - xo).max() <= 1e-8 * np.abs(xo).max()
        assert np.array_equal(o["x"][:NB + 1], o["x_in"][:NB + 1])
        xg[o["rows"]] = xl
    assert out[0]["it"] == out[1]["it"]  # every rank left the loop together
    tol = out[0]["tol"]
    assert np.linalg.norm(s.b - s.scipy() @ xg) < 1.01 * tol
    if prec != 2:  # one-domain preconditioner: the one-domain solution
        xs, *_ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x,
                              s.b, prec, 5000, 1e-3 * tol)
        xs = xs[s.NB + 1:]
        assert np.abs(xg - xs).max() <= 1e-7 * np.abs(xs).max()


def _rank_resid(rank, world):
    import torch
    torch.cuda.set_device(0)
    s = _make("pressure")
    sd = mesh.partition(s, world)[rank]
    rng = np.random.default_rng(5 + rank)
    x = rng.uniform(-1, 1, sd.NB + 1 + sd.N)  # buffer cells as a caller's exchange left them
    tflows.set_halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum())
    try:
        r = sd.b.copy()
        tflows.resid(sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Ab, x, r)
    finally:
        tflows.clear_halo()
    with oracle.halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, exchange(sd), glosum()):
        ro = oracle.resid(sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Ab, x, sd.b)
    return r, ro


def test_halo_resid_bit_for_bit():
    for r, ro in run_ranks(_rank_resid, 2):
        assert np.array_equal(r.view(np.uint64), ro.view(np.uint64))


def _rank_failures(rank, world):
    import torch
    torch.cuda.set_device(0)
    s = _make("pressure")
    sd = mesh.partition(s, world)[rank]
    tol = 1e-10 * float(np.linalg.norm(s.b))

    def broken(phi):
        raise ConnectionError("link down")

    tflows.set_halo(sd.Npro, sd.NB, sd.NBBs, sd.NBBe, sd.BufInd, broken, glosum())
    try:
        x, r = sd.x.copy(), sd.b.copy()
        out = tflows.solve_ex("cg", sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Adia, sd.Ab,
                              x, r, 1, 100, tol)
        try:
            tflows.solve_ex("cg", sd.N, sd.NB, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Adia, sd.Ab,
                            sd.x.copy(), sd.b.copy(), 1, 100, tol,
                            opts=tflows.options(precision=tflows.MIXED))
            mixed = "accepted"
        except tflows.SolverError as e:
            mixed = str(e)
        try:
            tflows.solve_ex("cg", sd.N, sd.NB + 1, sd.NONZ, sd.A, sd.Acol, sd.Arow, sd.Adia,
                            np.zeros(sd.NB + 1), np.zeros(sd.NB + 2 + sd.N), sd.b.copy(), 1, 100,
                            tol)
            nb_check = "accepted"
        except tflows.SolverError as e:
            nb_check = str(e)
    finally:
        tflows.clear_halo()
    return out.status, mixed, nb_check


def test_halo_errors_are_reported():
    """A failing exchange callback ends the solve with HALO_ERROR on every
    rank (the first exchange comes after the same global sums on all ranks);
    other precisions and a mismatched NB are rejected before any launch."""
    for status, mixed, nb_check in run_ranks(_rank_failures, 2):
        assert status == tflows.HALO_ERROR
        assert "unsupported" in mixed
        assert "bad input" in nb_check
