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


def test_set_halo_validates_maps_on_the_host():
    """tflows_set_halo checks its maps before any device work: ranges
    outside -NB..-1 and missing callbacks are rejected, an empty neighbour
    (NBBe > NBBs) is accepted, and Npro = 0 clears the registration."""
    import ctypes
    L = tflows.load_library()
    ip = ctypes.POINTER(ctypes.c_int)
    ex = tflows._native.EXCHANGE_FN(lambda user, phi, nb: 0)
    gs = tflows._native.GLOSUM_FN(lambda user, v: 0)

    def call(nbbs, nbbe, NB, exch=ex, gsum=gs):
        bs = np.array(nbbs, np.int32)
        be = np.array(nbbe, np.int32)
        bi = np.ones(max(NB, 1), np.int32)
        return L.tflows_set_halo(len(nbbs), NB, bs.ctypes.data_as(ip), be.ctypes.data_as(ip),
                                 bi.ctypes.data_as(ip), exch, gsum, None)

    try:
        assert call([-3, -1], [-6, 0], 6) == tflows.OK           # neighbour 2 empty
        assert call([-3, -1], [-7, 0], 6) == tflows.BAD_INPUT    # below -NB
        assert call([0, -1], [-2, 0], 6) == tflows.BAD_INPUT     # NBBs(1) not negative
        assert call([-3], [-6], 6, exch=tflows._native.EXCHANGE_FN()) == tflows.BAD_INPUT
        assert "halo" in tflows.last_error()
    finally:
        tflows.clear_halo()
    bs = np.zeros(1, np.int32)
    assert L.tflows_set_halo(0, 0, bs.ctypes.data_as(ip), bs.ctypes.data_as(ip), None,
                             ex, gs, None) == tflows.OK


def test_partition_layout_follows_bufloa():
    """mesh.partition: buffer ranges descend from -(n_phys+1) in neighbour
    order, connected pairs have equal segment lengths, every buffer cell
    maps to a local row, and the local matrices keep every entry once."""
    s = _system()
    subs = mesh.partition(s, 3)
    assert sum(d.N for d in subs) == s.N
    assert sum(d.NONZ - 1 for d in subs) + sum(
        int((d.BufInd > 0).sum()) for d in subs) == s.NONZ - 1
    for d in subs:
        first = True
        for q, lo, hi in d.segments():
            assert hi > lo
            if first:
                assert hi == d.NB - 2  # below the two physical boundary cells
                first = False
            other = subs[q]
            seg = [sg for sg in other.segments() if sg[0] == d.rank]
            assert seg and seg[0][2] - seg[0][1] == hi - lo
            assert np.all((d.BufInd[lo:hi] >= 1) & (d.BufInd[lo:hi] <= d.N))
        assert d.NBBs[d.rank] == -1 and d.NBBe[d.rank] == 0  # no connection with itself
