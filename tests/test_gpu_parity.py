"""GPU parity: the CUDA solvers through the C ABI against the golden vectors
and the oracle (FP64, reference semantics).

Tolerances: per-row arithmetic (Resid, Prec1, the IC sweeps, the SpMV) runs
in the reference's order without fused multiply-adds, so Resid and Prec1
match bit for bit; the Krylov scalars are grid reductions whose summation
order differs from the sequential loops, so iterates differ by rounding.
Solutions must agree to a relative difference of 1e-8 (FP64 mode bar) and
iteration counts exactly on the small golden cases, within 1 on larger ones.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
SOLVER_CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if not os.path.basename(p).startswith(("prec1_resid", "assembly_",
                                                                 "momentum_", "topolm_")))
PR_CASES = sorted(glob.glob(os.path.join(GOLDEN, "prec1_resid_*.npz")))
REL = 1e-8

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _defaults():
    tflows.set_options()
    yield


def rel_diff(a, b):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


@pytest.mark.parametrize("path", SOLVER_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_golden_solver_cases(path):
    g = np.load(path)
    for c in range(int(g["ncalls"])):
        p = f"c{c}_"
        x = g[p + "x_in"].copy()
        r = g[p + "r1_in"].copy()
        out = tflows.solve_ex(str(g[p + "method"]), int(g["N"]), int(g["NB"]), int(g["NONZ"]),
                              g["A"], g["Acol"], g["Arow"], g["Adia"], g["Ab"], x, r,
                              int(g[p + "prec"]), int(g[p + "niter_in"]), float(g[p + "tol"]),
                              float(g[p + "IniRes_in"]), float(g[p + "FinRes_in"]))
        assert out.niter == int(g[p + "niter_out"]), (c, out)
        xg, rg = g[p + "x_out"], g[p + "r1_out"]
        assert np.array_equal(np.isnan(x), np.isnan(xg))
        assert np.array_equal(np.isnan(r), np.isnan(rg))
        if np.isnan(rg).any():
            assert np.isnan(out.FinRes) and np.isnan(float(g[p + "FinRes_out"]))
            continue
        assert rel_diff(x, xg) <= REL, (c, rel_diff(x, xg))
        assert np.isfinite(r).all()
        ini_g, fin_g = float(g[p + "IniRes_out"]), float(g[p + "FinRes_out"])
        assert abs(out.IniRes - ini_g) <= 1e-12 * max(abs(ini_g), 1e-300), (out.IniRes, ini_g)
        # final residual norms: both below tol; rounding drift of the
        # recursive residual is bounded relative to the initial residual
        assert abs(out.FinRes - fin_g) <= 1e-6 * abs(fin_g) + 1e-9 * abs(ini_g)
        # the recursive residual tracks the golden one to rounding
        assert np.abs(r - rg).max() <= 1e-9 * max(np.abs(g[p + "r1_in"]).max(), 1.0)


@pytest.mark.parametrize("path", PR_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_golden_prec1_resid_bitwise(path):
    g = np.load(path)
    N, NONZ = int(g["N"]), int(g["NONZ"])
    for prec in (0, 1, 2):
        D = np.zeros(N)
        tflows.prec1(N, NONZ, g["A"], g["Acol"], g["Arow"], g["Adia"], D, prec)
        assert np.array_equal(D.view(np.uint64), g[f"D_prec{prec}"].view(np.uint64)), prec
    r = g["resid_r1_in"].copy()
    tflows.resid(N, int(g["NB"]), NONZ, g["A"], g["Acol"], g["Arow"], g["Ab"], g["resid_x"], r)
    assert np.array_equal(r.view(np.uint64), g["resid_r1_out"].view(np.uint64))


def _oracle_vs_gpu(s, method, prec, rel_tol, niter=2000, x0=None, it_slack=1, opts=None):
    tol = rel_tol * float(np.linalg.norm(s.b))
    x_in = s.x.copy() if x0 is None else x0
    xo, ro, ito, inio, fino = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                           s.Ab, x_in, s.b, prec, niter, tol)
    xg = x_in.copy()
    rg = s.b.copy()
    out = tflows.solve_ex(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, xg, rg,
                          prec, niter, tol, opts=opts)
    assert abs(out.niter - ito) <= it_slack, (out.niter, ito)
    assert rel_diff(xg, xo) <= REL, rel_diff(xg, xo)
    assert abs(out.IniRes - inio) <= 1e-11 * inio
    assert out.FinRes < tol and fino < tol
    return out, ito


def test_config1_jacobi_cg_32cube():
    s = mesh.config_system(1)
    out, ito = _oracle_vs_gpu(s, "cg", 1, 1e-12)
    assert out.status == tflows.OK


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_pressure_vd_cg(prec):
    s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    _oracle_vs_gpu(s, "cg", prec, 1e-12, niter=4000)


@pytest.mark.parametrize("method,prec", [("bicg", 1), ("bicg", 2), ("cgs", 0), ("cgs", 1),
                                         ("cgs", 2)])
def test_convection_diffusion(method, prec):
    s = mesh.convection_diffusion_system(24, 20, 18, perturb=0.2, seed=5)
    _oracle_vs_gpu(s, method, prec, 1e-12)


def test_bicg_equals_cg_bitwise_on_gpu():
    s = mesh.convection_diffusion_system(16, 16, 16, perturb=0.2, seed=1)
    outs = []
    for m in ("cg", "bicg"):
        x, r = s.x.copy(), s.b.copy()
        o = tflows.solve_ex(m, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1, 100,
                            s.tol)
        outs.append((x, r, o))
    assert outs[0][2].niter == outs[1][2].niter
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_state_chain_and_early_exits():
    s = mesh.pressure_system(8, 8, 8, seed=3)
    x, r = s.x.copy(), s.b.copy()
    o1 = tflows.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1, 500, s.tol)
    assert o1.status == tflows.OK and o1.FinRes < s.tol
    # zero RHS: exits on ||b|| < tol, x and r untouched, FinRes = previous error
    x2, r2 = s.x.copy(), np.zeros(s.N)
    o2 = tflows.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x2, r2, 1, 500, s.tol,
                   IniRes=-7.0)
    assert o2.niter == 0 and o2.FinRes == o1.FinRes and o2.IniRes == -7.0
    assert not x2.any() and not r2.any()
    # warm start at the solution: IniRes < tol, iter = 0
    x3, r3 = x.copy(), s.b.copy()
    o3 = tflows.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x3, r3, 1, 500,
                   s.tol * 10)
    assert o3.niter == 0 and o3.IniRes < s.tol * 10 and o3.FinRes == o3.IniRes
    # iteration limit: niter_in + 1 and NOT_CONVERGED
    x4, r4 = s.x.copy(), s.b.copy()
    o4 = tflows.cg(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x4, r4, 1, 3, 1e-30)
    assert o4.niter == 4 and o4.status == tflows.NOT_CONVERGED


def test_ic_rejects_unsorted_rows():
    s = mesh.pressure_system(4, 4, 4, seed=2)
    Arow = s.Arow.copy()
    A = s.A.copy()
    # swap the first two entries of row 30 so a lower entry follows the diagonal
    b, d = s.Acol[29] - 1, s.Adia[29] - 1
    Arow[[b, d]] = Arow[[d, b]]
    A[[b, d]] = A[[d, b]]
    Adia = s.Adia.copy()
    Adia[29] = b + 1
    x, r = s.x.copy(), s.b.copy()
    with pytest.raises(tflows.SolverError) as ei:
        tflows.solve_ex("cg", s.N, s.NB, s.NONZ, A, s.Acol, Arow, Adia, s.Ab, x, r, 2, 100, s.tol)
    assert ei.value.status == tflows.BAD_INPUT
    # prec 1 on the same pattern is fine
    out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, A, s.Acol, Arow, Adia, s.Ab, x, r, 1, 100,
                          s.tol)
    assert out.status == tflows.OK


def test_bad_layout_rejected():
    s = mesh.pressure_system(3, 3, 3, seed=2)
    bad = s.Arow.copy()
    bad[5] = s.N + 4
    x, r = s.x.copy(), s.b.copy()
    with pytest.raises(tflows.SolverError) as ei:
        tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, bad, s.Adia, s.Ab, x, r, 1, 10, 1e-8)
    assert ei.value.status == tflows.BAD_INPUT


def test_device_topology_api_matches_host_api():
    import torch
    s = mesh.convection_diffusion_system(12, 10, 9, perturb=0.2, seed=4)
    topo = tflows.Topology.from_system(s)
    dev = torch.device("cuda")
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    r = torch.empty_like(x)
    res = topo.solve(val, b, x, "cgs", 1, 200, s.tol, r_out=r)
    xh, rh = s.x.copy(), s.b.copy()
    out = tflows.cgs(s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, xh, rh, 1, 200, s.tol)
    assert res["iterations"] == out.niter
    assert np.array_equal(x.cpu().numpy(), xh[s.NB + 1:])
    assert np.array_equal(r.cpu().numpy(), rh)


def test_full_size_config2_properties():
    """128^3 convection-diffusion at the benchmark size: the recursive
    residual agrees with the true residual and reaches 1e-8 relative."""
    s = mesh.config_system(2)
    for method in ("bicg", "cgs"):
        x, r = s.x.copy(), s.b.copy()
        out = tflows.solve_ex(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r,
                              1, 200, s.tol)
        assert out.status == tflows.OK and out.FinRes < s.tol
        true_r = s.b - s.scipy() @ x[s.NB + 1:]
        assert np.linalg.norm(true_r) < 2 * s.tol
        assert abs(np.linalg.norm(r) - out.FinRes) <= 1e-10 * out.IniRes


def test_true_bicg_extension_converges_where_cg_recurrence_fails():
    """BICG_TRUE (shadow sequence multiplied by A^T) on a strongly
    nonsymmetric system: reaches the tolerance and the direct solution;
    not a reference method, so it is checked against scipy."""
    import scipy.sparse.linalg as spla
    s = mesh.convection_diffusion_system(14, 12, 10, perturb=0.2, seed=5, dt=1.0)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    for prec in (0, 1):
        x, r = s.x.copy(), s.b.copy()
        out = tflows.solve_ex("bicg_true", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                              x, r, prec, 2000, tol)
        assert out.status == tflows.OK, out
        xd = spla.spsolve(s.scipy().tocsc(), s.b)
        assert rel_diff(x[s.NB + 1:], xd) < 1e-7
        assert np.linalg.norm(s.b - s.scipy() @ x[s.NB + 1:]) < 2 * tol
    with pytest.raises(tflows.SolverError):
        tflows.solve_ex("bicg_true", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                        s.x.copy(), s.b.copy(), 2, 100, tol)


# ---- TFLOWS_FP64_FMA: the same recurrences with fused multiply-adds and a
# reciprocal diagonal; every result within the FP64 bar of the reference's.

def _fma():
    return tflows.options(precision=tflows.FP64_FMA)


@pytest.mark.parametrize("path", SOLVER_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_fp64_fma_golden_solver_cases(path):
    g = np.load(path)
    opts = _fma()
    for c in range(int(g["ncalls"])):
        p = f"c{c}_"
        x = g[p + "x_in"].copy()
        r = g[p + "r1_in"].copy()
        out = tflows.solve_ex(str(g[p + "method"]), int(g["N"]), int(g["NB"]), int(g["NONZ"]),
                              g["A"], g["Acol"], g["Arow"], g["Adia"], g["Ab"], x, r,
                              int(g[p + "prec"]), int(g[p + "niter_in"]), float(g[p + "tol"]),
                              float(g[p + "IniRes_in"]), float(g[p + "FinRes_in"]), opts=opts)
        assert abs(out.niter - int(g[p + "niter_out"])) <= 1, (c, out)
        xg, rg = g[p + "x_out"], g[p + "r1_out"]
        assert np.array_equal(np.isnan(x), np.isnan(xg))
        if np.isnan(rg).any():
            assert np.isnan(out.FinRes)
            continue
        assert rel_diff(x, xg) <= REL, (c, rel_diff(x, xg))
        ini_g = float(g[p + "IniRes_out"])
        # ||b - A x0|| differs by the rounding of the contracted products,
        # which scales with ||b|| (a warm start at the solution leaves only
        # rounding noise in IniRes)
        bnorm = float(np.linalg.norm(g[p + "r1_in"]))
        assert abs(out.IniRes - ini_g) <= 1e-12 * max(abs(ini_g), 1e-300) + 1e-13 * bnorm


def test_fp64_fma_config1():
    out, _ = _oracle_vs_gpu(mesh.config_system(1), "cg", 1, 1e-12, opts=_fma())
    assert out.status == tflows.OK


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_fp64_fma_pressure_vd_cg(prec):
    s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    _oracle_vs_gpu(s, "cg", prec, 1e-12, niter=4000, it_slack=2, opts=_fma())


@pytest.mark.parametrize("method,prec", [("bicg", 1), ("bicg", 2), ("cgs", 0), ("cgs", 1),
                                         ("cgs", 2)])
def test_fp64_fma_convection_diffusion(method, prec):
    s = mesh.convection_diffusion_system(24, 20, 18, perturb=0.2, seed=5)
    _oracle_vs_gpu(s, method, prec, 1e-12, it_slack=2, opts=_fma())


def test_fp64_fma_full_size_config2():
    """The 128^3 benchmark system: the same iteration counts as the
    reference arithmetic and solutions within the FP64 bar of each other."""
    s = mesh.config_system(2)
    for method in ("bicg", "cgs"):
        xs, its = {}, {}
        for name, opts in (("ref", tflows.options()), ("fma", _fma())):
            x, r = s.x.copy(), s.b.copy()
            out = tflows.solve_ex(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                  x, r, 1, 200, s.tol, opts=opts)
            assert out.status == tflows.OK and out.FinRes < s.tol
            xs[name], its[name] = x, out.niter
        assert abs(its["ref"] - its["fma"]) <= 1, its
        assert rel_diff(xs["fma"], xs["ref"]) <= REL
        true_r = s.b - s.scipy() @ xs["fma"][s.NB + 1:]
        assert np.linalg.norm(true_r) < 2 * s.tol


def test_fp64_fma_true_bicg_and_batched():
    import torch
    s = mesh.convection_diffusion_system(14, 12, 10, perturb=0.2, seed=5, dt=1.0)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    x, r = s.x.copy(), s.b.copy()
    out = tflows.solve_ex("bicg_true", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                          x, r, 1, 2000, tol, opts=_fma())
    assert out.status == tflows.OK
    assert np.linalg.norm(s.b - s.scipy() @ x[s.NB + 1:]) < 2 * tol
    p = mesh.pressure_system(12, 11, 10, perturb=0.2, seed=2, variable_density=True)
    systems = [(p, "cg", 2), (s, "cgs", 1)]
    topos = [tflows.Topology.from_system(m) for m, _, _ in systems]

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()

    vals = [dev(m.A[:-1]) for m, _, _ in systems]
    bs = [dev(m.b) for m, _, _ in systems]
    xs = [torch.zeros(m.N, dtype=torch.float64, device="cuda") for m, _, _ in systems]
    tols = [1e-10 * float(np.linalg.norm(m.b)) for m, _, _ in systems]
    res = tflows.solve_batched(topos, vals, bs, xs, [k for _, k, _ in systems],
                               [q for _, _, q in systems], [3000, 3000], tols, _fma())
    for k, (m, _, _) in enumerate(systems):
        assert res[k]["status"] == tflows.OK, res[k]
        assert np.linalg.norm(m.b - m.scipy() @ xs[k].cpu().numpy()) < 2 * tols[k]
    for t in topos:
        t.close()


def test_bad_precision_rejected():
    s = mesh.pressure_system(6, 6, 6, seed=1)
    with pytest.raises(tflows.SolverError) as e:
        tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x.copy(),
                        s.b.copy(), 1, 100, 1e-8, opts=tflows.options(precision=7))
    assert e.value.status == tflows.BAD_INPUT
