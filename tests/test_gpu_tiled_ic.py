"""Tiled IC(0) sweeps on box-numbered patterns.

On a 7-point box in natural numbering (what TopolM builds for a structured
block) the exact IC apply runs block-local wavefront steps over x-y tiles
instead of global level-ordered sweeps.  Each row still combines the same
operands in the same order as the sequential sweep of Process/CG.f90:135-156,
so in reference arithmetic one apply must equal the level-ordered apply and
the sequential loops bit for bit, at every block size; the contracted build
(which multiplies by a precomputed 1/(D+TINY)) must agree to rounding; whole
solves must meet the reference's parity bar against the oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


@pytest.mark.parametrize("dims", [(20, 13, 7), (16, 8, 5), (33, 17, 3), (5, 40, 6), (40, 36, 30)])
@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("block", [128, 256, 512])
def test_tiled_apply_equals_level_apply(dims, precision, block):
    import torch
    s = mesh.pressure_system(*dims, perturb=0.2, seed=sum(dims), variable_density=True)
    topo = tflows.Topology.from_system(s)
    val = _dev(s.A[:-1])
    r = _dev(np.random.default_rng(block).uniform(-1, 1, s.N))
    out = {}
    for tiled in (0, 1):
        z = torch.full((s.N,), float("nan"), dtype=torch.float64, device="cuda")
        opts = tflows.options(precision=precision, ic_tiled=tiled, block_size=block)
        res = topo.ic_apply(val, r, z, opts=opts)
        assert res["status"] == tflows.OK
        out[tiled] = z.cpu().numpy()
    topo.close()
    assert np.isfinite(out[1]).all()
    if precision == 0:
        assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))
    else:
        assert np.abs(out[0] - out[1]).max() <= 1e-12 * np.abs(out[0]).max()


def test_tiled_apply_matches_sequential_formula():
    """The apply against the sequential restatement of the reference loops
    (forward, /(D+TINY), backward) in numpy, reference arithmetic."""
    import torch
    s = mesh.pressure_system(12, 9, 7, perturb=0.2, seed=4, variable_density=True)
    D = oracle.prec1(s.N, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, 2)
    rp, col, dg, A = s.Acol - 1, s.Arow[:-1] - 1, s.Adia - 1, s.A[:-1]
    r = np.random.default_rng(0).uniform(-1, 1, s.N)
    w = np.zeros(s.N)
    for i in range(s.N):
        acc = r[i]
        for j in range(rp[i], dg[i]):
            acc = acc - A[j] * w[col[j]]
        w[i] = acc * D[i]
    z = np.zeros(s.N)
    for i in range(s.N - 1, -1, -1):
        acc = w[i] / (D[i] + 1e-64)
        for j in range(dg[i] + 1, rp[i + 1]):
            acc = acc - A[j] * z[col[j]]
        z[i] = acc * D[i]
    topo = tflows.Topology.from_system(s)
    zg = torch.empty(s.N, dtype=torch.float64, device="cuda")
    topo.ic_apply(_dev(A), _dev(r), zg, opts=tflows.options(ic_tiled=1))
    topo.close()
    assert np.array_equal(zg.cpu().numpy().view(np.uint64), z.view(np.uint64))


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("dims,seed", [((24, 20, 18), 1), ((32, 32, 32), 0), ((17, 35, 9), 3)])
def test_tiled_ic_cg_matches_oracle(precision, dims, seed):
    """IC-preconditioned CG through the Fortran-facing entry point with the
    tiled sweeps: within 1e-8 of the oracle, iteration counts within 1 (2 for
    the contracted build)."""
    s = mesh.pressure_system(*dims, perturb=0.2, seed=seed, variable_density=True)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    xo, _, ito, inio, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                       s.x, s.b, 2, 3000, tol)
    x, r = s.x.copy(), s.b.copy()
    out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 2,
                          3000, tol, opts=tflows.options(precision=precision, ic_tiled=1))
    assert out.status == tflows.OK
    assert abs(out.niter - ito) <= (1 if precision == 0 else 2), (out.niter, ito)
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()
    assert abs(out.IniRes - inio) <= 1e-12 * inio


@pytest.mark.parametrize("bf16", [0, 1])
@pytest.mark.parametrize("restart", [1, 0])
def test_tiled_ic_mixed_matches_level_and_oracle(bf16, restart):
    """Mixed precision (FP32 inner CG, IC in FP32 or BF16, FP64 refinement)
    with tiled and with level sweeps: both reach the FP64 tolerance and agree
    with the FP64 oracle solve to the accuracy the tolerance implies."""
    s = mesh.config_system(3, scale=28)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    xo, *_ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x, s.b,
                          2, 5000, 1e-3 * tol)
    scale = np.abs(xo).max()
    its = {}
    for tiled in (0, 1):
        x, r = s.x.copy(), s.b.copy()
        opts = tflows.options(precision=tflows.MIXED, ic_bf16=bf16, ic_tiled=tiled,
                              refine_restart=restart)
        out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r,
                              2, 20000, tol, opts=opts)
        res = tflows.last_result()
        assert out.status == tflows.OK, (tiled, out, res)
        assert np.linalg.norm(s.b - s.scipy() @ x[s.NB + 1:]) < tol
        assert np.abs(x - xo).max() <= 1e-6 * scale, tiled
        its[tiled] = res["inner_iterations"]
    # the same preconditioner: iteration counts differ by reduction rounding only
    assert abs(its[0] - its[1]) <= max(3, its[0] // 20), its


def test_non_box_numbering_falls_back_to_level_sweeps():
    """A symmetric renumbering of a box is not box-numbered: the tiled option
    is ignored and the apply equals the level-ordered one."""
    import torch
    s = mesh.pressure_system(9, 8, 7, perturb=0.2, seed=8, variable_density=True)
    A = s.scipy().tocsr()
    perm = np.random.default_rng(2).permutation(s.N)
    B = A[perm][:, perm].tocsr()
    B.sort_indices()
    rp = B.indptr.astype(np.int32)
    col = B.indices.astype(np.int32)
    dg = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(s.N)],
                  dtype=np.int32)
    topo = tflows.Topology(s.N, rp, col, dg)
    val, r = _dev(B.data), _dev(np.random.default_rng(3).uniform(-1, 1, s.N))
    z = {}
    for tiled in (0, 1):
        zz = torch.empty(s.N, dtype=torch.float64, device="cuda")
        topo.ic_apply(val, r, zz, opts=tflows.options(ic_tiled=tiled))
        z[tiled] = zz.cpu().numpy()
    topo.close()
    assert np.array_equal(z[0].view(np.uint64), z[1].view(np.uint64))


def test_tiled_ic_in_batched_plan():
    """Uneven IC systems in one graph-captured batched launch with the tiled
    sweeps (mixed, BF16 factor entries): every system meets its tolerance and
    agrees with the FP64 oracle."""
    import torch
    shapes = [(18, 16, 12), (24, 24, 20), (12, 10, 9), (30, 28, 16)]
    systems = [mesh.pressure_system(*d, perturb=0.2, seed=40 + k, variable_density=True)
               for k, d in enumerate(shapes)]
    topos = [tflows.Topology.from_system(s) for s in systems]
    vals = [_dev(s.A[:-1]) for s in systems]
    bs = [_dev(s.b) for s in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s in systems]
    tols = [1e-10 * float(np.linalg.norm(s.b)) for s in systems]
    opts = tflows.options(precision=tflows.MIXED, ic_bf16=1, ic_tiled=1)
    plan = tflows.Plan(topos, vals, bs, xs, ["cg"] * 4, [2] * 4, [20000] * 4, tols, opts)
    for _ in range(2):
        for x in xs:
            x.zero_()
        plan.launch()
        res = plan.results()
        for k, s in enumerate(systems):
            assert res[k]["status"] == tflows.OK, (k, res[k])
            xg = xs[k].cpu().numpy()
            assert np.linalg.norm(s.b - s.scipy() @ xg) < tols[k]
            xo, *_ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                  s.x, s.b, 2, 5000, 1e-3 * tols[k])
            xo = xo[s.NB + 1:]
            assert np.abs(xg - xo).max() <= 1e-6 * np.abs(xo).max(), k
    plan.close()
    for t in topos:
        t.close()
