"""Batched solves: many independent systems in one persistent launch.

Each system runs on its own group of blocks with its own barriers and
reductions; the results must agree with solving the systems one at a time
(same arithmetic; the reduction trees differ with the group size, so
iterates agree to rounding) and reach each system's tolerance.
"""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _systems():
    return [
        (mesh.pressure_system(10, 9, 8, perturb=0.2, seed=1, variable_density=True), "cg", 2),
        (mesh.convection_diffusion_system(12, 10, 9, perturb=0.2, seed=2), "bicg", 1),
        (mesh.pressure_system(16, 16, 16, perturb=0.2, seed=3, variable_density=True), "cg", 1),
        (mesh.convection_diffusion_system(7, 7, 30, perturb=0.2, seed=4), "cgs", 1),
        (mesh.pressure_system(5, 6, 7, seed=5), "cg", 0),
        (mesh.convection_diffusion_system(20, 18, 16, perturb=0.2, seed=6), "cgs", 2),
    ]


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("precision,ic", [(0, {}), (1, {}), (1, {"ic_bf16": 1, "ic_sweeps": 2})])
def test_batched_matches_one_at_a_time(precision, ic):
    import torch
    systems = _systems()
    opts = tflows.options(precision=precision, **ic)
    topos = [tflows.Topology.from_system(s) for s, _, _ in systems]
    vals = [_dev(s.A[:-1]) for s, _, _ in systems]
    bs = [_dev(s.b) for s, _, _ in systems]
    tols = [1e-10 * float(np.linalg.norm(s.b)) for s, _, _ in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s, _, _ in systems]
    res = tflows.solve_batched(topos, vals, bs, xs, [m for _, m, _ in systems],
                               [p for _, _, p in systems], [3000] * len(systems), tols, opts)
    for k, (s, m, p) in enumerate(systems):
        assert res[k]["status"] == tflows.OK, (k, res[k])
        x1 = torch.zeros(s.N, dtype=torch.float64, device="cuda")
        r1 = topos[k].solve(vals[k], bs[k], x1, m, p, 3000, tols[k], opts=opts)
        assert r1["status"] == tflows.OK
        assert abs(res[k]["iterations"] - r1["iterations"]) <= 2, (k, res[k], r1)
        xa, xb = xs[k].cpu().numpy(), x1.cpu().numpy()
        assert np.abs(xa - xb).max() <= 1e-7 * np.abs(xb).max(), k
        true_r = s.b - s.scipy() @ xa
        assert np.linalg.norm(true_r) < 2 * tols[k]


def test_batched_repeated_pattern():
    """Several right-hand sides on one pattern (as the equations of one
    SIMPLE step share the mesh topology) in one launch."""
    import torch
    s = mesh.convection_diffusion_system(16, 14, 12, perturb=0.2, seed=8)
    topo = tflows.Topology.from_system(s)
    rng = np.random.default_rng(0)
    rhs = [s.b * (1.0 + 0.1 * k) + rng.uniform(-1, 1, s.N) for k in range(5)]
    val = _dev(s.A[:-1])
    bs = [_dev(b) for b in rhs]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for _ in rhs]
    tols = [1e-10 * float(np.linalg.norm(b)) for b in rhs]
    res = tflows.solve_batched([topo] * 5, [val] * 5, bs, xs, ["bicg"] * 5, [1] * 5, [500] * 5,
                               tols)
    A = s.scipy()
    for k in range(5):
        assert res[k]["status"] == tflows.OK
        assert np.linalg.norm(rhs[k] - A @ xs[k].cpu().numpy()) < 2 * tols[k]


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_plan_replays_with_new_data(precision):
    """One CUDA graph holds the whole batched solve; each replay picks up new
    right-hand sides written in place (as a time loop would) and must reach
    the tolerance relative to them."""
    import torch
    systems = _systems()
    opts = tflows.options(precision=precision, tol_mode=tflows.TOL_RELATIVE)
    topos = [tflows.Topology.from_system(s) for s, _, _ in systems]
    vals = [_dev(s.A[:-1]) for s, _, _ in systems]
    bs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s, _, _ in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s, _, _ in systems]
    plan = tflows.Plan(topos, vals, bs, xs, [m for _, m, _ in systems],
                       [p for _, _, p in systems], [3000] * len(systems), [1e-10] * len(systems),
                       opts)
    rng = np.random.default_rng(1)
    for step in range(3):
        rhs = [s.b * (1.0 + step) + rng.uniform(-1, 1, s.N) for s, _, _ in systems]
        for k in range(len(systems)):
            bs[k].copy_(_dev(rhs[k]))
            xs[k].zero_()
        plan.launch()
        res = plan.results()
        for k, (s, m, p) in enumerate(systems):
            assert res[k]["status"] == tflows.OK, (step, k, res[k])
            x = xs[k].cpu().numpy()
            assert np.linalg.norm(rhs[k] - s.scipy() @ x) < 2e-10 * np.linalg.norm(rhs[k]), (step, k)
    plan.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_simple_step_plan_on_one_topology(precision):
    """The five solves of one SIMPLE outer iteration -- mixture fraction (cg),
    three momentum components (bicg) and pressure correction (cg, IC) -- on
    one mesh topology, replayed from one captured plan; each system must
    match its own single-system solve and the oracle's solve."""
    import torch
    cd = mesh.convection_diffusion_system(14, 12, 10, perturb=0.2, seed=21)
    zm = mesh.convection_diffusion_system(14, 12, 10, perturb=0.2, seed=22)
    pr = mesh.pressure_system(14, 12, 10, perturb=0.2, seed=23, variable_density=True)
    topo = tflows.Topology.from_system(pr)
    rng = np.random.default_rng(24)
    rhs = [zm.b] + [cd.b * (1.0 + 0.1 * k) + rng.uniform(-0.1, 0.1, cd.N) for k in range(3)] + [pr.b]
    mats = [zm, cd, cd, cd, pr]
    methods = ["cg", "bicg", "bicg", "bicg", "cg"]
    precs = [1, 1, 1, 1, 2]
    vals = [_dev(m.A[:-1]) for m in mats]
    bs = [_dev(b) for b in rhs]
    xs = [torch.zeros(pr.N, dtype=torch.float64, device="cuda") for _ in mats]
    tols = [1e-10 * float(np.linalg.norm(b)) for b in rhs]
    opts = tflows.options(precision=precision)
    plan = tflows.Plan([topo] * 5, vals, bs, xs, methods, precs, [3000] * 5, tols, opts)
    # each system's oracle solve (Process/CG.f90, BiCG.f90 restated), 1000x tighter
    xo = []
    for k in range(5):
        m = mats[k]
        xk, *_ = oracle.solve(methods[k], m.N, m.NB, m.NONZ, m.A, m.Acol, m.Arow, m.Adia, m.Ab,
                              m.x, rhs[k], precs[k], 20000, 1e-3 * tols[k])
        xo.append(xk[m.NB + 1:])
    for _ in range(2):
        for x in xs:
            x.zero_()
        plan.launch()
        res = plan.results()
        for k in range(5):
            assert res[k]["status"] == tflows.OK, (k, res[k])
            x1 = torch.zeros(pr.N, dtype=torch.float64, device="cuda")
            r1 = topo.solve(vals[k], bs[k], x1, methods[k], precs[k], 3000, tols[k], opts=opts)
            assert r1["status"] == tflows.OK
            assert abs(res[k]["iterations"] - r1["iterations"]) <= 2, (k, res[k], r1)
            xa, xb = xs[k].cpu().numpy(), x1.cpu().numpy()
            assert np.abs(xa - xb).max() <= 1e-7 * np.abs(xb).max(), k
            assert np.linalg.norm(rhs[k] - mats[k].scipy() @ xa) < 2 * tols[k]
            assert np.abs(xa - xo[k]).max() <= 1e-6 * np.abs(xo[k]).max(), k
    plan.close()
    topo.close()
