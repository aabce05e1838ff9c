"""Launch-shape autotuner and the runtime launch shapes it chooses between.

Block size, rows per warp (hence the grid) and the IC sweep warps change
only how the work is spread and how the reductions are grouped, so every
shape must give the reference's iterates to rounding and the same
iteration counts; the tuner must return the fastest shape it timed, keep it
in its table, and batched plans must balance their block groups without
changing any system's answer.
"""
import os

import numpy as np
import pytest

from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _solve(topo, s, method, prec, **kw):
    import torch
    opts = tflows.options(tol_mode=tflows.TOL_RELATIVE, **kw)
    x = torch.zeros(s.N, dtype=torch.float64, device="cuda")
    res = topo.solve(_dev(s.A[:-1]), _dev(s.b), x, method, prec, 5000, 1e-10, opts=opts)
    return x.cpu().numpy(), res


@pytest.mark.parametrize("method,prec,precision", [("cg", 1, 0), ("cg", 2, 0), ("cgs", 1, 0),
                                                   ("cg", 2, 1), ("bicg", 1, 1)])
@pytest.mark.parametrize("block,rpw", [(128, 0), (512, 0), (256, 256), (64, 1024)])
def test_launch_shapes_give_the_same_answer(method, prec, precision, block, rpw):
    if method == "cg":
        s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    else:
        s = mesh.convection_diffusion_system(20, 18, 16, perturb=0.2, seed=5)
    topo = tflows.Topology.from_system(s)
    # mixed: restarted refinement, whose iterates depend on the launch shape
    # only through rounding (reliable updates decide on direction restarts
    # by a threshold that rounding can flip; see the test below)
    kw = {"refine_restart": 1} if precision == 1 else {}
    x0, r0 = _solve(topo, s, method, prec, precision=precision, **kw)
    x1, r1 = _solve(topo, s, method, prec, precision=precision, block_size=block,
                    rows_per_warp=rpw, sweep_warps=2, **kw)
    assert r0["status"] == r1["status"] == tflows.OK, (r0, r1)
    assert r1["block_size"] == block
    assert abs(r0["iterations"] - r1["iterations"]) <= 1, (r0, r1)
    tol = 1e-8 if precision == 0 else 1e-7
    assert np.abs(x1 - x0).max() <= tol * np.abs(x0).max()
    topo.close()


@pytest.mark.parametrize("block,rpw", [(128, 0), (512, 0), (256, 256)])
def test_reliable_updates_across_launch_shapes(block, rpw):
    """Mixed CG with reliable updates (the default refinement): every launch
    shape reaches the tolerance with a solution within the refinement
    accuracy of the default shape's, and within 25 % of its iterations."""
    s = mesh.pressure_system(20, 18, 16, perturb=0.2, seed=11, variable_density=True)
    topo = tflows.Topology.from_system(s)
    x0, r0 = _solve(topo, s, "cg", 2, precision=1)
    x1, r1 = _solve(topo, s, "cg", 2, precision=1, block_size=block, rows_per_warp=rpw)
    assert r0["status"] == r1["status"] == tflows.OK, (r0, r1)
    assert abs(r0["iterations"] - r1["iterations"]) <= max(2, r0["iterations"] // 4), (r0, r1)
    assert np.abs(x1 - x0).max() <= 1e-7 * np.abs(x0).max()
    topo.close()


def test_bad_launch_shapes_are_rejected():
    import torch
    s = mesh.pressure_system(6, 6, 6, seed=1)
    topo = tflows.Topology.from_system(s)
    x = torch.zeros(s.N, dtype=torch.float64, device="cuda")
    for kw in ({"block_size": 100}, {"block_size": 1024}, {"rows_per_warp": -1}):
        with pytest.raises(tflows.SolverError) as e:
            topo.solve(_dev(s.A[:-1]), _dev(s.b), x, "cg", 1, 100, 1e-8,
                       opts=tflows.options(**kw))
        assert e.value.status == tflows.BAD_INPUT
    topo.close()


@pytest.mark.parametrize("prec,precision", [(1, 0), (2, 0), (1, 1)])
def test_autotune_returns_the_fastest_shape_and_remembers_it(prec, precision):
    tflows.autotune_clear()
    s = mesh.pressure_system(48, 40, 36, perturb=0.2, seed=3, variable_density=True)
    topo = tflows.Topology.from_system(s)
    opts = tflows.options(precision=precision)
    t1 = topo.autotune(_dev(s.A[:-1]), _dev(s.b), "cg", prec, opts=opts)
    assert t1["block_size"] in (128, 256, 512) and t1["candidates"] >= 3, t1
    assert 0 < t1["us_per_iteration"] <= t1["default_us_per_iteration"], t1
    assert t1["from_table"] == 0
    t2 = topo.autotune(_dev(s.A[:-1]), _dev(s.b), "cg", prec, opts=opts)
    assert t2["from_table"] == 1 and t2["block_size"] == t1["block_size"]
    # a solve asking for the tuned shape gets it, with the untuned answer
    x0, r0 = _solve(topo, s, "cg", prec, precision=precision)
    x1, r1 = _solve(topo, s, "cg", prec, precision=precision, autotune=1)
    assert r1["status"] == tflows.OK and r1["block_size"] == t1["block_size"], (t1, r1)
    assert abs(r0["iterations"] - r1["iterations"]) <= 1
    assert np.abs(x1 - x0).max() <= 1e-7 * np.abs(x0).max()
    topo.close()


def test_autotune_table_file_round_trip(tmp_path):
    path = str(tmp_path / "tune.txt")
    os.environ["TFLOWS_TUNE_FILE"] = path
    try:
        tflows.autotune_clear()
        s = mesh.convection_diffusion_system(30, 28, 26, perturb=0.2, seed=9)
        topo = tflows.Topology.from_system(s)
        t1 = topo.autotune(_dev(s.A[:-1]), _dev(s.b), "bicg", 1)
        assert t1["from_table"] == 0
        lines = open(path).read().split("\n")
        assert len([ln for ln in lines if ln.strip()]) == 1
        tflows.autotune_clear()  # forget; the next lookup reads the file
        t2 = topo.autotune(_dev(s.A[:-1]), _dev(s.b), "bicg", 1)
        assert t2["from_table"] == 1 and t2["block_size"] == t1["block_size"]
        assert t2["rows_per_warp"] == t1["rows_per_warp"]
        topo.close()
    finally:
        del os.environ["TFLOWS_TUNE_FILE"]
        tflows.autotune_clear()


def test_autotuned_plan_balances_groups_and_keeps_answers():
    import torch
    systems = [
        (mesh.pressure_system(10, 9, 8, perturb=0.2, seed=1, variable_density=True), "cg", 2),
        (mesh.convection_diffusion_system(12, 10, 9, perturb=0.2, seed=2), "bicg", 1),
        (mesh.pressure_system(32, 30, 28, perturb=0.2, seed=3, variable_density=True), "cg", 1),
        (mesh.convection_diffusion_system(7, 7, 30, perturb=0.2, seed=4), "cgs", 1),
        (mesh.pressure_system(24, 24, 24, perturb=0.2, seed=5, variable_density=True), "cg", 2),
    ]
    topos = [tflows.Topology.from_system(s) for s, _, _ in systems]
    vals = [_dev(s.A[:-1]) for s, _, _ in systems]
    bs = [_dev(s.b) for s, _, _ in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s, _, _ in systems]
    tols = [1e-10] * len(systems)
    opts = tflows.options(precision=tflows.MIXED, tol_mode=tflows.TOL_RELATIVE, autotune=1)
    plan = tflows.Plan(topos, vals, bs, xs, [m for _, m, _ in systems],
                       [p for _, _, p in systems], [5000] * len(systems), tols, opts)
    tun = plan.tuning()
    assert tun["runs"] >= 3 and tun["block_size"] in (128, 256, 512), tun
    assert 0 < tun["tuned_seconds"] <= tun["default_seconds"] * 1.0001, tun
    for rep in range(2):
        for x in xs:
            x.zero_()
        plan.launch()
        res = plan.results()
        for k, (s, m, p) in enumerate(systems):
            assert res[k]["status"] == tflows.OK, (k, res[k])
            assert res[k]["block_size"] == tun["block_size"]
            xa = xs[k].cpu().numpy()
            assert np.linalg.norm(s.b - s.scipy() @ xa) < 2e-10 * np.linalg.norm(s.b), k
    plan.close()
    for t in topos:
        t.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_gated_polling_changes_no_bit(precision):
    """Gated polling only changes when a warp looks at its inputs, not what
    it computes: with the same launch shape the solution is bit-identical."""
    s = mesh.pressure_system(24, 20, 18, perturb=0.2, seed=4, variable_density=True)
    topo = tflows.Topology.from_system(s)
    xs = []
    for gate in (0, 1):
        x, r = _solve(topo, s, "cg", 2, precision=precision, sweep_gate=gate)
        assert r["status"] == tflows.OK
        xs.append(x)
    assert np.array_equal(xs[0].view(np.uint64), xs[1].view(np.uint64))
    topo.close()
