"""The benchmark configurations' solver shapes at reduced size, against the oracle.

Config 3: CG + IC(0) on a variable-density pressure system (density ratio
1/0.14 ~ 7), mixed precision (FP32 inner solves, FP64 refinement), IC factor
entries in BF16, exact sweeps or Jacobi sweeps.  Config 4: uneven systems
(CG + IC(0) pressure, BiCG + diagonal transport) in one graph-captured
batched plan, mixed precision.  Every solution is compared with the oracle's
FP64 solve of the same system (Process/CG.f90, BiCG.f90 restated), tightened
1000x so that the oracle's own error is negligible, to the accuracy the
tolerance implies; iteration counts of mixed solves stay near the FP64
solve's with the same preconditioner.
"""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _oracle_x(s, method, prec, b, tol):
    xo, *_ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, s.x, b,
                          prec, 20000, 1e-3 * tol)
    return xo[s.NB + 1:]


def _mixed_vs_fp64(s, prec, sweeps):
    """Mixed (BF16 IC factors) and FP64-FMA solves of ``s`` from x0 = 0:
    the mixed solution at 1e-10 relative residual against the oracle, and
    both solvers' iteration counts at the configuration's 1e-8."""
    import torch
    topo = tflows.Topology.from_system(s)
    val, b = _dev(s.A[:-1]), _dev(s.b)
    bn = float(np.linalg.norm(s.b))
    its = {}
    for rel in (1e-10, 1e-8):
        for label, prec_mode in (("mixed", tflows.MIXED), ("fp64_fma", tflows.FP64_FMA)):
            if rel == 1e-10 and label != "mixed":
                continue
            opts = tflows.options(precision=prec_mode, ic_sweeps=sweeps,
                                  **({"ic_bf16": 1} if label == "mixed" else {}))
            x = torch.zeros(s.N, dtype=torch.float64, device="cuda")
            r = topo.solve(val, b, x, "cg", prec, 20000, rel * bn, opts=opts)
            assert r["status"] == tflows.OK, (label, rel, r)
            xg = x.cpu().numpy()
            assert np.linalg.norm(s.b - s.scipy() @ xg) < rel * bn, (label, rel)
            if rel == 1e-10:
                xo = _oracle_x(s, "cg", prec, s.b, rel * bn)
                assert np.abs(xg - xo).max() <= 1e-6 * np.abs(xo).max()
            else:
                its[label] = r["inner_iterations"] if label == "mixed" else r["iterations"]
    topo.close()
    return its


@pytest.mark.parametrize("sweeps", [0, 1, 2])
def test_config3_shape_mixed_ic_against_oracle(sweeps):
    """32^3 config-3 system, CG + IC(0) with BF16 factors (exact, one or two
    Jacobi sweeps per triangle): the mixed solve meets the FP64 tolerance
    and agrees with the oracle to 1e-6 of the solution's scale.  At the
    configuration's tolerance it needs at most 15 % more iterations than
    the FP64-FMA solve with the same sweeps (exact sweeps); with Jacobi
    sweeps the BF16 factors change the cheaper preconditioner itself, and
    the bound is 35 % at this size."""
    s = mesh.config_system(3, scale=32)
    its = _mixed_vs_fp64(s, 2, sweeps)
    assert its["mixed"] <= (1.15 if sweeps == 0 else 1.35) * its["fp64_fma"] + 2, its


def test_config3_shape_mixed_diagonal_iteration_ratio():
    """Diagonal preconditioning on the same system: the mixed solution within
    1e-6 of the oracle's, inner iterations within 15 % of FP64-FMA's at the
    configuration's tolerance."""
    s = mesh.config_system(3, scale=32)
    its = _mixed_vs_fp64(s, 1, 0)
    assert its["mixed"] <= 1.15 * its["fp64_fma"] + 2, its


@pytest.mark.parametrize("sweeps", [0, 1])
def test_config4_shape_batched_plan_against_oracle(sweeps):
    """Eight uneven systems (log-uniform sizes, odd ones CG + IC(0) pressure
    with density ratio ~7, even ones BiCG + diagonal transport), mixed
    precision with BF16 IC factors, in one graph-captured plan replayed
    twice: each system meets its tolerance and agrees with the oracle."""
    import torch
    shapes = mesh.batch_sizes(8, lo=8, hi=28, seed=3)
    systems = []
    for k, (nx, ny, nz) in enumerate(shapes):
        if k % 2:
            systems.append((mesh.pressure_system(nx, ny, nz, perturb=0.2, seed=200 + k,
                                                 variable_density=True), "cg", 2))
        else:
            systems.append((mesh.convection_diffusion_system(nx, ny, nz, perturb=0.2,
                                                             seed=200 + k), "bicg", 1))
    topos = [tflows.Topology.from_system(s) for s, _, _ in systems]
    vals = [_dev(s.A[:-1]) for s, _, _ in systems]
    bs = [_dev(s.b) for s, _, _ in systems]
    xs = [torch.zeros(s.N, dtype=torch.float64, device="cuda") for s, _, _ in systems]
    tols = [1e-10 * float(np.linalg.norm(s.b)) for s, _, _ in systems]
    opts = tflows.options(precision=tflows.MIXED, ic_bf16=1, ic_sweeps=sweeps)
    plan = tflows.Plan(topos, vals, bs, xs, [m for _, m, _ in systems],
                       [p for _, _, p in systems], [20000] * len(systems), tols, opts)
    xo = [_oracle_x(s, m, p, s.b, t) for (s, m, p), t in zip(systems, tols)]
    for _ in range(2):
        for x in xs:
            x.zero_()
        plan.launch()
        res = plan.results()
        for k, (s, m, p) in enumerate(systems):
            assert res[k]["status"] == tflows.OK, (k, res[k])
            xg = xs[k].cpu().numpy()
            assert np.linalg.norm(s.b - s.scipy() @ xg) < tols[k], k
            assert np.abs(xg - xo[k]).max() <= 1e-6 * np.abs(xo[k]).max(), k
    plan.close()
    for t in topos:
        t.close()
