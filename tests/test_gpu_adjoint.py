"""Hand-written adjoint of the GPU solve (torch.autograd.Function).

Config 5 of the benchmark suite: a perturbed-hex variable-density pressure
system assembled differentiably from its face coefficients (1/rho scaled,
float32), loss 0.5 ||x - x_target||^2.  The gradients with respect to the
right-hand side (float64) and the face coefficients come from one transposed
solve; they are checked against a dense FP64 adjoint at 16^3 and against
central finite differences (eps = 1e-6) on 200 random coefficients at 64^3.
"""
import numpy as np
import pytest

from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _setup(n, seed=0):
    import torch
    from tflows_gb300 import autograd as ag
    s = mesh.pressure_system(n, n, n, perturb=0.2, seed=seed, variable_density=True,
                             keep_faces=True)
    solver = ag.DifferentiableSolver.from_system(s, method="cg", prec=1, rtol=1e-13)
    asm = ag.FaceAssembly(s)
    rng = np.random.default_rng(seed + 100)
    xt = torch.as_tensor(rng.uniform(-1, 1, s.N), device="cuda")
    coef = torch.tensor(s.face_coef, dtype=torch.float32, device="cuda", requires_grad=True)
    b = torch.tensor(s.b, dtype=torch.float64, device="cuda", requires_grad=True)
    return s, solver, asm, xt, coef, b


def _loss(solver, asm, coef, b, xt):
    x = solver(asm(coef), b)
    return 0.5 * ((x - xt) ** 2).sum(), x


def test_adjoint_matches_dense_fp64_reference_16cube():
    s, solver, asm, xt, coef, b = _setup(16)
    L, x = _loss(solver, asm, coef, b, xt)
    L.backward()
    # dense FP64 reference with the float32-rounded coefficients
    val = asm(coef.detach()).cpu().numpy()
    rp, col, _, _ = s.csr0()
    A = np.zeros((s.N, s.N))
    rows = np.repeat(np.arange(s.N), np.diff(rp))
    A[rows, col] = val
    xd = np.linalg.solve(A, s.b)
    lam = np.linalg.solve(A.T, xd - xt.cpu().numpy())
    c1, c2 = asm.c1, asm.c2
    gc = -(lam[c1] - lam[c2]) * (xd[c1] - xd[c2])
    assert np.abs(x.detach().cpu().numpy() - xd).max() <= 1e-9 * np.abs(xd).max()
    gb = b.grad.cpu().numpy()
    assert np.abs(gb - lam).max() <= 1e-8 * np.abs(lam).max()
    ga = coef.grad.cpu().numpy().astype(np.float64)
    assert np.abs(ga - gc).max() <= 1e-5 * np.abs(gc).max()


def test_adjoint_matches_central_differences_64cube():
    import torch
    s, solver, asm, xt, coef, b = _setup(64, seed=1)
    L, _ = _loss(solver, asm, coef, b, xt)
    L.backward()
    ga = coef.grad.cpu().numpy().astype(np.float64)
    gb = b.grad.cpu().numpy()
    rng = np.random.default_rng(7)
    faces = rng.choice(coef.shape[0], 200, replace=False)
    eps = 1e-6
    c64 = coef.detach().to(torch.float64)
    fd = []
    with torch.no_grad():
        for f in faces:
            cp, cm = c64.clone(), c64.clone()
            cp[f] += eps
            cm[f] -= eps
            lp, _ = _loss(solver, asm, cp, b.detach(), xt)
            lm, _ = _loss(solver, asm, cm, b.detach(), xt)
            fd.append((float(lp) - float(lm)) / (2 * eps))
    fd = np.array(fd)
    scale = np.abs(ga).max()
    assert np.abs(ga[faces] - fd).max() <= 2e-4 * scale, np.abs(ga[faces] - fd).max() / scale
    # right-hand side: a few entries by central differences as well
    cells = rng.choice(s.N, 10, replace=False)
    with torch.no_grad():
        for c in cells:
            bp, bm = b.detach().clone(), b.detach().clone()
            bp[c] += eps
            bm[c] -= eps
            lp, _ = _loss(solver, asm, coef.detach(), bp, xt)
            lm, _ = _loss(solver, asm, coef.detach(), bm, xt)
            g = (float(lp) - float(lm)) / (2 * eps)
            assert abs(gb[c] - g) <= 1e-4 * np.abs(gb).max() + 1e-6 * abs(g)


def test_transpose_index_and_nonsymmetric_adjoint():
    """A nonsymmetric matrix: the adjoint solve really uses A^T."""
    import torch
    from tflows_gb300 import autograd as ag
    s = mesh.convection_diffusion_system(8, 7, 6, perturb=0.2, seed=3, dt=1.0)
    rp, col, val, _ = s.csr0()
    t = ag.transpose_index(rp, col)
    rows = np.repeat(np.arange(s.N), np.diff(rp))
    assert np.array_equal(rows[t], col) and np.array_equal(col[t], rows)
    solver = ag.DifferentiableSolver.from_system(s, method="cgs", prec=1, rtol=1e-13)
    v = torch.tensor(val, device="cuda", requires_grad=True)
    b = torch.tensor(s.b, device="cuda", requires_grad=True)
    w = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, s.N), device="cuda")
    x = solver(v, b)
    (w * x).sum().backward()
    A = s.scipy().toarray()
    lam = np.linalg.solve(A.T, w.cpu().numpy())
    assert np.abs(b.grad.cpu().numpy() - lam).max() <= 1e-8 * np.abs(lam).max()
    xd = np.linalg.solve(A, s.b)
    gv = -lam[rows] * xd[col]
    assert np.abs(v.grad.cpu().numpy() - gv).max() <= 1e-7 * np.abs(gv).max()
