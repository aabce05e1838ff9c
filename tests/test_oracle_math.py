"""Mathematical cross-checks of the oracle, beside its bit-for-bit pins to
the reference source: its solvers reach the dense solution, its IC(0)
preconditioner is the operator Process/CG.f90:135-156 describes, and a
one-cell system takes one iteration.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from conftest import tflows

mesh = tflows.mesh


def _dense(s):
    nnz = int(s.NONZ) - 1
    rows = np.repeat(np.arange(s.N), np.diff(s.Acol))
    return sp.csr_matrix((s.A[:nnz], (rows, s.Arow[:nnz] - 1)), shape=(s.N, s.N)).toarray()


@pytest.mark.parametrize("method,prec", [("cg", 0), ("cg", 1), ("cg", 2), ("cgs", 1),
                                         ("cgs", 2), ("bicg", 1)])
def test_oracle_reaches_the_dense_solution(method, prec):
    if method == "cg":
        s = mesh.pressure_system(7, 6, 5, perturb=0.2, seed=4, variable_density=True)
    else:
        s = mesh.convection_diffusion_system(7, 6, 5, perturb=0.2, seed=4)
    A = _dense(s)
    xd = np.linalg.solve(A, s.b)
    tol = 1e-12 * float(np.linalg.norm(s.b))
    x, r, it, _, _ = oracle.solve(method, s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                  np.zeros_like(s.x), s.b, prec, 5000, tol)
    assert it <= 5000
    xs = x[s.NB + 1:]
    assert np.abs(xs - xd).max() <= 1e-8 * np.abs(xd).max()
    # the returned r1 is the recursive residual: close to the true one
    assert np.linalg.norm((s.b - A @ xs) - r) <= 1e-6 * float(np.linalg.norm(s.b))


def test_ic_preconditioner_is_the_documented_operator():
    """Prec1 (prec 2) gives D_i = 1 / (a_ii - sum_{k<i} D_k a_ik^2); the apply is
    a forward solve of (D^-1 + L) y = r, a scaling by 1/(D + TINY) and a
    backward solve of (D^-1 + U) z = y, i.e. z = M^-1 r with
    M = (D^-1 + L) D (D^-1 + U).  One CG iteration from x0 = 0 moves along
    z0 = M^-1 b, so x1 is parallel to the dense M^-1 b."""
    s = mesh.pressure_system(6, 5, 4, perturb=0.2, seed=2, variable_density=True)
    A = _dense(s)
    D = oracle.prec1(s.N, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, 2)
    Dd = np.zeros(s.N)
    for i in range(s.N):
        Dd[i] = 1.0 / (A[i, i] - sum(Dd[k] * A[i, k] ** 2 for k in range(i) if A[i, k] != 0.0))
    assert np.allclose(D, Dd, rtol=1e-14, atol=0.0)
    L, U = np.tril(A, -1), np.triu(A, 1)
    M = (np.diag(1.0 / D) + L) @ np.diag(D) @ (np.diag(1.0 / D) + U)
    z0 = np.linalg.solve(M, s.b)
    x, _, it, _, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab,
                                  np.zeros_like(s.x), s.b, 2, 1, 0.0)
    assert it == 2  # one iteration, tolerance not reached: niter_in + 1
    x1 = x[s.NB + 1:]
    cos = float(x1 @ z0) / (np.linalg.norm(x1) * np.linalg.norm(z0))
    assert cos > 1.0 - 1e-12


def test_one_cell_system():
    """N = 1: D = a11 and x = b / a11 after one iteration."""
    A = np.array([4.0, 0.0])
    Acol, Arow, Adia = np.array([1, 2]), np.array([1, 0]), np.array([1])
    b = np.array([3.0])
    x, r, it, ini, fin = oracle.solve("cg", 1, 0, 2, A, Acol, Arow, Adia, np.zeros(1),
                                      np.zeros(1 + 1), b, 1, 10, 1e-12)
    assert it == 1 and x[1] == 0.75 and r[0] == 0.0
    assert ini == 3.0 and fin == 0.0
