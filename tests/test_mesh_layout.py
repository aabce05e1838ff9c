"""The synthetic mesh builder produces exactly the layout TopolM builds.

Process/TopolM.f90:24-98 (restated in the oracle) turns a face list into
Acol/Arow/Adia/SidAij; the vectorised box builder must agree element for
element, and the assembled matrices must have the properties the reference's
assembly gives them.
"""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 1, 1), (1, 4, 1), (2, 3, 4), (5, 4, 3),
                                   (7, 6, 5)])
def test_box_csr_matches_topolm(shape):
    nx, ny, nz = shape
    sc, (Acol, Arow, Adia, sid) = mesh.side_c(nx, ny, nz)
    rA, rR, rD, rS = oracle.topolm(nx * ny * nz, sc)
    assert np.array_equal(Acol, rA)
    assert np.array_equal(Arow, rR)
    assert np.array_equal(Adia, rD)
    assert np.array_equal(sid, rS)
    assert Arow[-1] == 0 and Acol[-1] == Arow.shape[0]


def test_nnz_formula():
    for n in (2, 5, 9):
        Acol, Arow, _, _ = mesh.box_csr(n, n, n)
        assert Acol[-1] - 1 == 7 * n**3 - 6 * n**2


def test_pressure_matrix_properties():
    s = mesh.pressure_system(6, 5, 4, perturb=0.2, seed=3, variable_density=True)
    A = s.scipy()
    assert abs(A - A.T).max() < 1e-14
    # rows sum to zero except the Dirichlet cell
    rs = np.asarray(A.sum(axis=1)).ravel()
    assert abs(rs[1:]).max() < 1e-12 and rs[0] > 0
    assert abs(s.b.mean()) < 1e-14
    w = np.linalg.eigvalsh(A.toarray())
    assert w.min() > 0


def test_convection_diffusion_flux_is_divergence_free():
    s = mesh.convection_diffusion_system(6, 5, 4, perturb=0.2, seed=2, nu=0.0, dt=1e30)
    A = s.scipy()
    # With nu = 0 and no time term the column sums of an upwind operator of a
    # divergence-free flux vanish (every outflow is someone's inflow).
    cs = np.asarray(A.sum(axis=0)).ravel()
    assert abs(cs).max() < 1e-10
    assert abs(A).max() > 0.1


def test_config_shapes():
    s = mesh.config_system(1, scale=8)
    assert s.N == 512 and s.nnz == 7 * 512 - 6 * 64 and s.NB == 6 * 64
    assert s.x.shape == (s.NB + s.N + 1,)
    shapes = mesh.batch_sizes()
    assert len(shapes) == 48
    Ns = [a * b * c for a, b, c in shapes]
    assert min(Ns) >= 16**3 * 0.8 and max(Ns) <= 160**3 * 1.2
