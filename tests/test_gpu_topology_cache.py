"""The legacy calls cache device copies of Acol/Arow/Adia keyed by the
arrays' addresses, sizes and a sampled content hash.  A caller that rewrites
the pattern in place calls tflows_forget_topologies; the next call must then
see the new pattern.  Prec1's IC(0) pivots (Prec1.f90:51-59) read D(Arow(j)),
so moving one lower-triangle column changes them."""
import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def test_forget_topologies_after_in_place_rewrite():
    nx, ny, nz = 24, 20, 18
    s = mesh.pressure_system(nx, ny, nz, perturb=0.2, seed=3, variable_density=True)
    Acol, Arow, Adia = s.Acol.copy(), s.Arow.copy(), s.Adia.copy()
    D0 = np.zeros(s.N)
    tflows.prec1(s.N, s.NONZ, s.A, Acol, Arow, Adia, D0, 2)
    assert np.array_equal(D0.view(np.uint64),
                          oracle.prec1(s.N, s.NONZ, s.A, Acol, Arow, Adia, 2).view(np.uint64))
    # move the (i, i - nx) entry of a middle row to column i - nx + 1: the
    # row's lower part stays ascending and below the diagonal
    i = nx * ny * (nz // 2) + nx * (ny // 2) + nx // 2  # 0-based interior row
    j = next(j for j in range(Acol[i] - 1, Adia[i] - 1) if Arow[j] - 1 == i - nx)
    Arow[j] += 1
    tflows.forget_topologies()
    D1 = np.zeros(s.N)
    tflows.prec1(s.N, s.NONZ, s.A, Acol, Arow, Adia, D1, 2)
    ref = oracle.prec1(s.N, s.NONZ, s.A, Acol, Arow, Adia, 2)
    assert not np.array_equal(ref, D0)
    assert np.array_equal(D1.view(np.uint64), ref.view(np.uint64))
