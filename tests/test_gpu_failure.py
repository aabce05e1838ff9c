"""Failure detection without faulting the GPU.

Every device-side wait is bounded.  The test hook `inject_stall` makes the
first block withhold its arrival at the first grid barrier, so the other
blocks' bounded waits run out: the solve must come back with TIMEOUT (and
the wait site), not hang, and the device must stay usable for the next
solve.  Host-side failures (bad input) are rejected before any launch.
"""
import numpy as np
import pytest

from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_withheld_barrier_arrival_times_out_cleanly(precision):
    s = mesh.pressure_system(24, 20, 16, perturb=0.2, seed=3)
    x, r = s.x.copy(), s.b.copy()
    bad = tflows.options(precision=precision, timeout_s=0.3, inject_stall=1)
    out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1,
                          500, s.tol, opts=bad, raise_on_error=False)
    assert out.status == tflows.TIMEOUT
    assert "timeout" in tflows.last_error()
    # the context is intact: the same solve without the hook succeeds
    x2, r2 = s.x.copy(), s.b.copy()
    ok = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia, s.Ab, x2, r2, 1,
                         500, s.tol, opts=tflows.options(precision=precision))
    assert ok.status == tflows.OK


def test_nonfinite_input_reports_nonfinite():
    s = mesh.pressure_system(8, 8, 8, seed=1)
    A = s.A.copy()
    A[10] = np.nan
    x, r = s.x.copy(), s.b.copy()
    out = tflows.solve_ex("cg", s.N, s.NB, s.NONZ, A, s.Acol, s.Arow, s.Adia, s.Ab, x, r, 1, 50,
                          s.tol, raise_on_error=False)
    assert out.status == tflows.NONFINITE and out.niter == 51
