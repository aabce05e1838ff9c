"""The allocation-free CG entry point (tflows_cg_noalloc) against the
regular device entry point (tflows_solve_device) and against the oracle,
through the C ABI.

Callers that may not allocate GPU memory while they run use this entry
point; its work vectors live in a static device array shared by all calls,
so two calls in a row must both reproduce the regular solver, and a smaller
system after a larger one must not pick up the larger one's leftovers.  This
file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
REL = 1e-8


def _call(L, n, rp, col, dg, val, b, x, r, prec, maxiter, tol):
    import torch
    it = ctypes.c_int(-1)
    ini = ctypes.c_double(-1.0)
    fin = ctypes.c_double(-1.0)
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    st = L.tflows_cg_noalloc(n, p(rp), p(col), p(dg), p(val), p(b), p(x), p(r), prec, maxiter,
                             tol, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                             ctypes.byref(it), ctypes.byref(ini), ctypes.byref(fin))
    return st, it.value, ini.value, fin.value


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [1, 0])
def test_noalloc_matches_device_entry_point_twice(prec):
    import torch
    L = tflows.load_library()
    s = mesh.pressure_system(24, 20, 16, perturb=0.2, seed=9, variable_density=True)
    dev = torch.device("cuda")
    rp = torch.from_numpy((s.Acol - 1).astype(np.int32)).to(dev)
    col = torch.from_numpy((s.Arow[:-1] - 1).astype(np.int32)).to(dev)
    dg = torch.from_numpy((s.Adia - 1).astype(np.int32)).to(dev)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    tol = 1e-10 * float(np.linalg.norm(s.b))

    topo = tflows.Topology.from_system(s)
    x_ref = torch.zeros(s.N, dtype=torch.float64, device=dev)
    r_ref = torch.empty_like(x_ref)
    ref = topo.solve(val, b, x_ref, "cg", prec, 3000, tol, r_out=r_ref)
    assert ref["status"] == tflows.OK
    scale = float(x_ref.abs().max())

    for call in range(2):
        x = torch.zeros(s.N, dtype=torch.float64, device=dev)
        r = torch.empty_like(x)
        st, it, ini, fin = _call(L, s.N, rp, col, dg, val, b, x, r, prec, 3000, tol)
        assert st == tflows.OK, (call, st)
        assert abs(it - ref["iterations"]) <= 1, (call, it, ref["iterations"])
        assert float((x - x_ref).abs().max()) <= REL * scale, call
        assert abs(ini - ref["ini_res"]) <= 1e-12 * ref["ini_res"]
        assert fin < tol
        assert float((r - r_ref).abs().max()) <= 1e-9 * ref["ini_res"]


def _device_csr(s, dev):
    import torch
    rp = torch.from_numpy((s.Acol - 1).astype(np.int32)).to(dev)
    col = torch.from_numpy((s.Arow[:-1] - 1).astype(np.int32)).to(dev)
    dg = torch.from_numpy((s.Adia - 1).astype(np.int32)).to(dev)
    val = torch.from_numpy(s.A[:-1].copy()).to(dev)
    b = torch.from_numpy(s.b.copy()).to(dev)
    return rp, col, dg, val, b


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [1, 0])
def test_noalloc_matches_oracle(prec):
    """Both calls in a row against the CPU restatement of Process/CG.f90:
    relative solution difference <= 1e-8, iteration counts within 1 % (at
    least 1): the device sums its dot products in a fixed tree, the oracle
    left to right, and without a preconditioner that rounding difference
    shifts the stopping iteration of this variable-density system by a few."""
    import torch
    L = tflows.load_library()
    oracle.build()
    s = mesh.pressure_system(24, 20, 16, perturb=0.2, seed=9, variable_density=True)
    dev = torch.device("cuda")
    rp, col, dg, val, b = _device_csr(s, dev)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    xo, ro, ito, inio, _ = oracle.solve("cg", s.N, s.NB, s.NONZ, s.A, s.Acol, s.Arow, s.Adia,
                                        s.Ab, s.x, s.b, prec, 3000, tol)
    xo = xo[s.NB + 1:]
    scale = float(np.abs(xo).max())
    for call in range(2):
        x = torch.zeros(s.N, dtype=torch.float64, device=dev)
        r = torch.empty_like(x)
        st, it, ini, fin = _call(L, s.N, rp, col, dg, val, b, x, r, prec, 3000, tol)
        assert st == tflows.OK, (call, st)
        assert abs(it - ito) <= max(1, ito // 100), (call, it, ito)
        assert float(np.abs(x.cpu().numpy() - xo).max()) <= REL * scale, call
        assert abs(ini - inio) <= 1e-12 * inio, (call, ini, inio)
        assert fin < tol


@pytest.mark.gpu
def test_noalloc_internal_residual_and_smaller_system_after_larger():
    """r_out = NULL (the residual lives in the static array) on a large
    system, then a smaller system with r_out = NULL: each matches
    tflows_solve_device, so nothing of the earlier call leaks into the next."""
    import torch
    L = tflows.load_library()
    dev = torch.device("cuda")
    for (nx, ny, nz, seed) in ((40, 36, 30, 3), (12, 10, 9, 4)):
        s = mesh.pressure_system(nx, ny, nz, perturb=0.2, seed=seed, variable_density=True)
        rp, col, dg, val, b = _device_csr(s, dev)
        tol = 1e-10 * float(np.linalg.norm(s.b))
        topo = tflows.Topology.from_system(s)
        x_ref = torch.zeros(s.N, dtype=torch.float64, device=dev)
        ref = topo.solve(val, b, x_ref, "cg", 1, 5000, tol)
        topo.close()
        assert ref["status"] == tflows.OK
        x = torch.zeros(s.N, dtype=torch.float64, device=dev)
        st, it, ini, fin = _call(L, s.N, rp, col, dg, val, b, x, None, 1, 5000, tol)
        assert st == tflows.OK, (nx, st)
        assert abs(it - ref["iterations"]) <= 1, (nx, it, ref["iterations"])
        assert float((x - x_ref).abs().max()) <= REL * float(x_ref.abs().max()), nx
        assert fin < tol


@pytest.mark.gpu
def test_noalloc_rejects_bad_indices():
    """A column index outside [0, n), a diagonal position outside its row and
    a decreasing row pointer are each rejected on the device with BAD_INPUT,
    leaving x untouched; a correct call right after still solves."""
    import torch
    L = tflows.load_library()
    s = mesh.pressure_system(8, 7, 6, perturb=0.2, seed=5, variable_density=True)
    dev = torch.device("cuda")
    rp, col, dg, val, b = _device_csr(s, dev)
    tol = 1e-10 * float(np.linalg.norm(s.b))
    bad_col = col.clone()
    bad_col[17] = s.N
    bad_dg = dg.clone()
    bad_dg[5] = int(rp[6])
    bad_rp = rp.clone()
    bad_rp[3] = bad_rp[4] + 1
    for args in ((rp, bad_col, dg), (rp, col, bad_dg), (bad_rp, col, dg)):
        x = torch.full((s.N,), 7.0, dtype=torch.float64, device=dev)
        st, *_ = _call(L, s.N, *args, val, b, x, None, 1, 100, tol)
        assert st == tflows.BAD_INPUT
        assert bool((x == 7.0).all())
    x = torch.zeros(s.N, dtype=torch.float64, device=dev)
    st, _, _, fin = _call(L, s.N, rp, col, dg, val, b, x, None, 1, 1000, tol)
    assert st == tflows.OK and fin < tol


@pytest.mark.gpu
def test_noalloc_rejects_oversized_system():
    import torch
    L = tflows.load_library()
    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    i = torch.zeros(4, dtype=torch.int32, device="cuda")
    st, *_ = _call(L, 262145, i, i, i, t, t, t, None, 1, 10, 1e-8)
    assert st == tflows.BAD_INPUT
    st, *_ = _call(L, 4, i, i, i, t, t, t, None, 2, 10, 1e-8)
    assert st == tflows.UNSUPPORTED
