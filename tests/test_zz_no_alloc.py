"""The allocation-free CG entry point (tflows_cg_noalloc) against the
regular device entry point (tflows_solve_device), through the C ABI.

Callers that may not allocate GPU memory while they run use this entry
point; its work vectors live in a static device array shared by all calls,
so two calls in a row must both reproduce the regular solver.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

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
