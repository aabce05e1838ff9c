"""The C-ABI library loads, exports every declared entry point, and rejects
bad arguments on the host before touching a device (no compute here)."""
import ctypes

import numpy as np

from conftest import tflows

native = tflows._native


def test_library_builds_and_exports_header_symbols():
    L = tflows.load_library()
    declared = tflows.header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(native.SIGNATURES), "ctypes bindings out of sync with header"


def test_status_strings():
    for st in range(9):
        assert tflows.status_string(st)
    assert tflows.status_string(tflows.NO_DEVICE) == "no CUDA device"


def test_options_roundtrip():
    o = tflows.options(precision=tflows.MIXED, inner_rtol=1e-3)
    assert o.precision == 1 and abs(o.inner_rtol - 1e-3) < 1e-18
    d = tflows.options()
    assert d.precision == 0 and d.tol_mode == 0 and d.timeout_s > 0


def test_null_arguments_rejected_on_host():
    L = tflows.load_library()
    res = native.Result()
    st = L.tflows_solve_ex(0, None, None, None, None, None, None, None, None, None, None, None,
                           None, None, None, None, None, ctypes.byref(res))
    assert st == tflows.BAD_INPUT
    assert "null" in tflows.last_error()


def test_empty_system_follows_reference_exit():
    # N = 0: ||b|| = 0 < tol exits with iter = 0 before any device work.
    x = np.zeros(1)
    r = np.zeros(1)
    out = tflows.solve_ex("cg", 0, 0, 1, np.zeros(1), np.array([1]), np.zeros(1, np.int32),
                          np.zeros(0, np.int32), np.zeros(0), x, r, 1, 100, 1e-8)
    assert out.niter == 0 and out.status == tflows.OK
