"""Column patterns of the SELL-32 products: a topology whose rows repeat a
few offset tuples (column - row) stores one pattern id per row instead of a
column index per entry; the FP64 products and the standalone product read
them (the FP32 inner solves keep explicit columns).  The products see the
same columns in the same order, so every solver and the standalone product
must give bit-identical results with and without them
(TFLOWS_SELL_PATTERNS=0 switches them off for topologies created
afterwards); a pattern with too many distinct rows falls back to explicit
columns.
"""
import os

import numpy as np
import pytest

from conftest import tflows

mesh = tflows.mesh
pytestmark = pytest.mark.gpu


def _topology(s, patterns_on):
    old = os.environ.get("TFLOWS_SELL_PATTERNS")
    os.environ["TFLOWS_SELL_PATTERNS"] = "1" if patterns_on else "0"
    try:
        return tflows.Topology.from_system(s)
    finally:
        if old is None:
            del os.environ["TFLOWS_SELL_PATTERNS"]
        else:
            os.environ["TFLOWS_SELL_PATTERNS"] = old


def _solve(s, method, prec, opts, patterns_on, maxiter=5000):
    import torch
    topo = _topology(s, patterns_on)
    npat = topo.patterns
    val = torch.from_numpy(s.A[:-1].copy()).cuda()
    b = torch.from_numpy(s.b.copy()).cuda()
    x = torch.zeros(s.N, dtype=torch.float64, device="cuda")
    r = torch.zeros(s.N, dtype=torch.float64, device="cuda")
    res = topo.solve(val, b, x, method, prec, maxiter, 1e-10 * float(np.linalg.norm(s.b)),
                     r_out=r, opts=opts)
    topo.close()
    return npat, x.cpu().numpy(), r.cpu().numpy(), res


CASES = [
    ("cg", 1, "FP64"), ("cg", 2, "FP64"), ("bicg", 1, "FP64_FMA"), ("cgs", 1, "FP64_FMA"),
    ("bicg_true", 1, "FP64_FMA"), ("cg", 1, "MIXED"), ("cg", 2, "MIXED"), ("cgs", 1, "MIXED"),
]


@pytest.mark.parametrize("method,prec,precision", CASES)
def test_patterns_give_identical_results(method, prec, precision):
    if method in ("bicg", "cgs", "bicg_true"):
        s = mesh.convection_diffusion_system(20, 17, 13, perturb=0.2, seed=3)
    else:
        s = mesh.pressure_system(20, 17, 13, perturb=0.2, seed=3, variable_density=True)
    opts = tflows.options(precision=getattr(tflows, precision))
    n1, x1, r1, res1 = _solve(s, method, prec, opts, True)
    n0, x0, r0, res0 = _solve(s, method, prec, opts, False)
    # a box: 27 stencils (interior, faces, edges, corners) and the empty
    # pattern of the padding rows of the last slice
    assert 0 < n1 <= 28 and n0 == 0
    assert res1["status"] == tflows.OK and res0["status"] == tflows.OK
    assert res1["iterations"] == res0["iterations"]
    assert np.array_equal(x1.view(np.uint64), x0.view(np.uint64))
    assert np.array_equal(r1.view(np.uint64), r0.view(np.uint64))
    # a pattern id per row instead of 4 bytes per entry
    assert res1["bytes"] < res0["bytes"]


@pytest.mark.parametrize("fp32", [False, True])
def test_standalone_product_identical_with_patterns(fp32):
    import torch
    s = mesh.convection_diffusion_system(33, 19, 7, perturb=0.2, seed=4)
    val = torch.from_numpy(s.A[:-1].copy()).cuda()
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, s.N)).cuda()
    out = []
    for on in (True, False):
        topo = _topology(s, on)
        assert (topo.patterns > 0) == on
        y = torch.zeros(s.N, dtype=torch.float64, device="cuda")
        topo.spmv(val, x, y, repeat=1, fp32=fp32)
        topo.close()
        out.append(y.cpu().numpy())
    assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))


def test_many_patterns_fall_back_to_explicit_columns():
    """Rows with random neighbours (more than 255 distinct offset tuples):
    the topology keeps explicit column indices and still solves."""
    import torch
    rng = np.random.default_rng(5)
    n = 4000
    rows = []
    for i in range(n):
        nb = set(rng.choice(n, size=3, replace=False).tolist()) - {i}
        rows.append(sorted(nb | {i}))
    # symmetric pattern: add the transposes, then cap rows at 8 entries
    sym = [set(r) for r in rows]
    for i, r in enumerate(rows):
        for j in r:
            sym[j].add(i)
    rowptr, col, diag, val = [0], [], [], []
    for i in range(n):
        cols = sorted(c for c in sym[i] if c == i or len(sym[i]) <= 8)
        for c in cols:
            if c == i:
                diag.append(len(col))
            col.append(c)
            val.append(10.0 if c == i else -1.0)
        rowptr.append(len(col))
    # symmetric after the cap: keep an entry only where its transpose stayed
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            A[i, col[k]] = val[k]
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 10.0)
    rowptr, col, diag, val = [0], [], [], []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        for c in nz:
            if c == i:
                diag.append(len(col))
            col.append(int(c))
            val.append(A[i, c])
        rowptr.append(len(col))
    topo = tflows.Topology(n, np.array(rowptr, np.int32), np.array(col, np.int32),
                           np.array(diag, np.int32))
    assert topo.patterns == 0
    b = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    res = topo.solve(torch.tensor(val, dtype=torch.float64, device="cuda"), b, x, "cg", 1, 500,
                     1e-10 * float(b.norm()))
    topo.close()
    assert res["status"] == tflows.OK
    r = b.cpu().numpy() - A @ x.cpu().numpy()
    assert np.linalg.norm(r) < 2e-10 * float(b.norm())
