"""Golden fixtures of the matrix layout, from the reference's own source text.

Extracts the body of Process/TopolM.f90 (stencil widths from SideC, the row
pointers Acol, the columns Arow sorted per row, the diagonal positions Adia
and the face positions SidAij) of a T-FlowS checkout (default
the path given as the first argument or in TFLOWS_REFERENCE) and executes it
statement by statement with fortran_subset.py.  Mechanical rewrites only:
the allocations, the progress messages and the deallocation are dropped
(the arrays are provided here, zeroed), and the call to the library sort
ISort (Library/ISort.f90, a quicksort) becomes an exchange sort of the same
stretch of Arow written in the translated subset -- sorting integers has a
single result, whatever the algorithm.  Runs on boxes and on boxes with a
repeated face (two faces joining the same cells).  Writes topolm_*.npz:
SideC and Acol, Arow, Adia, SidAij, NONZERO.

Run:  python tests/golden/make_golden_topolm.py [/path/to/T-FlowS]
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from fortran_subset import FArr, Module, load_subroutines  # noqa: E402
from make_golden import _mesh  # noqa: E402

SORT = """do i1 = Acol(c), Acol(c) + stencw(c) - 2
  do i2 = Acol(c), Acol(c) + stencw(c) - 2
    if (Arow(i2) > Arow(i2+1)) then
      kk = Arow(i2)
      Arow(i2) = Arow(i2+1)
      Arow(i2+1) = kk
    end if
  end do
end do"""


class F2W:
    """A writable two-dimensional Fortran array (column-major, lower bounds
    lo1, lo2), stored as a list of columns."""

    def __init__(self, cols, lo1, lo2):
        self.a, self.lo1, self.lo2 = cols, lo1, lo2

    def __getitem__(self, ij):
        i, j = ij
        return self.a[j - self.lo2][i - self.lo1]

    def __setitem__(self, ij, v):
        i, j = ij
        self.a[j - self.lo2][i - self.lo1] = v


def topolm_text(root):
    lines = open(os.path.join(root, "Process", "TopolM.f90")).read().splitlines()
    start = next(i for i, ln in enumerate(lines) if "allocate(stencw(NC))" in ln)
    end = next(i for i, ln in enumerate(lines) if "deallocate(stencw)" in ln)
    body = []
    for ln in lines[start:end]:
        low = ln.strip().lower()
        if low.startswith("allocate(stencw"):
            body.append("  stencw = 1")
            continue
        if low.startswith("allocate("):
            continue
        if re.match(r"if\s*\(\s*this\s*<\s*2\s*\)\s*write", low):
            continue
        body.append(ln)
    text = "\n".join(body)
    # the ISort call (two continuation lines) -> an exchange sort of the stretch
    text, n = re.subn(r"call\s+isort\s*\(\s*Arow\(Acol\(c\)\),\s*&\s*\n\s*Arow\(Acol\(c\)\),\s*"
                      r"stencw\(c\),\s*1\s*\)", SORT, text, flags=re.I)
    assert n == 1, "the ISort call of TopolM.f90 was not found"
    return ("subroutine topolm_layout()\n"
            "  integer :: c, s, j, n, c1, c2, i1, i2, kk\n"
            + text + "\nend subroutine topolm_layout\n")


def run_reference(root, NC, SideC):
    NS = SideC.shape[0]
    names = {n: "array" for n in ("sidec", "sidaij", "acol", "arow", "adia", "stencw")}
    names.update({n: "scalar" for n in ("nc", "ns", "nonzero")})
    subs, _ = load_subroutines([topolm_text(root)], names, {})
    M = Module(nc=NC, ns=NS, nonzero=0)
    M.sidec = F2W([[int(v) for v in row] for row in SideC], 0, 1)
    M.sidaij = F2W([[0, 0] for _ in range(NS)], 1, 1)
    M.acol = FArr([0] * (NC + 1), 0, 1)
    M.arow = FArr([0] * (NC + 2 * NS + 1), 0, 1)
    M.adia = FArr([0] * NC, 0, 1)
    M.stencw = FArr([0] * NC, 0, 1)
    subs["topolm_layout"](M)
    nonz = int(M.nonzero)
    return (np.array(M.acol.buf, np.int32), np.array(M.arow.buf[:nonz], np.int32),
            np.array(M.adia.buf, np.int32), np.array(M.sidaij.a, np.int32), nonz)


def case(root, name, shape, seed, dup=False):
    mesh = _mesh()
    msh = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    SideC = msh["SideC"]
    if dup:
        inner = np.nonzero(SideC[:, 2] > 0)[0]
        rng = np.random.default_rng(seed)
        picks = np.sort(rng.choice(inner, size=3, replace=False))
        order = np.arange(msh["NS"])
        for p in picks[::-1]:
            order = np.insert(order, int(np.nonzero(order == p)[0][0]) + 1, p)
        SideC = np.ascontiguousarray(SideC[order])
    Acol, Arow, Adia, SidAij, nonz = run_reference(root, msh["NC"], SideC)
    np.savez_compressed(os.path.join(HERE, f"topolm_{name}.npz"), NC=msh["NC"], SideC=SideC,
                        Acol=Acol, Arow=Arow, Adia=Adia, SidAij=SidAij, NONZERO=nonz)
    print(name, "NC", msh["NC"], "NS", SideC.shape[0], "NONZERO", nonz)


def main():
    root = reference_root()
    case(root, "box543", (5, 4, 3), 1)
    case(root, "box271", (2, 7, 1), 2)
    case(root, "box443_dupfaces", (4, 4, 3), 3, dup=True)



def reference_root():
    """The T-FlowS checkout to read: the first argument, else the
    TFLOWS_REFERENCE environment variable; one of them is required."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TFLOWS_REFERENCE")
    if not root:
        sys.exit(f"usage: {os.path.basename(sys.argv[0])} PATH_TO_T-FLOWS_CHECKOUT "
                 "(or set TFLOWS_REFERENCE)")
    return root

if __name__ == "__main__":
    main()
