"""Golden fixtures of the pressure-correction assembly, from the reference's
own source text.

Extracts Process/CalcPS.f90 lines 69-202 of a T-FlowS checkout (default
the path given as the first argument or in TFLOWS_REFERENCE) -- the face loop
that fills Aval through SidAij/Adia, Abou, the face fluxes and b, the errmax
loop, the density-derivative source and the removal of the volume-weighted
mean of b -- wraps them in a subroutine, translates it with
fortran_subset.py (derived-type components such as ``Rho % n`` become plain
names) and runs it on small perturbed boxes whose boundary cells carry every
boundary type of Library/allp_mod.f90, with Nmat = 1 and 2, and on a box with
one face repeated (two faces joining the same cells).  Writes
assembly_*.npz: the inputs and Aval, b, Abou, Flux, errmax.

Run:  python tests/golden/make_golden_assembly.py [/path/to/T-FlowS]
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

# Library/allp_mod.f90:16-24
BC = {"inflow": 1, "wall": 2, "outflow": 3, "symmetry": 4, "convect": 5, "wallfl": 6,
      "buffer": 11, "pressure": 12}
CELL_FIELDS = ("volume", "asave", "rho_n", "rho_o", "rho_oo", "u_n", "v_n", "w_n", "p_n", "px",
               "py", "pz")
FACE_GEOM = ("sx", "sy", "sz", "dx", "dy", "dz", "f")


class F2:
    """A two-dimensional Fortran array (column-major, lower bounds lo1, lo2)."""

    def __init__(self, a, lo1, lo2):
        self.a, self.lo1, self.lo2 = a, lo1, lo2

    def __getitem__(self, ij):
        i, j = ij
        return self.a[j - self.lo2][i - self.lo1]


def calcps_text(root):
    lines = open(os.path.join(root, "Process", "CalcPS.f90")).read().splitlines()
    body = lines[68:202]  # CalcPS.f90:69-202
    assert re.match(r"\s*do m = 1, Nmat", body[0]), body[0]
    assert "bc_sum/vol" in body[-3] and body[-1].strip().lower() == "end do", body[-3:]
    text = "\n".join(body)
    text = re.sub(r"(\w+)\s*%\s*(\w+)", r"\1_\2", text)
    return ("subroutine calcps_assembly()\n"
            "  integer :: s, c, c1, c2, m\n"
            "  real :: urs, vrs, wrs, a12, smdpn, dpxi, dpyi, dpzi, bc_sum, vol\n"
            + text + "\nend subroutine calcps_assembly\n")


def run_reference(root, msh, fields, typebc, nmat, dt):
    names = {n: "array" for n in ("sidec", "sidaij", "typebc", "aval", "adia", "abou", "b",
                                  "flux") + CELL_FIELDS + FACE_GEOM}
    names.update({n: "scalar" for n in ("nmat", "ns", "nc", "dt", "errmax")})
    subs, _ = load_subroutines([calcps_text(root)], names,
                               {k: str(v) for k, v in BC.items()})
    NC, NbC, NS = msh["NC"], msh["NbC"], msh["NS"]
    NONZ = int(msh["Acol"][-1])
    r = lambda a: [np.float64(v) for v in np.asarray(a, dtype=np.float64)]  # noqa: E731
    M = Module(nmat=nmat, ns=NS, nc=NC, dt=np.float64(dt), errmax=np.float64(0.0))
    M.sidec = F2([[int(v) for v in row] for row in msh["SideC"]], 0, 1)
    M.sidaij = F2([[int(v) for v in row] for row in msh["SidAij"]], 1, 1)
    M.typebc = FArr([int(v) for v in typebc], 0, -NbC)
    M.adia = FArr([int(v) for v in msh["Adia"]], 0, 1)
    M.aval = FArr(r(np.zeros(NONZ)), 0, 1)
    M.b = FArr(r(np.zeros(NC)), 0, 1)
    M.abou = FArr(r(np.zeros(max(NbC, 1))), 0, -NbC)
    M.flux = FArr(r(np.zeros(NS)), 0, 1)
    for k in FACE_GEOM:
        setattr(M, k, FArr(r(msh[k if k == "f" else k[0].upper() + k[1]]), 0, 1))
    for k in CELL_FIELDS:
        setattr(M, k, FArr(r(fields[k]), 0, -NbC))
    subs["calcps_assembly"](M)
    arr = lambda a: np.array([float(v) for v in a.buf])  # noqa: E731
    return arr(M.aval), arr(M.b), arr(M.abou)[:NbC], arr(M.flux), float(M.errmax)


def duplicate_face(msh, frac=0.5):
    """The box with one interior face repeated right after itself (two faces
    joining the same two cells, as a split face of a polyhedral mesh gives),
    the second one with a 1.5 times larger Sx so that face order shows.  The
    layout is rebuilt as Process/TopolM.f90 builds it (the C restatement in
    oracle/): the pair's row holds the neighbour twice and both faces get the
    last of its positions."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import oracle
    inner = np.nonzero(msh["SideC"][:, 2] > 0)[0]
    dup = int(inner[int(len(inner) * frac)])
    order = np.r_[np.arange(dup + 1), dup, np.arange(dup + 1, msh["NS"])]
    out = dict(msh)
    for k in ("SideC", "Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f"):
        out[k] = np.ascontiguousarray(msh[k][order])
    out["Sx"][dup + 1] *= 1.5
    out["NS"] = msh["NS"] + 1
    Acol, Arow, Adia, sid = oracle.topolm(msh["NC"], out["SideC"][:, 1:])
    out.update(Acol=Acol, Arow=Arow, Adia=Adia, SidAij=sid)
    return out


def case(root, name, shape, seed, nmat, dup=False):
    mesh = _mesh()
    msh = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    if dup:
        msh = duplicate_face(msh)
    NC, NbC = msh["NC"], msh["NbC"]
    rng = np.random.default_rng(seed + 1000)
    n = NbC + NC + 1
    fields = {}
    fields["volume"] = msh["volume"].copy()
    fields["volume"][:NbC] = rng.uniform(0.5, 1.5, NbC)  # buffer cells carry a volume
    fields["asave"] = rng.uniform(1.0, 2.0, n)
    for k in ("rho_n", "rho_o", "rho_oo"):
        fields[k] = rng.uniform(0.5, 1.5, n)
    for k in ("u_n", "v_n", "w_n", "p_n", "px", "py", "pz"):
        fields[k] = rng.uniform(-1.0, 1.0, n)
    typebc = np.zeros(n, np.int32)
    codes = np.array(sorted(BC.values()), np.int32)
    typebc[:NbC] = codes[rng.integers(0, len(codes), NbC)]
    dt = 0.01
    aval, b, abou, flux, errmax = run_reference(root, msh, fields, typebc, nmat, dt)
    out = dict(NC=NC, NbC=NbC, NS=msh["NS"], NONZ=int(msh["Acol"][-1]), Nmat=nmat, dt=dt,
               SideC=msh["SideC"], SidAij=msh["SidAij"], Adia=msh["Adia"], Acol=msh["Acol"],
               Arow=msh["Arow"], TypeBC=typebc, Aval=aval, b=b, Abou=abou, Flux=flux,
               errmax=errmax)
    for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f"):
        out[k] = msh[k]
    rename = {"volume": "volume", "asave": "Asave", "rho_n": "rho_n", "rho_o": "rho_o",
              "rho_oo": "rho_oo", "u_n": "U", "v_n": "V", "w_n": "W", "p_n": "P", "px": "Px",
              "py": "Py", "pz": "Pz"}
    for k, v in rename.items():
        out[v] = fields[k]
    np.savez_compressed(os.path.join(HERE, f"assembly_{name}.npz"), **out)
    print(name, "faces", msh["NS"], "types", np.bincount(typebc[:NbC]).nonzero()[0].tolist())


def main():
    root = reference_root()
    case(root, "box533_nmat1", (5, 3, 3), 3, 1)
    case(root, "box444_nmat2", (4, 4, 4), 4, 2)
    case(root, "box271_nmat1", (2, 7, 1), 5, 1)
    case(root, "box433_dupface", (4, 3, 3), 6, 1, dup=True)



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
