"""Golden fixtures of the momentum assembly, from the reference's own source
text.

Extracts Process/NewUVW.f90 lines 167-176 (the CalMinMax call when a material
blends, the zeroing of the convective and cross-diffusive sums) and 200-499
(the convection face loop, the diffusion face loop that fills Aval through
Adia/SidAij, b and Abou, the cross-diffusion, inertial, pressure and
under-relaxation terms), together with the whole of Process/ConvScheme.f90
and Process/CalMinMax.f90 of a T-FlowS checkout (the path given as the
first argument or in TFLOWS_REFERENCE).  Mechanical rewrites only: derived-type
components such as ``Ui % C`` become plain names, the `select case
(Moin_Problem())` inside the diffusion loop becomes an if/else on the same
value, and each statement on the array section ``(1:NC)`` becomes the
element loop it denotes.  The source term lines 177-199 are left out: they
call the test-problem functions of Moin_Problem_Mod, so `Ui % source` is an
input here.  The lines are translated with fortran_subset.py and run on small
perturbed boxes whose boundary cells carry every boundary type of
Library/allp_mod.f90, for every convection scheme of Process/IniPar.f90 and
each time-discretisation option, and on a box with one face repeated (two
faces joining the same cells).  Writes momentum_*.npz: the inputs and
Aval, b, Abou, Asave.

Run:  python tests/golden/make_golden_momentum.py [/path/to/T-FlowS]
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
from make_golden_assembly import F2, duplicate_face  # noqa: E402

# Library/allp_mod.f90:16-24 and Process/IniPar.f90:22-49
BC = {"inflow": 1, "wall": 2, "outflow": 3, "symmetry": 4, "convect": 5, "wallfl": 6,
      "buffer": 11, "pressure": 12, "periodic": 13}
CODES = {"ab": 1, "cn": 2, "fi": 3, "lin": 4, "par": 5, "yes": 10, "no": 11, "cds": 20,
         "quick": 21, "luds": 22, "minmod": 23, "smart": 24, "avl_smart": 25, "superbee": 26,
         "gamma": 27}
CELL_FIELDS = ("rho_n", "rho_o", "rho_oo", "ui_n", "ui_o", "ui_oo", "duidi", "duidj", "duidk",
               "dujdi", "dukdi", "dujdj", "dukdk", "pi", "ui_source")
FACE_FIELDS = ("flux_u", "flux", "ff", "scoef")
# Processor.f90:314-340: the face vectors each momentum component is given
FACE_VECTORS = {1: ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz"),
                2: ("Sy", "Sx", "Sz", "Dy", "Dx", "Dz"),
                3: ("Sz", "Sx", "Sy", "Dz", "Dx", "Dy")}


def _logical(text):
    """Fortran logical lines (comments dropped, continuations joined)."""
    out, buf = [], ""
    for raw in text.splitlines():
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        if line.endswith("&"):
            buf += line[:-1] + " "
            continue
        buf += line
        out.append(buf.strip())
        buf = ""
    return out


_SECTION = re.compile(r"\(\s*1\s*:\s*NC\s*\)", re.I)


def _expand_sections(lines):
    out = []
    for ln in lines:
        if not _SECTION.search(ln):
            out.append(ln)
            continue
        body = _SECTION.sub("(ii)", ln)
        m = re.match(r"if\s*\((.*?)\)\s*(\w+\s*\(.*)$", body, re.I)
        if m and "then" not in body.lower():
            out += [f"if ({m.group(1)}) then", "do ii = 1, NC", m.group(2), "end do", "end if"]
        else:
            out += ["do ii = 1, NC", body, "end do"]
    return out


def newuvw_text(root):
    lines = open(os.path.join(root, "Process", "NewUVW.f90")).read().splitlines()
    head = lines[166:176]   # NewUVW.f90:167-176
    body = lines[199:499]   # NewUVW.f90:200-499
    assert re.match(r"\s*do mat = 1, Nmat", head[0]), head[0]
    assert "Ui % X = 0.0" in head[-1], head[-1]
    assert body[-1].strip() == "Aval(Adia(1:NC)) = Aval(Adia(1:NC)) / U % URF", body[-1]
    logical = _logical("\n".join(head + body))
    # select case (Moin_Problem()) inside the diffusion loop -> if / else
    fixed, in_sel = [], False
    for ln in logical:
        low = ln.lower().replace(" ", "")
        if low == "selectcase(moin_problem())":
            in_sel = True
            continue
        if in_sel and low.startswith("case(4)"):
            fixed.append("if (moin_problem == 4) then")
            continue
        if in_sel and low == "casedefault":
            fixed.append("else")
            continue
        if in_sel and low == "endselect":
            fixed.append("end if")
            in_sel = False
            continue
        assert "select" not in low, ln
        fixed.append(ln)
    text = "\n".join(_expand_sections(fixed))
    text = re.sub(r"(\w+)\s*%\s*(\w+)", r"\1_\2", text)
    return ("subroutine newuvw_assembly()\n"
            "  integer :: c, c1, c2, s, mat, ii\n"
            "  real :: fex, fim, rhouis, a0, a12, a21, d12, d21, viseff, rhos\n"
            "  real :: duidis, duidjs, duidks, dujdis, dukdis, dujdjs, dukdks\n"
            + text + "\nend subroutine newuvw_assembly\n")


def run_reference(root, msh, inp):
    texts = [newuvw_text(root),
             open(os.path.join(root, "Process", "ConvScheme.f90")).read(),
             open(os.path.join(root, "Process", "CalMinMax.f90")).read()]
    arrays = ("sidec", "sidaij", "typebc", "material", "aval", "adia", "abou", "b", "asave",
              "volume", "blend", "blend_tem", "urfc", "rhoui", "ui_c", "ui_x", "phimax", "phimin",
              "f", "si", "sj", "sk", "di", "dj", "dk") + CELL_FIELDS + FACE_FIELDS
    names = {n: "array" for n in arrays}
    names.update({n: "scalar" for n in ("nmat", "ns", "nc", "nbc", "dt", "visc", "var", "u_urf",
                                        "convec", "cross", "diffus", "inert", "moin_problem")})
    params = {k: str(v) for k, v in {**BC, **CODES}.items()}
    subs, _ = load_subroutines(texts, names, params)
    NC, NbC, NS = msh["NC"], msh["NbC"], msh["NS"]
    NONZ = int(msh["Acol"][-1])
    ncell = NbC + NC + 1
    r = lambda a: [np.float64(v) for v in np.asarray(a, dtype=np.float64)]  # noqa: E731
    M = Module(nmat=inp["Nmat"], ns=NS, nc=NC, nbc=NbC, dt=np.float64(inp["dt"]),
               visc=np.float64(inp["visc"]), var=inp["var"], u_urf=np.float64(inp["urf"]),
               convec=inp["convec"], cross=inp["cross"], diffus=inp["diffus"],
               inert=inp["inert"], moin_problem=inp["moin_problem"])
    M.sidec = F2([[int(v) for v in row] for row in msh["SideC"]], 0, 1)
    M.sidaij = F2([[int(v) for v in row] for row in msh["SidAij"]], 1, 1)
    M.typebc = FArr([int(v) for v in inp["TypeBC"]], 0, -NbC)
    M.material = FArr([int(v) for v in inp["material"]], 0, -NbC)
    M.adia = FArr([int(v) for v in msh["Adia"]], 0, 1)
    M.blend = FArr([int(v) for v in inp["blend"]], 0, 1)
    M.blend_tem = FArr([int(v) for v in inp["blend_tem"]], 0, 1)
    M.urfc = FArr(r(inp["urfc"]), 0, 1)
    M.aval = FArr(r(np.zeros(NONZ)), 0, 1)                 # Aval(:) = 0.0   (:148)
    M.b = FArr(r(np.zeros(NC)), 0, 1)                      # b(:) = 0.0      (:149)
    M.abou = FArr(r(np.zeros(max(NbC, 1))), 0, -NbC)       # Abou(-NbC:-1) = 0.0 (:146)
    M.asave = FArr(r(np.zeros(ncell)), 0, -NbC)
    M.volume = FArr(r(inp["volume"]), 0, -NbC)
    M.f = FArr(r(msh["f"]), 0, 1)
    for k, src in zip(("si", "sj", "sk", "di", "dj", "dk"), FACE_VECTORS[inp["var"]]):
        setattr(M, k, FArr(r(msh[src]), 0, 1))
    for k in CELL_FIELDS:
        setattr(M, k, FArr(r(inp[k]), 0, -NbC))
    for k in FACE_FIELDS:
        setattr(M, k, FArr(r(inp[k]), 0, 1))
    # rhoUi = Rho % n * Ui % n (:138), the unknown the momentum solve updates
    M.rhoui = FArr(r(inp["rho_n"] * inp["ui_n"]), 0, -NbC)
    for k in ("ui_c", "ui_x", "phimax", "phimin"):
        setattr(M, k, FArr(r(np.zeros(ncell)), 0, -NbC))
    subs["newuvw_assembly"](M)
    arr = lambda a: np.array([float(v) for v in a.buf])  # noqa: E731
    return dict(Aval=arr(M.aval), b=arr(M.b), Abou=arr(M.abou)[:NbC],
                Asave=arr(M.asave)[NbC + 1:])


def make_inputs(msh, seed, nmat, blend, blend_tem, var, convec=3, cross=3, diffus=3, inert=4,
                moin_problem=0, flux_zero=0.05):
    NC, NbC, NS = msh["NC"], msh["NbC"], msh["NS"]
    rng = np.random.default_rng(seed + 2000)
    n = NbC + NC + 1
    inp = dict(Nmat=nmat, var=var, convec=convec, cross=cross, diffus=diffus, inert=inert,
               moin_problem=moin_problem, dt=0.01, visc=float(rng.uniform(1e-3, 1e-1)),
               urf=float(rng.uniform(0.5, 0.9)))
    vol = msh["volume"].copy()
    vol[:NbC] = rng.uniform(0.5, 1.5, NbC)
    inp["volume"] = vol
    for k in ("rho_n", "rho_o", "rho_oo"):
        inp[k] = rng.uniform(0.5, 1.5, n)
    for k in CELL_FIELDS[3:]:
        inp[k] = rng.uniform(-1.0, 1.0, n)
    for k in ("flux_u", "flux"):
        v = rng.uniform(-1.0, 1.0, NS)
        v[rng.random(NS) < flux_zero] = 0.0
        inp[k] = v
    ff = msh["f"].copy()
    pick = rng.random(NS)
    ff[pick < 0.1] = 1.0
    ff[(pick >= 0.1) & (pick < 0.2)] = 0.0
    inp["ff"] = ff
    # Scoef = |S|^2 / (S.d), Process/Calc3.f90:22-47
    S = (msh["Sx"] * msh["Sx"] + msh["Sy"] * msh["Sy"] + msh["Sz"] * msh["Sz"])
    inp["scoef"] = S / (msh["Dx"] * msh["Sx"] + msh["Dy"] * msh["Sy"] + msh["Dz"] * msh["Sz"])
    typebc = np.zeros(n, np.int32)
    codes = np.array(sorted(BC.values()), np.int32)
    typebc[:NbC] = codes[rng.integers(0, len(codes), NbC)]
    inp["TypeBC"] = typebc
    inp["material"] = rng.integers(1, nmat + 1, n).astype(np.int32)
    inp["material"][NbC] = 0  # cell 0 does not exist
    inp["blend"] = np.array(blend, np.int32)
    inp["blend_tem"] = np.array(blend_tem, np.int32)
    inp["urfc"] = rng.uniform(0.5, 1.0, nmat)
    return inp


def case(root, name, shape, seed, nmat, blend, blend_tem, var, dup=False, **kw):
    mesh = _mesh()
    msh = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    if dup:
        msh = duplicate_face(msh)
    inp = make_inputs(msh, seed, nmat, blend, blend_tem, var, **kw)
    res = run_reference(root, msh, inp)
    out = dict(NC=msh["NC"], NbC=msh["NbC"], NS=msh["NS"], NONZ=int(msh["Acol"][-1]),
               SideC=msh["SideC"], SidAij=msh["SidAij"], Adia=msh["Adia"], Acol=msh["Acol"],
               Arow=msh["Arow"])
    for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f"):
        out[k] = msh[k]
    out.update(inp)
    out.update(res)
    np.savez_compressed(os.path.join(HERE, f"momentum_{name}.npz"), **out)
    print(name, "faces", msh["NS"], "blend", blend, blend_tem,
          "types", np.bincount(inp["TypeBC"][:msh["NbC"]]).nonzero()[0].tolist())


def main():
    root = reference_root()
    C = CODES
    # no blending: central convection explicit, diffusion implicit
    case(root, "box533_no", (5, 3, 3), 3, 1, [C["no"]], [C["no"]], 1)
    # every scheme of ConvScheme, upwind sums on, three time levels on some
    for k, scheme in enumerate(("yes", "cds", "quick", "luds", "minmod", "smart", "avl_smart",
                                "superbee", "gamma")):
        case(root, f"box334_{scheme}", (3, 3, 4), 10 + k, 1, [C[scheme]], [C["yes"]],
             1 + k % 3, inert=C["par"] if k % 2 else C["lin"])
    # two materials with different schemes (max of the two codes on shared faces)
    case(root, "box444_smart_minmod_nmat2", (4, 4, 4), 4, 2, [C["smart"], C["minmod"]],
         [C["cds"], C["no"]], 2, moin_problem=4)
    # Crank-Nicolson diffusion flag, explicit terms off, no inertial term
    case(root, "box271_cn", (2, 7, 1), 5, 1, [C["quick"]], [C["no"]], 3, convec=C["ab"],
         cross=C["cn"], diffus=C["cn"], inert=C["ab"])
    # two faces joining the same two cells (one off-diagonal position each way)
    case(root, "box433_dupface_smart", (4, 3, 3), 6, 1, [C["smart"]], [C["yes"]], 1, dup=True)



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
