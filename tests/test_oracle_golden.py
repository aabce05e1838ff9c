"""The oracle against golden vectors produced by the reference's own source.

The fixtures in tests/golden/ come from executing Process/{CG,BiCG,CGS,
Prec1,Resid}.f90 statement by statement (tests/golden/make_golden.py); the C
restatement in oracle/ must reproduce every output bit for bit, including
the module state carried between calls and the early-exit and
non-convergence conventions.  The assembly (CalcPS, NewUVW with ConvScheme
and CalMinMax) and layout (TopolM) fixtures come from the same kind of
execution of those files (make_golden_assembly.py, make_golden_momentum.py,
make_golden_topolm.py).
"""
import glob
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
SOLVER_CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if not os.path.basename(p).startswith(("prec1_resid", "assembly_",
                                                                 "momentum_", "topolm_")))
PR_CASES = sorted(glob.glob(os.path.join(GOLDEN, "prec1_resid_*.npz")))


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64) if a.dtype == np.float64
                                                 else a, b.view(np.uint64)
                                                 if b.dtype == np.float64 else b)


def test_fixture_inventory():
    assert len(SOLVER_CASES) >= 20 and len(PR_CASES) == 2


@pytest.mark.parametrize("path", SOLVER_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_reference_solver(path):
    g = np.load(path)
    oracle.reset_state()
    for c in range(int(g["ncalls"])):
        p = f"c{c}_"
        x, r, it, ini, fin = oracle.solve(
            str(g[p + "method"]), int(g["N"]), int(g["NB"]), int(g["NONZ"]), g["A"], g["Acol"],
            g["Arow"], g["Adia"], g["Ab"], g[p + "x_in"], g[p + "r1_in"], int(g[p + "prec"]),
            int(g[p + "niter_in"]), float(g[p + "tol"]), float(g[p + "IniRes_in"]),
            float(g[p + "FinRes_in"]))
        assert it == int(g[p + "niter_out"])
        assert _same(x, g[p + "x_out"]), "x differs"
        assert _same(r, g[p + "r1_out"]), "r1 differs"
        assert _same(np.float64(ini), g[p + "IniRes_out"])
        assert _same(np.float64(fin), g[p + "FinRes_out"])
        assert _same(np.float64(oracle.error_state()), g[p + "error_state"])


@pytest.mark.parametrize("path", PR_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_reference_prec1_resid(path):
    g = np.load(path)
    for prec in (0, 1, 2):
        D = oracle.prec1(int(g["N"]), int(g["NONZ"]), g["A"], g["Acol"], g["Arow"], g["Adia"],
                         prec)
        assert _same(D, g[f"D_prec{prec}"])
    r = oracle.resid(int(g["N"]), int(g["NB"]), int(g["NONZ"]), g["A"], g["Acol"], g["Arow"],
                     g["Ab"], g["resid_x"], g["resid_r1_in"])
    assert _same(r, g["resid_r1_out"])


def test_bicg_iterates_equal_cg_bitwise():
    """The reference's BiCG multiplies its shadow sequence by A (not A^T)
    and starts it at r1, so it reproduces CG's outputs exactly
    (Process/BiCG.f90:93-95,193-212)."""
    for path in SOLVER_CASES:
        g = np.load(path)
        if int(g["ncalls"]) != 1 or str(g["c0_method"]) not in ("cg", "bicg"):
            continue
        args = (int(g["N"]), int(g["NB"]), int(g["NONZ"]), g["A"], g["Acol"], g["Arow"],
                g["Adia"], g["Ab"], g["c0_x_in"], g["c0_r1_in"], int(g["c0_prec"]),
                int(g["c0_niter_in"]), float(g["c0_tol"]))
        a = oracle.solve("cg", *args)
        b = oracle.solve("bicg", *args)
        assert a[2] == b[2]
        assert _same(a[0], b[0]) and _same(a[1], b[1])


ASM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "assembly_*.npz")))


@pytest.mark.parametrize("path", ASM_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_assembly_oracle_bitwise(path):
    """The C restatement of Process/CalcPS.f90:49-202 reproduces the
    reference source text's Aval, b, Abou, Flux and errmax bit for bit."""
    g = np.load(path)
    geom = {k: g[k] for k in oracle.FACE_GEOM}
    fields = {k: g[k] for k in oracle.CELL_FIELDS}
    aval, b, abou, flux, errmax = oracle.calcps_assembly(
        int(g["NC"]), int(g["NbC"]), int(g["NS"]), int(g["NONZ"]), int(g["Nmat"]),
        float(g["dt"]), g["SideC"], g["SidAij"], g["Adia"], g["TypeBC"], geom, fields)
    for name, mine in (("Aval", aval), ("b", b), ("Abou", abou), ("Flux", flux)):
        assert np.array_equal(mine.view(np.uint64), g[name].view(np.uint64)), name
    assert errmax == float(g["errmax"])


MOM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "momentum_*.npz")))


def momentum_oracle_case(g, **over):
    """Run the momentum oracle on the inputs of fixture ``g``."""
    geom = {k: g[k] for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "volume")}
    fields = {k: g[k] for k in oracle.MOMENTUM_CELL_FIELDS + oracle.MOMENTUM_FACE_FIELDS}
    kw = dict(Nmat=int(g["Nmat"]), var=int(g["var"]), blend=g["blend"],
              blend_tem=g["blend_tem"], urfc=g["urfc"], visc=float(g["visc"]),
              dt=float(g["dt"]), urf=float(g["urf"]), convec=int(g["convec"]),
              cross=int(g["cross"]), diffus=int(g["diffus"]), inert=int(g["inert"]),
              moin_problem=int(g["moin_problem"]))
    kw.update(over)
    material = kw.pop("material", g["material"])
    return oracle.momentum_assembly(int(g["NC"]), int(g["NbC"]), int(g["NS"]), int(g["NONZ"]),
                                    g["SideC"], g["SidAij"], g["Adia"], g["TypeBC"], material,
                                    geom, fields, **kw)


def test_momentum_fixture_inventory():
    names = {os.path.basename(p)[9:-4] for p in MOM_CASES}
    # every convection scheme of Process/IniPar.f90:42-49, no blending, YES
    for scheme in ("no", "yes", "cds", "quick", "luds", "minmod", "smart", "avl_smart",
                   "superbee", "gamma"):
        assert any(n.endswith("_" + scheme) or ("_" + scheme + "_") in n for n in names), scheme


@pytest.mark.parametrize("path", MOM_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_momentum_oracle_bitwise(path):
    """The C restatement of Process/NewUVW.f90:138-499, ConvScheme.f90 and
    CalMinMax.f90 reproduces the reference source text's Aval, b, Abou and
    Asave bit for bit."""
    g = np.load(path)
    aval, b, abou, asave, rhoui, st = momentum_oracle_case(g)
    assert st == 0
    for name, mine in (("Aval", aval), ("b", b), ("Abou", abou), ("Asave", asave)):
        assert np.array_equal(mine.view(np.uint64), g[name].view(np.uint64)), name
    assert np.array_equal(rhoui, g["rho_n"] * g["ui_n"])


def test_momentum_oracle_rejects_undefined_blending_and_materials():
    """A face between a material that blends with YES and one with NO hands
    ConvScheme the code NO, for which the reference reads an unset local;
    the restatement reports it instead of guessing.  Material indices
    outside 1..Nmat are reported too."""
    g = dict(np.load(os.path.join(GOLDEN, "momentum_box444_smart_minmod_nmat2.npz")))
    yes, no = oracle.SCHEME["yes"], oracle.SCHEME["no"]
    *_, st = momentum_oracle_case(g, blend=np.array([yes, no], np.int32))
    assert st == 1
    *_, st = momentum_oracle_case(g, blend=np.array([yes, yes], np.int32))
    assert st == 0
    mat = g["material"].copy()
    mat[int(g["NbC"]) + 3] = 3
    *_, st = momentum_oracle_case(g, material=mat)
    assert st == 2


TOPOLM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "topolm_*.npz")))


@pytest.mark.parametrize("path", TOPOLM_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_topolm_layouts_match_reference_source(path):
    """Process/TopolM.f90 executed from the reference source (its ISort call
    replaced by another sort of the same integers) gives Acol, Arow, Adia
    and SidAij; the oracle's restatement and the library's tflows_topolm
    (host code) reproduce them exactly -- including two faces joining the
    same cells, where the row holds the neighbour twice and both faces get
    its last position.  (The box mesh builder equals tflows_topolm on boxes,
    tests/test_mesh_files.py.)"""
    from conftest import tflows
    g = np.load(path)
    NC, SideC = int(g["NC"]), g["SideC"]
    oA, oR, oD, oS = oracle.topolm(NC, SideC[:, 1:])
    lA, lR, lD, lS = tflows.topolm(NC, SideC)
    for A, R, D, S in ((oA, oR, oD, oS), (lA, lR, lD, lS)):
        assert np.array_equal(A, g["Acol"]) and np.array_equal(R, g["Arow"])
        assert np.array_equal(D, g["Adia"])
        assert np.array_equal(np.asarray(S).reshape(-1, 2), g["SidAij"])
    assert int(g["NONZERO"]) == int(g["Acol"][-1])
