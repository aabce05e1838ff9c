"""GPU momentum assembly (Process/NewUVW.f90:138-499 with ConvScheme.f90 and
CalMinMax.f90) against the golden fixtures made from the reference's source
text and against the C oracle on larger boxes: Aval, b, Abou and Asave are
the reference's operations in the reference's order, bit for bit.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MOM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "momentum_*.npz")))
pytestmark = pytest.mark.gpu

CELL = oracle.MOMENTUM_CELL_FIELDS
FACE = oracle.MOMENTUM_FACE_FIELDS
# oracle field names -> tflows_newuvw_fields names
RENAME = {"ui_source": "source"}


def _same(a, b):
    a, b = np.ascontiguousarray(a, np.float64), np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def _run_gpu(d, scoef=True, abou_fill=5.0):
    import torch
    asm = tflows.Assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], d["SideC"], d["SidAij"],
                          d["Adia"], d["TypeBC"], {k: d[k] for k in tflows.Assembly.GEOM},
                          d["volume"])

    def f64(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()

    def i32(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()

    fields = {RENAME.get(k, k): f64(d[k]) for k in CELL + FACE}
    if not scoef:
        del fields["scoef"]
    fields.update(material=i32(d["material"]), blend=i32(d["blend"]),
                  blend_tem=i32(d["blend_tem"]), urfc=f64(d["urfc"]))
    aval = torch.full((d["NONZ"],), 7.0, dtype=torch.float64, device="cuda")
    b = torch.full((d["NC"],), 7.0, dtype=torch.float64, device="cuda")
    abou = torch.full((max(d["NbC"], 1),), abou_fill, dtype=torch.float64, device="cuda")
    asave = torch.zeros(d["NC"], dtype=torch.float64, device="cuda")
    rhoui = torch.zeros(d["NbC"] + d["NC"] + 1, dtype=torch.float64, device="cuda")
    try:
        asm.newuvw(int(d["var"]), fields, aval, b, abou, asave, rhoui, nmat=int(d["Nmat"]),
                   visc=float(d["visc"]), dt=float(d["dt"]), urf=float(d["urf"]),
                   convec=int(d["convec"]), cross=int(d["cross"]), diffus=int(d["diffus"]),
                   inert=int(d["inert"]), moin_problem=int(d["moin_problem"]))
    finally:
        asm.close()
    return (aval.cpu().numpy(), b.cpu().numpy(), abou.cpu().numpy()[:d["NbC"]],
            asave.cpu().numpy(), rhoui.cpu().numpy())


def _oracle(d):
    geom = {k: d[k] for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "volume")}
    fields = {k: d[k] for k in CELL + FACE}
    return oracle.momentum_assembly(
        d["NC"], d["NbC"], d["NS"], d["NONZ"], d["SideC"], d["SidAij"], d["Adia"], d["TypeBC"],
        d["material"], geom, fields, int(d["Nmat"]), int(d["var"]), d["blend"], d["blend_tem"],
        d["urfc"], float(d["visc"]), float(d["dt"]), float(d["urf"]), int(d["convec"]),
        int(d["cross"]), int(d["diffus"]), int(d["inert"]), int(d["moin_problem"]))


def _load(path):
    g = np.load(path)
    d = {k: g[k] for k in g.files}
    for k in ("NC", "NbC", "NS", "NONZ"):
        d[k] = int(d[k])
    return d


@pytest.mark.parametrize("path", MOM_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_momentum_matches_reference_fixtures(path):
    d = _load(path)
    aval, b, abou, asave, rhoui = _run_gpu(d)
    assert _same(aval, d["Aval"]), "Aval"
    assert _same(b, d["b"]), "b"
    assert _same(abou, d["Abou"]), "Abou"
    if int(d["var"]) == 1:
        assert _same(asave, d["Asave"]), "Asave"
    assert _same(rhoui, d["rho_n"] * d["ui_n"])


def test_momentum_default_scoef_is_calc3s():
    """Scoef left out: the mesh's |S|^2/(S.d), formed as Calc3.f90:22-47 forms
    it, gives the same bits."""
    d = _load(MOM_CASES[0])
    got = _run_gpu(d, scoef=False)
    assert _same(got[0], d["Aval"]) and _same(got[1], d["b"])


def _box_case(shape, seed, nmat, blend, blend_tem, var, **kw):
    """A perturbed box with the fixture generator's seeded fields."""
    import sys
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    from make_golden_momentum import make_inputs
    msh = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    d = dict(msh)
    d["NONZ"] = int(msh["Acol"][-1])
    d.update(make_inputs(msh, seed, nmat, blend, blend_tem, var, **kw))
    return d


C = oracle.SCHEME


@pytest.mark.parametrize("shape,nmat,blend,blend_tem,var,kw", [
    ((40, 33, 29), 1, [C["smart"]], [C["yes"]], 1, {}),
    ((24, 20, 18), 2, [C["gamma"], C["quick"]], [C["cds"], C["no"]], 2,
     {"inert": C["par"], "moin_problem": 4}),
    ((17, 31, 9), 2, [C["no"], C["superbee"]], [C["no"], C["no"]], 3, {"diffus": C["cn"]}),
])
def test_momentum_matches_oracle_on_larger_boxes(shape, nmat, blend, blend_tem, var, kw):
    d = _box_case(shape, 7, nmat, blend, blend_tem, var, **kw)
    aval, b, abou, asave, rhoui, st = _oracle(d)
    assert st == 0
    got = _run_gpu(d)
    for name, x, y in (("Aval", got[0], aval), ("b", got[1], b), ("Abou", got[2], abou),
                       ("rhoUi", got[4], rhoui)):
        assert _same(x, y), name
    if var == 1:
        assert _same(got[3], asave)


def test_momentum_two_faces_between_the_same_cells():
    """A mesh with two faces joining the same pair of cells: TopolM gives both
    faces the same off-diagonal positions and the reference adds both into
    them in face order; the GPU does too."""
    d = _box_case((6, 5, 4), 3, 1, [C["minmod"]], [C["yes"]], 1)
    sc = d["SideC"]
    inner = np.nonzero(sc[:, 2] > 0)[0]
    dup = int(inner[len(inner) // 2])
    order = np.r_[np.arange(dup + 1), dup, np.arange(dup + 1, d["NS"])]
    for k in ("SideC", "Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "flux_u", "flux", "ff",
              "scoef"):
        d[k] = np.ascontiguousarray(d[k][order])
    d["NS"] += 1
    Acol, Arow, Adia, sid = oracle.topolm(d["NC"], d["SideC"][:, 1:])
    d.update(Acol=Acol, Arow=Arow, Adia=Adia, SidAij=sid, NONZ=int(Acol[-1]))
    assert sid[dup, 0] == sid[dup + 1, 0] and sid[dup, 1] == sid[dup + 1, 1]
    aval, b, abou, asave, rhoui, st = _oracle(d)
    assert st == 0
    got = _run_gpu(d)
    assert _same(got[0], aval) and _same(got[1], b) and _same(got[2], abou)


def test_momentum_rejects_undefined_blending_and_bad_materials():
    d = _load(os.path.join(GOLDEN, "momentum_box444_smart_minmod_nmat2.npz"))
    d["blend"] = np.array([C["yes"], C["no"]], np.int32)
    with pytest.raises(tflows.SolverError) as e:
        _run_gpu(d)
    assert e.value.status == tflows.BAD_INPUT and "YES" in str(e.value)
    d = _load(os.path.join(GOLDEN, "momentum_box444_smart_minmod_nmat2.npz"))
    d["material"] = d["material"].copy()
    d["material"][d["NbC"] + 5] = 9
    with pytest.raises(tflows.SolverError) as e:
        _run_gpu(d)
    assert e.value.status == tflows.BAD_INPUT
    # the assembly object stays usable after a rejected call
    d = _load(os.path.join(GOLDEN, "momentum_box444_smart_minmod_nmat2.npz"))
    assert _same(_run_gpu(d)[0], d["Aval"])


def test_assembled_momentum_system_solves():
    """The GPU-assembled momentum system goes to the GPU BiCG as NewUVW hands
    it over (x = rhoUi, warm start; prec 1) and matches the oracle's BiCG on
    the oracle-assembled system."""
    import torch
    d = _box_case((22, 18, 14), 5, 1, [C["smart"]], [C["yes"]], 1)
    aval, b, abou, asave, rhoui, st = _oracle(d)
    assert st == 0
    got = _run_gpu(d)
    assert _same(got[0], aval) and _same(got[1], b)
    NC, NbC = d["NC"], d["NbC"]
    tol = 1e-10 * float(np.linalg.norm(b))
    xo, ro, ito, _, _ = oracle.solve("bicg", NC, NbC, d["NONZ"], aval, d["Acol"], d["Arow"],
                                     d["Adia"], abou if NbC else np.zeros(1), rhoui.copy(),
                                     b.copy(), 1, 200, tol)
    assert ito <= 200
    rp, col = d["Acol"] - 1, d["Arow"][:-1] - 1
    topo = tflows.Topology(NC, rp, col, d["Adia"] - 1)
    x = torch.from_numpy(got[4][NbC + 1:].copy()).cuda()
    res = topo.solve(torch.from_numpy(got[0][:-1].copy()).cuda(),
                     torch.from_numpy(got[1].copy()).cuda(), x, "bicg", 1, 200, tol)
    topo.close()
    assert res["status"] == tflows.OK, res
    assert abs(res["iterations"] - ito) <= 1
    xg = x.cpu().numpy()
    assert np.abs(xg - xo[NbC + 1:]).max() <= 1e-8 * np.abs(xo[NbC + 1:]).max()
