"""GPU pressure-correction assembly (Process/CalcPS.f90:49-202) against the
golden fixtures made from the reference's source text and against the C
oracle on larger boxes.

Aval, Abou, the face fluxes and errmax are sequences of the reference's
operations per face and per cell in the reference's order: bit for bit.  b
carries the removal of its volume-weighted mean, whose sum the GPU forms as
a tree reduction instead of the reference's left-to-right loop, so b - b_ref
is one constant (the two roundings of the mean) up to the rounding of each
cell's subtraction (an ulp of the larger of b and the mean).
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import tflows

mesh = tflows.mesh
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ASM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "assembly_*.npz")))
pytestmark = pytest.mark.gpu

FIELD_KEYS = {"rho_n": "rho_n", "rho_o": "rho_o", "rho_oo": "rho_oo", "u": "U", "v": "V",
              "w": "W", "p": "P", "px": "Px", "py": "Py", "pz": "Pz", "asave": "Asave"}


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _run_gpu(d, nmat, dt, abou_in=None):
    import torch
    asm = tflows.Assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], d["SideC"], d["SidAij"],
                          d["Adia"], d["TypeBC"], {k: d[k] for k in tflows.Assembly.GEOM},
                          d["volume"])
    fields = {k: _dev(d[v]) for k, v in FIELD_KEYS.items()}
    aval = torch.full((d["NONZ"],), 7.0, dtype=torch.float64, device="cuda")
    b = torch.full((d["NC"],), 7.0, dtype=torch.float64, device="cuda")
    abou = _dev(abou_in if abou_in is not None else np.zeros(max(d["NbC"], 1)))
    flux = torch.zeros(d["NS"], dtype=torch.float64, device="cuda")
    info = asm.calcps(fields, aval, b, abou, flux, Nmat=nmat, dt=dt)
    asm.close()
    return (aval.cpu().numpy(), b.cpu().numpy(), abou.cpu().numpy()[:d["NbC"]],
            flux.cpu().numpy(), info["errmax"])


def _check(got, ref):
    aval, b, abou, flux, em = got
    raval, rb, rabou, rflux, rem = ref
    for name, x, y in (("Aval", aval, raval), ("Abou", abou, rabou), ("Flux", flux, rflux)):
        assert np.array_equal(x.view(np.uint64), np.asarray(y).view(np.uint64)), name
    assert em == rem
    # b before the mean removal is bit-identical, so b - b_ref is one constant
    # (the difference of the two roundings of the mean) up to the rounding of
    # each subtraction
    diff = b - rb
    delta = float(np.median(diff))
    assert abs(delta) <= 1e-10 * np.abs(rb).max(), delta
    # (a cell whose b is much smaller than the mean loses the mean's ulps)
    assert np.all(np.abs(diff - delta) <= 4.5e-16 * (np.abs(rb) + np.abs(rb).max()))


@pytest.mark.parametrize("path", ASM_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_assembly_matches_reference_fixtures(path):
    g = np.load(path)
    d = {k: g[k] for k in g.files}
    for k in ("NC", "NbC", "NS", "NONZ", "Nmat"):
        d[k] = int(d[k])
    got = _run_gpu(d, d["Nmat"], float(d["dt"]))
    ref = (g["Aval"], g["b"], g["Abou"], g["Flux"], float(g["errmax"]))
    _check(got, ref)


def _box_case(shape, seed, nmat):
    msh = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    NC, NbC = msh["NC"], msh["NbC"]
    rng = np.random.default_rng(seed)
    n = NbC + NC + 1
    d = dict(msh)
    d["NONZ"] = int(msh["Acol"][-1])
    d["volume"] = msh["volume"].copy()
    d["volume"][:NbC] = rng.uniform(0.5, 1.5, NbC)
    d["Asave"] = rng.uniform(1.0, 2.0, n)
    for k in ("rho_n", "rho_o", "rho_oo"):
        d[k] = rng.uniform(0.5, 1.5, n)
    for k in ("U", "V", "W", "P", "Px", "Py", "Pz"):
        d[k] = rng.uniform(-1.0, 1.0, n)
    tb = np.zeros(n, np.int32)
    tb[:NbC] = np.array([1, 2, 3, 4, 5, 6, 11, 12], np.int32)[rng.integers(0, 8, NbC)]
    d["TypeBC"] = tb
    return d


@pytest.mark.parametrize("shape,nmat", [((40, 33, 29), 1), ((24, 20, 18), 2)])
def test_assembly_matches_oracle_on_larger_boxes(shape, nmat):
    d = _box_case(shape, 9, nmat)
    dt = 0.02
    fields = {k: d[k] for k in oracle.CELL_FIELDS}
    ref = oracle.calcps_assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], nmat, dt, d["SideC"],
                                 d["SidAij"], d["Adia"], d["TypeBC"],
                                 {k: d[k] for k in oracle.FACE_GEOM}, fields)
    abou0 = np.full(max(d["NbC"], 1), 3.0)  # entries of non-buffer cells stay as they were
    got = _run_gpu(d, nmat, dt, abou_in=abou0)
    ra = ref[2].copy()
    buf = d["TypeBC"][:d["NbC"]] == 11
    ra[~buf] = 3.0
    _check(got, (ref[0], ref[1], ra, ref[3], ref[4]))


def test_assembled_pressure_system_solves():
    """The GPU-assembled matrix and right-hand side feed the GPU solver
    directly (same TopolM layout): CG reaches the tolerance on an
    all-interior box with a pinned cell."""
    import torch
    d = _box_case((20, 18, 16), 3, 1)
    d["TypeBC"][:d["NbC"]] = 2  # walls: a pure Neumann problem, b has zero mean
    asm = tflows.Assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], d["SideC"], d["SidAij"],
                          d["Adia"], d["TypeBC"], {k: d[k] for k in tflows.Assembly.GEOM},
                          d["volume"])
    fields = {k: _dev(d[v]) for k, v in FIELD_KEYS.items()}
    aval = torch.zeros(d["NONZ"], dtype=torch.float64, device="cuda")
    b = torch.zeros(d["NC"], dtype=torch.float64, device="cuda")
    abou = torch.zeros(max(d["NbC"], 1), dtype=torch.float64, device="cuda")
    flux = torch.zeros(d["NS"], dtype=torch.float64, device="cuda")
    asm.calcps(fields, aval, b, abou, flux, Nmat=1, dt=0.01)
    # pin cell 1 (a Dirichlet value of 0) so that the singular system is regular
    A = aval.cpu().numpy()
    A[int(d["Adia"][0]) - 1] *= 2.0
    rp, col = d["Acol"] - 1, d["Arow"][:-1] - 1
    topo = tflows.Topology(d["NC"], rp, col, d["Adia"] - 1)
    x = torch.zeros(d["NC"], dtype=torch.float64, device="cuda")
    val = _dev(A[:-1])
    tol = 1e-10 * float(b.norm())
    res = topo.solve(val, b, x, "cg", 1, 5000, tol)
    assert res["status"] == tflows.OK, res
    import scipy.sparse as sp
    M = sp.csr_matrix((A[:-1], col, rp), shape=(d["NC"], d["NC"]))
    r = b.cpu().numpy() - M @ x.cpu().numpy()
    assert np.linalg.norm(r) < 2 * tol
    asm.close()
    topo.close()


def test_assembly_rejects_bad_indices():
    d = _box_case((4, 3, 2), 1, 1)
    bad = d["SideC"].copy()
    bad[5, 2] = d["NC"] + 3
    with pytest.raises(tflows.SolverError) as e:
        tflows.Assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], bad, d["SidAij"], d["Adia"],
                        d["TypeBC"], {k: d[k] for k in tflows.Assembly.GEOM}, d["volume"])
    assert e.value.status == tflows.BAD_INPUT


def test_mesh_files_to_gpu_solve(tmp_path):
    """A mesh read from T-FlowS files (NAME.cns / NAME.geo), its TopolM
    layout built by the library, the pressure-correction system assembled on
    the GPU and solved there: the chain a real T-FlowS case takes."""
    import torch
    from fortran_files import write_cns, write_geo
    m = mesh.box_faces(18, 16, 14, perturb=0.2, seed=6)
    NC, NbC, NS = m["NC"], m["NbC"], m["NS"]
    material = np.ones(NbC + NC + 1, np.int32)
    material[NbC] = 0
    zeros = np.zeros(NbC, np.int32)
    faces = {k: m[k] for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f")}
    for k in ("xsp", "ysp", "zsp"):
        faces[k] = np.zeros(NS)
    cns, geo = str(tmp_path / "case.cns"), str(tmp_path / "case.geo")
    write_cns(cns, NC, NbC, NS, 1, material, m["SideC"], zeros, zeros)
    write_geo(geo, NbC, m["xc"], m["yc"], m["zc"], m["volume"][NbC + 1:], np.ones(NC),
              np.ones(NC), faces)
    r = tflows.read_mesh(cns, geo)
    Acol, Arow, Adia, sid = tflows.topolm(r["NC"], r["SideC"])
    vol = np.concatenate([np.zeros(NbC + 1), r["volume"]])
    tb = np.zeros(NbC + NC + 1, np.int32)
    tb[:NbC] = 2
    tb[:NbC:7] = 12  # some pressure boundaries: the matrix is regular
    asm = tflows.Assembly(NC, NbC, NS, int(Acol[-1]), r["SideC"], sid, Adia, tb,
                          {k: r[k] for k in tflows.Assembly.GEOM}, vol)
    rng = np.random.default_rng(3)
    n = NbC + NC + 1
    fields = {"asave": _dev(rng.uniform(1.0, 2.0, n))}
    for k in ("rho_n", "rho_o", "rho_oo"):
        fields[k] = _dev(rng.uniform(0.5, 1.5, n))
    for k in ("u", "v", "w", "p", "px", "py", "pz"):
        fields[k] = _dev(rng.uniform(-1.0, 1.0, n))
    aval = torch.zeros(int(Acol[-1]), dtype=torch.float64, device="cuda")
    b = torch.zeros(NC, dtype=torch.float64, device="cuda")
    abou = torch.zeros(NbC, dtype=torch.float64, device="cuda")
    flux = torch.zeros(NS, dtype=torch.float64, device="cuda")
    asm.calcps(fields, aval, b, abou, flux, Nmat=1, dt=0.01)
    topo = tflows.Topology(NC, Acol - 1, Arow[:-1] - 1, Adia - 1)
    x = torch.zeros(NC, dtype=torch.float64, device="cuda")
    tol = 1e-10 * float(b.norm())
    res = topo.solve(aval[:-1].contiguous(), b, x, "cg", 2, 5000, tol)
    assert res["status"] == tflows.OK, res
    import scipy.sparse as sp
    M = sp.csr_matrix((aval[:-1].cpu().numpy(), Arow[:-1] - 1, Acol - 1), shape=(NC, NC))
    assert np.linalg.norm(b.cpu().numpy() - M @ x.cpu().numpy()) < 2 * tol
    asm.close()
    topo.close()


def test_assembly_two_faces_between_the_same_cells():
    """Two faces joining the same pair of cells share one off-diagonal entry
    (TopolM maps both to it): the reference assigns -A12 face by face, so the
    later face's value stays; both faces add to the diagonals.  The GPU
    matches the oracle bit for bit."""
    d = _box_case((6, 5, 4), 2, 1)
    inner = np.nonzero(d["SideC"][:, 2] > 0)[0]
    dup = int(inner[len(inner) // 3])
    order = np.r_[np.arange(dup + 1), dup, np.arange(dup + 1, d["NS"])]
    for k in ("SideC", "Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f"):
        d[k] = np.ascontiguousarray(d[k][order])
    d["Sx"][dup + 1] *= 1.5  # the second face differs, so the order shows
    d["NS"] += 1
    Acol, Arow, Adia, sid = oracle.topolm(d["NC"], d["SideC"][:, 1:])
    d.update(Acol=Acol, Arow=Arow, Adia=Adia, SidAij=sid, NONZ=int(Acol[-1]))
    dt = 0.02
    ref = oracle.calcps_assembly(d["NC"], d["NbC"], d["NS"], d["NONZ"], 1, dt, d["SideC"],
                                 d["SidAij"], d["Adia"], d["TypeBC"],
                                 {k: d[k] for k in oracle.FACE_GEOM},
                                 {k: d[k] for k in oracle.CELL_FIELDS})
    got = _run_gpu(d, 1, dt, abou_in=np.zeros(max(d["NbC"], 1)))
    ra = ref[2].copy()
    _check(got, (ref[0], ref[1], ra, ref[3], ref[4]))
