"""T-FlowS mesh files (NAME.cns / NAME.geo) and the TopolM layout (host code
of the library; no GPU needed).

The files are written here record by record in the order Process/CnsLoa.f90
and Library/GeoLoa.f90 read them (tests/fortran_files.py); the library must
return every array, handle gfortran's subrecords, reject damaged files with a
message, and build the same compressed-row layout as the oracle's TopolM
restatement and the mesh builder.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import tflows
from fortran_files import write_cns, write_geo

mesh = tflows.mesh


def _case(shape=(5, 4, 3), seed=2):
    m = mesh.box_faces(*shape, perturb=0.2, seed=seed)
    NC, NbC = m["NC"], m["NbC"]
    rng = np.random.default_rng(seed)
    material = np.ones(NbC + NC + 1, np.int32)
    material[:NbC] = rng.integers(1, 3, NbC)
    material[NbC] = 0  # there is no cell 0
    bcmark = rng.integers(1, 7, NbC).astype(np.int32)
    copyc = np.zeros(NbC, np.int32)
    faces = {k: m[k] for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f")}
    for k in ("xsp", "ysp", "zsp"):
        faces[k] = rng.uniform(-1, 1, m["NS"])
    vol = m["volume"][NbC + 1:]
    delta = rng.uniform(0.5, 1.0, NC)
    walld = rng.uniform(0.0, 3.0, NC)
    return m, material, bcmark, copyc, faces, vol, delta, walld


@pytest.mark.parametrize("split", [None, 40])
def test_mesh_files_round_trip(tmp_path, split):
    m, material, bcmark, copyc, faces, vol, delta, walld = _case()
    NC, NbC, NS = m["NC"], m["NbC"], m["NS"]
    cns, geo = str(tmp_path / "box.cns"), str(tmp_path / "box.geo")
    write_cns(cns, NC, NbC, NS, 2, material, m["SideC"], bcmark, copyc, NSsh=7, split=split)
    write_geo(geo, NbC, m["xc"], m["yc"], m["zc"], vol, delta, walld, faces, split=split)
    r = tflows.read_mesh(cns, geo)
    assert (r["NC"], r["NbC"], r["NS"], r["NSsh"], r["Nmat"]) == (NC, NbC, NS, 7, 2)
    assert np.array_equal(r["material"], material)
    assert np.array_equal(r["SideC"], m["SideC"])
    assert np.array_equal(r["bcmark"], bcmark) and np.array_equal(r["CopyC"], copyc)
    for k in ("xc", "yc", "zc"):
        assert np.array_equal(r[k], m[k]), k
    for k, v in (("volume", vol), ("delta", delta), ("WallDs", walld)):
        assert np.array_equal(r[k], v), k
    for k, v in faces.items():
        assert np.array_equal(r[k], v), k
    # without the .geo file only the topology part is read
    r2 = tflows.read_mesh(cns)
    assert "Sx" not in r2 and np.array_equal(r2["SideC"], m["SideC"])


def test_damaged_files_are_rejected(tmp_path):
    m, material, bcmark, copyc, faces, vol, delta, walld = _case((3, 3, 2), 4)
    NC, NbC, NS = m["NC"], m["NbC"], m["NS"]
    cns = str(tmp_path / "a.cns")
    write_cns(cns, NC, NbC, NS, 1, material, m["SideC"], bcmark, copyc)
    data = open(cns, "rb").read()
    short = str(tmp_path / "short.cns")
    open(short, "wb").write(data[: len(data) // 2])
    with pytest.raises(tflows.SolverError) as e:
        tflows.read_mesh(short)
    assert e.value.status == tflows.BAD_INPUT and "short.cns" in str(e.value)
    wrong = m["SideC"].copy()
    wrong[3, 2] = NC + 5
    bad = str(tmp_path / "bad.cns")
    write_cns(bad, NC, NbC, NS, 1, material, wrong, bcmark, copyc)
    with pytest.raises(tflows.SolverError) as e:
        tflows.read_mesh(bad)
    assert "SideC" in str(e.value)
    with pytest.raises(tflows.SolverError):
        tflows.read_mesh(str(tmp_path / "missing.cns"))


@pytest.mark.parametrize("shape", [(5, 4, 3), (1, 6, 2), (7, 1, 1)])
def test_topolm_matches_oracle_and_mesh_builder(shape):
    m = mesh.box_faces(*shape, perturb=0.1, seed=1)
    NC, NS = m["NC"], m["NS"]
    Acol, Arow, Adia, sid = tflows.topolm(NC, m["SideC"])
    assert np.array_equal(Acol, m["Acol"]) and np.array_equal(Arow, m["Arow"])
    assert np.array_equal(Adia, m["Adia"])
    inner = m["SideC"][:, 2] > 0
    assert np.array_equal(sid[inner], m["SidAij"][inner]) and not sid[~inner].any()
    oAcol, oArow, oAdia, osid = oracle.topolm(NC, m["SideC"][:, 1:])
    assert np.array_equal(oAcol, Acol) and np.array_equal(oArow, Arow)
    assert np.array_equal(oAdia, Adia) and np.array_equal(osid, sid)
