"""Writers of T-FlowS mesh files for the tests: gfortran sequential
unformatted records (a 4-byte length before and after each record, 4-byte
INTEGER, 8-byte REAL), laid out record by record as Process/CnsLoa.f90 and
Library/GeoLoa.f90 read them, which is also the order the reference's
writer (Library/GeoSav.f90) emits them in."""
import struct

import numpy as np


def _record(fh, payload, split=None):
    """One record; with `split`, as subrecords of at most `split` bytes (the
    leading length of every subrecord but the last is negative)."""
    data = payload.tobytes() if isinstance(payload, np.ndarray) else payload
    if split is None or len(data) <= split:
        fh.write(struct.pack("<i", len(data)) + data + struct.pack("<i", len(data)))
        return
    chunks = [data[i:i + split] for i in range(0, len(data), split)]
    for k, ch in enumerate(chunks):
        # gfortran: the leading length is negative while more subrecords
        # follow, the trailing one negative on every subrecord but the first
        head = -len(ch) if k < len(chunks) - 1 else len(ch)
        tail = len(ch) if k == 0 else -len(ch)
        fh.write(struct.pack("<i", head) + ch + struct.pack("<i", tail))


def i4(a):
    return np.ascontiguousarray(a, dtype="<i4")


def r8(a):
    return np.ascontiguousarray(a, dtype="<f8")


def write_cns(path, NC, NbC, NS, Nmat, material, SideC, bcmark, CopyC, NSsh=0, split=None):
    """material over cells -NbC..NC, SideC (NS, 3), bcmark / CopyC over
    -NbC..-1 (element c at index c + NbC)."""
    with open(path, "wb") as fh:
        for v in (NC, NbC, NS, NSsh, Nmat):
            _record(fh, i4([v]))
        _record(fh, i4(material[NbC + 1:]), split)
        _record(fh, i4(material[:NbC][::-1]))          # (material(c), c=-1,-NbC,-1)
        for k in range(3):
            _record(fh, i4(SideC[:, k]), split)
        _record(fh, i4(bcmark[::-1]))
        _record(fh, i4(CopyC[::-1]))


def write_geo(path, NbC, xc, yc, zc, volume, delta, WallDs, faces, split=None):
    """xc/yc/zc over cells -NbC..NC; volume, delta, WallDs over 1..NC;
    faces: Sx, Sy, Sz, Dx, Dy, Dz, f, xsp, ysp, zsp over 1..NS."""
    with open(path, "wb") as fh:
        for a in (xc, yc, zc):
            _record(fh, r8(a[NbC + 1:]), split)
        for a in (xc, yc, zc):
            _record(fh, r8(a[:NbC][::-1]))
        for a in (volume, delta, WallDs):
            _record(fh, r8(a), split)
        for k in ("Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "xsp", "ysp", "zsp"):
            _record(fh, r8(faces[k]), split)
