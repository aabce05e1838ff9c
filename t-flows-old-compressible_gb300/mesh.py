"""Synthetic hexahedral box meshes stored in the T-FlowS compressed-row layout.

The solver interface takes a matrix in the layout that Process/TopolM.f90:24-98
builds: 1-based row pointers ``Acol(N+1)``, column indices ``Arow(NONZ)``
sorted ascending within each row, diagonal positions ``Adia(N)``, values
``A(NONZ)`` and ``NONZ = nnz + 1`` (the last slot is unused and 0).  This
module builds that layout for a box of ``nx*ny*nz`` hex cells (cell numbering
x fastest), with optional seeded node perturbation, and fills it with the
coefficients the reference's assembly routines produce:

* pressure correction (Process/CalcPS.f90:77-102): off-diagonal ``-A12``,
  diagonal ``sum A12``, with ``A12 = |S|^2/(S.d)``, optionally divided by the
  harmonic face density; Neumann walls and one Dirichlet cell;
* momentum / scalar transport (Process/NewUVW.f90:323-367,447-456): first
  order upwind convection from a discretely divergence-free face flux,
  diffusion ``A0/rho`` with ``A0 = nu*|S|^2/(S.d)``, and the time term
  ``rho*V/dt`` on the diagonal.

Faces are stored as the reference's ``SideC`` list would hold them (interior
x-, y-, z-faces in cell order, then the six walls), and ``SidAij``-style
positions map each interior face to its two off-diagonal entries
(Process/TopolM.f90:81-94).  Everything is vectorised numpy so that a 256^3
box (16.8 M cells, 117 M stored entries) builds in seconds.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

__all__ = [
    "System", "box_csr", "box_geometry", "pressure_system",
    "convection_diffusion_system", "config_system", "batch_sizes",
    "side_c", "interior_faces", "structured_levels", "box_faces",
]


@dataclasses.dataclass
class System:
    """One linear system in the reference's argument layout.

    ``x`` holds ``x(-NB:N)`` (so ``x[NB + i]`` is Fortran ``x(i)``; ``x[NB]``
    is the unused ``x(0)``), ``Ab`` holds ``Ab(-NB:-1)``.  ``tol`` is the
    absolute tolerance that equals ``rel_tol * ||b||`` (the reference tests
    ``||r|| < tol`` in absolute terms, Process/CG.f90:248-255).
    """

    name: str
    shape: tuple
    N: int
    NB: int
    NONZ: int
    A: np.ndarray
    Acol: np.ndarray
    Arow: np.ndarray
    Adia: np.ndarray
    Ab: np.ndarray
    b: np.ndarray
    x: np.ndarray
    symmetric: bool
    rel_tol: float = 1e-8
    face_coef: np.ndarray | None = None
    fixed_diag: np.ndarray | None = None

    @property
    def nnz(self) -> int:
        return self.NONZ - 1

    @property
    def tol(self) -> float:
        return self.rel_tol * float(np.sqrt(np.dot(self.b, self.b)))

    def x0(self) -> np.ndarray:
        return self.x[self.NB + 1:]

    def csr0(self):
        """0-based (rowptr, col, val, diag) views of the stored entries."""
        return (self.Acol - 1, self.Arow[:-1] - 1, self.A[:-1], self.Adia - 1)

    def scipy(self):
        import scipy.sparse as sp
        rp, col, val, _ = self.csr0()
        return sp.csr_matrix((val, col, rp), shape=(self.N, self.N))


def box_csr(nx: int, ny: int, nz: int):
    """Compressed-row topology of a 7-point hex box, as TopolM builds it.

    Returns ``(Acol, Arow, Adia, slot)`` with 1-based int32 arrays and
    ``slot[(axis, side)]`` (axis 0/1/2 = x/y/z, side -1/+1) the 1-based
    position of the entry for that neighbour in each row (0 where the
    neighbour does not exist).
    """
    N = nx * ny * nz
    cell = np.arange(N, dtype=np.int64)
    i = cell % nx
    j = (cell // nx) % ny
    k = cell // (nx * ny)
    offs = (-nx * ny, -nx, -1, 0, 1, nx, nx * ny)
    keys = ((2, -1), (1, -1), (0, -1), 0, (0, 1), (1, 1), (2, 1))
    masks = (k > 0, j > 0, i > 0, None, i < nx - 1, j < ny - 1, k < nz - 1)
    del i, j, k
    rowlen = np.ones(N, np.int64)
    for m in masks:
        if m is not None:
            rowlen += m
    nnz = int(rowlen.sum())
    if nnz + 1 >= 2**31:
        raise ValueError("box too large for 32-bit Fortran INTEGER indices")
    Acol = np.empty(N + 1, np.int32)
    Acol[0] = 1
    np.cumsum(rowlen, out=Acol[1:])
    Acol[1:] += 1
    del rowlen
    run = Acol[:-1].astype(np.int64)
    Arow = np.zeros(nnz + 1, np.int32)
    slot = {}
    for off, key, m in zip(offs, keys, masks):
        if m is None:
            Arow[run - 1] = cell + 1
            slot[0] = run.astype(np.int32)
            run += 1
        else:
            pos = run[m]
            Arow[pos - 1] = cell[m] + off + 1
            full = np.zeros(N, np.int32)
            full[m] = pos
            slot[key] = full
            run += m
    Adia = slot[0]
    return Acol, Arow, Adia, slot


class V3:
    """Three same-shaped component arrays (structure of arrays): slicing,
    +, -, scalar *, dot and cross act componentwise without ever stacking
    the components into one (..., 3) array."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x, y, z):
        self.x, self.y, self.z = x, y, z

    def __getitem__(self, idx):
        return V3(self.x[idx], self.y[idx], self.z[idx])

    def __add__(self, o):
        return V3(self.x + o.x, self.y + o.y, self.z + o.z)

    def __sub__(self, o):
        return V3(self.x - o.x, self.y - o.y, self.z - o.z)

    def __mul__(self, k):
        return V3(self.x * k, self.y * k, self.z * k)

    __rmul__ = __mul__

    def dot(self, o):
        return self.x * o.x + self.y * o.y + self.z * o.z

    def cross(self, o):
        return V3(self.y * o.z - self.z * o.y, self.z * o.x - self.x * o.z,
                  self.x * o.y - self.y * o.x)

    def ravel(self):
        return V3(self.x.ravel(), self.y.ravel(), self.z.ravel())


def _dot(a, b):
    return a.dot(b)


def box_geometry(nx, ny, nz, h=1.0, perturb=0.0, rng=None):
    """Node, face and cell geometry of a (perturbed) hex box.

    Nodes are displaced by ``uniform(-perturb*h, perturb*h)`` per coordinate
    (one draw of shape (nz+1, ny+1, nx+1, 3)).  Face area vectors are
    ``0.5 * (c - a) x (d - b)`` for the quad a-b-c-d, oriented along +x, +y,
    +z; cell volumes come from the divergence theorem.  Returns a dict of
    V3 arrays: nodes ``P`` (nz+1, ny+1, nx+1), face vectors ``Sx, Sy, Sz``
    and face centres ``Fx, Fy, Fz``, cell centres ``C``, and volumes ``V``
    (nz, ny, nx).
    """
    shape = (nz + 1, ny + 1, nx + 1)
    X = np.broadcast_to(np.arange(nx + 1, dtype=np.float64)[None, None, :] * h, shape).copy()
    Y = np.broadcast_to(np.arange(ny + 1, dtype=np.float64)[None, :, None] * h, shape).copy()
    Z = np.broadcast_to(np.arange(nz + 1, dtype=np.float64)[:, None, None] * h, shape).copy()
    if perturb > 0.0:
        d = rng.uniform(-perturb * h, perturb * h, size=shape + (3,))
        X += d[..., 0]
        Y += d[..., 1]
        Z += d[..., 2]
        del d
    P = V3(X, Y, Z)

    def quad(a, b_, c, d):
        return 0.5 * (c - a).cross(d - b_), 0.25 * (a + b_ + c + d)

    # x-faces on node plane i: a=(k,j), b=(k,j+1), c=(k+1,j+1), d=(k+1,j)
    Sx, Fx = quad(P[:-1, :-1, :], P[:-1, 1:, :], P[1:, 1:, :], P[1:, :-1, :])
    # y-faces on node plane j: a=(k,i), b=(k+1,i), c=(k+1,i+1), d=(k,i+1)
    Sy, Fy = quad(P[:-1, :, :-1], P[1:, :, :-1], P[1:, :, 1:], P[:-1, :, 1:])
    # z-faces on node plane k: a=(j,i), b=(j,i+1), c=(j+1,i+1), d=(j+1,i)
    Sz, Fz = quad(P[:, :-1, :-1], P[:, :-1, 1:], P[:, 1:, 1:], P[:, 1:, :-1])
    C = 0.125 * (P[:-1, :-1, :-1] + P[:-1, :-1, 1:] + P[:-1, 1:, :-1] + P[:-1, 1:, 1:]
                 + P[1:, :-1, :-1] + P[1:, :-1, 1:] + P[1:, 1:, :-1] + P[1:, 1:, 1:])
    fx, fy, fz = Fx.dot(Sx), Fy.dot(Sy), Fz.dot(Sz)
    Vol = (fx[:, :, 1:] - fx[:, :, :-1] + fy[:, 1:, :] - fy[:, :-1, :]
           + fz[1:, :, :] - fz[:-1, :, :]) / 3.0
    return dict(P=P, Sx=Sx, Sy=Sy, Sz=Sz, Fx=Fx, Fy=Fy, Fz=Fz, C=C, V=Vol)


# Slot order of a 7-point row (ascending column offset): -z, -y, -x, diag,
# +x, +y, +z; the (c1, c2) entry of an axis-d face sits in slot PLUS[d] of
# row c1 and the (c2, c1) entry in slot MINUS[d] of row c2.
PLUS = (4, 5, 6)
MINUS = (2, 1, 0)
DIAG = 3


def _face_slices(axis):
    """(lo, hi) index tuples over the (nz, ny, nx) cell grid selecting the
    lower / upper cell of every interior face normal to `axis`."""
    lo = [slice(None)] * 3
    hi = [slice(None)] * 3
    dim = 2 - axis
    lo[dim] = slice(0, -1)
    hi[dim] = slice(1, None)
    return tuple(lo), tuple(hi)


def _interior_geometry(geo, axis):
    """Area vectors and centre-to-centre vectors of the interior faces normal
    to `axis`, shaped like the face grid."""
    S = (geo["Sx"][:, :, 1:-1], geo["Sy"][:, 1:-1, :], geo["Sz"][1:-1])[axis]
    lo, hi = _face_slices(axis)
    C = geo["C"]
    return S, C[hi] - C[lo]


class _SlotMatrix:
    """Dense (nz, ny, nx, 7) slot array compressed into the TopolM layout."""

    def __init__(self, nx, ny, nz):
        self.shape = (nx, ny, nz)
        self.A7 = np.zeros((nz, ny, nx, 7))

    def face(self, axis, off12, off21, d1, d2):
        """Add one direction's interior faces: entry (c1,c2) = -off12,
        entry (c2,c1) = -off21, diag(c1) += d1, diag(c2) += d2."""
        lo, hi = _face_slices(axis)
        self.A7[lo + (PLUS[axis],)] -= off12
        self.A7[hi + (MINUS[axis],)] -= off21
        self.A7[lo + (DIAG,)] += d1
        self.A7[hi + (DIAG,)] += d2

    def diag(self):
        return self.A7[..., DIAG]

    def compress(self):
        nx, ny, nz = self.shape
        Acol, Arow, Adia, _ = box_csr(nx, ny, nz)
        k = np.arange(nz)[:, None, None]
        j = np.arange(ny)[None, :, None]
        i = np.arange(nx)[None, None, :]
        mask = np.empty((nz, ny, nx, 7), bool)
        mask[..., 0] = k > 0
        mask[..., 1] = j > 0
        mask[..., 2] = i > 0
        mask[..., 3] = True
        mask[..., 4] = i < nx - 1
        mask[..., 5] = j < ny - 1
        mask[..., 6] = k < nz - 1
        A = np.zeros(Arow.shape[0])
        A[:-1] = self.A7[mask]
        return A, Acol, Arow, Adia


def _wall_faces(nx, ny, nz, geo):
    """Boundary faces (x-min, x-max, y-min, y-max, z-min, z-max) with the
    adjacent cell, outward area vector and centre-to-face vector (V3)."""
    N = nx * ny * nz
    cell = np.arange(N, dtype=np.int64).reshape(nz, ny, nx)
    C = geo["C"]
    cs, Ss, ds = [], [], []
    for S, F, cidx, cc, sign in (
        (geo["Sx"][:, :, 0], geo["Fx"][:, :, 0], cell[:, :, 0], C[:, :, 0], -1.0),
        (geo["Sx"][:, :, nx], geo["Fx"][:, :, nx], cell[:, :, nx - 1], C[:, :, nx - 1], 1.0),
        (geo["Sy"][:, 0, :], geo["Fy"][:, 0, :], cell[:, 0, :], C[:, 0, :], -1.0),
        (geo["Sy"][:, ny, :], geo["Fy"][:, ny, :], cell[:, ny - 1, :], C[:, ny - 1, :], 1.0),
        (geo["Sz"][0], geo["Fz"][0], cell[0], C[0], -1.0),
        (geo["Sz"][nz], geo["Fz"][nz], cell[nz - 1], C[nz - 1], 1.0),
    ):
        cs.append(cidx.ravel())
        Ss.append((S * sign).ravel())
        ds.append((F - cc).ravel())
    cat = lambda vs: V3(*(np.concatenate([getattr(v, a) for v in vs]) for a in "xyz"))  # noqa
    return np.concatenate(cs), cat(Ss), cat(ds)


def interior_faces(nx, ny, nz):
    """Interior faces in SideC order (x-, y-, z-faces, each in cell order):
    0-based cells c1 < c2 and 0-based positions of entries (c1,c2) in row c1
    and (c2,c1) in row c2 (the reference's SidAij minus 1)."""
    N = nx * ny * nz
    _, _, _, slot = box_csr(nx, ny, nz)
    cell = np.arange(N, dtype=np.int64).reshape(nz, ny, nx)
    c1s, c2s, p12s, p21s = [], [], [], []
    for axis, off in ((0, 1), (1, nx), (2, nx * ny)):
        lo, _ = _face_slices(axis)
        c1 = cell[lo].ravel()
        c2 = c1 + off
        c1s.append(c1)
        c2s.append(c2)
        p12s.append(slot[(axis, 1)][c1].astype(np.int64) - 1)
        p21s.append(slot[(axis, -1)][c2].astype(np.int64) - 1)
    return (np.concatenate(c1s), np.concatenate(c2s), np.concatenate(p12s),
            np.concatenate(p21s))


def side_c(nx, ny, nz):
    """The face list as the reference stores it: SideC(2,NS), 1-based cells,
    boundary faces with negative second cell (-1, -2, ...), plus the layout
    TopolM would build from it (Acol, Arow, Adia, SidAij(NS,2))."""
    Acol, Arow, Adia, _ = box_csr(nx, ny, nz)
    c1, c2, p12, p21 = interior_faces(nx, ny, nz)
    cell = np.arange(nx * ny * nz, dtype=np.int64).reshape(nz, ny, nx)
    cw = np.concatenate([cell[:, :, 0].ravel(), cell[:, :, nx - 1].ravel(), cell[:, 0, :].ravel(),
                         cell[:, ny - 1, :].ravel(), cell[0].ravel(), cell[nz - 1].ravel()])
    nb = cw.shape[0]
    ni = c1.shape[0]
    sc = np.empty((ni + nb, 2), np.int32)
    sc[:ni, 0] = c1 + 1
    sc[:ni, 1] = c2 + 1
    sc[ni:, 0] = cw + 1
    sc[ni:, 1] = -np.arange(1, nb + 1)
    sid = np.zeros((sc.shape[0], 2), np.int32)
    sid[:ni, 0] = p12 + 1
    sid[:ni, 1] = p21 + 1
    return sc, (Acol, Arow, Adia, sid)


def box_faces(nx, ny, nz, perturb=0.0, seed=0):
    """Every face of a (perturbed) hex box with the geometry the reference
    keeps per face and cell (Library/GeoLoa.f90: Sx..Sz, Dx..Dz, f, volume),
    in SideC order: interior x-, y-, z-faces in cell order (as
    ``interior_faces``), then the six walls (x-min, x-max, y-min, y-max,
    z-min, z-max, each in cell order) whose second cell is the boundary cell
    -1, -2, ...  Area vectors point from c1 to c2 (outward on walls);
    D = centre(c2) - centre(c1), a boundary cell sitting at its face centre;
    f is the weight of c1 in face interpolation (distance based, 0 on walls).

    Returns a dict: NC, NbC, NS, SideC (NS, 3) = SideC(0:2, NS) in memory
    order (SideC(0, s) = 0), SidAij (NS, 2), Acol, Arow, Adia (TopolM layout),
    geometry arrays Sx..Dz and f (NS,), volume (NbC + NC + 1,) over cells
    -NbC..NC (boundary cells get volume 0), centres xc/yc/zc likewise.
    """
    rng = np.random.default_rng(seed)
    geo = box_geometry(nx, ny, nz, perturb=perturb, rng=rng)
    sc, (Acol, Arow, Adia, sid) = side_c(nx, ny, nz)
    C, V = geo["C"], geo["V"]
    cx, cy, cz = (a.ravel() for a in (C.x, C.y, C.z))
    S_parts, F_parts = [], []
    for axis, Sk, Fk in ((0, geo["Sx"], geo["Fx"]), (1, geo["Sy"], geo["Fy"]),
                         (2, geo["Sz"], geo["Fz"])):
        sl = (slice(None), slice(None), slice(1, -1)) if axis == 0 else \
             (slice(None), slice(1, -1), slice(None)) if axis == 1 else \
             (slice(1, -1), slice(None), slice(None))
        S_parts.append([a[sl].ravel() for a in (Sk.x, Sk.y, Sk.z)])
        F_parts.append([a[sl].ravel() for a in (Fk.x, Fk.y, Fk.z)])
    for axis, Sk, Fk in ((0, geo["Sx"], geo["Fx"]), (1, geo["Sy"], geo["Fy"]),
                         (2, geo["Sz"], geo["Fz"])):
        for side, sign in ((0, -1.0), (-1, 1.0)):
            sl = [slice(None)] * 3
            sl[2 - axis] = side
            sl = tuple(sl)
            S_parts.append([sign * a[sl].ravel() for a in (Sk.x, Sk.y, Sk.z)])
            F_parts.append([a[sl].ravel() for a in (Fk.x, Fk.y, Fk.z)])
    S = [np.concatenate([p[k] for p in S_parts]) for k in range(3)]
    F = [np.concatenate([p[k] for p in F_parts]) for k in range(3)]
    NS = sc.shape[0]
    NC = nx * ny * nz
    c1 = sc[:, 0].astype(np.int64) - 1
    c2 = sc[:, 1].astype(np.int64)
    inner = c2 > 0
    NbC = int(-c2.min()) if (~inner).any() else 0
    x1 = [cx[c1], cy[c1], cz[c1]]
    x2 = [np.where(inner, c[np.maximum(c2 - 1, 0)], Fk) for c, Fk in zip((cx, cy, cz), F)]
    D = [b - a for a, b in zip(x1, x2)]
    d1 = np.sqrt(sum((Fk - a) ** 2 for Fk, a in zip(F, x1)))
    d2 = np.sqrt(sum((Fk - b) ** 2 for Fk, b in zip(F, x2)))
    f = np.where(inner, d2 / (d1 + d2), 0.0)
    vol = np.zeros(NbC + NC + 1)
    vol[NbC + 1:] = V.ravel()
    cen = []
    for k, c in enumerate((cx, cy, cz)):
        a = np.zeros(NbC + NC + 1)
        a[NbC + 1:] = c
        a[NbC + c2[~inner]] = F[k][~inner]
        cen.append(a)
    SideC = np.zeros((NS, 3), np.int32)
    SideC[:, 1:] = sc
    return dict(NC=NC, NbC=NbC, NS=NS, SideC=SideC, SidAij=sid, Acol=Acol, Arow=Arow, Adia=Adia,
                Sx=S[0], Sy=S[1], Sz=S[2], Dx=D[0], Dy=D[1], Dz=D[2], f=f, volume=vol,
                xc=cen[0], yc=cen[1], zc=cen[2])


def _smooth_field(shape, sigma, rng):
    from scipy.ndimage import gaussian_filter
    f = rng.standard_normal(shape)
    return gaussian_filter(f, sigma=sigma, mode="wrap")


def _density(shape, rng, lo=0.14, hi=1.0, sigma=3.0):
    f = _smooth_field(shape, sigma, rng)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-300)
    return lo + (hi - lo) * f


def _geom_coef(S, d):
    return _dot(S, S) / _dot(S, d)


def pressure_system(nx, ny, nz, perturb=0.0, seed=0, variable_density=False,
                    rel_tol=1e-8, name=None, keep_faces=False):
    """Pressure-correction matrix (Process/CalcPS.f90:77-102 pattern).

    A12 = |S|^2/(S.d) (divided by the harmonic face density when
    ``variable_density``); Neumann walls; cell 1 gets a Dirichlet face (its
    x-min wall coefficient added to the diagonal).  RHS ~ uniform[-1, 1]
    (``numpy.random.default_rng(seed)``), mean removed; x0 = 0.
    Random draws in order: node perturbation, density field, RHS.
    With ``keep_faces`` the per-face coefficients are kept (interior_faces
    order) together with the fixed diagonal part, for differentiable
    assembly.
    """
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    geo = box_geometry(nx, ny, nz, perturb=perturb, rng=rng)
    rho = _density((nz, ny, nx), rng) if variable_density else None
    M = _SlotMatrix(nx, ny, nz)
    coefs = []
    for axis in range(3):
        S, d = _interior_geometry(geo, axis)
        c = _geom_coef(S, d)
        if rho is not None:
            lo, hi = _face_slices(axis)
            c = c * (0.5 * (1.0 / rho[lo] + 1.0 / rho[hi]))
        M.face(axis, c, c, c, c)
        if keep_faces:
            coefs.append(c.ravel())
    # Dirichlet face: the x-min wall of cell 1.
    S0 = geo["Sx"][0, 0, 0]
    d0 = geo["C"][0, 0, 0] - geo["Fx"][0, 0, 0]
    gw0 = float(S0.dot(S0) / abs(S0.dot(d0)))
    fixed = np.zeros(N)
    fixed[0] = gw0 / (rho[0, 0, 0] if rho is not None else 1.0)
    M.diag().reshape(-1)[0] += fixed[0]
    NB = 2 * (nx * ny + ny * nz + nx * nz)
    del geo
    A, Acol, Arow, Adia = M.compress()
    del M
    b = rng.uniform(-1.0, 1.0, N)
    b -= b.mean()
    x = np.zeros(NB + N + 1)
    return System(
        name=name or f"pressure{'-vd' if variable_density else ''}-{nx}x{ny}x{nz}",
        shape=(nx, ny, nz), N=N, NB=NB, NONZ=int(Arow.shape[0]), A=A, Acol=Acol, Arow=Arow,
        Adia=Adia, Ab=np.zeros(NB), b=b, x=x, symmetric=True, rel_tol=rel_tol,
        face_coef=np.concatenate(coefs) if keep_faces else None,
        fixed_diag=fixed if keep_faces else None)


def convection_diffusion_system(nx, ny, nz, perturb=0.2, seed=0, nu=1e-2, dt=1e-2,
                                variable_density=False, sigma=2.0, rel_tol=1e-8,
                                name=None):
    """Momentum / scalar transport matrix (Process/NewUVW.f90:323-367,447-456).

    Face flux F is the circulation of a vector potential psi (Gaussian-smoothed
    seeded noise, sigma in cells, zero on the boundary nodes) around the face,
    so every cell's net flux is exactly zero and walls carry none; it is
    scaled to an RMS face velocity of 1.  For face s with cells c1 < c2:
    row c1 diagonal += max(F,0) + A0/rho1, entry (c1,c2) = -(max(-F,0) + A0/rho2);
    row c2 diagonal += max(-F,0) + A0/rho2, entry (c2,c1) = -(max(F,0) + A0/rho1);
    A0 = nu*|S|^2/(S.d).  Walls are Dirichlet (diagonal += A0_wall/rho); the
    time term rho*V/dt is on the diagonal; b = rho*V/dt * u_old with
    u_old ~ uniform[-1, 1]; x0 = 0.
    Random draws in order: node perturbation, psi (3 components), density, u_old.
    """
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    geo = box_geometry(nx, ny, nz, perturb=perturb, rng=rng)
    P = geo["P"]
    comps = []
    for _ in range(3):
        f = _smooth_field(P.x.shape, sigma, rng)
        f[0] = f[-1] = 0.0
        f[:, 0] = f[:, -1] = 0.0
        f[:, :, 0] = f[:, :, -1] = 0.0
        comps.append(f)
    psi = V3(*comps)
    del comps

    def circ(a, b_, c, d, pa, pb, pc, pd):
        return ((pa + pb).dot(b_ - a) + (pb + pc).dot(c - b_) + (pc + pd).dot(d - c)
                + (pd + pa).dot(a - d)) * 0.5

    # Same quad orderings as box_geometry, so the circulation is the flux
    # through the oriented area vector (Stokes).  Interior faces only.
    F = [
        circ(P[:-1, :-1, 1:-1], P[:-1, 1:, 1:-1], P[1:, 1:, 1:-1], P[1:, :-1, 1:-1],
             psi[:-1, :-1, 1:-1], psi[:-1, 1:, 1:-1], psi[1:, 1:, 1:-1], psi[1:, :-1, 1:-1]),
        circ(P[:-1, 1:-1, :-1], P[1:, 1:-1, :-1], P[1:, 1:-1, 1:], P[:-1, 1:-1, 1:],
             psi[:-1, 1:-1, :-1], psi[1:, 1:-1, :-1], psi[1:, 1:-1, 1:], psi[:-1, 1:-1, 1:]),
        circ(P[1:-1, :-1, :-1], P[1:-1, :-1, 1:], P[1:-1, 1:, 1:], P[1:-1, 1:, :-1],
             psi[1:-1, :-1, :-1], psi[1:-1, :-1, 1:], psi[1:-1, 1:, 1:], psi[1:-1, 1:, :-1]),
    ]
    del psi
    geoms = [_interior_geometry(geo, a) for a in range(3)]
    ssum, cnt = 0.0, 0
    for a in range(3):
        area2 = _dot(geoms[a][0], geoms[a][0])
        ssum += float(np.sum(F[a] * F[a] / area2))
        cnt += F[a].size
    rms = math.sqrt(ssum / cnt) if cnt else 1.0
    rho = _density((nz, ny, nx), rng) if variable_density else np.ones((nz, ny, nx))
    M = _SlotMatrix(nx, ny, nz)
    for a in range(3):
        S, d = geoms[a]
        Fa = F[a] / max(rms, 1e-300)
        A0 = nu * _geom_coef(S, d)
        lo, hi = _face_slices(a)
        a12 = np.maximum(-Fa, 0.0)
        a21 = np.maximum(Fa, 0.0)
        D12 = A0 / rho[hi]
        D21 = A0 / rho[lo]
        M.face(a, a12 + D12, a21 + D21, a21 + D21, a12 + D12)
    del F, geoms
    cw, Sw, dw = _wall_faces(nx, ny, nz, geo)
    NB = int(cw.shape[0])
    rho_f = rho.ravel()
    V = geo["V"].ravel()
    diag = M.diag().reshape(-1)
    diag += np.bincount(cw, weights=nu * _dot(Sw, Sw) / _dot(Sw, dw) / rho_f[cw], minlength=N)
    diag += rho_f * V / dt
    del geo
    A, Acol, Arow, Adia = M.compress()
    del M
    u_old = rng.uniform(-1.0, 1.0, N)
    b = rho_f * V / dt * u_old
    x = np.zeros(NB + N + 1)
    return System(
        name=name or f"convdiff-{nx}x{ny}x{nz}", shape=(nx, ny, nz), N=N, NB=NB,
        NONZ=int(Arow.shape[0]), A=A, Acol=Acol, Arow=Arow, Adia=Adia, Ab=np.zeros(NB), b=b, x=x,
        symmetric=False, rel_tol=rel_tol)


def config_system(index: int, scale: int | None = None, seed: int = 0) -> System:
    """The workloads of the benchmark suite, by number (1-5).

    1: 32^3 unit-cube pressure Poisson (Jacobi CG, FP64).
    2: 128^3 perturbed convection-diffusion (BiCG / CGS, diagonal).
    3: 256^3 perturbed variable-density pressure (IC CG, mixed + refinement).
    5: 64^3 perturbed variable-density pressure (differentiable solve).
    ``scale`` overrides the edge length (for parity tests at small sizes).
    """
    if index == 1:
        n = scale or 32
        return pressure_system(n, n, n, perturb=0.0, seed=seed, name=f"cfg1-pressure-{n}^3")
    if index == 2:
        n = scale or 128
        return convection_diffusion_system(n, n, n, perturb=0.2, seed=seed,
                                           name=f"cfg2-convdiff-{n}^3")
    if index == 3:
        n = scale or 256
        return pressure_system(n, n, n, perturb=0.2, seed=seed, variable_density=True,
                               name=f"cfg3-vd-pressure-{n}^3")
    if index == 5:
        n = scale or 64
        return pressure_system(n, n, n, perturb=0.2, seed=seed, variable_density=True,
                               name=f"cfg5-vd-pressure-{n}^3")
    raise ValueError(f"no single-system workload {index}")


def batch_sizes(count=48, lo=16, hi=160, seed=0):
    """Box shapes of the batched workload: N log-uniform in [lo^3, hi^3],
    boxes close to cubes (n, n, round(N/n^2))."""
    rng = np.random.default_rng(seed)
    Ns = np.exp(rng.uniform(math.log(lo**3), math.log(hi**3), count))
    shapes = []
    for Nt in Ns:
        n = max(2, int(round(Nt ** (1.0 / 3.0))))
        nz = max(2, int(round(Nt / (n * n))))
        shapes.append((n, n, nz))
    return shapes


def structured_levels(nx, ny, nz):
    """Wavefront level of each cell of a 7-point box in natural numbering:
    i + j + k (the forward IC sweep's dependency depth)."""
    N = nx * ny * nz
    cell = np.arange(N, dtype=np.int64)
    return (cell % nx) + (cell // nx) % ny + cell // (nx * ny)


@dataclasses.dataclass
class Subdomain:
    """One rank's part of a system split into subdomains, in the layout a
    T-FlowS rank holds after Parallel/Double/BufLoa.f90:35-84.

    Rows are the rank's cells (``rows`` their global 0-based indices, in
    order); the matrix keeps the local couplings, and each coupling to a
    cell of neighbour ``sub`` becomes a buffer cell k (negative, inside
    x(-NB:-1)) with ``Ab`` holding the coefficient and ``BufInd`` the local
    row: ``Ab[NB + k]`` = Ab(k), ``BufInd[NB + k]`` = BufInd(k).  ``NBBs``,
    ``NBBe`` hold NBBs(sub), NBBe(sub) for sub = 1..Npro; the first
    ``n_phys`` boundary cells x(-n_phys:-1) stand for the physical boundary
    cells and carry no coupling.  Both sides of a neighbour pair order their
    shared couplings by the global (row, column) of the lower-numbered side,
    so that the k-th cell of one rank's segment meets the k-th of the
    other's when the segments are swapped."""

    rank: int
    Npro: int
    N: int
    NB: int
    NONZ: int
    A: np.ndarray
    Acol: np.ndarray
    Arow: np.ndarray
    Adia: np.ndarray
    Ab: np.ndarray
    b: np.ndarray
    x: np.ndarray
    NBBs: np.ndarray
    NBBe: np.ndarray
    BufInd: np.ndarray
    rows: np.ndarray

    def segments(self):
        """(partner rank, lo, hi) slices of the PHI(-NB:-1) array that are
        exchanged with each connected neighbour, in neighbour order."""
        out = []
        for sub in range(1, self.Npro + 1):
            s0, e0 = int(self.NBBs[sub - 1]), int(self.NBBe[sub - 1])
            if e0 <= s0:
                out.append((sub - 1, self.NB + e0, self.NB + s0 + 1))
        return out


def partition(s: System, nparts: int, n_phys: int = 2) -> list:
    """Split ``s`` into ``nparts`` subdomains of consecutive rows (slabs of
    a box in natural numbering), returning one Subdomain per rank."""
    N = s.N
    rp = s.Acol.astype(np.int64) - 1
    col = s.Arow[:-1].astype(np.int64) - 1
    val = s.A[:-1]
    owner = (np.arange(N) * nparts) // N
    subs = []
    for r in range(nparts):
        rows = np.nonzero(owner == r)[0]
        loc = np.full(N, -1, np.int64)
        loc[rows] = np.arange(rows.size)
        Acol = [1]
        Arow, A, Adia = [], [], []
        links = {q: [] for q in range(nparts) if q != r}  # (key, local row, coefficient)
        for i in rows:
            for j in range(rp[i], rp[i + 1]):
                c = col[j]
                if owner[c] == r:
                    if c == i:
                        Adia.append(len(A) + 1)
                    Arow.append(loc[c] + 1)
                    A.append(val[j])
                else:
                    links[owner[c]].append(((min(i, c), max(i, c)), loc[i] + 1, val[j]))
            Acol.append(len(A) + 1)
        nbuf = sum(len(v) for v in links.values())
        NB = n_phys + nbuf
        NBBs = np.zeros(nparts, np.int32)
        NBBe = np.zeros(nparts, np.int32)
        Ab = np.zeros(NB)
        BufInd = np.zeros(NB, np.int32)
        prev_e = -n_phys  # NBBe(0) = -NBC (BufLoa.f90:47-50)
        for sub in range(1, nparts + 1):
            q = sub - 1
            lst = sorted(links.get(q, []), key=lambda t: t[0])
            if q == r or not lst:
                NBBs[q], NBBe[q] = prev_e - 1, prev_e  # empty: NBBe > NBBs
                continue
            s0 = prev_e - 1
            e0 = s0 - len(lst) + 1
            for m, (_, i_loc, a) in enumerate(lst):
                k = s0 - m
                Ab[NB + k] = a
                BufInd[NB + k] = i_loc
            NBBs[q], NBBe[q] = s0, e0
            prev_e = e0
        for q in range(nparts):  # BufLoa.f90:74-80: empty ranges become (-1, 0)
            if NBBe[q] > NBBs[q]:
                NBBs[q], NBBe[q] = -1, 0
        A = np.array(A + [0.0])
        subs.append(Subdomain(
            rank=r, Npro=nparts, N=int(rows.size), NB=NB, NONZ=len(A), A=A,
            Acol=np.array(Acol, np.int32), Arow=np.array(Arow + [0], np.int32),
            Adia=np.array(Adia, np.int32), Ab=Ab, b=s.b[rows].copy(),
            x=np.zeros(NB + 1 + rows.size), NBBs=NBBs, NBBe=NBBe, BufInd=BufInd, rows=rows))
    return subs
