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
    "side_c", "structured_levels",
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
    c1: np.ndarray
    c2: np.ndarray
    pos12: np.ndarray
    pos21: np.ndarray
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


def _cross(a, b):
    return np.stack([
        a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
        a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
        a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0],
    ], axis=-1)


def _dot(a, b):
    return np.einsum("...i,...i->...", a, b)


def box_geometry(nx, ny, nz, h=1.0, perturb=0.0, rng=None):
    """Node, face and cell geometry of a (perturbed) hex box.

    Nodes are displaced by ``uniform(-perturb*h, perturb*h)`` per coordinate.
    Face area vectors are ``0.5 * (c - a) x (d - b)`` for the quad a-b-c-d,
    oriented along +x, +y, +z; cell volumes come from the divergence theorem.
    Returns a dict with node array ``P`` (nz+1, ny+1, nx+1, 3), face arrays
    ``Sx, Sy, Sz`` and face centres ``Fx, Fy, Fz``, cell centres ``C`` and
    volumes ``V`` (nz, ny, nx).
    """
    z, y, x = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1),
                          indexing="ij")
    P = np.stack([x, y, z], axis=-1).astype(np.float64) * h
    del x, y, z
    if perturb > 0.0:
        P += rng.uniform(-perturb * h, perturb * h, size=P.shape)
    # x-faces on node plane i: a=(k,j), b=(k,j+1), c=(k+1,j+1), d=(k+1,j)
    a, b_, c, d = P[:-1, :-1, :], P[:-1, 1:, :], P[1:, 1:, :], P[1:, :-1, :]
    Sx = 0.5 * _cross(c - a, d - b_)
    Fx = 0.25 * (a + b_ + c + d)
    # y-faces on node plane j: a=(k,i), b=(k+1,i), c=(k+1,i+1), d=(k,i+1)
    a, b_, c, d = P[:-1, :, :-1], P[1:, :, :-1], P[1:, :, 1:], P[:-1, :, 1:]
    Sy = 0.5 * _cross(c - a, d - b_)
    Fy = 0.25 * (a + b_ + c + d)
    # z-faces on node plane k: a=(j,i), b=(j,i+1), c=(j+1,i+1), d=(j+1,i)
    a, b_, c, d = P[:, :-1, :-1], P[:, :-1, 1:], P[:, 1:, 1:], P[:, 1:, :-1]
    Sz = 0.5 * _cross(c - a, d - b_)
    Fz = 0.25 * (a + b_ + c + d)
    del a, b_, c, d
    C = 0.125 * (P[:-1, :-1, :-1] + P[:-1, :-1, 1:] + P[:-1, 1:, :-1] + P[:-1, 1:, 1:]
                 + P[1:, :-1, :-1] + P[1:, :-1, 1:] + P[1:, 1:, :-1] + P[1:, 1:, 1:])
    fx, fy, fz = _dot(Fx, Sx), _dot(Fy, Sy), _dot(Fz, Sz)
    V = (fx[:, :, 1:] - fx[:, :, :-1] + fy[:, 1:, :] - fy[:, :-1, :]
         + fz[1:, :, :] - fz[:-1, :, :]) / 3.0
    return dict(P=P, Sx=Sx, Sy=Sy, Sz=Sz, Fx=Fx, Fy=Fy, Fz=Fz, C=C, V=V)


def _interior_faces(nx, ny, nz, slot, geo):
    """Interior faces in SideC order with SidAij positions and geometry."""
    N = nx * ny * nz
    cell = np.arange(N, dtype=np.int64).reshape(nz, ny, nx)
    C = geo["C"]
    out = []
    for axis, off, sl_lo, sl_hi, S in (
        (0, 1, (slice(None), slice(None), slice(0, nx - 1)),
         (slice(None), slice(None), slice(1, nx)), geo["Sx"][:, :, 1:nx]),
        (1, nx, (slice(None), slice(0, ny - 1), slice(None)),
         (slice(None), slice(1, ny), slice(None)), geo["Sy"][:, 1:ny, :]),
        (2, nx * ny, (slice(0, nz - 1), slice(None), slice(None)),
         (slice(1, nz), slice(None), slice(None)), geo["Sz"][1:nz, :, :]),
    ):
        c1 = cell[sl_lo].ravel()
        c2 = c1 + off
        d = (C[sl_hi] - C[sl_lo]).reshape(-1, 3)
        S = S.reshape(-1, 3)
        out.append((c1, c2, slot[(axis, 1)][c1], slot[(axis, -1)][c2], S, d))
    cat = lambda n: np.concatenate([o[n] for o in out])  # noqa: E731
    return cat(0), cat(1), cat(2).astype(np.int64) - 1, cat(3).astype(np.int64) - 1, cat(4), cat(5)


def _wall_faces(nx, ny, nz, geo):
    """Boundary faces (x-min, x-max, y-min, y-max, z-min, z-max) with the
    adjacent cell, outward area vector and centre-to-face vector."""
    N = nx * ny * nz
    cell = np.arange(N, dtype=np.int64).reshape(nz, ny, nx)
    C = geo["C"]
    res = []
    for S, F, cidx, sign in (
        (geo["Sx"][:, :, 0], geo["Fx"][:, :, 0], cell[:, :, 0], -1.0),
        (geo["Sx"][:, :, nx], geo["Fx"][:, :, nx], cell[:, :, nx - 1], 1.0),
        (geo["Sy"][:, 0, :], geo["Fy"][:, 0, :], cell[:, 0, :], -1.0),
        (geo["Sy"][:, ny, :], geo["Fy"][:, ny, :], cell[:, ny - 1, :], 1.0),
        (geo["Sz"][0], geo["Fz"][0], cell[0], -1.0),
        (geo["Sz"][nz], geo["Fz"][nz], cell[nz - 1], 1.0),
    ):
        c = cidx.ravel()
        Sout = sign * S.reshape(-1, 3)
        d = F.reshape(-1, 3) - C.reshape(-1, 3)[c]
        res.append((c, Sout, d))
    return (np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res]),
            np.concatenate([r[2] for r in res]))


def side_c(nx, ny, nz):
    """The face list as the reference stores it: SideC(2,NS), 1-based cells,
    boundary faces with negative second cell (-1, -2, ...)."""
    Acol, Arow, Adia, slot = box_csr(nx, ny, nz)
    geo = dict(C=np.zeros((nz, ny, nx, 3)), Sx=np.zeros((nz, ny, nx + 1, 3)),
               Sy=np.zeros((nz, ny + 1, nx, 3)), Sz=np.zeros((nz + 1, ny, nx, 3)),
               Fx=np.zeros((nz, ny, nx + 1, 3)), Fy=np.zeros((nz, ny + 1, nx, 3)),
               Fz=np.zeros((nz + 1, ny, nx, 3)))
    c1, c2, p12, p21, _, _ = _interior_faces(nx, ny, nz, slot, geo)
    cw, _, _ = _wall_faces(nx, ny, nz, geo)
    nb = cw.shape[0]
    sc = np.empty((c1.shape[0] + nb, 2), np.int32)
    sc[: c1.shape[0], 0] = c1 + 1
    sc[: c1.shape[0], 1] = c2 + 1
    sc[c1.shape[0]:, 0] = cw + 1
    sc[c1.shape[0]:, 1] = -np.arange(1, nb + 1)
    sid = np.zeros((sc.shape[0], 2), np.int32)
    sid[: c1.shape[0], 0] = p12 + 1
    sid[: c1.shape[0], 1] = p21 + 1
    return sc, (Acol, Arow, Adia, sid)


def _smooth_field(shape, sigma, rng):
    from scipy.ndimage import gaussian_filter
    f = rng.standard_normal(shape)
    return gaussian_filter(f, sigma=sigma, mode="wrap")


def _density(shape, rng, lo=0.14, hi=1.0, sigma=3.0):
    f = _smooth_field(shape, sigma, rng)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-300)
    return lo + (hi - lo) * f


def _assemble(N, NONZ, Adia, c1, c2, pos12, pos21, a12_off, a21_off, d1_add, d2_add,
              diag_extra):
    A = np.zeros(NONZ, np.float64)
    A[pos12] = -a12_off
    A[pos21] = -a21_off
    diag = np.zeros(N, np.float64)
    diag += np.bincount(c1, weights=d1_add, minlength=N)
    diag += np.bincount(c2, weights=d2_add, minlength=N)
    diag += diag_extra
    A[Adia.astype(np.int64) - 1] = diag
    return A


def pressure_system(nx, ny, nz, perturb=0.0, seed=0, variable_density=False,
                    rel_tol=1e-8, name=None):
    """Pressure-correction matrix (Process/CalcPS.f90:77-102 pattern).

    A12 = |S|^2/(S.d) (divided by the harmonic face density when
    ``variable_density``); Neumann walls; cell 1 gets a Dirichlet face (its
    x-min wall coefficient added to the diagonal).  RHS ~ uniform[-1, 1]
    (``numpy.random.default_rng(seed)``), mean removed; x0 = 0.
    Random draws in order: node perturbation, density field, RHS.
    """
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    Acol, Arow, Adia, slot = box_csr(nx, ny, nz)
    NONZ = int(Arow.shape[0])
    geo = box_geometry(nx, ny, nz, perturb=perturb, rng=rng)
    c1, c2, p12, p21, S, d = _interior_faces(nx, ny, nz, slot, geo)
    g = _dot(S, S) / _dot(S, d)
    if variable_density:
        rho = _density((nz, ny, nx), rng).ravel()
        inv_rho_f = 0.5 * (1.0 / rho[c1] + 1.0 / rho[c2])
    else:
        rho = np.ones(N)
        inv_rho_f = np.ones_like(g)
    coef = g * inv_rho_f
    cw, Sw, dw = _wall_faces(nx, ny, nz, geo)
    NB = int(cw.shape[0])
    diag_extra = np.zeros(N)
    # Dirichlet face: the first wall face (x-min) of cell 1.
    gw0 = float(_dot(Sw[0], Sw[0]) / _dot(Sw[0], dw[0]))
    diag_extra[cw[0]] += gw0 / rho[cw[0]]
    A = _assemble(N, NONZ, Adia, c1, c2, p12, p21, coef, coef, coef, coef, diag_extra)
    b = rng.uniform(-1.0, 1.0, N)
    b -= b.mean()
    x = np.zeros(NB + N + 1)
    return System(
        name=name or f"pressure{'-vd' if variable_density else ''}-{nx}x{ny}x{nz}",
        shape=(nx, ny, nz), N=N, NB=NB, NONZ=NONZ, A=A, Acol=Acol, Arow=Arow,
        Adia=Adia, Ab=np.zeros(NB), b=b, x=x, c1=c1, c2=c2, pos12=p12, pos21=p21,
        symmetric=True, rel_tol=rel_tol, face_coef=coef, fixed_diag=diag_extra)


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
    Acol, Arow, Adia, slot = box_csr(nx, ny, nz)
    NONZ = int(Arow.shape[0])
    geo = box_geometry(nx, ny, nz, perturb=perturb, rng=rng)
    P = geo["P"]
    psi = np.stack([_smooth_field(P.shape[:3], sigma, rng) for _ in range(3)], axis=-1)
    psi[0] = psi[-1] = 0.0
    psi[:, 0] = psi[:, -1] = 0.0
    psi[:, :, 0] = psi[:, :, -1] = 0.0

    def circ(a, b_, c, d, pa, pb, pc, pd):
        return (_dot(0.5 * (pa + pb), b_ - a) + _dot(0.5 * (pb + pc), c - b_)
                + _dot(0.5 * (pc + pd), d - c) + _dot(0.5 * (pd + pa), a - d))

    # Same quad orderings as box_geometry, so the circulation is the flux
    # through the oriented area vector (Stokes).
    Gx = circ(P[:-1, :-1, :], P[:-1, 1:, :], P[1:, 1:, :], P[1:, :-1, :],
              psi[:-1, :-1, :], psi[:-1, 1:, :], psi[1:, 1:, :], psi[1:, :-1, :])
    Gy = circ(P[:-1, :, :-1], P[1:, :, :-1], P[1:, :, 1:], P[:-1, :, 1:],
              psi[:-1, :, :-1], psi[1:, :, :-1], psi[1:, :, 1:], psi[:-1, :, 1:])
    Gz = circ(P[:, :-1, :-1], P[:, :-1, 1:], P[:, 1:, 1:], P[:, 1:, :-1],
              psi[:, :-1, :-1], psi[:, :-1, 1:], psi[:, 1:, 1:], psi[:, 1:, :-1])
    del psi
    F = np.concatenate([Gx[:, :, 1:nx].ravel(), Gy[:, 1:ny, :].ravel(), Gz[1:nz].ravel()])
    c1, c2, p12, p21, S, d = _interior_faces(nx, ny, nz, slot, geo)
    area = np.sqrt(_dot(S, S))
    rms = math.sqrt(float(np.mean((F / area) ** 2))) if F.size else 1.0
    F = F / max(rms, 1e-300)
    if variable_density:
        rho = _density((nz, ny, nx), rng).ravel()
    else:
        rho = np.ones(N)
    A0 = nu * _dot(S, S) / _dot(S, d)
    a12 = np.maximum(-F, 0.0)
    a21 = np.maximum(F, 0.0)
    D12 = A0 / rho[c2]
    D21 = A0 / rho[c1]
    cw, Sw, dw = _wall_faces(nx, ny, nz, geo)
    NB = int(cw.shape[0])
    V = geo["V"].ravel()
    diag_extra = np.zeros(N, np.float64)
    diag_extra += np.bincount(cw, weights=nu * _dot(Sw, Sw) / _dot(Sw, dw) / rho[cw],
                              minlength=N)
    diag_extra += rho * V / dt
    A = _assemble(N, NONZ, Adia, c1, c2, p12, p21, a12 + D12, a21 + D21, a21 + D21,
                  a12 + D12, diag_extra)
    u_old = rng.uniform(-1.0, 1.0, N)
    b = rho * V / dt * u_old
    x = np.zeros(NB + N + 1)
    return System(
        name=name or f"convdiff-{nx}x{ny}x{nz}", shape=(nx, ny, nz), N=N, NB=NB,
        NONZ=NONZ, A=A, Acol=Acol, Arow=Arow, Adia=Adia, Ab=np.zeros(NB), b=b, x=x,
        c1=c1, c2=c2, pos12=p12, pos21=p21, symmetric=False, rel_tol=rel_tol)


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
