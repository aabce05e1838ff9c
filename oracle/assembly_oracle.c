/*
 * ORACLE -- test infrastructure only.  C restatement of the pressure-
 * correction assembly of T-FlowS, Process/CalcPS.f90:49-202: the face loop
 * that fills Aval (through SidAij and Adia), Abou, the face mass fluxes and
 * the right-hand side, then the density time-derivative source and the
 * removal of the volume-weighted mean of b.  Statement order, loop order
 * (including the outer `do m = 1, Nmat` loops, which repeat the face loop
 * and the source loop Nmat times) and left-to-right evaluation of every
 * expression follow the source; compiled with -ffp-contract=off like the
 * solver restatement.  Only tests/ use it, to compare the GPU assembly
 * kernels against.
 *
 * Parity pin: tests/golden/assembly_*.npz hold the outputs of the reference's
 * own source text of those lines executed statement by statement
 * (tests/golden/make_golden_assembly.py); tests/test_oracle_golden.py
 * requires this file to reproduce them bit for bit.
 *
 * Array conventions: cell arrays that the reference declares (-NbC:NC) are
 * passed at their element -NbC (index c + NbC); b is (1:NC); Abou is
 * (-NbC:-1) passed at -NbC; face arrays are (1:NS); SideC is SideC(0:2,NS)
 * and SidAij SidAij(2,NS) in Fortran (column-major) order; Adia holds 1-based
 * positions into Aval(1:NONZ).  Boundary-type codes: Library/allp_mod.f90.
 */
#include <math.h>

enum { INFLOW = 1, WALL = 2, OUTFLOW = 3, SYMMETRY = 4, CONVECT = 5, WALLFL = 6,
       BUFFER = 11, PRESSURE = 12 };

/* cell array with bounds (-NbC:NC) */
#define CELL(a, c) ((a)[(c) + NbC])

void oracle_calcps_assembly(int NC, int NbC, int NS, int NONZ, int Nmat, double dt,
                            const int *SideC, const int *SidAij, const int *Adia,
                            const int *TypeBC, const double *Sx, const double *Sy,
                            const double *Sz, const double *Dx, const double *Dy,
                            const double *Dz, const double *f, const double *volume,
                            const double *Asave, const double *rho_n, const double *rho_o,
                            const double *rho_oo, const double *U, const double *V,
                            const double *W, const double *P, const double *Px,
                            const double *Py, const double *Pz, double *Aval, double *b,
                            double *Abou, double *Flux, double *errmax_out)
{
    /* Aval(:) = 0.0, b(:) = 0.0 (CalcPS.f90:49,55) */
    for (int k = 0; k < NONZ; ++k) Aval[k] = 0.0;
    for (int c = 0; c < NC; ++c) b[c] = 0.0;
    for (int m = 1; m <= Nmat; ++m) {
        for (int s = 1; s <= NS; ++s) {
            const int c1 = SideC[3 * (s - 1) + 1], c2 = SideC[3 * (s - 1) + 2];
            const int i = s - 1;
            if (c2 > 0 || (c2 < 0 && CELL(TypeBC, c2) == BUFFER)) {
                const double SMDPN = (Sx[i] * Sx[i] + Sy[i] * Sy[i] + Sz[i] * Sz[i]) /
                                     (Sx[i] * Dx[i] + Sy[i] * Dy[i] + Sz[i] * Dz[i]);
                const double Urs = f[i] * CELL(rho_n, c1) * CELL(U, c1) +
                                   (1.0 - f[i]) * CELL(rho_n, c2) * CELL(U, c2);
                const double Vrs = f[i] * CELL(rho_n, c1) * CELL(V, c1) +
                                   (1.0 - f[i]) * CELL(rho_n, c2) * CELL(V, c2);
                const double Wrs = f[i] * CELL(rho_n, c1) * CELL(W, c1) +
                                   (1.0 - f[i]) * CELL(rho_n, c2) * CELL(W, c2);
                double A12;
                if (c2 > 0) {
                    A12 = 0.5 * SMDPN *
                          (CELL(volume, c1) / CELL(Asave, c1) + CELL(volume, c2) / CELL(Asave, c2));
                    Aval[SidAij[2 * i] - 1] = -A12;
                    Aval[SidAij[2 * i + 1] - 1] = -A12;
                    Aval[Adia[c1 - 1] - 1] = Aval[Adia[c1 - 1] - 1] + A12;
                    Aval[Adia[c2 - 1] - 1] = Aval[Adia[c2 - 1] - 1] + A12;
                } else {
                    A12 = 0.5 * SMDPN *
                          (CELL(volume, c1) / CELL(Asave, c1) + CELL(volume, c2) / CELL(Asave, c2));
                    Aval[Adia[c1 - 1] - 1] = Aval[Adia[c1 - 1] - 1] + A12;
                    Abou[c2 + NbC] = -A12;
                }
                const double dPxi = .5 * (CELL(Px, c1) + CELL(Px, c2)) * Dx[i];
                const double dPyi = .5 * (CELL(Py, c1) + CELL(Py, c2)) * Dy[i];
                const double dPzi = .5 * (CELL(Pz, c1) + CELL(Pz, c2)) * Dz[i];
                Flux[i] = (Urs * Sx[i] + Vrs * Sy[i] + Wrs * Sz[i]) +
                          A12 * (CELL(P, c1) - CELL(P, c2)) + A12 * (dPxi + dPyi + dPzi);
                b[c1 - 1] = b[c1 - 1] - Flux[i];
                if (c2 > 0) b[c2 - 1] = b[c2 - 1] + Flux[i];
            } else {
                const int t = CELL(TypeBC, c2);
                if (t == INFLOW) {
                    const double Urs = f[i] * CELL(rho_n, c1) * CELL(U, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(U, c2);
                    const double Vrs = f[i] * CELL(rho_n, c1) * CELL(V, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(V, c2);
                    const double Wrs = f[i] * CELL(rho_n, c1) * CELL(W, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(W, c2);
                    Flux[i] = (Urs * Sx[i] + Vrs * Sy[i] + Wrs * Sz[i]);
                    b[c1 - 1] = b[c1 - 1] - Flux[i];
                } else if (t == OUTFLOW || t == CONVECT) {
                    const double Urs = f[i] * CELL(rho_n, c1) * CELL(U, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(U, c2);
                    const double Vrs = f[i] * CELL(rho_n, c1) * CELL(V, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(V, c2);
                    const double Wrs = f[i] * CELL(rho_n, c1) * CELL(W, c1) +
                                       (1.0 - f[i]) * CELL(rho_n, c2) * CELL(W, c2);
                    const double SMDPN = (Sx[i] * Sx[i] + Sy[i] * Sy[i] + Sz[i] * Sz[i]) /
                                         (Sx[i] * Dx[i] + Sy[i] * Dy[i] + Sz[i] * Dz[i]);
                    const double A12 = SMDPN * CELL(volume, c1) / CELL(Asave, c1);
                    Aval[Adia[c1 - 1] - 1] = Aval[Adia[c1 - 1] - 1] + A12;
                    Flux[i] = (Urs * Sx[i] + Vrs * Sy[i] + Wrs * Sz[i]);
                    b[c1 - 1] = b[c1 - 1] - Flux[i];
                } else if (t == PRESSURE) {
                    const double Urs = CELL(rho_n, c1) * CELL(U, c1);
                    const double Vrs = CELL(rho_n, c1) * CELL(V, c1);
                    const double Wrs = CELL(rho_n, c1) * CELL(W, c1);
                    Flux[i] = (Urs * Sx[i] + Vrs * Sy[i] + Wrs * Sz[i]);
                    b[c1 - 1] = b[c1 - 1] - Flux[i];
                    const double SMDPN = (Sx[i] * Sx[i] + Sy[i] * Sy[i] + Sz[i] * Sz[i]) /
                                         (Sx[i] * Dx[i] + Sy[i] * Dy[i] + Sz[i] * Dz[i]);
                    const double A12 = SMDPN * CELL(volume, c1) / CELL(Asave, c1);
                    Aval[Adia[c1 - 1] - 1] = Aval[Adia[c1 - 1] - 1] + A12;
                } else {
                    Flux[i] = 0.0;
                }
            }
        }
    }
    /* CalcPS.f90:171-174 */
    double errmax = 0.0;
    for (int c = 1; c <= NC; ++c) errmax = fmax(errmax, fabs(b[c - 1]));
    *errmax_out = errmax;
    /* CalcPS.f90:183-202 */
    double bc_sum = 0.0, vol = 0.0;
    for (int m = 1; m <= Nmat; ++m)
        for (int c = 1; c <= NC; ++c) {
            b[c - 1] = b[c - 1] - CELL(volume, c) / dt *
                                  (1.5 * CELL(rho_n, c) - 2.0 * CELL(rho_o, c) + 0.5 * CELL(rho_oo, c));
            bc_sum = bc_sum + b[c - 1] * CELL(volume, c);
            vol = vol + CELL(volume, c);
        }
    for (int c = 1; c <= NC; ++c) b[c - 1] = b[c - 1] - bc_sum / vol;
}
