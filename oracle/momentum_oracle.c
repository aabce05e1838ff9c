/*
 * ORACLE -- test infrastructure only.  C restatement of the momentum
 * assembly of T-FlowS, Process/NewUVW.f90:138-499 (one component Ui of
 * rho*u): the CalMinMax bounds when a material blends (CalMinMax.f90:20-36),
 * the convection face loop with the blended face values of ConvScheme.f90
 * and the upwind sums, the explicit convection term, the diffusion face loop
 * that fills Aval through Adia and SidAij, b and Abou, the cross-diffusion,
 * inertial (two or three time levels) and pressure terms and the
 * under-relaxation of the diagonal.  Statement order, loop order and the
 * left-to-right evaluation of every expression follow the source; compiled
 * with -ffp-contract=off like the solver restatement.  Only tests/ use it,
 * to compare the GPU momentum assembly against.
 *
 * MIN and MAX take the first argument unless a later one is strictly
 * smaller (larger), as the statement-by-statement execution of the
 * reference's text does; the Fortran standard leaves the result for equal
 * signed zeros and NaN arguments to the compiler.
 *
 * Parity pin: tests/golden/momentum_*.npz hold the outputs of the
 * reference's own source text of those lines executed statement by statement
 * (tests/golden/make_golden_momentum.py); tests/test_oracle_golden.py
 * requires this file to reproduce them bit for bit.
 *
 * Not restated: the old-value shift `if (ini == 1)` (NewUVW.f90:153-156;
 * the caller passes Ui % o and Ui % oo as they are after it) and the source
 * term (:177-199, test-problem functions; the caller passes Ui % source).
 *
 * Array conventions: cell arrays (-NbC:NC) are passed at element -NbC;
 * b and Asave are (1:NC); Abou (-NbC:-1) at -NbC; face arrays (1:NS);
 * SideC(0:2,NS) and SidAij(2,NS) in column-major order; Adia 1-based into
 * Aval(1:NONZ); material arrays (1:Nmat).
 *
 * iopt = {Nmat, var, Moin_Problem, CONVEC, CROSS, DIFFUS, INERT}
 * dopt = {VISc, dt, U % URF}
 * face_vec = {Si, Sj, Sk, Di, Dj, Dk}   face = {Flux_u, Flux, fF, Scoef}
 * cell = {Rho%n, Rho%o, Rho%oo, Ui%n, Ui%o, Ui%oo, dUidi, dUidj, dUidk,
 *         dUjdi, dUkdi, dUjdj, dUkdk, Pi, Ui%source}
 * *status: 0, 1 = a face whose blending code is undefined in ConvScheme
 * (one material YES, the other NO: the reference reads an unset Phij),
 * 2 = a material index outside 1..Nmat.
 */
#include <stdlib.h>

/* Library/allp_mod.f90:16-24 */
enum { INFLOW = 1, WALL = 2, OUTFLOW = 3, CONVECT = 5, WALLFL = 6, BUFFER = 11 };
/* Process/IniPar.f90:22-49 */
enum { CN = 2, FI = 3, LIN = 4, PAR = 5, YES = 10, NO = 11, CDS = 20, QUICK = 21, LUDS = 22,
       MINMOD = 23, SMART = 24, AVL_SMART = 25, SUPERBEE = 26, GAMMA = 27 };

#define CELL(a, c) ((a)[(c) + NbC])

static double min2(double a, double b) { return b < a ? b : a; }
static double max2(double a, double b) { return b > a ? b : a; }

struct conv_ctx {
    int NbC;
    const int *SideC;
    const double *Flux, *f, *PhiMax, *PhiMin;
};

/* ConvScheme.f90:52-135 for face s (1-based).  Returns 1 when blenda is
 * none of the codes the routine handles. */
static int conv_scheme(const struct conv_ctx *x, double *Phis, int s, const double *Phi,
                       const double *dPhidi, const double *dPhidj, const double *dPhidk,
                       const double *Di, const double *Dj, const double *Dk, int blenda)
{
    const int NbC = x->NbC, i = s - 1;
    const int c1 = x->SideC[3 * i + 1], c2 = x->SideC[3 * i + 2];
    double fj, sign, PhiUstar, Phij = 0.0;
    int C, D;
    if (x->Flux[i] > 0.0) {
        fj = 1.0 - x->f[i];
        C = c1;
        D = c2;
        sign = +1.0;
    } else {
        fj = x->f[i];
        C = c2;
        D = c1;
        sign = -1.0;
    }
    if (x->Flux[i] > 0.0)
        PhiUstar = CELL(Phi, D) - 2.0 * (CELL(dPhidi, C) * Di[i] + CELL(dPhidj, C) * Dj[i] +
                                         CELL(dPhidk, C) * Dk[i]);
    else
        PhiUstar = CELL(Phi, D) + 2.0 * (CELL(dPhidi, C) * Di[i] + CELL(dPhidj, C) * Dj[i] +
                                         CELL(dPhidk, C) * Dk[i]);
    const double PhiU = max2(CELL(x->PhiMin, C), min2(PhiUstar, CELL(x->PhiMax, C)));
    double rj = (CELL(Phi, C) - PhiU) / (CELL(Phi, D) - CELL(Phi, C) + 1.0e-16);
    const double gD = 0.5 * fj * (1.0 + fj);
    const double gU = 0.5 * fj * (1.0 - fj);
    if (blenda == CDS) {
        Phij = fj;
    } else if (blenda == QUICK) {
        rj = (CELL(Phi, C) - PhiU) / (CELL(Phi, D) - CELL(Phi, C) + 1.0e-12);
        const double alfa = 0.0;
        Phij = (gD - alfa) + (gU + alfa) * rj;
    } else if (blenda == LUDS) {
        const double alfa = 0.5 * fj * (1.0 + fj);
        Phij = (gD - alfa) + (gU + alfa) * rj;
    } else if (blenda == MINMOD) {
        Phij = fj * max2(0.0, min2(rj, 1.0));
    } else if (blenda == SMART) {
        const double beta1 = 3.0, beta2 = 1.0;
        Phij = max2(0.0, min2(min2((beta1 - 1.0) * rj, gD + gU * rj), beta2));
    } else if (blenda == AVL_SMART) {
        const double beta1 = 1.0 + fj * (2.0 + fj);
        const double beta2 = fj * (2.0 - fj);
        Phij = max2(0.0, min2(min2((beta1 - 1.0) * rj, gD + gU * rj), beta2));
    } else if (blenda == SUPERBEE) {
        Phij = 0.5 * max2(max2(0.0, min2(2.0 * rj, 1.0)), min2(rj, 2.0));
    } else if (blenda == YES) {
        return 0;
    } else if (blenda != GAMMA) {
        return 1;
    }
    if (blenda != GAMMA) {
        *Phis = CELL(Phi, C) + Phij * sign * (CELL(Phi, c2) - CELL(Phi, c1));
        return 0;
    }
    /* GAMMA (:111-133): the value above is overwritten in every branch */
    const double Beta = 0.1;
    const double den = 2.0 * (CELL(dPhidi, C) * Di[i] + CELL(dPhidj, C) * Dj[i] +
                              CELL(dPhidk, C) * Dk[i]);
    if (x->Flux[i] > 0.0)
        PhiUstar = 1.0 - (CELL(Phi, D) - CELL(Phi, C)) / den;
    else
        PhiUstar = 1.0 + (CELL(Phi, D) - CELL(Phi, C)) / den;
    const double GammaC = PhiUstar / Beta;
    if (PhiUstar < Beta && PhiUstar > 0.0)
        *Phis = (1.0 - GammaC * (1.0 - x->f[i])) * CELL(Phi, C) +
                GammaC * (1.0 - x->f[i]) * CELL(Phi, D);
    else if (PhiUstar < 1.0 && PhiUstar >= Beta)
        *Phis = x->f[i] * CELL(Phi, C) + (1.0 - x->f[i]) * CELL(Phi, D);
    else
        *Phis = CELL(Phi, C);
    return 0;
}

void oracle_newuvw_assembly(int NC, int NbC, int NS, int NONZ, const int *iopt,
                            const double *dopt, const int *SideC, const int *SidAij,
                            const int *Adia, const int *TypeBC, const int *material,
                            const int *BLEND, const int *BLEND_TEM, const double *URFC,
                            const double *f, const double *volume,
                            const double *const *face_vec, const double *const *face,
                            const double *const *cell, double *Aval, double *b, double *Abou,
                            double *Asave, double *rhoUi, int *status)
{
    const int Nmat = iopt[0], var = iopt[1], moin = iopt[2], CONVEC = iopt[3],
              CROSS = iopt[4], DIFFUS = iopt[5], INERT = iopt[6];
    const double VISc = dopt[0], dt = dopt[1], URF = dopt[2];
    const double *Si = face_vec[0], *Sj = face_vec[1], *Sk = face_vec[2];
    const double *Di = face_vec[3], *Dj = face_vec[4], *Dk = face_vec[5];
    const double *Flux_u = face[0], *Flux = face[1], *fF = face[2], *Scoef = face[3];
    const double *rho_n = cell[0], *rho_o = cell[1], *rho_oo = cell[2], *ui_o = cell[4],
                 *ui_oo = cell[5], *dUidi = cell[6], *dUidj = cell[7], *dUidk = cell[8],
                 *dUjdi = cell[9], *dUkdi = cell[10], *dUjdj = cell[11], *dUkdk = cell[12],
                 *Pi = cell[13], *source = cell[14];
    const int ncell = NbC + NC + 1;
    double *C = calloc((size_t)ncell, sizeof(double));
    double *X = calloc((size_t)ncell, sizeof(double));
    double *PhiMax = calloc((size_t)ncell, sizeof(double));
    double *PhiMin = calloc((size_t)ncell, sizeof(double));
    *status = 0;
    for (int s = 0; s < NS; ++s)
        for (int k = 1; k <= 2; ++k) {
            const int m = CELL(material, SideC[3 * s + k]);
            if (m < 1 || m > Nmat) *status = 2;
        }
    for (int c = 1; c <= NC; ++c)
        if (CELL(material, c) < 1 || CELL(material, c) > Nmat) *status = 2;
    if (*status) goto done;

    /* rhoUi = Rho % n * Ui % n (:138) */
    for (int c = -NbC; c <= NC; ++c) CELL(rhoUi, c) = CELL(rho_n, c) * CELL(cell[3], c);
    for (int c = 0; c < NbC; ++c) Abou[c] = 0.0; /* :146 */
    for (int k = 0; k < NONZ; ++k) Aval[k] = 0.0; /* :148 */
    for (int c = 0; c < NC; ++c) b[c] = 0.0;      /* :149 */

    /* :167-173: CalMinMax(rhoUi) when any material blends */
    for (int mat = 1; mat <= Nmat; ++mat)
        if (BLEND[mat - 1] != NO) {
            for (int c = -NbC; c <= NC; ++c) {
                CELL(PhiMax, c) = CELL(rhoUi, c);
                CELL(PhiMin, c) = CELL(rhoUi, c);
            }
            for (int s = 0; s < NS; ++s) {
                const int c1 = SideC[3 * s + 1], c2 = SideC[3 * s + 2];
                if (c2 > 0 || (c2 < 0 && CELL(TypeBC, c2) == BUFFER)) {
                    CELL(PhiMax, c1) = max2(CELL(PhiMax, c1), CELL(rhoUi, c2));
                    CELL(PhiMin, c1) = min2(CELL(PhiMin, c1), CELL(rhoUi, c2));
                    CELL(PhiMax, c2) = max2(CELL(PhiMax, c2), CELL(rhoUi, c1));
                    CELL(PhiMin, c2) = min2(CELL(PhiMin, c2), CELL(rhoUi, c1));
                }
            }
            break;
        }
    /* Ui % C = 0.0, Ui % X = 0.0 (:175-176): calloc */
    const struct conv_ctx cx = {NbC, SideC, Flux, f, PhiMax, PhiMin};

    /* convection (:205-236) */
    for (int s = 1; s <= NS; ++s) {
        const int i = s - 1;
        const int c1 = SideC[3 * i + 1], c2 = SideC[3 * i + 2];
        const int m1 = CELL(material, c1), m2 = CELL(material, c2);
        double rhoUiS = f[i] * CELL(rhoUi, c1) + (1.0 - f[i]) * CELL(rhoUi, c2);
        if (BLEND[m1 - 1] != NO || BLEND[m2 - 1] != NO) {
            const int blenda = BLEND[m1 - 1] > BLEND[m2 - 1] ? BLEND[m1 - 1] : BLEND[m2 - 1];
            if (conv_scheme(&cx, &rhoUiS, s, rhoUi, dUidi, dUidj, dUidk, Di, Dj, Dk, blenda)) {
                *status = 1;
                goto done;
            }
        }
        if (c2 > 0) {
            CELL(C, c1) = CELL(C, c1) - Flux_u[i] * rhoUiS;
            CELL(C, c2) = CELL(C, c2) + Flux_u[i] * rhoUiS;
        } else {
            CELL(C, c1) = CELL(C, c1) - Flux_u[i] * rhoUiS;
        }
        if (BLEND_TEM[m1 - 1] != NO || BLEND_TEM[m2 - 1] != NO) {
            if (Flux_u[i] < 0) {
                CELL(X, c1) = CELL(X, c1) - Flux_u[i] * CELL(rhoUi, c2);
                if (c2 > 0) CELL(X, c2) = CELL(X, c2) + Flux_u[i] * CELL(rhoUi, c2);
            } else {
                CELL(X, c1) = CELL(X, c1) - Flux_u[i] * CELL(rhoUi, c1);
                if (c2 > 0) CELL(X, c2) = CELL(X, c2) + Flux_u[i] * CELL(rhoUi, c1);
            }
        }
    }
    /* :250-255 */
    if (CONVEC == FI)
        for (int c = 1; c <= NC; ++c)
            b[c - 1] = b[c - 1] + URFC[CELL(material, c) - 1] * (CELL(C, c) - CELL(X, c));
    for (int c = 1; c <= NC; ++c) CELL(X, c) = 0.0; /* :262-264 */

    /* diffusion (:276-416) */
    for (int s = 1; s <= NS; ++s) {
        const int i = s - 1;
        double A12 = 0.0, A21 = 0.0, D12 = 0.0, D21 = 0.0;
        const int c1 = SideC[3 * i + 1], c2 = SideC[3 * i + 2];
        const double RhoS = fF[i] * CELL(rho_n, c1) + (1.0 - fF[i]) * CELL(rho_n, c2);
        const double VISeff = moin == 4 ? VISc * RhoS : VISc;
        const double dUidiS = fF[i] * CELL(dUidi, c1) + (1.0 - fF[i]) * CELL(dUidi, c2);
        const double dUidjS = fF[i] * CELL(dUidj, c1) + (1.0 - fF[i]) * CELL(dUidj, c2);
        const double dUidkS = fF[i] * CELL(dUidk, c1) + (1.0 - fF[i]) * CELL(dUidk, c2);
        const double dUjdiS = fF[i] * CELL(dUjdi, c1) + (1.0 - fF[i]) * CELL(dUjdi, c2);
        const double dUkdiS = fF[i] * CELL(dUkdi, c1) + (1.0 - fF[i]) * CELL(dUkdi, c2);
        const double dUjdjS = fF[i] * CELL(dUjdj, c1) + (1.0 - fF[i]) * CELL(dUjdj, c2);
        const double dUkdkS = fF[i] * CELL(dUkdk, c1) + (1.0 - fF[i]) * CELL(dUkdk, c2);
        const double Fex = VISeff * (4.0 / 3.0 * dUidiS * Si[i] + (dUidjS + dUjdiS) * Sj[i] +
                                     (dUidkS + dUkdiS) * Sk[i] -
                                     2.0 / 3.0 * (dUjdjS + dUkdkS) * Si[i]);
        const double A0 = VISeff * Scoef[i];
        const double Fim = A0 * (dUidiS * Di[i] + dUidjS * Dj[i] + dUidkS * Dk[i]);
        CELL(X, c1) = CELL(X, c1) + Fex - Fim;
        if (c2 > 0) CELL(X, c2) = CELL(X, c2) - Fex + Fim;
        if (DIFFUS == CN || DIFFUS == FI) {
            if (DIFFUS == FI) {
                D12 = D12 + A0 / CELL(rho_n, c2);
                D21 = D21 + A0 / CELL(rho_n, c1);
            }
            const int m1 = CELL(material, c1), m2 = CELL(material, c2);
            if (BLEND[m1 - 1] != NO || BLEND[m2 - 1] != NO) {
                A12 = A12 - min2(Flux_u[i], 0.0);
                A21 = A21 + max2(Flux_u[i], 0.0);
            }
            const int d1 = Adia[c1 - 1] - 1;
            if (c2 > 0) {
                const int d2 = Adia[c2 - 1] - 1;
                const int s1 = SidAij[2 * i] - 1, s2 = SidAij[2 * i + 1] - 1;
                Aval[d1] = Aval[d1] + A21 + D21;
                Aval[s2] = Aval[s2] - A21 - D21;
                Aval[d2] = Aval[d2] + A12 + D12;
                Aval[s1] = Aval[s1] - A12 - D12;
            } else if (c2 < 0) {
                const int t = CELL(TypeBC, c2);
                if (t == WALL || t == CONVECT || t == INFLOW || t == WALLFL) {
                    Aval[d1] = Aval[d1] + A21 + D21;
                    b[c1 - 1] = b[c1 - 1] + (A12 + D12) * CELL(rhoUi, c2);
                } else if (t == OUTFLOW) {
                    Aval[d1] = Aval[d1] + A21;
                    b[c1 - 1] = b[c1 - 1] + (A12)*CELL(rhoUi, c2);
                } else if (t == BUFFER) {
                    Aval[d1] = Aval[d1] + A21 + D21;
                    Abou[c2 + NbC] = -A12 - D12;
                }
            }
        }
    }
    /* :438-442 */
    if (CROSS == FI)
        for (int c = 1; c <= NC; ++c) b[c - 1] = b[c - 1] + CELL(X, c);
    /* :451-460 */
    if (INERT == LIN) {
        for (int c = 1; c <= NC; ++c)
            Aval[Adia[c - 1] - 1] = Aval[Adia[c - 1] - 1] + CELL(volume, c) / dt;
        for (int c = 1; c <= NC; ++c)
            b[c - 1] = b[c - 1] + CELL(volume, c) / dt * CELL(rho_o, c) * CELL(ui_o, c) +
                       CELL(source, c) * CELL(volume, c);
    }
    if (INERT == PAR) {
        for (int c = 1; c <= NC; ++c)
            Aval[Adia[c - 1] - 1] = Aval[Adia[c - 1] - 1] + 1.5 * CELL(volume, c) / dt;
        for (int c = 1; c <= NC; ++c)
            b[c - 1] = b[c - 1] + 2.0 * CELL(volume, c) / dt * CELL(rho_o, c) * CELL(ui_o, c) -
                       0.5 * CELL(volume, c) / dt * CELL(rho_oo, c) * CELL(ui_oo, c) +
                       CELL(source, c) * CELL(volume, c);
    }
    /* :488 */
    for (int c = 1; c <= NC; ++c) b[c - 1] = b[c - 1] - CELL(Pi, c) * CELL(volume, c);
    /* :497-499 */
    if (var == 1)
        for (int c = 1; c <= NC; ++c) Asave[c - 1] = Aval[Adia[c - 1] - 1];
    for (int c = 1; c <= NC; ++c)
        b[c - 1] = b[c - 1] + Aval[Adia[c - 1] - 1] * (1.0 - URF) * CELL(rhoUi, c) / URF;
    for (int c = 1; c <= NC; ++c) Aval[Adia[c - 1] - 1] = Aval[Adia[c - 1] - 1] / URF;
done:
    free(C);
    free(X);
    free(PhiMax);
    free(PhiMin);
}
