/* A C caller of the Fortran-facing entry points, with the array layout a
 * Fortran caller of Process/CG.f90 hands over:
 *
 *   A(1:NONZ), Arow(1:NONZ)   stored entries, NONZ = entries + 1 (TopolM)
 *   Acol(1:N+1), Adia(1:N)    1-based row starts and diagonal positions
 *   x(-NB:N)                  passed by its first element x(-NB); x(0) and
 *                             the boundary part x(-NB:-1) are not the
 *                             solver's to change
 *   Ab(-NB:-1), r1(1:N)       r1 holds b on entry, the residual on exit
 *
 * System: a 7-point variable-coefficient diffusion operator on an
 * nx x ny x nz box in natural numbering, columns ascending in each row,
 * with a Dirichlet coefficient on the x-min wall (symmetric positive
 * definite).  For prec = 1 and 2 it calls tflows_prec1 and checks D bit for
 * bit against the Prec1.f90:43-59 loops restated here, runs tflows_cg from
 * x = 0 and checks the status, IniRes = ||b||, the true residual against
 * the tolerance and that x(-NB:0) is untouched, then checks tflows_resid bit
 * for bit against the Resid.f90:29-35 loop.  Built with -ffp-contract=off
 * so that the restated loops round every product and sum as the reference
 * arithmetic does.
 *
 * Exit status: 0 all checks passed, 3 no CUDA device (the library's
 * TFLOWS_NO_DEVICE), 1 a solver status other than TFLOWS_OK, 4 a check
 * failed.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tflows_krylov.h"

static double coef(int a, int b) {
    /* a smooth positive face coefficient between cells a and b (1-based) */
    return 1.0 + 0.5 * sin(0.37 * (double)(a + b)) * cos(0.11 * (double)(a - b));
}

int main(int argc, char **argv) {
    int nx = argc > 1 ? atoi(argv[1]) : 12;
    int ny = argc > 2 ? atoi(argv[2]) : 10;
    int nz = argc > 3 ? atoi(argv[3]) : 9;
    const int N = nx * ny * nz;
    const int NB = 2 * (nx * ny + ny * nz + nz * nx);

    int entries = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                entries += 1 + (x > 0) + (x < nx - 1) + (y > 0) + (y < ny - 1) + (z > 0) +
                           (z < nz - 1);
    const int NONZ = entries + 1;

    double *A = calloc((size_t)NONZ, sizeof(double));
    int *Arow = calloc((size_t)NONZ, sizeof(int));
    int *Acol = calloc((size_t)N + 1, sizeof(int));
    int *Adia = calloc((size_t)N, sizeof(int));
    double *Ab = calloc((size_t)NB, sizeof(double));
    double *xbuf = calloc((size_t)NB + 1 + N, sizeof(double));
    double *b = calloc((size_t)N, sizeof(double));
    double *r1 = calloc((size_t)N, sizeof(double));
    double *r2 = calloc((size_t)N, sizeof(double));
    double *D = calloc((size_t)N, sizeof(double));
    double *Dref = calloc((size_t)N, sizeof(double));
    if (!A || !Arow || !Acol || !Adia || !Ab || !xbuf || !b || !r1 || !r2 || !D || !Dref) {
        fprintf(stderr, "allocation failed\n");
        return 4;
    }

    /* 1-based CSR in natural numbering, columns ascending */
    int pos = 1;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int i = 1 + x + nx * (y + ny * z);
                int nb[6], n = 0;
                if (z > 0) nb[n++] = i - nx * ny;
                if (y > 0) nb[n++] = i - nx;
                if (x > 0) nb[n++] = i - 1;
                const int lower = n;
                if (x < nx - 1) nb[n++] = i + 1;
                if (y < ny - 1) nb[n++] = i + nx;
                if (z < nz - 1) nb[n++] = i + nx * ny;
                Acol[i - 1] = pos;
                double diag = x == 0 ? 2.0 * coef(i, 0) : 0.0; /* Dirichlet wall */
                for (int k = 0; k < n; ++k) {
                    if (k == lower) {
                        Adia[i - 1] = pos;
                        Arow[pos - 1] = i;
                        ++pos;
                    }
                    const double c = coef(i, nb[k]);
                    Arow[pos - 1] = nb[k];
                    A[pos - 1] = -c;
                    diag += c;
                    ++pos;
                }
                if (lower == n) {
                    Adia[i - 1] = pos;
                    Arow[pos - 1] = i;
                    ++pos;
                }
                A[Adia[i - 1] - 1] = diag;
            }
    Acol[N] = pos;
    if (pos != NONZ) {
        fprintf(stderr, "layout: %d entries written, NONZ %d\n", pos - 1, NONZ);
        return 4;
    }

    /* x(-NB:-1) and x(0) hold markers the solver must leave alone */
    double *x = xbuf; /* x(i) is x[NB + i] */
    for (int k = 0; k < NB; ++k) x[k] = 7.25 + k;
    x[NB] = -3.5;
    for (int k = 0; k < NB; ++k) Ab[k] = 1.0e300; /* serial run: never read */
    unsigned long long s = 12345u;
    double bn = 0.0;
    for (int i = 0; i < N; ++i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        b[i] = (double)(s >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        bn += b[i] * b[i];
    }
    bn = sqrt(bn);

    int failed = 0;
    for (int prec = 1; prec <= 2; ++prec) {
        /* Prec1.f90:43-59 */
        for (int i = 1; i <= N; ++i) {
            if (prec == 1) {
                Dref[i - 1] = A[Adia[i - 1] - 1];
            } else {
                double sum1 = A[Adia[i - 1] - 1];
                for (int j = Acol[i - 1]; j <= Adia[i - 1] - 1; ++j) {
                    const int k = Arow[j - 1];
                    sum1 = sum1 - Dref[k - 1] * A[j - 1] * A[j - 1];
                }
                Dref[i - 1] = 1.0 / sum1;
            }
        }
        tflows_prec1(&N, &NONZ, A, Acol, Arow, Adia, D, &prec);
        int st = tflows_last_status();
        if (st == TFLOWS_NO_DEVICE) {
            printf("prec1: status %d (%s)\n", st, tflows_status_string(st));
            return 3;
        }
        if (st != TFLOWS_OK) {
            printf("prec1: status %d (%s): %s\n", st, tflows_status_string(st), tflows_last_error());
            return 1;
        }
        if (memcmp(D, Dref, (size_t)N * sizeof(double)) != 0) {
            printf("prec %d: D differs from Prec1.f90\n", prec);
            failed = 1;
        }

        for (int i = 1; i <= N; ++i) x[NB + i] = 0.0;
        memcpy(r1, b, (size_t)N * sizeof(double));
        int niter = 2000;
        const double tol = 1e-10 * bn;
        double ini = 0.0, fin = 0.0;
        tflows_cg(&N, &NB, &NONZ, A, Acol, Arow, Adia, Ab, x, r1, &prec, &niter, &tol, &ini, &fin);
        st = tflows_last_status();
        printf("cg prec %d: status %d (%s) niter %d IniRes %.6e FinRes %.6e tol %.6e\n", prec, st,
               tflows_status_string(st), niter, ini, fin, tol);
        if (st != TFLOWS_OK) return 1;

        /* the true residual, and the untouched markers */
        double rn = 0.0;
        for (int i = 1; i <= N; ++i) {
            double acc = b[i - 1];
            for (int j = Acol[i - 1]; j <= Acol[i] - 1; ++j) acc -= A[j - 1] * x[NB + Arow[j - 1]];
            rn += acc * acc;
        }
        rn = sqrt(rn);
        if (!(fin < tol) || !(rn < 1.01 * tol)) {
            printf("prec %d: residual %.6e / recursive %.6e above tol %.6e\n", prec, rn, fin, tol);
            failed = 1;
        }
        if (fabs(ini - bn) > 1e-12 * bn) {
            printf("prec %d: IniRes %.17g, ||b|| %.17g\n", prec, ini, bn);
            failed = 1;
        }
        for (int k = 0; k < NB; ++k)
            if (x[k] != 7.25 + k) {
                printf("prec %d: x(%d) changed\n", prec, k - NB);
                failed = 1;
                break;
            }
        if (x[NB] != -3.5) {
            printf("prec %d: x(0) changed\n", prec);
            failed = 1;
        }

        /* Resid.f90:29-35 on the returned x, bit for bit */
        memcpy(r2, b, (size_t)N * sizeof(double));
        tflows_resid(&N, &NB, &NONZ, A, Acol, Arow, Ab, x, r2);
        if (tflows_last_status() != TFLOWS_OK) return 1;
        for (int i = 1; i <= N; ++i) {
            double ri = b[i - 1];
            for (int j = Acol[i - 1]; j <= Acol[i] - 1; ++j) ri = ri - A[j - 1] * x[NB + Arow[j - 1]];
            if (memcmp(&ri, &r2[i - 1], sizeof(double)) != 0) {
                printf("prec %d: resid row %d differs (%.17g vs %.17g)\n", prec, i, r2[i - 1], ri);
                failed = 1;
                break;
            }
        }
    }
    tflows_finalize();
    printf(failed ? "FAILED\n" : "PASSED\n");
    return failed ? 4 : 0;
}
