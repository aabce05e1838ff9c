/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.  Nothing in the product path links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it, always as the reference
 * results are compared with or as the timed CPU baseline, never as the thing measured or shipped.
 *
 * A plain-C, statement-by-statement restatement of the Krylov linear-solver
 * path of T-FlowS (FP64, Fortran REAL with -fdefault-real-8):
 *
 *   oracle_prec1   Process/Prec1.f90:45-67   D <- diag | IC(0) pivots | 1
 *   oracle_resid   Process/Resid.f90:28-42   r1 <- r1 - A x  (halo loop empty)
 *   oracle_cg      Process/CG.f90:55-262     preconditioned CG
 *   oracle_bicg    Process/BiCG.f90:43-254   "BiCG" (shadow sequence uses A)
 *   oracle_cgs     Process/CGS.f90:55-337    preconditioned CGS
 *   oracle_topolm  Process/TopolM.f90:24-98  face list -> CSR layout
 *
 * Same loop order, same left-to-right sums, the q/(D+TINY) middle step of the
 * IC apply (TINY = 1e-64, Library/allp_mod.f90:31), the module variable
 * `error` that persists between calls (Library/sol_mod.f90:9; reported as
 * FinRes on the ||b|| < tol early exit), and the Fortran DO-loop exit value
 * (niter_in+1 when not converged).  Compiled with -ffp-contract=off so that no
 * multiply-add is fused (gfortran on x86-64 without -march emits none).
 *
 * Parity pin: the .npz fixtures in tests/golden/ hold outputs of the reference's own Fortran
 * source text executed statement by statement (tests/golden/fortran_subset.py
 * run over Process/{CG,BiCG,CGS,Prec1,Resid}.f90); tests/test_oracle_golden.py
 * requires this file to reproduce them bit for bit.
 *
 * Single-domain run: glosum and Exchng are the identity and the subdomain
 * loops `do sub=1,Npro` have no iterations (Npro = 0 for one rank,
 * Parallel/Double/StaPar.f90:31-34), so the Ab halo terms never contribute.
 * Subdomain run (oracle_set_halo on the calling thread, one thread or
 * process per rank): the halo maps of par_mod (NBBs, NBBe, BufInd as
 * Parallel/Double/BufLoa.f90:35-84 leaves them), Exchng
 * (Parallel/Double/Exchng.f90:26-62: buffer cells take the values of the
 * cells they mirror, then the caller's exchange callback swaps each
 * neighbour's segment, as MPI_SENDRECV_REPLACE does) and glosum (the
 * caller's sum over ranks, Parallel/Double/GloSum.f90) are called where the
 * reference calls them, and the halo loops add Ab(k) p(k) to row BufInd(k)
 * (CG.f90:200-208, BiCG.f90:202-211, CGS.f90:201-208 and :301-308,
 * Resid.f90:36-42).
 *
 * Array conventions follow the Fortran dummies: 1-based Acol/Arow/Adia;
 * x_base points at x(-NB) and Ab_base at Ab(-NB).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TINY 1.0e-64

/* 1-based element access, a(i) in Fortran. */
#define F1(a, i) ((a)[(i) - 1])

/* sol_mod :: error, which outlives a call (Library/sol_mod.f90:9).  One copy
 * per thread: threads stand in for MPI ranks, each with its own module. */
static _Thread_local double s_error = 0.0;

/* par_mod's halo maps and the rank-coupling callbacks of the calling thread.
 * exchange(user, phi, NB): phi points at PHI(-NB); swap each neighbour's
 * segment PHI(NBBe(sub):NBBs(sub)) in place.  glosum(user, v): replace *v by
 * the sum over ranks.  A nonzero return marks the halo as failed. */
typedef int (*halo_exchange_fn)(void *user, double *phi, int NB);
typedef int (*halo_glosum_fn)(void *user, double *value);
typedef struct {
    int on, Npro, NB, failed;
    const int *NBBs, *NBBe; /* NBBs(sub) = NBBs[sub - 1], sub = 1..Npro */
    const int *BufInd;      /* BufInd(k) = BufInd[k + NB], k = -NB..-1 */
    halo_exchange_fn exchange;
    halo_glosum_fn glosum;
    void *user;
} HaloCtx;
static _Thread_local HaloCtx s_halo;

void oracle_set_halo(int Npro, int NB, const int *NBBs, const int *NBBe, const int *BufInd_base,
                     halo_exchange_fn exchange, halo_glosum_fn glosum, void *user)
{
    s_halo.on = 1;
    s_halo.Npro = Npro;
    s_halo.NB = NB;
    s_halo.failed = 0;
    s_halo.NBBs = NBBs;
    s_halo.NBBe = NBBe;
    s_halo.BufInd = BufInd_base;
    s_halo.exchange = exchange;
    s_halo.glosum = glosum;
    s_halo.user = user;
}
void oracle_clear_halo(void) { memset(&s_halo, 0, sizeof(s_halo)); }
int oracle_halo_failed(void) { return s_halo.failed; }

/* Parallel/Double/GloSum.f90 */
static void glosum(double *v)
{
    if (s_halo.on && s_halo.glosum(s_halo.user, v) != 0) s_halo.failed = 1;
}

/* Parallel/Double/Exchng.f90:26-62 on a vector whose buffer part is
 * addressable: F1(phi, k) for k = -NB..N. */
static void exchng(double *phi)
{
    if (!s_halo.on) return;
    for (int sub = 1; sub <= s_halo.Npro; ++sub) {
        const int s0 = s_halo.NBBs[sub - 1], e0 = s_halo.NBBe[sub - 1];
        if (e0 <= s0)
            for (int c2 = s0; c2 >= e0; --c2) F1(phi, c2) = F1(phi, s_halo.BufInd[c2 + s_halo.NB]);
    }
    if (s_halo.exchange(s_halo.user, &F1(phi, -s_halo.NB), s_halo.NB) != 0) s_halo.failed = 1;
}

/* The halo loop after a product: q(BufInd(k)) = q(BufInd(k)) + Ab(k)*p(k),
 * sub ascending, k from NBBs(sub) down to NBBe(sub). */
static void halo_add(double *q, const double *p, const double *Ab_base)
{
    if (!s_halo.on) return;
    for (int sub = 1; sub <= s_halo.Npro; ++sub) {
        const int s0 = s_halo.NBBs[sub - 1], e0 = s_halo.NBBe[sub - 1];
        if (e0 <= s0)
            for (int k = s0; k >= e0; --k) {
                const int i = s_halo.BufInd[k + s_halo.NB];
                F1(q, i) = F1(q, i) + Ab_base[k + s_halo.NB] * F1(p, k);
            }
    }
}

/* Vectors that are exchanged carry the buffer part in front: F1(v, k) is
 * valid for k = -NB..N (NB = 0 leaves the one-domain layout unchanged). */
static double *hvec(int N, int NB) { return (double *)calloc((size_t)N + NB + 2, sizeof(double)) + NB + 1; }
static void hvec_free(double *v, int NB) { free(v - NB - 1); }

void oracle_reset_state(void) { s_error = 0.0; }
double oracle_error_state(void) { return s_error; }

/* Process/Prec1.f90:45-67 */
void oracle_prec1(int N, int NONZ, const double *A, const int *Acol,
                  const int *Arow, const int *Adia, double *D, int prec)
{
    (void)NONZ;
    if (prec == 1) {
        for (int i = 1; i <= N; ++i) F1(D, i) = F1(A, F1(Adia, i));
    } else if (prec == 2) {
        for (int i = 1; i <= N; ++i) {
            double sum1 = F1(A, F1(Adia, i));
            for (int j = F1(Acol, i); j <= F1(Adia, i) - 1; ++j) {
                int k = F1(Arow, j);
                sum1 = sum1 - F1(D, k) * F1(A, j) * F1(A, j);
            }
            F1(D, i) = 1.0 / sum1;
        }
    } else {
        for (int i = 1; i <= N; ++i) F1(D, i) = 1.0;
    }
}

/* Process/Resid.f90:28-42 (the Npro loop is empty for one domain) */
void oracle_resid(int N, int NB, int NONZ, const double *A, const int *Acol,
                  const int *Arow, const double *Ab_base, const double *x_base,
                  double *r1)
{
    (void)NONZ;
    for (int i = 1; i <= N; ++i)
        for (int j = F1(Acol, i); j <= F1(Acol, i + 1) - 1; ++j) {
            int k = F1(Arow, j);
            F1(r1, i) = F1(r1, i) - F1(A, j) * x_base[k + NB];
        }
    /* Resid.f90:36-42: x's buffer cells as the caller left them (no Exchng) */
    if (s_halo.on)
        for (int sub = 1; sub <= s_halo.Npro; ++sub) {
            const int s0 = s_halo.NBBs[sub - 1], e0 = s_halo.NBBe[sub - 1];
            if (e0 <= s0)
                for (int k = s0; k >= e0; --k) {
                    const int i = s_halo.BufInd[k + NB];
                    F1(r1, i) = F1(r1, i) - Ab_base[k + NB] * x_base[k + NB];
                }
        }
}

/* Shared IC(0) apply: forward sweep, q/(D+TINY), backward sweep, in place on
 * q (CG.f90:135-156, BiCG.f90:124-152, CGS.f90:156-177 and :249-270).  The
 * forward sum starts from rhs(i); q(k) for k<i are this sweep's values. */
static void ic_apply(int N, const double *A, const int *Acol, const int *Arow,
                     const int *Adia, const double *D, const double *rhs,
                     double *q)
{
    for (int i = 1; i <= N; ++i) {
        double sum1 = F1(rhs, i);
        for (int j = F1(Acol, i); j <= F1(Adia, i) - 1; ++j) {
            int k = F1(Arow, j);
            sum1 = sum1 - F1(A, j) * F1(q, k);
        }
        F1(q, i) = sum1 * F1(D, i);
    }
    for (int i = 1; i <= N; ++i) F1(q, i) = F1(q, i) / (F1(D, i) + TINY);
    for (int i = N; i >= 1; --i) {
        double sum1 = F1(q, i);
        for (int j = F1(Adia, i) + 1; j <= F1(Acol, i + 1) - 1; ++j) {
            int k = F1(Arow, j);
            sum1 = sum1 - F1(A, j) * F1(q, k);
        }
        F1(q, i) = sum1 * F1(D, i);
    }
}

/* q(i) = sum_j A(j) p(Arow(j)), left to right from 0.0 (CG.f90:193-199) */
static void spmv(int N, const double *A, const int *Acol, const int *Arow,
                 const double *p, double *q)
{
    for (int i = 1; i <= N; ++i) {
        F1(q, i) = 0.0;
        for (int j = F1(Acol, i); j <= F1(Acol, i + 1) - 1; ++j) {
            int k = F1(Arow, j);
            F1(q, i) = F1(q, i) + F1(A, j) * F1(p, k);
        }
    }
}

static double norm2(int N, const double *r)
{
    double e = 0.0;
    for (int i = 1; i <= N; ++i) e = e + F1(r, i) * F1(r, i);
    glosum(&e);
    return sqrt(e);
}

/* Process/CG.f90:55-262 */
void oracle_cg(int N, int NB, int NONZ, const double *A, const int *Acol,
               const int *Arow, const int *Adia, const double *Ab_base,
               double *x_base, double *r1, int prec, int *niter, double tol,
               double *IniRes, double *FinRes)
{
    double *D = calloc((size_t)N + 1, sizeof(double));
    double *p1 = hvec(N, NB);
    double *q1 = calloc((size_t)N + 1, sizeof(double));
    double *x = x_base + NB; /* x[i] == x(i) */
    double rho = 0.0, rhoold = 0.0, alfa, beta, bnrm2;
    int iter;

    oracle_prec1(N, NONZ, A, Acol, Arow, Adia, D, prec);

    bnrm2 = norm2(N, r1);
    if (bnrm2 < tol) {
        iter = 0;
        goto done;
    }

    oracle_resid(N, NB, NONZ, A, Acol, Arow, Ab_base, x_base, r1);

    for (int i = 1; i <= N; ++i) F1(p1, i) = F1(r1, i);

    s_error = norm2(N, r1);
    *IniRes = s_error;
    if (s_error < tol) {
        iter = 0;
        goto done;
    }

    for (iter = 1; iter <= *niter; ++iter) {
        if (prec == 1) {
            for (int i = 1; i <= N; ++i) F1(q1, i) = F1(r1, i) / F1(D, i);
        } else if (prec == 2) {
            ic_apply(N, A, Acol, Arow, Adia, D, r1, q1);
        } else {
            for (int i = 1; i <= N; ++i) F1(q1, i) = F1(r1, i);
        }

        rho = 0.0;
        for (int i = 1; i <= N; ++i) rho = rho + F1(r1, i) * F1(q1, i);
        glosum(&rho);

        if (iter == 1) {
            for (int i = 1; i <= N; ++i) F1(p1, i) = F1(q1, i);
        } else {
            beta = rho / rhoold;
            for (int i = 1; i <= N; ++i) F1(p1, i) = F1(q1, i) + beta * F1(p1, i);
        }

        spmv(N, A, Acol, Arow, p1, q1);
        exchng(p1);
        halo_add(q1, p1, Ab_base);

        alfa = 0.0;
        for (int i = 1; i <= N; ++i) alfa = alfa + F1(p1, i) * F1(q1, i);
        glosum(&alfa);
        alfa = rho / alfa;

        for (int i = 1; i <= N; ++i) {
            x[i] = x[i] + alfa * F1(p1, i);
            F1(r1, i) = F1(r1, i) - alfa * F1(q1, i);
        }

        s_error = norm2(N, r1);
        if (s_error < tol) goto done;

        rhoold = rho;
    }

done:
    *FinRes = s_error;
    *niter = iter;
    free(D);
    hvec_free(p1, NB);
    free(q1);
}

/* Process/BiCG.f90:43-254.  The shadow sequence r2 starts equal to r1 and is
 * multiplied by A (not A^T), exactly as the reference does. */
void oracle_bicg(int N, int NB, int NONZ, const double *A, const int *Acol,
                 const int *Arow, const int *Adia, const double *Ab_base,
                 double *x_base, double *r1, int prec, int *niter, double tol,
                 double *IniRes, double *FinRes)
{
    size_t n1 = (size_t)N + 1;
    double *D = calloc(n1, sizeof(double));
    double *p1 = hvec(N, NB), *p2 = hvec(N, NB);
    double *q1 = calloc(n1, sizeof(double)), *q2 = calloc(n1, sizeof(double));
    double *r2 = calloc(n1, sizeof(double));
    double *x = x_base + NB;
    double rho = 0.0, rhoold = 0.0, alfa, beta, bnrm2;
    int iter;

    oracle_prec1(N, NONZ, A, Acol, Arow, Adia, D, prec);

    bnrm2 = norm2(N, r1);
    if (bnrm2 < tol) {
        iter = 0;
        goto done;
    }

    oracle_resid(N, NB, NONZ, A, Acol, Arow, Ab_base, x_base, r1);

    s_error = norm2(N, r1);
    *IniRes = s_error;
    if (s_error < tol) {
        iter = 0;
        goto done;
    }

    for (int i = 1; i <= N; ++i) F1(r2, i) = F1(r1, i);

    for (iter = 1; iter <= *niter; ++iter) {
        if (prec == 1) {
            for (int i = 1; i <= N; ++i) {
                F1(q1, i) = F1(r1, i) / F1(D, i);
                F1(q2, i) = F1(r2, i) / F1(D, i);
            }
        } else if (prec == 2) {
            /* BiCG.f90:124-152 interleaves the two sweeps row by row; each
             * sequence only reads its own vector, so applying them one after
             * the other gives the same values. */
            ic_apply(N, A, Acol, Arow, Adia, D, r1, q1);
            ic_apply(N, A, Acol, Arow, Adia, D, r2, q2);
        } else {
            for (int i = 1; i <= N; ++i) {
                F1(q1, i) = F1(r1, i);
                F1(q2, i) = F1(r2, i);
            }
        }

        rho = 0.0;
        for (int i = 1; i <= N; ++i) rho = rho + F1(q1, i) * F1(r2, i);
        glosum(&rho);

        if (iter == 1) {
            for (int i = 1; i <= N; ++i) {
                F1(p1, i) = F1(q1, i);
                F1(p2, i) = F1(q2, i);
            }
        } else {
            beta = rho / rhoold;
            for (int i = 1; i <= N; ++i) {
                F1(p1, i) = F1(q1, i) + beta * F1(p1, i);
                F1(p2, i) = F1(q2, i) + beta * F1(p2, i);
            }
        }

        spmv(N, A, Acol, Arow, p1, q1);
        spmv(N, A, Acol, Arow, p2, q2);
        exchng(p1);
        exchng(p2);
        halo_add(q1, p1, Ab_base);
        halo_add(q2, p2, Ab_base);

        alfa = 0.0;
        for (int i = 1; i <= N; ++i) alfa = alfa + F1(p2, i) * F1(q1, i);
        glosum(&alfa);
        alfa = rho / alfa;

        for (int i = 1; i <= N; ++i) {
            x[i] = x[i] + alfa * F1(p1, i);
            F1(r1, i) = F1(r1, i) - alfa * F1(q1, i);
            F1(r2, i) = F1(r2, i) - alfa * F1(q2, i);
        }

        s_error = norm2(N, r1);
        if (s_error < tol) goto done;

        rhoold = rho;
    }

done:
    *FinRes = s_error;
    *niter = iter;
    free(D);
    hvec_free(p1, NB);
    hvec_free(p2, NB);
    free(q1);
    free(q2);
    free(r2);
}

/* Process/CGS.f90:55-337 */
void oracle_cgs(int N, int NB, int NONZ, const double *A, const int *Acol,
                const int *Arow, const int *Adia, const double *Ab_base,
                double *x_base, double *r1, int prec, int *niter, double tol,
                double *IniRes, double *FinRes)
{
    size_t n1 = (size_t)N + 1;
    double *D = calloc(n1, sizeof(double));
    double *p1 = hvec(N, NB), *p2 = hvec(N, NB);
    double *q1 = calloc(n1, sizeof(double)), *q2 = calloc(n1, sizeof(double));
    double *r2 = calloc(n1, sizeof(double));
    double *u1 = calloc(n1, sizeof(double)), *u2 = calloc(n1, sizeof(double));
    double *v2 = calloc(n1, sizeof(double)), *w = calloc(n1, sizeof(double));
    double *x = x_base + NB;
    double rho = 0.0, rhoold = 0.0, alfa, beta, bnrm2;
    int iter;

    oracle_prec1(N, NONZ, A, Acol, Arow, Adia, D, prec);

    bnrm2 = norm2(N, r1);
    if (bnrm2 < tol) {
        iter = 0;
        goto done;
    }

    oracle_resid(N, NB, NONZ, A, Acol, Arow, Ab_base, x_base, r1);

    for (int i = 1; i <= N; ++i) F1(r2, i) = F1(r1, i);

    s_error = norm2(N, r1);
    *IniRes = s_error;
    if (s_error < tol) {
        iter = 0;
        goto done;
    }

    for (iter = 1; iter <= *niter; ++iter) {
        rho = 0.0;
        for (int i = 1; i <= N; ++i) rho = rho + F1(r1, i) * F1(r2, i);
        glosum(&rho);

        if (iter == 1) {
            for (int i = 1; i <= N; ++i) {
                F1(u1, i) = F1(r1, i);
                F1(u2, i) = F1(u1, i);
            }
        } else {
            beta = rho / rhoold;
            for (int i = 1; i <= N; ++i) {
                F1(u1, i) = F1(r1, i) + beta * F1(q1, i);
                F1(u2, i) = F1(u1, i) + beta * (F1(q1, i) + beta * F1(u2, i));
            }
        }

        /* p2 = M^-1 u2 (CGS.f90:145-187) */
        if (prec == 1) {
            for (int i = 1; i <= N; ++i) F1(p2, i) = F1(u2, i) / F1(D, i);
        } else if (prec == 2) {
            ic_apply(N, A, Acol, Arow, Adia, D, u2, p2);
        } else {
            for (int i = 1; i <= N; ++i) F1(p2, i) = F1(u2, i);
        }

        /* v2 = A p2 (CGS.f90:193-200; the stray alfa sum at :199 is
         * overwritten at :215 and changes nothing) */
        spmv(N, A, Acol, Arow, p2, v2);
        exchng(p2);
        halo_add(v2, p2, Ab_base);

        alfa = 0.0;
        for (int i = 1; i <= N; ++i) alfa = alfa + F1(r2, i) * F1(v2, i);
        glosum(&alfa);
        alfa = rho / alfa;

        for (int i = 1; i <= N; ++i) F1(q1, i) = F1(u1, i) - alfa * F1(v2, i);

        /* p1 = M^-1 (u1 + q1) (CGS.f90:238-280) */
        if (prec == 1) {
            for (int i = 1; i <= N; ++i)
                F1(p1, i) = (F1(u1, i) + F1(q1, i)) / F1(D, i);
        } else if (prec == 2) {
            for (int i = 1; i <= N; ++i) F1(w, i) = F1(u1, i) + F1(q1, i);
            ic_apply(N, A, Acol, Arow, Adia, D, w, p1);
        } else {
            for (int i = 1; i <= N; ++i) F1(p1, i) = F1(u1, i) + F1(q1, i);
        }

        for (int i = 1; i <= N; ++i) x[i] = x[i] + alfa * F1(p1, i);

        spmv(N, A, Acol, Arow, p1, q2);
        exchng(p1);
        halo_add(q2, p1, Ab_base);

        for (int i = 1; i <= N; ++i) F1(r1, i) = F1(r1, i) - alfa * F1(q2, i);

        s_error = norm2(N, r1);
        if (s_error < tol) goto done;

        rhoold = rho;
    }

done:
    *FinRes = s_error;
    *niter = iter;
    free(D);
    hvec_free(p1, NB);
    hvec_free(p2, NB);
    free(q1);
    free(q2);
    free(r2);
    free(u1);
    free(u2);
    free(v2);
    free(w);
}

/* Process/TopolM.f90:24-98: from the face list SideC(2,NS) (c2 <= 0 marks a
 * boundary face) build Acol (N+1), Arow (NONZ), Adia (N) and SidAij(2,NS),
 * all 1-based.  Per row the columns end up in ascending order, as ISORT
 * leaves them.  Returns NONZERO = nnz+1 (the last Arow slot stays 0). */
static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

int oracle_topolm(int NC, int NS, const int *SideC, int *Acol, int *Arow,
                  int *Adia, int *SidAij)
{
    int *stencw = malloc(((size_t)NC + 1) * sizeof(int));
    for (int c = 1; c <= NC; ++c) stencw[c] = 1;
    for (int s = 1; s <= NS; ++s) {
        int c1 = SideC[2 * (s - 1)], c2 = SideC[2 * (s - 1) + 1];
        if (c2 > 0) {
            stencw[c1] += 1;
            stencw[c2] += 1;
        }
    }
    int n = 0;
    for (int c = 1; c <= NC; ++c) n += stencw[c];
    for (int j = 1; j <= n + 1; ++j) F1(Arow, j) = 0;
    F1(Acol, 1) = 1;
    for (int c = 1; c <= NC; ++c) {
        F1(Acol, c + 1) = F1(Acol, c) + stencw[c];
        F1(Arow, F1(Acol, c)) = c;
        stencw[c] = 1;
    }
    for (int s = 1; s <= NS; ++s) {
        int c1 = SideC[2 * (s - 1)], c2 = SideC[2 * (s - 1) + 1];
        if (c2 > 0) {
            F1(Arow, F1(Acol, c1) + stencw[c1]) = c2;
            F1(Arow, F1(Acol, c2) + stencw[c2]) = c1;
            stencw[c1] += 1;
            stencw[c2] += 1;
        }
    }
    for (int c = 1; c <= NC; ++c) {
        qsort(&F1(Arow, F1(Acol, c)), (size_t)stencw[c], sizeof(int), cmp_int);
        for (int j = F1(Acol, c); j <= F1(Acol, c + 1) - 1; ++j)
            if (F1(Arow, j) == c) F1(Adia, c) = j;
    }
    for (int s = 1; s <= NS; ++s) {
        int c1 = SideC[2 * (s - 1)], c2 = SideC[2 * (s - 1) + 1];
        SidAij[2 * (s - 1)] = 0;
        SidAij[2 * (s - 1) + 1] = 0;
        if (c2 > 0) {
            for (int c = F1(Acol, c1); c <= F1(Acol, c1 + 1) - 1; ++c)
                if (F1(Arow, c) == c2) SidAij[2 * (s - 1)] = c;
            for (int c = F1(Acol, c2); c <= F1(Acol, c2 + 1) - 1; ++c)
                if (F1(Arow, c) == c1) SidAij[2 * (s - 1) + 1] = c;
        }
    }
    free(stencw);
    return n + 1;
}
