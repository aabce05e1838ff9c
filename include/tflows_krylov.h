/*
 * tflows_krylov.h -- C ABI of libtflows_krylov.so, the GB300 (sm_103a)
 * Krylov linear-solver core that replaces the T-FlowS solver subroutines.
 *
 * Legacy entry points keep the Fortran subroutine interfaces unchanged: all
 * arguments by reference, 1-based compressed-row arrays exactly as
 * Process/TopolM.f90 builds them (Acol = row pointers N+1, Arow = column
 * indices, Adia = diagonal positions, NONZ = stored entries + 1), x passed at
 * x(-NB) and Ab at Ab(-NB).  They mirror the reference outputs: x, r1 (the
 * final recursive residual), niter (iterations used, or niter_in+1 when the
 * tolerance was not reached), IniRes, FinRes.  Nothing here aborts the
 * calling process; tflows_last_status() reports what happened.  Ab and the
 * buffer part x(-NB:-1) are read only while a subdomain halo is registered
 * (tflows_set_halo); otherwise the calls are the reference's one-domain run.
 *
 * Every call is synchronous and returns after x and r1 are back in host
 * memory.  The library keeps a per-device context (stream, workspace and a
 * cache of device copies of the matrix topology keyed by its pointers, sizes
 * and a sampled content hash); tflows_finalize() releases it.
 */
#ifndef TFLOWS_KRYLOV_H
#define TFLOWS_KRYLOV_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TFLOWS_OK             0 /* tolerance reached (or an early exit)    */
#define TFLOWS_NOT_CONVERGED  1 /* iteration limit reached                 */
#define TFLOWS_BREAKDOWN      2 /* (p,Ap) or rho vanished (mixed mode)      */
#define TFLOWS_NONFINITE      3 /* residual norm became Inf/NaN            */
#define TFLOWS_TIMEOUT        4 /* a device-side wait exceeded its limit   */
#define TFLOWS_BAD_INPUT      5 /* rejected on the host before any launch  */
#define TFLOWS_CUDA_ERROR     6 /* a CUDA runtime call failed              */
#define TFLOWS_NO_DEVICE      7 /* no CUDA device available                */
#define TFLOWS_UNSUPPORTED    8 /* option combination not implemented      */
#define TFLOWS_HALO_ERROR     9 /* a halo exchange or global-sum callback
                                   returned nonzero (tflows_set_halo)      */

/* ---- methods, precisions, tolerance modes -------------------------------- */
#define TFLOWS_METHOD_CG        0 /* Process/CG.f90                          */
#define TFLOWS_METHOD_BICG      1 /* Process/BiCG.f90 (shadow uses A)        */
#define TFLOWS_METHOD_CGS       2 /* Process/CGS.f90                         */
#define TFLOWS_METHOD_BICG_TRUE 3 /* extension: shadow sequence uses A^T     */

#define TFLOWS_FP64  0 /* reference arithmetic: FP64 throughout, every a*b+c
                          a rounded product then a rounded sum, the diagonal
                          preconditioner a division (as the reference)      */
#define TFLOWS_MIXED 1 /* FP32 inner Krylov solves inside FP64 refinement    */
#define TFLOWS_FP64_FMA 2 /* FP64 throughout with fused multiply-adds and a
                          reciprocal diagonal: the reference's recurrences
                          with about half the FP64 instructions, results
                          that differ from the reference's by rounding only */

#define TFLOWS_TOL_ABSOLUTE 0 /* stop when ||r||_2 < tol (the reference)    */
#define TFLOWS_TOL_RELATIVE 1 /* stop when ||r||_2 < tol * ||b||_2           */

typedef struct tflows_options {
    int precision;       /* TFLOWS_FP64 (default), TFLOWS_MIXED or
                            TFLOWS_FP64_FMA                                 */
    int tol_mode;        /* TFLOWS_TOL_ABSOLUTE (default) or _RELATIVE       */
    double inner_rtol;   /* mixed: FP32 residual reduction between FP64
                            refinements (default 1e-1)                      */
    int inner_maxiter;   /* mixed, restarted: inner iterations per step     */
    int max_refinements; /* mixed, restarted: refinement steps cap          */
    int refine_restart;  /* mixed: 0 = reliable updates (default for CG and
                            BiCG): one FP32 CG stream whose residual is
                            replaced by the FP64 true residual at each
                            refinement, keeping the search direction while
                            the replaced residual had drifted by less than
                            0.3 of its norm; 1 = restart the inner solve at
                            each refinement (always for CGS)                */
    int ic_sweeps;       /* prec 2 in mixed or TFLOWS_FP64_FMA solves: 0 =
                            exact triangular sweeps, k > 0 = k Jacobi sweeps
                            per triangle                                    */
    int ic_bf16;         /* mixed + prec 2: IC off-diagonals stored in BF16 */
    double timeout_s;    /* limit for any single device-side wait           */
    int block_size;      /* threads per block (multiple of 32, 64..512),
                            0 = 256 or the tuned value                      */
    int grid_blocks;     /* persistent blocks, 0 = from rows_per_warp       */
    int device;          /* CUDA device ordinal, -1 = current                */
    int inject_stall;    /* test hook: 1 = the first block withholds its
                            arrival at the first grid barrier, so every
                            bounded wait runs out and the solve returns
                            TFLOWS_TIMEOUT (the device stays usable)        */
    int autotune;        /* 1 = launch shapes from the tuning table, timing
                            candidates on the first solve of a new system
                            class (block_size and grid_blocks 0); batched
                            launches also balance their block groups       */
    int rows_per_warp;   /* rows each warp owns, sets the grid (0 = 32)     */
    int sweep_warps;     /* IC sweeps: warps per chunk of the widest
                            wavefront level (0 = 4)                         */
    int sweep_gate;      /* IC sweeps: 1 = a waiting warp polls one
                            representative cell until it is ready, 0 = every
                            lane polls every input, -1 = the default (on,
                            TFLOWS_SWEEP_GATE=0 turns it off)              */
    int ic_tiled;        /* exact IC(0) on a box-numbered pattern (row =
                            x + nx (y + ny z), 7-point TopolM rows): 1 =
                            tiled sweeps (block-local wavefront steps, bulk
                            copies into shared memory), 0 = level-ordered
                            sweeps, -1 = the default (tiled, TFLOWS_IC_TILED=0
                            turns it off).  In reference arithmetic both give
                            the same apply bit for bit.  Other patterns always
                            use the level sweeps                            */
} tflows_options;

typedef struct tflows_result {
    int status;           /* TFLOWS_* status code                           */
    int iterations;       /* reference-visible iteration count              */
    int inner_iterations; /* mixed: total inner iterations                  */
    int refinements;      /* mixed: FP64 refinement steps                   */
    double ini_res;       /* ||b - A x0||_2                                 */
    double fin_res;       /* final recursive (FP64) or true (mixed) norm    */
    double seconds;       /* device time of the solve kernels               */
    double bytes;         /* algorithmic bytes moved by the solve kernels   */
    int block_size;       /* launch shape used: threads per block           */
    int grid_blocks;      /* blocks (batched: this system's block group)    */
    double group_seconds; /* batched: this system's own solve time          */
} tflows_result;

/* Launch shape chosen by the autotuner for one system class. */
typedef struct tflows_tuning {
    int block_size;      /* threads per block                               */
    int rows_per_warp;   /* rows per warp (0 = one 32-row slice)            */
    int grid_blocks;     /* the grid that gives for the tuned system        */
    int sweep_warps;     /* IC sweep warps per chunk (0 = default 4)        */
    int candidates;      /* launch shapes timed (0 when from the table)     */
    int from_table;      /* 1 = the table already held this class           */
    double us_per_iteration;         /* chosen shape                        */
    double default_us_per_iteration; /* 256 threads, one slice per warp     */
    int sweep_gate;      /* IC sweeps: gated polling chosen (-1 = default)  */
} tflows_tuning;

/* Batched-launch tuning of a plan: block size and block-group balance. */
typedef struct tflows_batch_tuning {
    int block_size;
    int runs;               /* full batched solves timed                    */
    double default_seconds; /* N^(4/3) group split, 256 threads             */
    double tuned_seconds;   /* chosen block size and group split            */
} tflows_batch_tuning;

/* Fill *opt with the defaults (reference arithmetic and tolerance). */
void tflows_default_options(tflows_options *opt);
/* Options used by the legacy entry points below (copied). */
int tflows_set_options(const tflows_options *opt);

/* ---- legacy Fortran-facing entry points ---------------------------------- */
/* Replaces SUBROUTINE cg (Process/CG.f90:2-34). */
void tflows_cg(const int *N, const int *NB, const int *NONZ, const double *A,
               const int *Acol, const int *Arow, const int *Adia,
               const double *Ab, double *x, double *r1, const int *prec,
               int *niter, const double *tol, double *IniRes, double *FinRes);
/* Replaces SUBROUTINE bicg (Process/BiCG.f90:2-34). */
void tflows_bicg(const int *N, const int *NB, const int *NONZ, const double *A,
                 const int *Acol, const int *Arow, const int *Adia,
                 const double *Ab, double *x, double *r1, const int *prec,
                 int *niter, const double *tol, double *IniRes,
                 double *FinRes);
/* Replaces SUBROUTINE CGS (Process/CGS.f90:2-34). */
void tflows_cgs(const int *N, const int *NB, const int *NONZ, const double *A,
                const int *Acol, const int *Arow, const int *Adia,
                const double *Ab, double *x, double *r1, const int *prec,
                int *niter, const double *tol, double *IniRes, double *FinRes);
/* Replaces SUBROUTINE Prec1 (Process/Prec1.f90:2-18): D <- diag | IC(0)
 * inverse pivots | 1 for prec = 1 | 2 | other. */
void tflows_prec1(const int *N, const int *NONZ, const double *A,
                  const int *Acol, const int *Arow, const int *Adia,
                  double *D, const int *prec);
/* Replaces SUBROUTINE Resid (Process/Resid.f90:2-16): r1 <- r1 - A x. */
void tflows_resid(const int *N, const int *NB, const int *NONZ,
                  const double *A, const int *Acol, const int *Arow,
                  const double *Ab, const double *x, double *r1);

/* Status of the last call made on this thread, and a readable message. */
int tflows_last_status(void);
const char *tflows_status_string(int status);
const char *tflows_last_error(void);
/* Result details of the last solve made on this thread. */
void tflows_last_result(tflows_result *res);
/* Drop the device copies of Acol/Arow/Adia that the legacy calls keep,
 * keyed by the arrays' addresses, sizes and a sampled content hash; call it
 * after rewriting those arrays in place (or set TFLOWS_TOPOLOGY_CHECK=full
 * to hash every element). */
void tflows_forget_topologies(void);
/* Release every device resource the library holds. */
void tflows_finalize(void);

/* ---- subdomain coupling: halo maps and rank callbacks -------------------- */
/* A run split into subdomains, one per rank (T-FlowS with Npro > 0), couples
 * its rows to buffer cells k = -NB..-1 of x(-NB:N) whose values live on the
 * neighbouring ranks.  Without a registered halo, Ab is not read: the
 * reference's one-domain run (Npro = 0), where the subdomain loops are
 * empty.  With one, the legacy entry points (and tflows_solve_ex with
 * TFLOWS_FP64; other precisions return TFLOWS_UNSUPPORTED) run the
 * reference's coupled algorithm on the device in reference arithmetic:
 *   - after every product q = A p the buffer cells of p are exchanged and
 *     q(BufInd(k)) += Ab(k) p(k) is added (Process/CG.f90:200-208,
 *     BiCG.f90:202-211, CGS.f90:201-208 and :301-308);
 *   - every inner product and norm is summed over the ranks (glosum);
 *   - tflows_resid subtracts Ab(k) x(k) with the caller's x(-NB:-1)
 *     (Resid.f90:36-42; no exchange, as the reference).
 * The transport stays with the caller, through two callbacks:
 *   exchange(user, phi, NB): phi points at PHI(-NB) of a host copy whose
 *     buffer cells already hold the values of the cells they mirror,
 *     PHI(c) = PHI(BufInd(c)) (Parallel/Double/Exchng.f90:36-43); swap each
 *     neighbour's segment PHI(NBBe(sub):NBBs(sub)) with rank sub-1 in place,
 *     as MPI_SENDRECV_REPLACE does (Exchng.f90:46-60);
 *   glosum(user, value): replace *value by its sum over the ranks
 *     (Parallel/Double/GloSum.f90, MPI_ALLREDUCE).
 * Both return 0 on success; anything else ends the call with
 * TFLOWS_HALO_ERROR.  Every rank makes the same solver calls: the number of
 * exchanges and sums per call is the same on all ranks.
 * Maps as par_mod holds them after Parallel/Double/BufLoa.f90:35-84:
 * NBBs[sub-1] = NBBs(sub), NBBe[sub-1] = NBBe(sub) for sub = 1..Npro (a
 * neighbour without connections has NBBe(sub) > NBBs(sub)); BufInd passed
 * from BufInd(-NB), so BufInd[NB + k] = BufInd(k) in 1..N for every buffer
 * cell k.  NB must equal the NB of the solver calls.  The registration is
 * process-wide, as par_mod is; Npro = 0 or tflows_clear_halo removes it. */
typedef int (*tflows_exchange_fn)(void *user, double *phi, int NB);
typedef int (*tflows_glosum_fn)(void *user, double *value);
int tflows_set_halo(int Npro, int NB, const int *NBBs, const int *NBBe, const int *BufInd,
                    tflows_exchange_fn exchange, tflows_glosum_fn glosum, void *user);
void tflows_clear_halo(void);

/* ---- extended host-pointer entry point ------------------------------------ */
/* Same arguments and outputs as tflows_cg/bicg/cgs plus a method, options
 * (NULL = the legacy options) and a result record (may be NULL).  Returns
 * the status code. */
int tflows_solve_ex(int method, const int *N, const int *NB, const int *NONZ,
                    const double *A, const int *Acol, const int *Arow,
                    const int *Adia, const double *Ab, double *x, double *r1,
                    const int *prec, int *niter, const double *tol,
                    double *IniRes, double *FinRes,
                    const tflows_options *opt, tflows_result *res);

/* ---- device-pointer interface (used by the PyTorch binding) -------------- */
typedef struct tflows_topology tflows_topology;

/* Register a compressed-row pattern.  rowptr (n+1), col (nnz), diag (n) use
 * `index_base` (0 or 1); they are device pointers when `on_device` is 1 and
 * host pointers otherwise.  The library copies what it needs. */
int tflows_topology_create(tflows_topology **out, int n, int nnz,
                           const int *rowptr, const int *col, const int *diag,
                           int index_base, int on_device);
void tflows_topology_destroy(tflows_topology *topo);
/* Positions of the transposed entries: tpos[k] = stored position of (j,i)
 * for the entry k at (i,j); -1 where the pattern has no such entry.
 * Device int array of nnz elements, valid while the topology lives. */
const int *tflows_topology_transpose_map(tflows_topology *topo);
/* Column patterns of the topology's products: the number of distinct
 * per-row offset tuples (column - row) the products read instead of column
 * indices (1..255), or 0 when they read explicit column indices (a row with
 * more than 8 entries, more than 255 tuples, or TFLOWS_SELL_PATTERNS=0 when
 * the topology was created).  Either way the products see the same columns
 * in the same order. */
int tflows_topology_patterns(tflows_topology *topo);

/* Solve A x = b with device arrays in the topology's stored order: val
 * (nnz FP64), b (n), x (n, in/out: initial guess and solution), r_out (n,
 * may be NULL: final recursive residual).  `stream` is a cudaStream_t (NULL
 * = the library's own).  Synchronous: returns when the result is final. */
int tflows_solve_device(tflows_topology *topo, int method, int prec,
                        const tflows_options *opt, const double *val,
                        const double *b, double *x, double *r_out,
                        int maxiter, double tol, void *stream,
                        tflows_result *res);

/* Batched solve: `count` independent systems, each with its own topology,
 * method and preconditioner, run by one persistent launch.  Arrays of
 * per-system device pointers as in tflows_solve_device. */
int tflows_solve_batched_device(int count, tflows_topology *const *topos,
                                const int *methods, const int *precs,
                                const tflows_options *opt,
                                const double *const *vals,
                                const double *const *bs, double *const *xs,
                                const int *maxiters, const double *tols,
                                void *stream, tflows_result *results);

/* Graph-captured batched solve.  tflows_plan_create records, for fixed
 * device pointers, everything a batched solve does -- value layout, staging
 * of x and b, the one persistent cooperative launch, result records and the
 * copy of x back -- into a CUDA graph with its own workspaces;
 * tflows_plan_launch replays it on `stream` (asynchronous; the caller may
 * change the contents of vals/bs/xs between replays, e.g. once per time
 * step); tflows_plan_results waits for the last replay and fills one result
 * per system. */
typedef struct tflows_plan tflows_plan;
int tflows_plan_create(tflows_plan **out, int count,
                       tflows_topology *const *topos, const int *methods,
                       const int *precs, const tflows_options *opt,
                       const double *const *vals, const double *const *bs,
                       double *const *xs, const int *maxiters,
                       const double *tols);
int tflows_plan_launch(tflows_plan *plan, void *stream);
int tflows_plan_results(tflows_plan *plan, tflows_result *results);
void tflows_plan_destroy(tflows_plan *plan);

/* Autotuner (no counterpart in the reference).  Times candidate launch
 * shapes -- threads per block, rows per warp (hence the grid), IC sweep
 * warps -- for this pattern, method, preconditioner and options on the given
 * device values and right-hand side (capped solves from x0 = 0; x is not
 * touched), stores the fastest per iteration in the process-wide tuning
 * table and returns it.  The table is keyed by device, method,
 * preconditioner, precision options and size class (quarter octaves of n);
 * with TFLOWS_TUNE_FILE set it is read from and appended to that file.
 * Solves with options.autotune = 1 use it. */
int tflows_autotune(tflows_topology *topo, int method, int prec,
                    const tflows_options *opt, const double *val,
                    const double *b, void *stream, tflows_tuning *out);
/* Forget every tuned entry of this process; the next lookup reads the
 * TFLOWS_TUNE_FILE table again (the file is left as it is). */
void tflows_autotune_clear(void);
/* The batched-launch tuning a plan made at creation (options.autotune = 1:
 * block size and group sizes from timed full solves, each starting from the
 * contents of vals/bs/xs at creation -- give the plan the kind of initial
 * guesses its replays will use, not converged solutions). */
int tflows_plan_tuning(const tflows_plan *plan, tflows_batch_tuning *out);

/* grad_val[k] = -lambda[row(k)] * x[col(k)] over the stored pattern: the
 * gradient of a scalar loss with respect to the matrix entries, given the
 * adjoint solution lambda (A^T lambda = dL/dx) and the solution x. */
int tflows_pattern_outer(tflows_topology *topo, const double *lambda,
                         const double *x, double *grad_val, void *stream);

/* Standalone compressed-row product y = A x on device arrays (FP64 or, with
 * fp32 = 1, values/vectors converted to FP32 on the fly).  For tests and
 * bandwidth measurement; returns the kernel time in seconds through *sec. */
/* The IC(0) preconditioner of Process/Prec1.f90:51-59 and CG.f90:124-166 as
 * an operator on device arrays: the pivots D, then z = M^-1 r with the
 * reference's forward sweep, TINY middle step and backward sweep, in FP64
 * (opt->precision TFLOWS_FP64: reference arithmetic, bit-identical per row to
 * the sequential loops; TFLOWS_FP64_FMA: contracted).  opt->ic_tiled picks
 * the tiled or the level-ordered sweeps; NULL opt = defaults.  Synchronous
 * on `stream`; *res (may be NULL) gets the status and the device time. */
int tflows_ic_apply_device(tflows_topology *topo, const tflows_options *opt,
                           const double *val, const double *r, double *z,
                           void *stream, tflows_result *res);

int tflows_spmv_device(tflows_topology *topo, const double *val,
                       const double *x, double *y, int repeat, int fp32,
                       void *stream, double *sec);

/* ---- T-FlowS mesh files ---------------------------------------------------- */
/* A mesh as the solver loads it: NAME.cns (Process/CnsLoa.f90) and NAME.geo
 * (Library/GeoLoa.f90), gfortran sequential unformatted files (4-byte record
 * markers, 4-byte INTEGER, 8-byte REAL, native byte order).  Arrays the
 * reference declares over (-NbC:NC) point at element -NbC; bcmark and CopyC
 * (-NbC:-1) at -NbC; SideC is SideC(0:2,NS) column-major; volume, delta,
 * WallDs (1:NC); face arrays (1:NS).  Geometry pointers are NULL when no
 * .geo file was given. */
typedef struct tflows_mesh {
    int NC, NbC, NS, NSsh, Nmat;
    int *material, *SideC, *bcmark, *CopyC;
    double *xc, *yc, *zc;
    double *volume, *delta, *WallDs;
    double *Sx, *Sy, *Sz, *Dx, *Dy, *Dz, *f, *xsp, *ysp, *zsp;
} tflows_mesh;
/* Reads the files (geo_path may be NULL); TFLOWS_BAD_INPUT with a message
 * naming the record on a short, truncated or inconsistent file. */
int tflows_mesh_read(const char *cns_path, const char *geo_path,
                     tflows_mesh **out);
void tflows_mesh_free(tflows_mesh *m);
/* Process/TopolM.f90:24-98: the compressed-row layout of the face list
 * SideC(0:2,NS): *NONZ <- stored entries + 1; with Acol (NC+1), Arow
 * (NONZ), Adia (NC) given (else a size query) the 1-based row pointers,
 * ascending column indices and diagonal positions; with SidAij (2*NS) given
 * the positions of each interior face's (c1,c2) and (c2,c1) entries (0 on
 * boundary faces). */
int tflows_topolm(int NC, int NS, const int *SideC, int *Acol, int *Arow,
                  int *Adia, int *SidAij, int *NONZ);

/* ---- pressure-correction and momentum assembly on the GPU ---------------- */
/* Mesh data of the assemblies, resident on the device (host arrays in, copied):
 * SideC(0:2,NS) and SidAij(2,NS) as the reference holds them (column-major),
 * Adia(NC) 1-based, TypeBC(-NbC:NC) and volume(-NbC:NC) passed at their
 * element -NbC, face geometry Sx..Sz, Dx..Dz, f(1:NS) (Library/GeoLoa.f90).
 * Every index is checked here; bad ones give TFLOWS_BAD_INPUT.  An object
 * keeps per-call scratch on the device, so it serves one assembly call at a
 * time (calls on different objects may overlap). */
typedef struct tflows_assembly tflows_assembly;
int tflows_assembly_create(tflows_assembly **out, int NC, int NbC, int NS,
                           int NONZ, const int *SideC, const int *SidAij,
                           const int *Adia, const int *TypeBC,
                           const double *Sx, const double *Sy, const double *Sz,
                           const double *Dx, const double *Dy, const double *Dz,
                           const double *f, const double *volume, int device);
void tflows_assembly_destroy(tflows_assembly *a);

/* Per-call cell fields of the assembly: device arrays over cells -NbC..NC,
 * each passed at its element -NbC (Rho % n, Rho % o, Rho % oo, U/V/W % n,
 * P % n, the pressure gradient Px/Py/Pz and the momentum diagonal Asave). */
typedef struct tflows_calcps_fields {
    const double *rho_n, *rho_o, *rho_oo;
    const double *u, *v, *w;
    const double *p, *px, *py, *pz;
    const double *asave;
} tflows_calcps_fields;

/* Replaces the assembly part of SUBROUTINE CalcPS (Process/CalcPS.f90:49-202):
 * Aval(1:NONZ) <- the pressure-correction matrix (zero where no face
 * writes), Abou(-NbC:-1) <- -A12 on BUFFER faces (passed at -NbC, other
 * entries untouched), Flux(1:NS) <- the face mass fluxes, b(1:NC) <- the
 * right-hand side with the density-derivative source and its volume-weighted
 * mean removed; *errmax (host, may be NULL) <- max |b| before the source.
 * Device arrays; asynchronous on `stream` unless errmax or seconds is
 * requested.  Aval, Abou, Flux and errmax are bit-identical to the
 * reference's sequential loop; b differs from it only by the rounding of
 * the mean (a tree reduction instead of a left-to-right sum).  *seconds (may
 * be NULL) <- device time. */
int tflows_calcps_assemble_device(tflows_assembly *a, int Nmat, double dt,
                                  const tflows_calcps_fields *fields,
                                  double *aval, double *b, double *abou,
                                  double *flux, double *errmax, void *stream,
                                  double *seconds);

/* Inputs of the momentum assembly of one component Ui (NewUVW's dummies and
 * the module fields it reads), all device arrays.  Cell arrays span cells
 * -NbC..NC (element c at [c + NbC]); face arrays faces 1..NS; material
 * arrays materials 1..Nmat (element m at [m - 1]).  dUidi..dUkdk are the
 * seven gradient dummies of NewUVW in its order (for U: Ux, Uy, Uz, Vx, Wx,
 * Vy, Wz; Processor.f90:314-340 gives V and W). */
typedef struct tflows_newuvw_fields {
    const int *material;                   /* material(c), 1..Nmat */
    const double *rho_n, *rho_o, *rho_oo;  /* Rho % n, o, oo */
    const double *ui_n, *ui_o, *ui_oo;     /* Ui % n, o, oo (after the old-value shift) */
    const double *duidi, *duidj, *duidk, *dujdi, *dukdi, *dujdj, *dukdk;
    const double *pi;                      /* Pi: the pressure-gradient component */
    const double *source;                  /* Ui % source */
    const double *flux_u;                  /* faces: Flux_u, the convected mass flux */
    const double *flux;                    /* faces: Flux, orients the blended schemes */
    const double *ff;                      /* faces: fF */
    const double *scoef;                   /* faces: Scoef; NULL = |S|^2/(S.d) of the
                                              mesh, as Process/Calc3.f90:22-47 forms it */
    const int *blend, *blend_tem;          /* materials: BLEND, BLEND_TEM codes */
    const double *urfc;                    /* materials: URFC */
} tflows_newuvw_fields;

/* Scalars of the same call.  Codes as Process/IniPar.f90:22-49 sets them:
 * AB 1, CN 2, FI 3, LIN 4, PAR 5, YES 10, NO 11, CDS 20, QUICK 21, LUDS 22,
 * MINMOD 23, SMART 24, AVL_SMART 25, SUPERBEE 26, GAMMA 27. */
typedef struct tflows_newuvw_params {
    int var;           /* 1, 2, 3: the component; picks the face vectors
                          (Si..Dk, Processor.f90:314-340) and Asave on 1 */
    int nmat;          /* Nmat */
    int moin_problem;  /* Moin_Problem(): 4 gives VISeff = VISc * RhoS */
    int convec, cross, diffus, inert;  /* CONVEC, CROSS, DIFFUS, INERT */
    double visc, dt, urf;              /* VISc, dt, U % URF */
} tflows_newuvw_params;

/* Replaces the assembly part of SUBROUTINE NewUVW (Process/NewUVW.f90:
 * 138-499, with ConvScheme.f90 and CalMinMax.f90) for one component:
 * Aval(1:NONZ) <- the momentum matrix, b(1:NC) <- its right-hand side,
 * Abou(-NbC:-1) <- 0 and -A12-D12 on BUFFER faces, asave(1:NC) <- the
 * diagonal before under-relaxation when var == 1 (may be NULL),
 * rhoui(-NbC:NC) <- Rho % n * Ui % n, the unknown the solve updates in place
 * (may be NULL).  Ui % o / oo must already hold the shifted old values and
 * Ui % source the source term (NewUVW.f90:153-199 stay with the caller).
 * Aval, b, Abou and Asave are bit-identical to the reference's sequential
 * loops.  A face between a material blending with YES and one with NO hands
 * ConvScheme a code it does not handle (the reference then reads an unset
 * local): TFLOWS_BAD_INPUT, as for material indices outside 1..nmat.  The
 * call waits for the stream to read that check; *seconds (may be NULL) <-
 * device time. */
int tflows_newuvw_assemble_device(tflows_assembly *a, const tflows_newuvw_params *params,
                                  const tflows_newuvw_fields *fields, double *aval,
                                  double *b, double *abou, double *asave, double *rhoui,
                                  void *stream, double *seconds);

/* ---- allocation-free solve ------------------------------------------------ */
/* No counterpart in the reference.  For callers that may not allocate GPU
 * memory while they run (device memory reserved up front by another
 * allocator, a fixed memory budget, or no room for the device-wide
 * synchronisation of cudaMalloc/cudaFree): CG as in Process/CG.f90 with
 * prec 1 (diagonal) or any other value but 2 (none) on device arrays -- a
 * 0-based compressed-row matrix (rowptr n+1, col, diag, val), b, x (in/out)
 * and r_out (final recursive residual, may be NULL) -- that allocates
 * nothing.  Its work vectors live in one static device array of about
 * 10.2 MB that every GPU loading the library keeps until exit; n is limited
 * to 262144 rows (larger: TFLOWS_BAD_INPUT; prec 2: TFLOWS_UNSUPPORTED).
 * All calls share that array, so calls that overlap on the GPU race.  The
 * first call on a device looks up the array's address (cudaGetSymbolAddress)
 * and should come before any stream capture; the lookup is repeated after
 * the device's context has been replaced (cudaDeviceReset).  Every call
 * waits for `stream` to finish before it returns, to read its status.  The
 * pattern is checked on the device before use: row pointers starting at 0
 * and never decreasing, columns in [0, n), with prec 1 diagonal positions
 * inside their rows; otherwise TFLOWS_BAD_INPUT and x, r_out untouched.
 * rowptr[n] must not exceed the length of col and val (not checkable here).
 * Returns the status; *iterations, *ini_res, *fin_res as in tflows_cg (on the
 * ||b|| < tol exit *ini_res and *fin_res are left as they were). */
int tflows_cg_noalloc(int n, const int *rowptr, const int *col,
                      const int *diag, const double *val, const double *b,
                      double *x, double *r_out, int prec, int maxiter,
                      double tol, void *stream, int *iterations,
                      double *ini_res, double *fin_res);

#ifdef __cplusplus
}
#endif

#endif /* TFLOWS_KRYLOV_H */
