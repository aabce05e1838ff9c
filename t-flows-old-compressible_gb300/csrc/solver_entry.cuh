// Kernel entry points of the persistent solvers and their parameter blocks.
//
// Included by two translation units that compile the same solver code with
// different arithmetic: krylov.cu (namespace tflows::ref) with --fmad=false,
// where every a*b+c is a rounded product followed by a rounded sum and the
// diagonal preconditioner divides, as the reference does; krylov_fma.cu
// (namespace tflows::fma) with contraction into fused multiply-adds and a
// reciprocal diagonal, for the TFLOWS_FP64_FMA solves and the mixed-precision
// solves.  The parameter blocks are shared types; the kernels of each unit
// live in its own namespace so that the two builds never merge.
#pragma once

#include "krylov_kernels.cuh"

#ifndef TFLOWS_KNS
#error "define TFLOWS_KNS (the kernel namespace of this translation unit) first"
#endif

namespace tflows {

// Threads per block of the persistent kernels unless a launch asks for
// another multiple of 32 up to kMaxBlock (the tuner's choice).  Register
// budget: 65536 / (kBlock * kMinBlocks) per thread, i.e. kMinBlocks resident
// blocks of kBlock threads per SM.
constexpr int kBlock = 256;
constexpr int kMaxBlock = 512;
#ifndef TFLOWS_MINBLOCKS
#define TFLOWS_MINBLOCKS 4
#endif
constexpr int kMinBlocks = TFLOWS_MINBLOCKS;
constexpr int kMinBlocksAtMax = kMinBlocks * kBlock / kMaxBlock > 0 ? kMinBlocks * kBlock / kMaxBlock : 1;

template <typename T>
struct KParams {
    Mat<T> m;
    Mat<T> mT;  // A^T values in A's pattern (true BiCG only)
    Vecs<T> v;
    SolveCfg cfg;
    DevCtl* ctl;
    DevState* state;
    double* partials;
    long long timeout_cyc;
    int mode;  // 0 solve, 1 Prec1 only
    int stall;
};

struct MixedParams {
    Mat<double> m64;
    Mat<float> m32;
    double* x64;
    double* r64;
    const double* b64;
    double* D64;
    double* xbest;
    Vecs<float> v32;
    MixedCfg cfg;
    DevCtl* ctl;
    DevState* state;
    double* partials;
    long long timeout_cyc;
    int stall;
};

struct BatchItem {
    int b0;       // first block of the group
    int nb;       // blocks in the group
    int mixed;    // 0: FP64 params, 1: mixed params
    int method;   // 0 CG, 2 CGS
    KParams<double> P64;
    MixedParams PM;
};

namespace TFLOWS_KNS {

__device__ int status_of(const SolveOut& o, const DevCtl* ctl) {
    if (ctl->status != 0) return ctl->status;
    switch (o.exit_kind) {
        case EXIT_MAXITER: return isfinite(o.fin_res) ? ST_NOT_CONVERGED : ST_NONFINITE;
        case EXIT_NONFINITE: return ST_NONFINITE;
        case EXIT_ABORT: return ST_TIMEOUT;
        default: return ST_OK;
    }
}

// METHOD: 0 CG (and BiCG), 2 CGS, 3 true BiCG, 9 Prec1 only, 8 the IC(0)
// pivots (Prec1 prec 2) and one apply z = M^-1 r (v.r in, v.z out).
template <typename T, int METHOD>
__global__ void __launch_bounds__(kMaxBlock, kMinBlocksAtMax) krylov_kernel(KParams<T> P) {
    Grid g;
    grid_init(g, P.ctl, P.partials, P.timeout_cyc);
    g.stall = P.stall;
    SolveOut out;
    out.exit_kind = 0;
    out.iterations = 0;
    out.ini_res = 0.0;
    out.fin_res = 0.0;
    out.bnrm2 = 0.0;
    if (METHOD == 9) {
        bool ok = prec1_phase(g, P.m, P.v.D, P.cfg.prec);
        out.exit_kind = ok ? EXIT_CONVERGED : EXIT_ABORT;
    } else if (METHOD == 8) {
        bool ok = prec1_phase(g, P.m, P.v.D, 2);  // ends with a barrier
        if (ok && P.m.tile.on) {
            tiles_init(g, P.m, P.v.D);
            ok = grid_sync(g, 14);
        }
        if (ok) ok = ic_precond(g, P.m, P.v, P.cfg.ic_sweeps, P.v.r, P.v.z, [](int, T, T) {});
        out.exit_kind = ok ? EXIT_CONVERGED : EXIT_ABORT;
    } else if (METHOD == 2) {
        cgs_solve(g, P.m, P.v, P.cfg, out);
    } else if (METHOD == 3) {
        bicg_true_solve(g, P.m, P.mT, P.v, P.cfg, out);
    } else {
        cg_solve(g, P.m, P.v, P.cfg, out);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        DevState* s = P.state;
        s->status = status_of(out, P.ctl);
        s->exit_kind = out.exit_kind;
        s->iterations = out.iterations;
        s->inner_iters = 0;
        s->refinements = 0;
        s->ini_res = out.ini_res;
        s->fin_res = out.fin_res;
        s->bnrm2 = out.bnrm2;
        s->timeout_where = P.ctl->where;
    }
}


// KIND: 0 restarted CG, 2 restarted CGS, 1 CG with reliable updates.
template <int KIND>
__global__ void __launch_bounds__(kMaxBlock, kMinBlocksAtMax) mixed_kernel(MixedParams P) {
    Grid g;
    grid_init(g, P.ctl, P.partials, P.timeout_cyc);
    g.stall = P.stall;
    MixedOut out;
    out.exit_kind = 0;
    out.iterations = 0;
    out.refinements = 0;
    out.ini_res = 0.0;
    out.fin_res = 0.0;
    out.bnrm2 = 0.0;
    if (KIND == 1)
        mixed_cg_reliable(g, P.m64, P.m32, P.x64, P.r64, P.b64, P.D64, P.xbest, P.v32, P.cfg,
                          out);
    else
        mixed_solve(g, P.m64, P.m32, P.x64, P.r64, P.b64, P.D64, P.v32, P.cfg, out);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        DevState* s = P.state;
        SolveOut o;
        o.exit_kind = out.exit_kind;
        o.fin_res = out.fin_res;
        s->status = status_of(o, P.ctl);
        s->exit_kind = out.exit_kind;
        s->iterations = out.iterations;
        s->inner_iters = out.iterations;
        s->refinements = out.refinements;
        s->ini_res = out.ini_res;
        s->fin_res = out.fin_res;
        s->bnrm2 = out.bnrm2;
        s->timeout_where = P.ctl->where;
    }
}

// ---- batched solves: one cooperative launch, one block group per system ------

template <int MIXED>
__global__ void __launch_bounds__(kMaxBlock, kMinBlocksAtMax)
    batch_kernel(const BatchItem* __restrict__ items, const int* __restrict__ block_item) {
    const BatchItem& it = items[block_item[blockIdx.x]];
    const unsigned long long t_start = globaltimer_ns();
    Grid g;
    if (!MIXED) {
        KParams<double> P = it.P64;
        grid_init_group(g, P.ctl, P.partials, P.timeout_cyc, it.b0, it.nb);
        SolveOut out;
        out.exit_kind = 0;
        out.iterations = 0;
        out.ini_res = 0.0;
        out.fin_res = 0.0;
        out.bnrm2 = 0.0;
        if (it.method == 2) cgs_solve(g, P.m, P.v, P.cfg, out);
        else cg_solve(g, P.m, P.v, P.cfg, out);
        if (g.bid == 0 && threadIdx.x == 0) {
            DevState* s = P.state;
            s->status = status_of(out, P.ctl);
            s->exit_kind = out.exit_kind;
            s->iterations = out.iterations;
            s->inner_iters = 0;
            s->refinements = 0;
            s->ini_res = out.ini_res;
            s->fin_res = out.fin_res;
            s->bnrm2 = out.bnrm2;
            s->timeout_where = P.ctl->where;
            s->group_ns = (double)(globaltimer_ns() - t_start);
        }
    } else {
        MixedParams P = it.PM;
        grid_init_group(g, P.ctl, P.partials, P.timeout_cyc, it.b0, it.nb);
        MixedOut out;
        out.exit_kind = 0;
        out.iterations = 0;
        out.refinements = 0;
        out.ini_res = 0.0;
        out.fin_res = 0.0;
        out.bnrm2 = 0.0;
        // the refinement the system asked for, as in its single-system solve
        if (it.method != 2 && !P.cfg.restart)
            mixed_cg_reliable(g, P.m64, P.m32, P.x64, P.r64, P.b64, P.D64, P.xbest, P.v32, P.cfg,
                              out);
        else
            mixed_solve(g, P.m64, P.m32, P.x64, P.r64, P.b64, P.D64, P.v32, P.cfg, out);
        if (g.bid == 0 && threadIdx.x == 0) {
            DevState* s = P.state;
            SolveOut o;
            o.exit_kind = out.exit_kind;
            o.fin_res = out.fin_res;
            s->status = status_of(o, P.ctl);
            s->exit_kind = out.exit_kind;
            s->iterations = out.iterations;
            s->inner_iters = out.iterations;
            s->refinements = out.refinements;
            s->ini_res = out.ini_res;
            s->fin_res = out.fin_res;
            s->bnrm2 = out.bnrm2;
            s->timeout_where = P.ctl->where;
            s->group_ns = (double)(globaltimer_ns() - t_start);
        }
    }
}


}  // namespace TFLOWS_KNS

}  // namespace tflows
