// Persistent Krylov solvers (CG / CGS with diagonal or IC(0) preconditioning)
// for the T-FlowS compressed-row systems, in FP64 (reference arithmetic) or
// FP32 (inner solves of the mixed-precision refinement).
//
// Matrix storage on the device is SELL-32: the rows are cut into slices of
// 32 consecutive rows; within a slice entry t of row (32*s + lane) sits at
// soff[s] + 32*t + lane, so a warp reading entry t of its 32 rows touches
// 32 consecutive words.  Each row keeps its entries in the caller's stored
// order, so every per-row sum runs left to right exactly as the reference's
// loops do (Process/CG.f90:193-199, Resid.f90:28-33); padding slots carry
// column -1 and are skipped.  With --fmad=false every a*b+c is a rounded
// product followed by a rounded sum, as in the reference.
//
// One cooperative launch runs a whole solve.  Phases are separated by the
// bounded grid barrier of device_common.cuh; the three scalar all-reduces
// per iteration of the reference (glosum, Parallel/Double/GloSum.f90:20-28)
// become block partial sums combined in a fixed order by every block, so
// alpha, beta and the convergence test never leave the device.
//
// IC(0) preconditioning (Process/Prec1.f90:51-59 and CG.f90:135-156) runs as
// sync-free triangular sweeps: rows are visited in wavefront-level order
// (levels padded to whole warps, so no warp waits on itself) and each row
// waits only for the specific earlier rows it reads, through value-as-flag
// cells.  Rows therefore combine the same operands in the same order as the
// sequential sweep: the preconditioner output is bit-identical to it.
#pragma once

#include "device_common.cuh"

namespace tflows {

constexpr double kTiny = 1.0e-64;  // Library/allp_mod.f90:31

// Reduction slots in the partials array (each slot = one value per block).
enum : int { SLOT_A = 0, SLOT_B = 4, SLOT_C = 8, SLOT_D = 12, NUM_SLOTS = 16 };

template <typename T>
struct Mat {
    int n;
    int nslices;
    const long long* __restrict__ soff;  // nslices + 1 slice offsets (elements)
    const int* __restrict__ scol;        // SELL column indices, -1 = padding
    const T* __restrict__ sval;          // SELL values
    const int* __restrict__ meta;        // per row: length | diag slot << 16
    const int* __restrict__ perm_f;      // forward level order, 32-padded, -1 pads
    const int* __restrict__ perm_b;      // backward level order
    int nchunk_f;
    int nchunk_b;
};

template <typename T>
struct Vecs {
    T* x;   // solution (in/out)
    T* r;   // in: right-hand side, out: final recursive residual
    T* p;   // search direction (CGS: p1)
    T* q;   // A p (CGS: q1)
    T* z;   // preconditioned residual (CG)
    T* w;   // IC forward-sweep cells (sentinel between sweeps)
    T* D;   // Prec1 output
    T* r2;  // CGS: shadow residual
    T* u1;
    T* u2;
    T* v2;
    T* p2;
    T* t;   // CGS: u1 + q1
};

struct SolveCfg {
    int method;     // 0 CG, 2 CGS (BiCG runs as CG)
    int prec;       // 1 diagonal, 2 IC(0), other = none
    int maxiter;
    double tol;     // absolute, compared as error < tol
    int x_is_zero;  // skip Resid's product (x0 = 0)
    int do_prec1;   // compute D (Prec1) in this launch
    int tol_is_relative;  // tol multiplies ||b||
};

struct SolveOut {
    int exit_kind;
    int iterations;
    double ini_res;
    double fin_res;
    double bnrm2;
};

#define TF_FOR_ROWS(g, m, i)                                        \
    for (int s__ = (g).wg; s__ < (m).nslices; s__ += (g).nw)        \
        for (int i = s__ * kWarp + (g).lane, once__ = 1; once__; once__ = 0) \
            if (i < (m).n)

// q_i = sum_j a_ij x_j over row i = 32*s + lane, left to right from 0.
template <typename T, typename X>
__device__ __forceinline__ T sell_row(const Mat<T>& m, int s, int lane, const X* __restrict__ xv) {
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const T* vp = m.sval + b0 + lane;
    T acc = T(0);
    int t = 0;
    for (; t + 4 <= w; t += 4) {
        const int c0 = cp[0], c1 = cp[32], c2 = cp[64], c3 = cp[96];
        const T v0 = vp[0], v1 = vp[32], v2 = vp[64], v3 = vp[96];
        const T x0 = c0 >= 0 ? T(xv[c0]) : T(0);
        const T x1 = c1 >= 0 ? T(xv[c1]) : T(0);
        const T x2 = c2 >= 0 ? T(xv[c2]) : T(0);
        const T x3 = c3 >= 0 ? T(xv[c3]) : T(0);
        if (c0 >= 0) acc = acc + v0 * x0;
        if (c1 >= 0) acc = acc + v1 * x1;
        if (c2 >= 0) acc = acc + v2 * x2;
        if (c3 >= 0) acc = acc + v3 * x3;
        cp += 128;
        vp += 128;
    }
    for (; t < w; ++t) {
        const int c = cp[0];
        const T v = vp[0];
        if (c >= 0) acc = acc + v * T(xv[c]);
        cp += 32;
        vp += 32;
    }
    return acc;
}

// r_i <- r_i - a_i1 x_1 - a_i2 x_2 - ... (Process/Resid.f90:28-33 order).
template <typename T, typename X>
__device__ __forceinline__ T sell_resid_row(const Mat<T>& m, int s, int lane, T ri,
                                            const X* __restrict__ xv) {
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const T* vp = m.sval + b0 + lane;
    for (int t = 0; t < w; ++t) {
        const int c = cp[32 * t];
        if (c >= 0) ri = ri - vp[32 * t] * T(xv[c]);
    }
    return ri;
}

template <typename T>
__device__ __forceinline__ T diag_value(const Mat<T>& m, int i) {
    const int dslot = m.meta[i] >> 16;
    return m.sval[m.soff[i >> 5] + (i & 31) + 32LL * dslot];
}

// ---- Prec1 -----------------------------------------------------------------
// prec 1: D_i = a_ii; prec 2: D_i = 1 / (a_ii - sum_{k<i} D_k a_ik a_ik);
// otherwise D_i = 1 (Process/Prec1.f90:45-67).  Ends with a grid barrier.
template <typename T>
__device__ bool prec1_phase(Grid& g, const Mat<T>& m, T* D, int prec) {
    if (prec == 2) {
        TF_FOR_ROWS(g, m, i) { D[i] = Cell<T>::sentinel(); }
        if (!grid_sync(g, 10)) return false;
        bool ok = true;
        for (int c = g.wg; c < m.nchunk_f && ok; c += g.nw) {
            const int row = m.perm_f[c * kWarp + g.lane];
            if (row >= 0) {
                const int meta = m.meta[row];
                const int dslot = meta >> 16;
                const long long base = m.soff[row >> 5] + (row & 31);
                T sum = m.sval[base + 32LL * dslot];
                for (int t = 0; t < dslot && ok; ++t) {
                    const int k = m.scol[base + 32LL * t];
                    const T a = m.sval[base + 32LL * t];
                    T dk;
                    ok = wait_cell(D + k, dk, g.ctl, g.timeout_ns, 11);
                    sum = sum - dk * a * a;
                }
                Cell<T>::store(D + row, T(1) / sum);
            }
        }
        return grid_sync(g, 12);
    }
    TF_FOR_ROWS(g, m, i) { D[i] = (prec == 1) ? diag_value(m, i) : T(1); }
    return true;  // made visible by the caller's next barrier
}

// ---- IC(0) apply -------------------------------------------------------------
// z = [(D~+U)^-1 D~ (D~+L)^-1] rhs with D~ = 1/D, computed as the reference
// does: forward w_i = D_i (rhs_i - sum_{k<i} a_ik w_k); middle
// w_i / (D_i + TINY); backward z_i = D_i (mid_i - sum_{k>i} a_ik z_k).
// `w` cells must hold the sentinel on entry and hold it again on exit.
// The backward phase calls `epi(row, z_row)` for fused per-row work.
template <typename T, typename Epi>
__device__ bool ic_apply(Grid& g, const Mat<T>& m, const T* D, const T* rhs, T* w, T* z, Epi epi) {
    bool ok = true;
    for (int c = g.wg; c < m.nchunk_f && ok; c += g.nw) {
        const int row = m.perm_f[c * kWarp + g.lane];
        if (row >= 0) {
            const int dslot = m.meta[row] >> 16;
            const long long base = m.soff[row >> 5] + (row & 31);
            T sum = rhs[row];
            for (int t = 0; t < dslot && ok; ++t) {
                const int k = m.scol[base + 32LL * t];
                const T a = m.sval[base + 32LL * t];
                T wk;
                ok = wait_cell(w + k, wk, g.ctl, g.timeout_ns, 20);
                sum = sum - a * wk;
            }
            Cell<T>::store(w + row, sum * D[row]);
            z[row] = Cell<T>::sentinel();
        }
    }
    if (!grid_sync(g, 21)) return false;
    for (int c = g.wg; c < m.nchunk_b && ok; c += g.nw) {
        const int row = m.perm_b[c * kWarp + g.lane];
        if (row >= 0) {
            const int meta = m.meta[row];
            const int len = meta & 0xFFFF, dslot = meta >> 16;
            const long long base = m.soff[row >> 5] + (row & 31);
            const T d = D[row];
            T sum = w[row] / (d + T(kTiny));
            for (int t = dslot + 1; t < len && ok; ++t) {
                const int k = m.scol[base + 32LL * t];
                const T a = m.sval[base + 32LL * t];
                T zk;
                ok = wait_cell(z + k, zk, g.ctl, g.timeout_ns, 22);
                sum = sum - a * zk;
            }
            const T zi = sum * d;
            Cell<T>::store(z + row, zi);
            w[row] = Cell<T>::sentinel();
            epi(row, zi);
        }
    }
    return ok;
}

template <typename T>
__device__ __forceinline__ bool finite_val(T v) { return isfinite(v); }

// ---- the reference prologue: Prec1, ||b||, Resid, IniRes -------------------
// Returns false when the launch aborted or an early exit was taken (out
// records which).  On return true, `err` holds ||r0|| and, for prec 1 / 0,
// rho0 = (r0, M^-1 r0) is in `rho0` (z written for prec 1).
template <typename T>
__device__ bool prologue(Grid& g, const Mat<T>& m, Vecs<T>& v, const SolveCfg& cfg, SolveOut& out,
                         double& tol, double& err, double& rho0, bool store_z) {
    if (cfg.do_prec1 && !prec1_phase(g, m, v.D, cfg.prec)) {
        out.exit_kind = EXIT_ABORT;
        return false;
    }
    double acc[1] = {0.0};
    TF_FOR_ROWS(g, m, i) {
        const double ri = v.r[i];
        acc[0] += ri * ri;
    }
    publish<1>(g, SLOT_A, acc);
    if (!grid_sync(g, 30)) { out.exit_kind = EXIT_ABORT; return false; }
    double tot[1];
    totals<1>(g, SLOT_A, tot);
    const double bnrm2 = sqrt(tot[0]);
    out.bnrm2 = bnrm2;
    if (cfg.tol_is_relative) tol = tol * bnrm2;
    if (bnrm2 < tol || (cfg.tol_is_relative && bnrm2 == 0.0)) {
        out.exit_kind = EXIT_BNRM;
        out.iterations = 0;
        return false;
    }
    double a2[2] = {0.0, 0.0};
    for (int s = g.wg; s < m.nslices; s += g.nw) {
        const int i = s * kWarp + g.lane;
        T ri = i < m.n ? v.r[i] : T(0);
        if (!cfg.x_is_zero) ri = sell_resid_row(m, s, g.lane, ri, v.x);
        if (i < m.n) {
            v.r[i] = ri;
            a2[0] += double(ri) * double(ri);
            if (store_z) {
                if (cfg.prec == 1) {
                    const T zi = ri / v.D[i];
                    v.z[i] = zi;
                    a2[1] += double(ri) * double(zi);
                }
            }
        }
    }
    publish<2>(g, SLOT_B, a2);
    if (!grid_sync(g, 31)) { out.exit_kind = EXIT_ABORT; return false; }
    double t2[2];
    totals<2>(g, SLOT_B, t2);
    err = sqrt(t2[0]);
    out.ini_res = err;
    out.fin_res = err;
    rho0 = cfg.prec == 1 ? t2[1] : t2[0];
    if (err < tol) {
        out.exit_kind = EXIT_INIRES;
        out.iterations = 0;
        return false;
    }
    return true;
}

// ---- CG (Process/CG.f90:113-259; also BiCG, whose iterates are CG's) --------
template <typename T>
__device__ void cg_solve(Grid& g, const Mat<T>& m, Vecs<T>& v, const SolveCfg& cfg, SolveOut& out) {
    double tol = cfg.tol, err = 0.0, rho_next = 0.0;
    if (!prologue(g, m, v, cfg, out, tol, err, rho_next, true)) return;
    const int prec = (cfg.prec == 1 || cfg.prec == 2) ? cfg.prec : 0;
    const T* z = prec == 0 ? v.r : v.z;
    double rho = 0.0, rhoold = 0.0;
    bool nonfinite = false;
    int iter = 1;
    for (; iter <= cfg.maxiter; ++iter) {
        if (prec == 2) {
            double a[1] = {0.0};
            const T* rr = v.r;
            if (!ic_apply(g, m, v.D, v.r, v.w, v.z, [&](int row, T zi) {
                    a[0] += double(rr[row]) * double(zi);
                })) {
                grid_sync(g, 40);
                out.exit_kind = EXIT_ABORT;
                return;
            }
            publish<1>(g, SLOT_A, a);
            if (!grid_sync(g, 41)) { out.exit_kind = EXIT_ABORT; return; }
            double t[1];
            totals<1>(g, SLOT_A, t);
            rho = t[0];
        } else {
            rho = rho_next;
        }
        // p = z + beta p  (CG.f90:178-187)
        if (iter == 1) {
            TF_FOR_ROWS(g, m, i) { v.p[i] = z[i]; }
        } else {
            const T beta = T(rho / rhoold);
            TF_FOR_ROWS(g, m, i) { v.p[i] = z[i] + beta * v.p[i]; }
        }
        if (!grid_sync(g, 42)) { out.exit_kind = EXIT_ABORT; return; }
        // q = A p; (p, q)  (CG.f90:193-218)
        double a1[1] = {0.0};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T qi = sell_row(m, s, g.lane, v.p);
            if (i < m.n) {
                v.q[i] = qi;
                a1[0] += double(v.p[i]) * double(qi);
            }
        }
        publish<1>(g, SLOT_C, a1);
        if (!grid_sync(g, 43)) { out.exit_kind = EXIT_ABORT; return; }
        double t1[1];
        totals<1>(g, SLOT_C, t1);
        const double alfa_d = rho / t1[0];
        const T alfa = T(alfa_d);
        // x += alfa p; r -= alfa q; ||r||; next z and rho  (CG.f90:226-253)
        double a3[3] = {0.0, 0.0, 0.0};
        TF_FOR_ROWS(g, m, i) {
            const T xi = v.x[i] + alfa * v.p[i];
            const T ri = v.r[i] - alfa * v.q[i];
            v.x[i] = xi;
            v.r[i] = ri;
            a3[0] += double(ri) * double(ri);
            if (prec == 1) {
                const T zi = ri / v.D[i];
                v.z[i] = zi;
                a3[1] += double(ri) * double(zi);
            }
            if (nonfinite) a3[2] += (xi == xi ? 1.0 : 0.0) + (ri == ri ? 1.0 : 0.0);
        }
        publish<3>(g, SLOT_D, a3);
        if (!grid_sync(g, 44)) { out.exit_kind = EXIT_ABORT; return; }
        double t3[3];
        totals<3>(g, SLOT_D, t3);
        err = sqrt(t3[0]);
        out.fin_res = err;
        if (err < tol) {
            out.exit_kind = EXIT_CONVERGED;
            out.iterations = iter;
            return;
        }
        rho_next = prec == 1 ? t3[1] : t3[0];
        if (!finite_val(err)) {
            // From here on the reference keeps iterating on non-finite
            // values; once every x and r entry is NaN nothing changes any
            // more, so the remaining iterations can be skipped.
            if (nonfinite && t3[2] == 0.0) {
                out.exit_kind = EXIT_NONFINITE;
                out.iterations = cfg.maxiter + 1;
                return;
            }
            nonfinite = true;
        }
        rhoold = rho;
    }
    out.exit_kind = EXIT_MAXITER;
    out.iterations = iter;
}

// ---- CGS (Process/CGS.f90:112-333) -------------------------------------------
template <typename T>
__device__ void cgs_solve(Grid& g, const Mat<T>& m, Vecs<T>& v, const SolveCfg& cfg, SolveOut& out) {
    double tol = cfg.tol, err = 0.0, dummy = 0.0;
    if (!prologue(g, m, v, cfg, out, tol, err, dummy, false)) return;
    const int prec = (cfg.prec == 1 || cfg.prec == 2) ? cfg.prec : 0;
    // r2 = r1 (CGS.f90:84-86); rho = (r1, r2) for the first iteration.
    double a0[1] = {0.0};
    TF_FOR_ROWS(g, m, i) {
        const T ri = v.r[i];
        v.r2[i] = ri;
        a0[0] += double(ri) * double(ri);
    }
    publish<1>(g, SLOT_A, a0);
    if (!grid_sync(g, 50)) { out.exit_kind = EXIT_ABORT; return; }
    double t0[1];
    totals<1>(g, SLOT_A, t0);
    double rho = t0[0], rhoold = 0.0;
    bool nonfinite = false;
    int iter = 1;
    for (; iter <= cfg.maxiter; ++iter) {
        // u1 = r1 + beta q1; u2 = u1 + beta (q1 + beta u2); p2 = M^-1 u2
        const T beta = T(iter == 1 ? 0.0 : rho / rhoold);
        TF_FOR_ROWS(g, m, i) {
            T u1, u2;
            if (iter == 1) {
                u1 = v.r[i];
                u2 = u1;
            } else {
                const T q1 = v.q[i];
                u1 = v.r[i] + beta * q1;
                u2 = u1 + beta * (q1 + beta * v.u2[i]);
            }
            v.u1[i] = u1;
            v.u2[i] = u2;
            if (prec == 1) v.p2[i] = u2 / v.D[i];
            else if (prec != 2) v.p2[i] = u2;
        }
        if (!grid_sync(g, 51)) { out.exit_kind = EXIT_ABORT; return; }
        if (prec == 2) {
            if (!ic_apply(g, m, v.D, v.u2, v.w, v.p2, [](int, T) {})) {
                grid_sync(g, 52);
                out.exit_kind = EXIT_ABORT;
                return;
            }
            if (!grid_sync(g, 53)) { out.exit_kind = EXIT_ABORT; return; }
        }
        // v2 = A p2; alfa = rho / (r2, v2)
        double a1[1] = {0.0};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T vi = sell_row(m, s, g.lane, v.p2);
            if (i < m.n) {
                v.v2[i] = vi;
                a1[0] += double(v.r2[i]) * double(vi);
            }
        }
        publish<1>(g, SLOT_B, a1);
        if (!grid_sync(g, 54)) { out.exit_kind = EXIT_ABORT; return; }
        double t1[1];
        totals<1>(g, SLOT_B, t1);
        const T alfa = T(rho / t1[0]);
        // q1 = u1 - alfa v2; p1 = M^-1 (u1 + q1); x += alfa p1
        TF_FOR_ROWS(g, m, i) {
            const T u1 = v.u1[i];
            const T q1 = u1 - alfa * v.v2[i];
            v.q[i] = q1;
            const T tt = u1 + q1;
            if (prec == 2) {
                v.t[i] = tt;
            } else {
                const T p1 = prec == 1 ? tt / v.D[i] : tt;
                v.p[i] = p1;
                v.x[i] = v.x[i] + alfa * p1;
            }
        }
        if (!grid_sync(g, 55)) { out.exit_kind = EXIT_ABORT; return; }
        if (prec == 2) {
            T* xx = v.x;
            if (!ic_apply(g, m, v.D, v.t, v.w, v.p, [&](int row, T p1) {
                    xx[row] = xx[row] + alfa * p1;
                })) {
                grid_sync(g, 56);
                out.exit_kind = EXIT_ABORT;
                return;
            }
            if (!grid_sync(g, 57)) { out.exit_kind = EXIT_ABORT; return; }
        }
        // q2 = A p1; r1 -= alfa q2; ||r1||; next rho = (r1, r2)
        double a3[3] = {0.0, 0.0, 0.0};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T q2 = sell_row(m, s, g.lane, v.p);
            if (i < m.n) {
                const T ri = v.r[i] - alfa * q2;
                v.r[i] = ri;
                a3[0] += double(ri) * double(ri);
                a3[1] += double(ri) * double(v.r2[i]);
                if (nonfinite) {
                    const T xi = v.x[i];
                    a3[2] += (xi == xi ? 1.0 : 0.0) + (ri == ri ? 1.0 : 0.0);
                }
            }
        }
        publish<3>(g, SLOT_C, a3);
        if (!grid_sync(g, 58)) { out.exit_kind = EXIT_ABORT; return; }
        double t3[3];
        totals<3>(g, SLOT_C, t3);
        err = sqrt(t3[0]);
        out.fin_res = err;
        if (err < tol) {
            out.exit_kind = EXIT_CONVERGED;
            out.iterations = iter;
            return;
        }
        if (!finite_val(err)) {
            if (nonfinite && t3[2] == 0.0) {
                out.exit_kind = EXIT_NONFINITE;
                out.iterations = cfg.maxiter + 1;
                return;
            }
            nonfinite = true;
        }
        rhoold = rho;
        rho = t3[1];
    }
    out.exit_kind = EXIT_MAXITER;
    out.iterations = iter;
}

}  // namespace tflows
