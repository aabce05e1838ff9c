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
// column -1 and are skipped.  In the reference-arithmetic build (--fmad=false)
// every a*b+c is a rounded product followed by a rounded sum, as in the
// reference; the contracted build fuses them (solver_entry.cuh).
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
// TINY in the working precision: FP32 has no such number and 1e-64 rounds
// to zero there, so the FP32 inner solves divide by D itself.
template <typename T>
__device__ __forceinline__ T tiny_v() {
    if constexpr (sizeof(T) == 8) return T(kTiny);
    else return T(0);
}

// Reduction slots in the partials array (each slot = one value per block).
enum : int { SLOT_A = 0, SLOT_B = 4, SLOT_C = 8, SLOT_D = 12, NUM_SLOTS = 16 };

// Tiled IC(0) sweeps on a box-numbered pattern (row = x + nx (y + ny z),
// 7-point stencil in TopolM order).  Each block owns tiles of 16 x ty
// columns (ty = block size / 16) that run through all z; its threads walk
// their columns along the wavefront step s = lx + ly + z.  Everything a step
// reads sits in one contiguous record per (tile, step), fields of `block`
// entries each, so one bulk copy stages it:
//   forward record:  lower coefficients (z-1, y-1, x-1) | D | rhs | [1/(D+TINY)]
//   backward record: upper coefficients (x+1, y+1, z+1) | D | mid | rhs
// (mid = w / (D + TINY), written by the forward sweep; the reciprocal field
// exists only where the forward sweep multiplies by it: the contracted FP64
// build).  The cells of slot (k, s, t) = (k * steps + s) * block + t carry
// the results a neighbouring tile reads.
constexpr int kTileX = 16;     // tile width in x (columns per tile row)
// The staged records form two halves of `half` steps each: one bulk copy
// fills a half while the block works through the other.  The ring takes at
// most kTileRingBytes of shared memory (so four 256-thread blocks still fit
// on an SM) and a half at most kTileHalfMax steps.
constexpr unsigned kTileRingBytes = 48u * 1024u;
constexpr int kTileHalfMax = 4;

template <typename T>
struct Tiles {
    int on;                 // 1: IC applies of this solve run the tiled sweeps
    int nx, ny, nz;         // box dimensions
    int ty;                 // tile height in y (block size / 16)
    int ntx, nty;           // tiles along x and y
    int steps;              // wavefront steps per tile: 16 + ty + nz - 2
    int lu_bf16;            // coefficients stored as BF16 bit patterns (FP32 solves)
    int recip;              // forward: mid = w * (1/(D+TINY)) instead of w / (D+TINY)
    int half;               // steps per ring half (tile_half)
    unsigned rec_f, rec_b;  // bytes of one forward / backward record
    unsigned char* fwd;     // [tile][step] forward records
    unsigned char* bwd;     // [tile][step] backward records
    T* wt;                  // forward results by slot (value-as-flag cells)
    T* zt;                  // backward results by slot (value-as-flag cells)
};

// Bytes of one ring slot (the larger record: three coefficients and three
// value fields), rounded to 128; steps per ring half; and the whole dynamic
// shared-memory block of a tiled solve (barriers and flags, the ring, the
// neighbour exchange).
__host__ __device__ constexpr unsigned tile_slot_bytes(unsigned block, unsigned coef_bytes,
                                                       unsigned val_bytes) {
    return (block * (3 * coef_bytes + 3 * val_bytes) + 127u) / 128u * 128u;
}
__host__ __device__ constexpr int tile_half(unsigned block, unsigned coef_bytes, unsigned val_bytes) {
    return kTileRingBytes / (2u * tile_slot_bytes(block, coef_bytes, val_bytes)) < 1u
               ? 1
               : (kTileRingBytes / (2u * tile_slot_bytes(block, coef_bytes, val_bytes)) >
                          (unsigned)kTileHalfMax
                      ? kTileHalfMax
                      : (int)(kTileRingBytes / (2u * tile_slot_bytes(block, coef_bytes, val_bytes))));
}
__host__ __device__ constexpr unsigned tile_smem_bytes(unsigned block, unsigned coef_bytes,
                                                       unsigned val_bytes) {
    return 128u + 2u * tile_half(block, coef_bytes, val_bytes) *
                      tile_slot_bytes(block, coef_bytes, val_bytes) +
           2u * block * val_bytes;
}

template <typename T>
struct Mat {
    int n;
    int nslices;
    const long long* __restrict__ soff;  // nslices + 1 slice offsets (elements)
    const int* __restrict__ scol;        // SELL column indices, -1 = padding
    // Column patterns (null when the topology has none): row i's entry t is
    // at column i + poff[8 * spat[i] + t], absent where that offset is
    // kNoCol (i + kNoCol < 0 for every row); the same columns as `scol`, in
    // the same order, read as one byte per row instead of four per entry.
    const unsigned char* __restrict__ spat;
    const int* __restrict__ poff;
    const T* __restrict__ sval;          // SELL values
    const int* __restrict__ meta;        // per row: length | diag slot << 16
    const int* __restrict__ perm_f;      // forward level order, 32-padded, -1 pads
    const int* __restrict__ perm_b;      // backward level order
    // BF16 copy of the SELL values (bit patterns), read by the IC sweeps in
    // place of `sval` when set (the off-diagonal factor entries)
    const unsigned short* __restrict__ lu16;
    int nchunk_f;
    int nchunk_b;
    int wide_f;  // chunks in the widest forward / backward level
    int wide_b;
    int sweep_mult;  // sweep warps per chunk of the widest level (0 = default)
    int sweep_sleep; // longest pause between polls of a sweep cell, ns (0: none)
    int sweep_gate;  // 1: a waiting warp polls one representative cell first
    Tiles<T> tile;   // tiled IC sweeps (tile.on = 0: level-ordered sweeps)
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
    T* s;   // scratch of the Jacobi-sweep IC apply (FP32 inner solves)
};

struct SolveCfg {
    int method;     // 0 CG, 2 CGS (BiCG runs as CG)
    int prec;       // 1 diagonal, 2 IC(0), other = none
    int maxiter;
    double tol;     // absolute, compared as error < tol
    int x_is_zero;  // skip Resid's product (x0 = 0)
    int do_prec1;   // compute D (Prec1) in this launch
    int tol_is_relative;  // tol multiplies ||b||
    int ic_sweeps;  // prec 2: 0 = exact triangular sweeps, k > 0 = k Jacobi sweeps each
    int fuse_dir;   // FP64 CG: form the search direction inside the product
};

struct SolveOut {
    int exit_kind;
    int iterations;
    double ini_res;
    double fin_res;
    double bnrm2;
};

// Rows in SELL order: row i = 32*slice + lane (used by the matrix phases).
#define TF_FOR_ROWS(g, m, i)                                        \
    for (int s__ = (g).wg; s__ < (m).nslices; s__ += (g).nw)        \
        for (int i = s__ * kWarp + (g).lane, once__ = 1; once__; once__ = 0) \
            if (i < (m).n)

// Four consecutive rows per thread with 16-byte vector accesses (the vector
// phases).  Every work vector is padded to a multiple of 32 elements, so the
// group i..i+3 is in bounds; contributions of rows >= n are masked.
#define TF_FOR4(g, m, i) for (int i = 4 * (g).tid; i < (m).n; i += 4 * (g).nt)

template <typename T>
struct V4 {
    T a[4];
};
__device__ __forceinline__ V4<float> ld4(const float* p) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    return {{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ void st4(float* p, const V4<float>& v) {
    *reinterpret_cast<float4*>(p) = make_float4(v.a[0], v.a[1], v.a[2], v.a[3]);
}
__device__ __forceinline__ V4<double> ld4(const double* p) {
    const double2 u = reinterpret_cast<const double2*>(p)[0];
    const double2 w = reinterpret_cast<const double2*>(p)[1];
    return {{u.x, u.y, w.x, w.y}};
}
__device__ __forceinline__ void st4(double* p, const V4<double>& v) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v.a[0], v.a[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v.a[2], v.a[3]);
}

// Dot-product partials accumulate per thread in the working precision (FP64
// sums in FP64 mode; FP32 sums in the FP32 inner solves, where a per-element
// FP64 accumulation would load GB300's narrow FP64 pipe) and are combined
// across threads and blocks in FP64.
template <int K, typename T>
__device__ __forceinline__ void publish_t(Grid& g, int slot, const T (&v)[K]) {
    double d[K];
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] = (double)v[k];
    publish<K>(g, slot, d);
}

// Jacobi step z = r / D.  The reference-arithmetic build keeps the
// reference's correctly rounded division; the contracted build
// (TFLOWS_FP64_RECIP_DIAG) and the FP32 inner solves hold 1/D and multiply.
#ifdef TFLOWS_FP64_RECIP_DIAG
constexpr bool kRecipDiag64 = true;
__device__ __forceinline__ double jacobi(double r, double dinv) { return r * dinv; }
#else
constexpr bool kRecipDiag64 = false;
__device__ __forceinline__ double jacobi(double r, double d) { return r / d; }
#endif
__device__ __forceinline__ float jacobi(float r, float dinv) { return r * dinv; }

// Offset marking an absent entry of a column pattern: patterns are built
// only for fewer than 2^30 rows, so i + kNoCol is negative for every row.
constexpr int kNoCol = -(1 << 30);

// The first 8 column indices of row i = 32*s + lane of a slice of width
// w <= 8 (negative where the row has no entry): from the row's column
// pattern (two 16-byte loads of a table that stays in L1, one add per
// entry) when the topology has patterns, else from the SELL column array.
template <typename T>
__device__ __forceinline__ void sell_cols8(const Mat<T>& m, int s, int lane, int w, long long b0,
                                          int (&c)[8]) {
    if (m.spat) {
        const int i = s * kWarp + lane;
        const int4* po = reinterpret_cast<const int4*>(m.poff) + 2 * (int)m.spat[i];
        const int4 a = __ldg(po), b = __ldg(po + 1);
        c[0] = i + a.x;
        c[1] = i + a.y;
        c[2] = i + a.z;
        c[3] = i + a.w;
        c[4] = i + b.x;
        c[5] = i + b.y;
        c[6] = i + b.z;
        c[7] = i + b.w;
    } else {
        const int* cp = m.scol + b0 + lane;
#pragma unroll
        for (int t = 0; t < 8; ++t) c[t] = t < w ? cp[32 * t] : -1;
    }
}

// FP32 products in difference form.  The FP32 copy of a matrix keeps its
// off-diagonal entries rounded to FP32 but holds, in the diagonal slot, the
// row sum c_i (summed in FP64, then rounded); a product is then formed as
//     q_i = c_i x_i + sum_{j != i} a_ij (x_j - x_i),
// the same number in exact arithmetic.  Rounding each entry separately would
// perturb every row sum by ~6e-8 |a_ii|; for the pressure-correction
// operator -- a graph Laplacian whose rows sum to zero except at Dirichlet
// cells -- that shifts the smallest eigenvalues, so FP32 inner CG iterations
// converge towards a different operator and each FP64 refinement pays for
// it (measured: 112 instead of 84 iterations at 24^3; reliable updates
// stalling at 256^3).  In difference form the rounding error of a product
// scales with the variation of x, and the near null space of the operator
// (smooth x) is kept.  The FP64 matrices keep the reference's plain sums.
template <typename T>
__device__ __forceinline__ T diff_term(T a, T xj, T xi, bool diag) {
    return diag ? a * xi : a * (xj - xi);
}

// q_i = sum_j a_ij x_j over row i = 32*s + lane, left to right from 0 (FP32:
// in difference form).  Rows of at most 8 stored entries (every hex or prism
// cell) take a fully unrolled path: all index and value loads issue before
// the gathers.
template <typename T, typename X>
__device__ __forceinline__ T sell_row(const Mat<T>& m, int s, int lane, const X* __restrict__ xv) {
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const T* vp = m.sval + b0 + lane;
    const int i = s * kWarp + lane;
    T acc = T(0);
    if (w <= 8) {
        int c[8];
        T v[8], xx[8];
        sell_cols8(m, s, lane, w, b0, c);
#pragma unroll
        for (int t = 0; t < 8; ++t) v[t] = t < w ? vp[32 * t] : T(0);
#pragma unroll
        for (int t = 0; t < 8; ++t) xx[t] = c[t] >= 0 ? T(xv[c[t]]) : T(0);
        if constexpr (sizeof(T) == 4) {
            T xi = T(0);
#pragma unroll
            for (int t = 0; t < 8; ++t)
                if (c[t] == i) xi = xx[t];
#pragma unroll
            for (int t = 0; t < 8; ++t)
                if (c[t] >= 0) acc = acc + diff_term(v[t], xx[t], xi, c[t] == i);
            return acc;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (c[t] >= 0) acc = acc + v[t] * xx[t];
        return acc;
    }
    if constexpr (sizeof(T) == 4) {
        const T xi = i < m.n ? T(xv[i]) : T(0);
        for (int t = 0; t < w; ++t) {
            const int c = cp[32 * t];
            if (c >= 0) acc = acc + diff_term(vp[32 * t], T(xv[c]), xi, c == i);
        }
        return acc;
    }
    for (int t = 0; t < w; ++t) {
        const int c = cp[32 * t];
        if (c >= 0) acc = acc + vp[32 * t] * T(xv[c]);
    }
    return acc;
}

// q_i = sum_j a_ij (z_j + beta p_j): the product with the next search
// direction formed inside the gather (FP32 inner solves), so the update
// p = z + beta p needs no pass of its own and no grid barrier.  `first`:
// p = z.  The direction is formed with one fused multiply-add, exactly as
// the row's owner forms its own entry (fused_dir), so every product sees the
// same vector the iteration stores.
__device__ __forceinline__ float fused_dir(float z, float beta, float p, bool first) {
    return first ? z : __fmaf_rn(beta, p, z);
}
// FP64: z + beta p written as the separate update pass writes it, so each
// build (contracted or not) forms the same value either way.
__device__ __forceinline__ double fused_dir(double z, double beta, double p, bool first) {
    return first ? z : z + beta * p;
}

// The FP64 product with the next search direction formed in the gather
// (column patterns where the topology has them, plain left-to-right sums as
// the reference's product): the same direction and the same q as the
// separate update pass followed by the product, bit for bit, with one vector
// pass and one grid barrier less per iteration.
__device__ __forceinline__ double sell_row_dir(const Mat<double>& m, int s, int lane,
                                               const double* __restrict__ z,
                                               const double* __restrict__ p, double beta,
                                               bool first) {
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const double* vp = m.sval + b0 + lane;
    double acc = 0.0;
    if (w <= 8) {
        int c[8];
        double v[8], zz[8], pp[8];
        sell_cols8(m, s, lane, w, b0, c);
#pragma unroll
        for (int t = 0; t < 8; ++t) v[t] = t < w ? vp[32 * t] : 0.0;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            zz[t] = c[t] >= 0 ? z[c[t]] : 0.0;
            pp[t] = c[t] >= 0 && !first ? p[c[t]] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (c[t] >= 0) acc = acc + v[t] * fused_dir(zz[t], beta, pp[t], first);
        return acc;
    }
    for (int t = 0; t < w; ++t) {
        const int c = cp[32 * t];
        if (c >= 0) acc = acc + vp[32 * t] * fused_dir(z[c], beta, first ? 0.0 : p[c], first);
    }
    return acc;
}


__device__ __forceinline__ float sell_row_dir(const Mat<float>& m, int s, int lane,
                                              const float* __restrict__ z,
                                              const float* __restrict__ p, float beta, bool first) {
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const float* vp = m.sval + b0 + lane;
    float acc = 0.f;
    if (w <= 8) {
        // the FP32 inner solves read explicit columns (their matrices carry no
        // patterns), so this loop has no pattern branch
        int c[8];
        float v[8], zz[8], pp[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            c[t] = t < w ? cp[32 * t] : -1;
            v[t] = t < w ? vp[32 * t] : 0.f;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            zz[t] = c[t] >= 0 ? z[c[t]] : 0.f;
            pp[t] = c[t] >= 0 && !first ? p[c[t]] : 0.f;
        }
        // difference form (see sell_row): the row's own direction first
        const int i = s * kWarp + lane;
        float di = 0.f;
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (c[t] == i) di = fused_dir(zz[t], beta, pp[t], first);
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (c[t] >= 0) acc = acc + diff_term(v[t], fused_dir(zz[t], beta, pp[t], first), di, c[t] == i);
        return acc;
    }
    const int i = s * kWarp + lane;
    const float di = i < m.n ? fused_dir(z[i], beta, first ? 0.f : p[i], first) : 0.f;
    for (int t = 0; t < w; ++t) {
        const int c = cp[32 * t];
        if (c >= 0)
            acc = acc + diff_term(vp[32 * t], fused_dir(z[c], beta, first ? 0.f : p[c], first), di,
                                  c == i);
    }
    return acc;
}

// r_i <- r_i - a_i1 x_1 - a_i2 x_2 - ... (Process/Resid.f90:28-33 order;
// FP32: r_i - (the difference-form product)).
template <typename T, typename X>
__device__ __forceinline__ T sell_resid_row(const Mat<T>& m, int s, int lane, T ri,
                                            const X* __restrict__ xv) {
    if constexpr (sizeof(T) == 4) return ri - sell_row(m, s, lane, xv);
    const long long b0 = m.soff[s];
    const int w = (int)((m.soff[s + 1] - b0) >> 5);
    const int* cp = m.scol + b0 + lane;
    const T* vp = m.sval + b0 + lane;
    if (w <= 8) {
        int c[8];
        T v[8], xx[8];
        sell_cols8(m, s, lane, w, b0, c);
#pragma unroll
        for (int t = 0; t < 8; ++t) v[t] = t < w ? vp[32 * t] : T(0);
#pragma unroll
        for (int t = 0; t < 8; ++t) xx[t] = c[t] >= 0 ? T(xv[c[t]]) : T(0);
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (c[t] >= 0) ri = ri - v[t] * xx[t];
        return ri;
    }
    for (int t = 0; t < w; ++t) {
        const int c = cp[32 * t];
        if (c >= 0) ri = ri - vp[32 * t] * T(xv[c]);
    }
    return ri;
}

// An off-diagonal factor entry for the IC sweeps: the BF16 copy when the
// matrix carries one (FP32 inner solves with ic_bf16), else the SELL value.
// BF16 -> FP32 is exact (the bit pattern shifted into the high half).
template <typename T>
__device__ __forceinline__ T lu_val(const Mat<T>& m, long long k) {
    if constexpr (sizeof(T) == 4) {
        if (m.lu16) return __uint_as_float((unsigned)m.lu16[k] << 16);
    }
    return m.sval[k];
}

template <typename T>
__device__ __forceinline__ T diag_value(const Mat<T>& m, int i) {
    const int dslot = m.meta[i] >> 16;
    return m.sval[m.soff[i >> 5] + (i & 31) + 32LL * dslot];
}

// ---- sync-free level-ordered sweeps ----------------------------------------
// Rows are visited in wavefront-level order in chunks of 32 rows of one
// level (levels padded to whole warps); warp w takes chunks w, w+nw, ... in
// increasing order.  A row waits only for the specific earlier rows it reads,
// through their value-as-flag cells; every index, coefficient and own-row
// operand is loaded before the first wait, so a row's critical path is one
// cell load per dependency.  A chunk only ever waits on rows of lower levels,
// which sit in chunks of lower index, so with all warps resident the sweep
// cannot deadlock.
constexpr int kSweepMax = 8;  // dependencies prefetched per row
// Longest pause between polls of not-yet-ready cells, in ns (0: poll back to
// back).
// Warps taking part in a sweep: at most `per_chunk` (a tuning parameter,
// default 4) per chunk of the widest level, so that a warp's next chunk is
// only a few levels ahead of the front and its polls rarely spin long.
constexpr int kSweepWarpsPerChunk = 4;

__device__ __forceinline__ int sweep_warps(const Grid& g, int wide, int per_chunk) {
    const int want = max(1, wide * (per_chunk > 0 ? per_chunk : kSweepWarpsPerChunk));
    return want < g.nw ? want : g.nw;
}

// One chunk of a level-ordered sweep.  Each lane owns one row; every index,
// coefficient and own-row operand is loaded before the first poll.  The
// warp then polls its rows' not-yet-ready dependency cells together, and a
// lane computes and publishes its row as soon as its own dependencies are
// in, without waiting for the other lanes, so a level's rows become visible
// one handoff after their inputs rather than after the slowest lane of the
// chunk.  Rows with more than kSweepMax dependencies wait one cell at a time.
// KIND 0: forward  acc = rhs - sum a_t cell_t,   result = acc * D_row
// KIND 1: backward acc = mid - sum a_t cell_t,   result = acc * D_row
// KIND 2: pivots   acc = a_ii - sum cell_t a_t a_t, result = 1 / acc
template <int KIND, typename T, typename Pub>
__device__ __forceinline__ bool sweep_chunk(const Grid& g, const Mat<T>& m, int row, int t0, int t1,
                                            long long base, T acc, T dmul, const T* cells,
                                            int where, Pub publish_row) {
    using C = Cell<T>;
    const int n = row >= 0 ? t1 - t0 : 0;
    const bool longrow = n > kSweepMax;  // rare: walked with a cursor instead
    int c[kSweepMax];
    T a[kSweepMax], v[kSweepMax];
    unsigned pending = 0;
#pragma unroll
    for (int u = 0; u < kSweepMax; ++u) {
        const bool use = !longrow && u < n;
        c[u] = use ? m.scol[base + 32LL * (t0 + u)] : 0;
        a[u] = use ? lu_val(m, base + 32LL * (t0 + u)) : T(0);
        v[u] = T(0);
        if (use) pending |= 1u << u;
    }
    int cursor = t0;
    bool done = row < 0;
    // Gate: while the chunk's inputs are far from ready, one lane polls one
    // representative cell (its dependency nearest in row order: the last
    // lower entry forward, the first upper entry backward) instead of every
    // lane polling every cell; the whole warp polls once it is in.  This
    // keeps thousands of early warps from loading L2 with polls.
    int gate_lane = -1, gate_col = 0;
    if (m.sweep_gate) {
        int rc = 0;
#pragma unroll
        for (int u = 0; u < kSweepMax; ++u)
            if (KIND == 1 ? u == 0 : u == n - 1) rc = c[u];
        const unsigned has = __ballot_sync(0xffffffffu, !longrow && n > 0);
        gate_lane = has ? __ffs(has) - 1 : -1;
        gate_col = __shfl_sync(0xffffffffu, rc, gate_lane < 0 ? 0 : gate_lane);
    }
    bool gated = gate_lane >= 0;
    const long long start = clock64();
    unsigned spins = 0;
    while (true) {
        if (gated) {
            int ready = 0;
            if (g.lane == gate_lane) ready = C::load(cells + gate_col) != C::kSentinel;
            gated = !__shfl_sync(0xffffffffu, ready, gate_lane);
        }
        if (!done && !gated) {
            if (longrow) {
                while (cursor < t1) {
                    const auto b = C::load(cells + m.scol[base + 32LL * cursor]);
                    if (b == C::kSentinel) break;
                    const T av = lu_val(m, base + 32LL * cursor);
                    const T vv = C::value(b);
                    acc = KIND == 2 ? acc - vv * av * av : acc - av * vv;
                    ++cursor;
                }
                if (cursor == t1) {
                    publish_row(KIND == 2 ? T(1) / acc : acc * dmul);
                    done = true;
                }
            } else {
#pragma unroll
                for (int u = 0; u < kSweepMax; ++u) {
                    if (pending & (1u << u)) {
                        const auto b = C::load(cells + c[u]);
                        if (b != C::kSentinel) {
                            v[u] = C::value(b);
                            pending &= ~(1u << u);
                        }
                    }
                }
                if (!pending) {
                    // every input present: sum in slot order (the reference's order)
#pragma unroll
                    for (int u = 0; u < kSweepMax; ++u)
                        if (u < n) acc = KIND == 2 ? acc - v[u] * a[u] * a[u] : acc - a[u] * v[u];
                    publish_row(KIND == 2 ? T(1) / acc : acc * dmul);
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) return true;
        // back off while the inputs are far from ready (a chunk several
        // levels ahead of the front), never more than m.sweep_sleep ns
        ++spins;
        if (m.sweep_sleep > 0 && spins > 4u)
            __nanosleep(min((unsigned)m.sweep_sleep, 8u << min(spins - 4u, 10u)));
        if ((spins & 63u) == 0u) {
            bool quit = ld_relaxed_s32(&g.ctl->abort) != 0;
            if (!quit && clock64() - start > g.timeout_cyc) {
                raise_abort(g.ctl, ST_TIMEOUT, where);
                quit = true;
            }
            if (__any_sync(0xffffffffu, quit)) return false;
        }
    }
}

// ---- Prec1 -----------------------------------------------------------------
// prec 1: D_i = a_ii; prec 2: D_i = 1 / (a_ii - sum_{k<i} D_k a_ik a_ik);
// otherwise D_i = 1 (Process/Prec1.f90:45-67).  IC ends with a grid barrier.
template <typename T>
__device__ bool prec1_phase(Grid& g, const Mat<T>& m, T* D, int prec) {
    if (prec == 2) {
        TF_FOR_ROWS(g, m, i) { D[i] = Cell<T>::sentinel(); }
        if (!grid_sync(g, 10)) return false;
        bool ok = true;
        const int nws = sweep_warps(g, m.wide_f, m.sweep_mult);
        for (int ch = g.wg; g.wg < nws && ch < m.nchunk_f && ok; ch += nws) {
            const int row = m.perm_f[ch * kWarp + g.lane];
            int dslot = 0;
            long long base = 0;
            T aii = T(1);
            if (row >= 0) {
                dslot = m.meta[row] >> 16;
                base = m.soff[row >> 5] + (row & 31);
                aii = m.sval[base + 32LL * dslot];
            }
            ok = sweep_chunk<2>(g, m, row, 0, dslot, base, aii, T(1), D, 11,
                                [&](T d) { Cell<T>::store(D + row, d); });
        }
        const bool synced = grid_sync(g, 12);
        return ok && synced;
    }
    // with a reciprocal diagonal (contracted FP64 build) D holds 1 / a_ii
    TF_FOR_ROWS(g, m, i) {
        D[i] = (prec == 1) ? (sizeof(T) == 8 && kRecipDiag64 ? T(1) / diag_value(m, i)
                                                            : diag_value(m, i))
                           : T(1);
    }
    return true;  // made visible by the caller's next barrier
}

// ---- IC(0) apply -------------------------------------------------------------
// z = [(D~+U)^-1 D~ (D~+L)^-1] rhs with D~ = 1/D, computed as the reference
// does: forward w_i = D_i (rhs_i - sum_{k<i} a_ik w_k); middle
// w_i / (D_i + TINY); backward z_i = D_i (mid_i - sum_{k>i} a_ik z_k).
// `w` cells must hold the sentinel on entry and hold it again on exit.
// The backward phase calls `epi(row, z_row, rhs_row)` for fused per-row work.
template <typename T, typename Epi>
__device__ bool ic_apply(Grid& g, const Mat<T>& m, const T* D, const T* rhs, T* w, T* z, Epi epi) {
    bool ok = true;
    const int nwf = sweep_warps(g, m.wide_f, m.sweep_mult);
    for (int ch = g.wg; g.wg < nwf && ch < m.nchunk_f && ok; ch += nwf) {
        const int row = m.perm_f[ch * kWarp + g.lane];
        int dslot = 0;
        long long base = 0;
        T r0 = T(0), d = T(0);
        if (row >= 0) {
            dslot = m.meta[row] >> 16;
            base = m.soff[row >> 5] + (row & 31);
            r0 = rhs[row];
            d = D[row];
            z[row] = Cell<T>::sentinel();
        }
        ok = sweep_chunk<0>(g, m, row, 0, dslot, base, r0, d, w, 20,
                            [&](T val) { Cell<T>::store(w + row, val); });
    }
    if (!grid_sync(g, 21) || !ok) return false;
    const int nwb = sweep_warps(g, m.wide_b, m.sweep_mult);
    for (int ch = g.wg; g.wg < nwb && ch < m.nchunk_b && ok; ch += nwb) {
        const int row = m.perm_b[ch * kWarp + g.lane];
        int dslot = 0, len = 0;
        long long base = 0;
        T mid = T(0), d = T(0);
        if (row >= 0) {
            const int meta = m.meta[row];
            len = meta & 0xFFFF;
            dslot = meta >> 16;
            base = m.soff[row >> 5] + (row & 31);
            d = D[row];
            mid = w[row] / (d + tiny_v<T>());
        }
        ok = sweep_chunk<1>(g, m, row, dslot + 1, row >= 0 ? len : dslot + 1, base, mid, d, z, 22,
                            [&](T zi) {
                                Cell<T>::store(z + row, zi);
                                w[row] = Cell<T>::sentinel();
                                epi(row, zi, rhs[row]);
                            });
    }
    return ok;
}

// ---- IC(0) apply by Jacobi sweeps (FP32 inner solves, ic_sweeps = k > 0) ----
// Each triangular solve of the exact apply is replaced by k Jacobi sweeps
//     y^s_i = D_i (f_i - sum_{t in the triangle of row i} a_it y^(s-1)_t),
//     y^0   = D f,
// every sweep one fully parallel pass over one triangle (no waits between
// rows, a grid barrier between sweeps); the middle step y_i / (D_i + TINY)
// is folded into the last forward sweep.  For a symmetric matrix the
// backward sweeps are the transposes of the forward ones, so the operator is
// fixed and symmetric and CG stays valid; it tends to the exact IC(0) apply
// as k grows (after k = number of levels it is exact).
template <bool FWD, typename T, typename Fin>
__device__ __forceinline__ void tri_jacobi(const Grid& g, const Mat<T>& m, const T* __restrict__ D,
                                           const T* __restrict__ f, const T* __restrict__ y,
                                           T* __restrict__ out, Fin fin) {
    for (int s = g.wg; s < m.nslices; s += g.nw) {
        const int i = s * kWarp + g.lane;
        if (i >= m.n) continue;
        const int meta = m.meta[i];
        const int dslot = meta >> 16;
        const int t0 = FWD ? 0 : dslot + 1;
        const int nt = (FWD ? dslot : (meta & 0xFFFF)) - t0;
        const long long base = m.soff[s] + g.lane + 32LL * t0;
        T acc = f[i];
        const T di = D[i];
        if (nt <= kSweepMax) {
            int c[kSweepMax];
            T a[kSweepMax], yv[kSweepMax];
#pragma unroll
            for (int u = 0; u < kSweepMax; ++u) {
                c[u] = u < nt ? m.scol[base + 32LL * u] : 0;
                a[u] = u < nt ? lu_val(m, base + 32LL * u) : T(0);
            }
#pragma unroll
            for (int u = 0; u < kSweepMax; ++u)
                yv[u] = u < nt ? (y ? y[c[u]] : D[c[u]] * f[c[u]]) : T(0);
#pragma unroll
            for (int u = 0; u < kSweepMax; ++u)
                if (u < nt) acc = acc - a[u] * yv[u];
        } else {
            for (int u = 0; u < nt; ++u) {
                const int c = m.scol[base + 32LL * u];
                acc = acc - lu_val(m, base + 32LL * u) * (y ? y[c] : D[c] * f[c]);
            }
        }
        out[i] = fin(i, acc * di);
    }
}

// k forward sweeps ping-pong between w and s (the last one stores the middle
// vector), k backward sweeps between z and the other buffer, the last one
// into z with `epi(row, z_row, rhs_row)` fused.  No barrier after the last sweep.
template <typename T, typename Epi>
__device__ bool ic_jacobi_apply(Grid& g, const Mat<T>& m, const T* D, const T* rhs, T* w, T* sb,
                                T* z, int k, Epi epi) {
    T* fb[2] = {w, sb};
    for (int sw = 1; sw <= k; ++sw) {
        const T* y = sw == 1 ? nullptr : fb[(sw - 1) & 1];
        T* o = fb[sw & 1];
        if (sw < k)
            tri_jacobi<true>(g, m, D, rhs, y, o, [](int, T v) { return v; });
        else
            tri_jacobi<true>(g, m, D, rhs, y, o, [&](int i, T v) { return v / (D[i] + tiny_v<T>()); });
        if (!grid_sync(g, 23)) return false;
    }
    const T* mid = fb[k & 1];
    T* bb[2] = {z, fb[(k + 1) & 1]};
    for (int sw = 1; sw <= k; ++sw) {
        const T* y = sw == 1 ? nullptr : bb[(k - sw + 1) & 1];
        T* o = bb[(k - sw) & 1];
        if (sw < k) {
            tri_jacobi<false>(g, m, D, mid, y, o, [](int, T v) { return v; });
            if (!grid_sync(g, 24)) return false;
        } else {
            tri_jacobi<false>(g, m, D, mid, y, o, [&](int i, T v) {
                epi(i, v, rhs[i]);
                return v;
            });
        }
    }
    return true;
}

// ---- tiled IC(0) sweeps (box-numbered patterns) --------------------------------
// Forward: row (x, y, z) needs (x, y, z-1), (x, y-1, z), (x-1, y, z), in the
// stored order of its lower entries (columns ascending, CG.f90:135-142).
// Thread (lx, ly) of a tile walks its column: at step s it computes the row
// with z = s - lx - ly.  Its z-1 input is its own result of step s-1, its
// y-1 and x-1 inputs are the results of threads (lx, ly-1) and (lx-1, ly)
// at step s-1, exchanged through shared memory with one block barrier per
// step -- or, on the tile's low edges, the cells of the neighbouring tiles,
// which run the same steps ahead of this one (tiles are taken in increasing
// index, each depending only on lower ones, all blocks resident, so the
// sweep cannot deadlock).  Backward mirrors it (x+1, y+1, z+1; tiles and
// steps in decreasing order).  Each row combines the same operands in the
// same order as the sequential sweep (CG.f90:135-156), so in the
// reference-arithmetic build the result is bit-identical to it and to the
// level-ordered sweeps.
//
// The records are staged into a ring of two halves of `half` consecutive
// steps each; one bulk async copy (one elected thread, one mbarrier per half)
// fills a half while the block works through the other, so the issue cost is
// paid once per `half` steps.  The right-hand side enters the forward records
// through a gather each block runs for its own tiles before their first
// step; the neighbour tiles' edge cells are loaded two steps ahead and
// polled again only if they were not ready yet.

struct TileSmem {
    unsigned long long* bar;  // two barriers, one per ring half
    volatile int* fail;       // set by a thread whose wait gave up
    int* phase;               // the halves' phase parities between sweeps
    unsigned char* ring;      // two halves of `half` records (at most tile_slot_bytes each)
    unsigned slot;            // bytes of the largest record
};

template <typename T>
__device__ __forceinline__ TileSmem tile_smem(const Tiles<T>& tl) {
    extern __shared__ __align__(128) unsigned char tf_smem[];
    TileSmem m;
    m.bar = reinterpret_cast<unsigned long long*>(tf_smem);
    m.fail = reinterpret_cast<volatile int*>(tf_smem + 64);
    m.phase = reinterpret_cast<int*>(tf_smem + 68);
    m.ring = tf_smem + 128;
    m.slot = tile_slot_bytes(blockDim.x, tl.lu_bf16 ? 2u : (unsigned)sizeof(T), (unsigned)sizeof(T));
    return m;
}

// Byte offset of value field v (0 = D, 1 = rhs / mid, 2 = 1/(D+TINY) / rhs)
// in a record, after the three coefficient fields.
template <typename T>
__device__ __forceinline__ unsigned tile_vfield(const Tiles<T>& tl, int v) {
    return blockDim.x * (3u * (tl.lu_bf16 ? 2u : (unsigned)sizeof(T)) + v * (unsigned)sizeof(T));
}

// Coefficient f of thread t in a staged record.
template <typename T>
__device__ __forceinline__ T tile_coef(const Tiles<T>& tl, const unsigned char* rec, int f, int t) {
    if constexpr (sizeof(T) == 4) {
        if (tl.lu_bf16) {
            const unsigned short u =
                reinterpret_cast<const unsigned short*>(rec + (size_t)f * blockDim.x * 2)[t];
            return __uint_as_float((unsigned)u << 16);
        }
    }
    return reinterpret_cast<const T*>(rec + (size_t)f * blockDim.x * sizeof(T))[t];
}

// The same for a record staged in shared memory, at shared address `rec`.
template <typename T>
__device__ __forceinline__ T tile_coef_s(const Tiles<T>& tl, unsigned rec, int f, int t) {
    if constexpr (sizeof(T) == 4) {
        if (tl.lu_bf16)
            return __uint_as_float((unsigned)lds<unsigned short>(rec + (f * blockDim.x + t) * 2u)
                                   << 16);
    }
    return lds<T>(rec + (f * blockDim.x + t) * (unsigned)sizeof(T));
}

template <typename T>
__device__ __forceinline__ T& tile_val(const Tiles<T>& tl, unsigned char* rec, int v, int t) {
    return reinterpret_cast<T*>(rec + tile_vfield(tl, v))[t];
}

// `count` consecutive records of `rec_bytes` each (a multiple of 128) into a
// ring half, packed as they are in global memory: one copy, completing on
// the half's barrier.
__device__ __forceinline__ void tile_issue(unsigned char* dst, unsigned long long* bar,
                                           const unsigned char* rec, unsigned rec_bytes,
                                           int count) {
    mbar_expect_tx(bar, rec_bytes * count);
    bulk_g2s(dst, rec, rec_bytes * count, bar);
}

// A prefetched neighbour cell, polled again (bounded) while it still holds
// the sentinel.  On giving up: abort raised, the block's fail flag set.
// (`ctl` and the limit `tmo` come as values: the sweeps keep everything
// they use per step in registers.)
template <typename T>
__device__ __forceinline__ T tile_cell(DevCtl* ctl, long long tmo, const TileSmem& sm, const T* p,
                                       T v, int where) {
    using C = Cell<T>;
    if (C::bits(v) != C::kSentinel) return v;
    const long long t0 = clock64();
    unsigned spins = 0;
    while (true) {
        const auto b = C::load(p);
        if (b != C::kSentinel) return C::value(b);
        if ((++spins & 63u) == 0u) {
            const bool quit = ld_relaxed_s32(&ctl->abort) != 0;
            if (quit || clock64() - t0 > tmo) {
                if (!quit) raise_abort(ctl, ST_TIMEOUT, where);
                *sm.fail = 1;
                return T(0);
            }
        }
    }
}

// Waits for a ring half's copy (bounded).  False: abort raised, fail set.
__device__ __forceinline__ bool tile_wait(DevCtl* ctl, long long tmo, const TileSmem& sm, int h,
                                          unsigned parity, int where) {
    if (mbar_try_wait(sm.bar + h, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(sm.bar + h, parity)) {
        if (clock64() - t0 > tmo) {
            raise_abort(ctl, ST_TIMEOUT, where);
            *sm.fail = 1;
            return false;
        }
    }
    return true;
}

// After a failure: thread 0 waits (bounded) for the copies still in flight
// into the ring (the halves issued and not yet waited for, bits of `pend`).
__device__ __forceinline__ void tile_drain(long long tmo, const TileSmem& sm, unsigned pend,
                                           unsigned phase) {
    if (threadIdx.x != 0) return;
    for (int h = 0; h < 2; ++h) {
        if (!(pend & (1u << h))) continue;
        const long long t0 = clock64();
        while (!mbar_try_wait(sm.bar + h, (phase >> h) & 1u))
            if (clock64() - t0 > tmo) break;
    }
}

// Once per solve, before the first apply (a grid barrier must follow): the
// pivots (and the reciprocals) into both record kinds, sentinels into both
// cell arrays, the ring barriers initialised.
template <typename T>
__device__ void tiles_init(Grid& g, const Mat<T>& m, const T* __restrict__ D) {
    const Tiles<T>& tl = m.tile;
    const int B = blockDim.x;
    const long long total = (long long)tl.ntx * tl.nty * tl.steps * B;
    const T sen = Cell<T>::sentinel();
    for (long long i = g.tid; i < total; i += g.nt) {
        const int t = (int)(i % B);
        const long long ks = i / B;
        const int s = (int)(ks % tl.steps), k = (int)(ks / tl.steps);
        const int lx = t % kTileX, ly = t / kTileX;
        const int x = (k % tl.ntx) * kTileX + lx, y = (k / tl.ntx) * tl.ty + ly, z = s - lx - ly;
        const bool act = x < tl.nx && y < tl.ny && z >= 0 && z < tl.nz;
        const T d = act ? D[x + tl.nx * (y + tl.ny * z)] : T(0);
        unsigned char* rf = tl.fwd + ks * tl.rec_f;
        unsigned char* rb = tl.bwd + ks * tl.rec_b;
        tile_val(tl, rf, 0, t) = d;
        tile_val(tl, rb, 0, t) = d;
        if (tl.recip) tile_val(tl, rf, 2, t) = act ? T(1) / (d + tiny_v<T>()) : T(0);
        tl.wt[i] = sen;
        tl.zt[i] = sen;
    }
    const TileSmem sm = tile_smem(tl);
    if (threadIdx.x == 0) {
        mbar_init(sm.bar, 1);
        mbar_init(sm.bar + 1, 1);
        *sm.fail = 0;
        *sm.phase = 0;
        mbar_init_fence();
    }
    __syncthreads();
}

template <typename T>
__device__ bool tile_forward(Grid& g, const Mat<T>& m, const T* __restrict__ rhs) {
    const Tiles<T> tl = m.tile;  // a copy: the per-step fields stay in registers
    DevCtl* const ctl = g.ctl;
    const long long tmo = g.timeout_cyc;
    const TileSmem sm = tile_smem(tl);
    const int B = blockDim.x, t = threadIdx.x, lx = t % kTileX, ly = t / kTileX;
    const int S = tl.steps, ntiles = tl.ntx * tl.nty, H = tl.half;
    const size_t plane = (size_t)S * B;
    // shared addresses of the ring and of the neighbour exchange (two step
    // parities of B values); this thread's own offsets within a record
    const unsigned ring_a = smem_u32(sm.ring);
    const unsigned nbv_a = ring_a + 2 * H * sm.slot;
    const unsigned sz = (unsigned)sizeof(T);
    const unsigned vf0 = tile_vfield(tl, 0) + t * sz, vf1 = tile_vfield(tl, 1) + t * sz,
                   vf2 = tile_vfield(tl, 2) + t * sz;
    __syncthreads();
    unsigned phase = (unsigned)*sm.phase, pend = 0;
    bool ok = true;
    for (int k = g.bid; k < ntiles && ok; k += g.nblocks) {
        const int x = (k % tl.ntx) * kTileX + lx, y = (k / tl.ntx) * tl.ty + ly;
        const bool inb = x < tl.nx && y < tl.ny;
        const size_t base = (size_t)k * plane;
        unsigned char* recf = tl.fwd + (size_t)k * S * tl.rec_f;
        unsigned char* recb = tl.bwd + (size_t)k * S * tl.rec_b;
        // gather this tile's right-hand side into its forward records
        // (eight independent loads in flight per thread)
        for (int s0 = 0; s0 < S; s0 += 8) {
            T v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int z = s0 + q - lx - ly;
                v[q] = inb && z >= 0 && z < tl.nz && s0 + q < S ? rhs[x + tl.nx * (y + tl.ny * z)]
                                                                : T(0);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (s0 + q < S) *reinterpret_cast<T*>(recf + (size_t)(s0 + q) * tl.rec_f + vf1) = v[q];
        }
        __syncthreads();
        // edge cells of the left (x-1) and lower (y-1) tiles at step s
        // (used only where that tile exists: x > 0 resp. y > 0)
        const long long sb = (long long)base, sp = (long long)plane;
        const T* xcell = tl.wt + (sb - sp + (long long)(kTileX - 1) * B + ly * kTileX + (kTileX - 1));
        const T* ycell =
            tl.wt + (sb - tl.ntx * sp + (long long)(tl.ty - 1) * B + (tl.ty - 1) * kTileX + lx);
        if (t == 0) {
            // the gathered words (and the records written before the sweep)
            // and the previous tile's reads of the ring before the bulk copies
            fence_proxy_async_global();
            fence_proxy_async_smem();
            for (int h = 0; h < 2 && h * H < S; ++h) {
                tile_issue(sm.ring + h * H * tl.rec_f, sm.bar + h, recf + (size_t)h * H * tl.rec_f,
                           tl.rec_f, min(H, S - h * H));
                pend |= 1u << h;
            }
        }
        // neighbour cells two steps ahead, by step parity
        T xp0 = T(0), xp1 = T(0), yp0 = T(0), yp1 = T(0);
        auto prefetch = [&](int s) {
            const int z = s - lx - ly;
            if (inb && z >= 0 && z < tl.nz) {
                T xv = T(0), yv = T(0);
                if (lx == 0 && x > 0) xv = Cell<T>::value(Cell<T>::load(xcell + (size_t)s * B));
                if (ly == 0 && y > 0) yv = Cell<T>::value(Cell<T>::load(ycell + (size_t)s * B));
                if (s & 1) { xp1 = xv; yp1 = yv; } else { xp0 = xv; yp0 = yv; }
            }
        };
        prefetch(0);
        if (S > 1) prefetch(1);
        T ycur = T(0);
        // one ring half per outer pass (no index arithmetic by a runtime
        // divisor per step); a failed wait ends the tile at the half's end
        int hb = 0;
        for (int s0 = 0; s0 < S; s0 += H, hb ^= 1) {
            tile_wait(ctl, tmo, sm, hb, (phase >> hb) & 1u, 26);
            phase ^= 1u << hb;
            pend &= ~(1u << hb);
            const int cnt = min(H, S - s0);
            const unsigned half = ring_a + (unsigned)(hb * H) * tl.rec_f;
            for (int q = 0; q < cnt; ++q) {
                const int s = s0 + q;
                const int z = s - lx - ly;
                if (inb && z >= 0 && z < tl.nz) {
                    const unsigned sl = half + (unsigned)q * tl.rec_f;
                    const unsigned nb_prev = nbv_a + ((unsigned)((s - 1) & 1) * B + t) * sz;
                    const T ri = lds<T>(sl + vf1);
                    T acc = ri;
                    if (z > 0) acc = acc - tile_coef_s(tl, sl, 0, t) * ycur;
                    if (y > 0) {
                        const T v = ly > 0 ? lds<T>(nb_prev - kTileX * sz)
                                           : tile_cell(ctl, tmo, sm, ycell + (size_t)s * B,
                                                       (s & 1) ? yp1 : yp0, 27);
                        acc = acc - tile_coef_s(tl, sl, 1, t) * v;
                    }
                    if (x > 0) {
                        const T v = lx > 0 ? lds<T>(nb_prev - sz)
                                           : tile_cell(ctl, tmo, sm, xcell + (size_t)s * B,
                                                       (s & 1) ? xp1 : xp0, 27);
                        acc = acc - tile_coef_s(tl, sl, 2, t) * v;
                    }
                    const T d = lds<T>(sl + vf0);
                    const T yv = acc * d;
                    sts(nbv_a + ((unsigned)(s & 1) * B + t) * sz, yv);
                    ycur = yv;
                    const size_t idx = base + (size_t)s * B + t;
                    Cell<T>::store(tl.wt + idx, yv);
                    // the middle step of CG.f90:144-146, for the backward sweep
                    const T mid = tl.recip ? yv * lds<T>(sl + vf2) : yv / (d + tiny_v<T>());
                    unsigned char* rb = recb + (size_t)s * tl.rec_b;
                    *reinterpret_cast<T*>(rb + vf1) = mid;
                    *reinterpret_cast<T*>(rb + vf2) = ri;
                    tl.zt[idx] = Cell<T>::sentinel();
                }
                __syncthreads();
                if (s + 2 < S) prefetch(s + 2);
            }
            if (*sm.fail) {
                tile_drain(tmo, sm, pend, phase);
                ok = false;
                break;
            }
            // this half consumed: refill it with the steps after the other half
            const int first = s0 + 2 * H;
            if (t == 0 && first < S) {
                fence_proxy_async_smem();  // the half's reads before its refill
                tile_issue(sm.ring + (size_t)hb * H * tl.rec_f, sm.bar + hb,
                           recf + (size_t)first * tl.rec_f, tl.rec_f, min(H, S - first));
                pend |= 1u << hb;
            }
        }
    }
    __syncthreads();
    if (t == 0) *sm.phase = (int)phase;
    __syncthreads();
    return ok;
}

template <typename T, typename Epi>
__device__ bool tile_backward(Grid& g, const Mat<T>& m, T* __restrict__ zout, Epi epi) {
    const Tiles<T> tl = m.tile;  // a copy: the per-step fields stay in registers
    DevCtl* const ctl = g.ctl;
    const long long tmo = g.timeout_cyc;
    const TileSmem sm = tile_smem(tl);
    const int B = blockDim.x, t = threadIdx.x, lx = t % kTileX, ly = t / kTileX;
    const int S = tl.steps, ntiles = tl.ntx * tl.nty, H = tl.half;
    const size_t plane = (size_t)S * B;
    const unsigned ring_a = smem_u32(sm.ring);
    const unsigned nbv_a = ring_a + 2 * H * sm.slot;
    const unsigned sz = (unsigned)sizeof(T);
    const unsigned vf0 = tile_vfield(tl, 0) + t * sz, vf1 = tile_vfield(tl, 1) + t * sz,
                   vf2 = tile_vfield(tl, 2) + t * sz;
    __syncthreads();
    unsigned phase = (unsigned)*sm.phase, pend = 0;
    if (t == 0) fence_proxy_async_global();  // the records written before the barrier
    bool ok = true;
    // this block's tiles (g.bid, g.bid + nblocks, ...) in decreasing order
    const int mine = g.bid < ntiles ? (ntiles - 1 - g.bid) / g.nblocks + 1 : 0;
    for (int q = mine - 1; q >= 0 && ok; --q) {
        const int k = g.bid + q * g.nblocks;
        const int x = (k % tl.ntx) * kTileX + lx, y = (k / tl.ntx) * tl.ty + ly;
        const bool inb = x < tl.nx && y < tl.ny;
        const size_t base = (size_t)k * plane;
        const unsigned char* recb = tl.bwd + (size_t)k * S * tl.rec_b;
        // edge cells of the right (x+1) and upper (y+1) tiles at step s
        // (used only where that tile exists: x < nx-1 resp. y < ny-1)
        const long long sb = (long long)base, sp = (long long)plane;
        const T* xcell = tl.zt + (sb + sp + ly * kTileX - (long long)(kTileX - 1) * B);
        const T* ycell = tl.zt + (sb + tl.ntx * sp + lx - (long long)(tl.ty - 1) * B);
        // half h holds the steps of indices j in [h H, h H + H), j = S-1-s;
        // they are the records S-1-j, in decreasing order, so the copy
        // starts at the lowest step of the range and slot u holds step
        // S-1-j at position (H-1-(j mod H)) from the half's start
        auto issue = [&](int h, int j0) {
            const int cnt = min(H, S - j0);
            const int slo = S - 1 - (j0 + cnt - 1);  // lowest step of the range
            tile_issue(sm.ring + (size_t)(h * H + H - cnt) * tl.rec_b, sm.bar + h,
                       recb + (size_t)slo * tl.rec_b, tl.rec_b, cnt);
            pend |= 1u << h;
        };
        if (t == 0) {
            fence_proxy_async_smem();
            for (int h = 0; h < 2 && h * H < S; ++h) issue(h, h * H);
        }
        T xp0 = T(0), xp1 = T(0), yp0 = T(0), yp1 = T(0);
        auto prefetch = [&](int j) {
            const int s = S - 1 - j, z = s - lx - ly;
            if (inb && z >= 0 && z < tl.nz) {
                T xv = T(0), yv = T(0);
                if (lx == kTileX - 1 && x < tl.nx - 1)
                    xv = Cell<T>::value(Cell<T>::load(xcell + (size_t)s * B));
                if (ly == tl.ty - 1 && y < tl.ny - 1)
                    yv = Cell<T>::value(Cell<T>::load(ycell + (size_t)s * B));
                if (j & 1) { xp1 = xv; yp1 = yv; } else { xp0 = xv; yp0 = yv; }
            }
        };
        prefetch(0);
        if (S > 1) prefetch(1);
        T zcur = T(0);
        int hb = 0;
        for (int j0 = 0; j0 < S; j0 += H, hb ^= 1) {
            tile_wait(ctl, tmo, sm, hb, (phase >> hb) & 1u, 28);
            phase ^= 1u << hb;
            pend &= ~(1u << hb);
            const int cnt = min(H, S - j0);
            // step S-1-(j0+q) sits at slot H-1-q of the half
            const unsigned half = ring_a + (unsigned)(hb * H + H - 1) * tl.rec_b;
            for (int q = 0; q < cnt; ++q) {
                const int j = j0 + q;
                const int s = S - 1 - j;
                const int z = s - lx - ly;
                if (inb && z >= 0 && z < tl.nz) {
                    const unsigned sl = half - (unsigned)q * tl.rec_b;
                    const unsigned nb_prev = nbv_a + ((unsigned)((j - 1) & 1) * B + t) * sz;
                    const T d = lds<T>(sl + vf0);
                    T acc = lds<T>(sl + vf1);  // mid
                    const T ri = lds<T>(sl + vf2);
                    if (x < tl.nx - 1) {
                        const T v = lx < kTileX - 1
                                        ? lds<T>(nb_prev + sz)
                                        : tile_cell(ctl, tmo, sm, xcell + (size_t)s * B,
                                                    (j & 1) ? xp1 : xp0, 29);
                        acc = acc - tile_coef_s(tl, sl, 0, t) * v;
                    }
                    if (y < tl.ny - 1) {
                        const T v = ly < tl.ty - 1
                                        ? lds<T>(nb_prev + kTileX * sz)
                                        : tile_cell(ctl, tmo, sm, ycell + (size_t)s * B,
                                                    (j & 1) ? yp1 : yp0, 29);
                        acc = acc - tile_coef_s(tl, sl, 1, t) * v;
                    }
                    if (z < tl.nz - 1) acc = acc - tile_coef_s(tl, sl, 2, t) * zcur;
                    const T zi = acc * d;
                    sts(nbv_a + ((unsigned)(j & 1) * B + t) * sz, zi);
                    zcur = zi;
                    const size_t idx = base + (size_t)s * B + t;
                    Cell<T>::store(tl.zt + idx, zi);
                    tl.wt[idx] = Cell<T>::sentinel();
                    const int row = x + tl.nx * (y + tl.ny * z);
                    zout[row] = zi;
                    epi(row, zi, ri);
                }
                __syncthreads();
                if (j + 2 < S) prefetch(j + 2);
            }
            if (*sm.fail) {
                tile_drain(tmo, sm, pend, phase);
                ok = false;
                break;
            }
            const int jn = j0 + 2 * H;
            if (t == 0 && jn < S) {
                fence_proxy_async_smem();
                issue(hb, jn);
            }
        }
    }
    __syncthreads();
    if (t == 0) *sm.phase = (int)phase;
    __syncthreads();
    return ok;
}

// z = IC(0) apply of rhs by the tiled sweeps; epi(row, z_row, rhs_row) per row.
template <typename T, typename Epi>
__device__ bool ic_tiled_apply(Grid& g, const Mat<T>& m, const T* rhs, T* z, Epi epi) {
    const bool ok = tile_forward(g, m, rhs);
    if (!grid_sync(g, 25) || !ok) return false;
    return tile_backward(g, m, z, epi);
}

// The IC(0) apply the solve was configured for: `sweeps` Jacobi sweeps per
// triangle (FP32 inner solves and contracted FP64 solves), else the exact
// apply -- tiled sweeps on a box-numbered pattern, level-ordered sync-free
// sweeps otherwise.  epi(row, z_row, rhs_row) runs once per row.
template <typename T, typename Epi>
__device__ __forceinline__ bool ic_precond(Grid& g, const Mat<T>& m, Vecs<T>& v, int sweeps,
                                           const T* rhs, T* z, Epi epi) {
    if (sweeps > 0) return ic_jacobi_apply(g, m, v.D, rhs, v.w, v.s, z, sweeps, epi);
    if (m.tile.on) return ic_tiled_apply(g, m, rhs, z, epi);
    return ic_apply(g, m, v.D, rhs, v.w, z, epi);
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
    // (IC pivots complete: prec1_phase ends with a barrier; the barrier
    // below orders the tiled layout before the first apply)
    if (cfg.do_prec1 && cfg.prec == 2 && m.tile.on) tiles_init(g, m, v.D);
    T acc[1] = {T(0)};
    TF_FOR4(g, m, i) {
        const V4<T> r = ld4(v.r + i);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u < m.n) acc[0] += r.a[u] * r.a[u];
    }
    publish_t<1>(g, SLOT_A, acc);
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
    T a2[2] = {T(0), T(0)};
    for (int s = g.wg; s < m.nslices; s += g.nw) {
        const int i = s * kWarp + g.lane;
        T ri = i < m.n ? v.r[i] : T(0);
        if (!cfg.x_is_zero) ri = sell_resid_row(m, s, g.lane, ri, v.x);
        if (i < m.n) {
            v.r[i] = ri;
            a2[0] += ri * ri;
            if (store_z) {
                if (cfg.prec == 1) {
                    const T zi = jacobi(ri, v.D[i]);
                    v.z[i] = zi;
                    a2[1] += ri * zi;
                }
            }
        }
    }
    publish_t<2>(g, SLOT_B, a2);
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
    // search direction; the FP32 inner solves alternate between p and t
    T* pcur = v.p;
    T* pnext = v.t;
    for (; iter <= cfg.maxiter; ++iter) {
        if (prec == 2) {
            T a[1] = {T(0)};
            const bool ok = ic_precond(g, m, v, cfg.ic_sweeps, v.r, v.z, [&](int, T zi, T ri) {
                a[0] += ri * zi;
            });
            publish_t<1>(g, SLOT_A, a);
            if (!grid_sync(g, 41) || !ok) { out.exit_kind = EXIT_ABORT; return; }
            double t[1];
            totals<1>(g, SLOT_A, t);
            rho = t[0];
        } else {
            rho = rho_next;
        }
        // The new search direction formed inside the product, into the other
        // p buffer (no separate update pass, one barrier less per
        // iteration): always in the FP32 inner solves; in FP64 where the
        // host asked for it (systems whose vectors stay in L2 -- on larger
        // ones gathering z and p and forming z + beta p per neighbour on the
        // FP64 pipe costs more than the pass it saves).
        const bool fused = sizeof(T) == 4 || cfg.fuse_dir;
        if (fused) {
            const T beta = iter == 1 ? T(0) : T(rho / rhoold);
            const bool first = iter == 1;
            const T* pold = pcur;
            T* pnew = pnext;
            T a1[1] = {T(0)};
            for (int s = g.wg; s < m.nslices; s += g.nw) {
                const int i = s * kWarp + g.lane;
                const T qi = sell_row_dir(m, s, g.lane, z, pold, beta, first);
                if (i < m.n) {
                    const T pi = fused_dir(z[i], beta, first ? T(0) : pold[i], first);
                    pnew[i] = pi;
                    v.q[i] = qi;
                    a1[0] += pi * qi;
                }
            }
            pcur = pnew;
            pnext = const_cast<T*>(pold);
            publish_t<1>(g, SLOT_C, a1);
            if (!grid_sync(g, 43)) { out.exit_kind = EXIT_ABORT; return; }
        }
        if (!fused) {
        // p = z + beta p  (CG.f90:178-187)
        if (iter == 1) {
            TF_FOR4(g, m, i) { st4(v.p + i, ld4(z + i)); }
        } else {
            const T beta = T(rho / rhoold);
            TF_FOR4(g, m, i) {
                const V4<T> zz = ld4(z + i);
                V4<T> pp = ld4(v.p + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) pp.a[u] = zz.a[u] + beta * pp.a[u];
                st4(v.p + i, pp);
            }
        }
        if (!grid_sync(g, 42)) { out.exit_kind = EXIT_ABORT; return; }
        // q = A p; (p, q)  (CG.f90:193-218)
        T a1[1] = {T(0)};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T qi = sell_row(m, s, g.lane, v.p);
            if (i < m.n) {
                v.q[i] = qi;
                a1[0] += v.p[i] * qi;
            }
        }
        publish_t<1>(g, SLOT_C, a1);
        if (!grid_sync(g, 43)) { out.exit_kind = EXIT_ABORT; return; }
        }
        double t1[1];
        totals<1>(g, SLOT_C, t1);
        const double alfa_d = rho / t1[0];
        const T alfa = T(alfa_d);
        // x += alfa p; r -= alfa q; ||r||; next z and rho  (CG.f90:226-253)
        T a3[3] = {T(0), T(0), T(0)};
        TF_FOR4(g, m, i) {
            V4<T> xx = ld4(v.x + i), rr = ld4(v.r + i);
            const V4<T> pp = ld4(pcur + i), qq = ld4(v.q + i);
            V4<T> dd, zz;
            if (prec == 1) dd = ld4(v.D + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                xx.a[u] = xx.a[u] + alfa * pp.a[u];
                rr.a[u] = rr.a[u] - alfa * qq.a[u];
                if (prec == 1) zz.a[u] = jacobi(rr.a[u], dd.a[u]);
                if (i + u < m.n) {
                    a3[0] += rr.a[u] * rr.a[u];
                    if (prec == 1) a3[1] += rr.a[u] * zz.a[u];
                    if (nonfinite)
                        a3[2] += (xx.a[u] == xx.a[u] ? T(1) : T(0)) + (rr.a[u] == rr.a[u] ? T(1) : T(0));
                }
            }
            st4(v.x + i, xx);
            st4(v.r + i, rr);
            if (prec == 1) st4(v.z + i, zz);
        }
        publish_t<3>(g, SLOT_D, a3);
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
    T a0[1] = {T(0)};
    TF_FOR4(g, m, i) {
        const V4<T> r = ld4(v.r + i);
        st4(v.r2 + i, r);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u < m.n) a0[0] += r.a[u] * r.a[u];
    }
    publish_t<1>(g, SLOT_A, a0);
    if (!grid_sync(g, 50)) { out.exit_kind = EXIT_ABORT; return; }
    double t0[1];
    totals<1>(g, SLOT_A, t0);
    double rho = t0[0], rhoold = 0.0;
    bool nonfinite = false;
    int iter = 1;
    for (; iter <= cfg.maxiter; ++iter) {
        // u1 = r1 + beta q1; u2 = u1 + beta (q1 + beta u2); p2 = M^-1 u2
        const T beta = T(iter == 1 ? 0.0 : rho / rhoold);
        TF_FOR4(g, m, i) {
            const V4<T> rr = ld4(v.r + i);
            V4<T> u1, u2, p2;
            if (iter == 1) {
                u1 = rr;
                u2 = rr;
            } else {
                const V4<T> q1 = ld4(v.q + i);
                u2 = ld4(v.u2 + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    u1.a[u] = rr.a[u] + beta * q1.a[u];
                    u2.a[u] = u1.a[u] + beta * (q1.a[u] + beta * u2.a[u]);
                }
            }
            st4(v.u1 + i, u1);
            st4(v.u2 + i, u2);
            if (prec == 1) {
                const V4<T> dd = ld4(v.D + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) p2.a[u] = jacobi(u2.a[u], dd.a[u]);
                st4(v.p2 + i, p2);
            } else if (prec != 2) {
                st4(v.p2 + i, u2);
            }
        }
        if (!grid_sync(g, 51)) { out.exit_kind = EXIT_ABORT; return; }
        if (prec == 2) {
            const bool ok = ic_precond(g, m, v, cfg.ic_sweeps, v.u2, v.p2, [](int, T, T) {});
            if (!grid_sync(g, 53) || !ok) { out.exit_kind = EXIT_ABORT; return; }
        }
        // v2 = A p2; alfa = rho / (r2, v2)
        T a1[1] = {T(0)};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T vi = sell_row(m, s, g.lane, v.p2);
            if (i < m.n) {
                v.v2[i] = vi;
                a1[0] += v.r2[i] * vi;
            }
        }
        publish_t<1>(g, SLOT_B, a1);
        if (!grid_sync(g, 54)) { out.exit_kind = EXIT_ABORT; return; }
        double t1[1];
        totals<1>(g, SLOT_B, t1);
        const T alfa = T(rho / t1[0]);
        // q1 = u1 - alfa v2; p1 = M^-1 (u1 + q1); x += alfa p1
        TF_FOR4(g, m, i) {
            const V4<T> u1 = ld4(v.u1 + i), v2 = ld4(v.v2 + i);
            V4<T> q1, tt;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                q1.a[u] = u1.a[u] - alfa * v2.a[u];
                tt.a[u] = u1.a[u] + q1.a[u];
            }
            st4(v.q + i, q1);
            if (prec == 2) {
                st4(v.t + i, tt);
            } else {
                V4<T> p1 = tt, xx = ld4(v.x + i);
                if (prec == 1) {
                    const V4<T> dd = ld4(v.D + i);
#pragma unroll
                    for (int u = 0; u < 4; ++u) p1.a[u] = jacobi(tt.a[u], dd.a[u]);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) xx.a[u] = xx.a[u] + alfa * p1.a[u];
                st4(v.p + i, p1);
                st4(v.x + i, xx);
            }
        }
        if (!grid_sync(g, 55)) { out.exit_kind = EXIT_ABORT; return; }
        if (prec == 2) {
            T* xx = v.x;
            const bool ok = ic_precond(g, m, v, cfg.ic_sweeps, v.t, v.p, [&](int row, T p1, T) {
                xx[row] = xx[row] + alfa * p1;
            });
            if (!grid_sync(g, 57) || !ok) { out.exit_kind = EXIT_ABORT; return; }
        }
        // q2 = A p1; r1 -= alfa q2; ||r1||; next rho = (r1, r2)
        T a3[3] = {T(0), T(0), T(0)};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T q2 = sell_row(m, s, g.lane, v.p);
            if (i < m.n) {
                const T ri = v.r[i] - alfa * q2;
                v.r[i] = ri;
                a3[0] += ri * ri;
                a3[1] += ri * v.r2[i];
                if (nonfinite) {
                    const T xi = v.x[i];
                    a3[2] += (xi == xi ? T(1) : T(0)) + (ri == ri ? T(1) : T(0));
                }
            }
        }
        publish_t<3>(g, SLOT_C, a3);
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

// ---- BiCG with the transposed shadow sequence (extension) ---------------------
// The textbook preconditioned BiCG (the shadow residual is multiplied by A^T,
// whose values mT holds in A's pattern), for nonsymmetric systems where the
// reference's "bicg" (shadow multiplied by A, i.e. CG) may fail.  Diagonal
// or no preconditioning (M^T = M).  Same control flow and outputs as cg_solve.
template <typename T>
__device__ void bicg_true_solve(Grid& g, const Mat<T>& m, const Mat<T>& mT, Vecs<T>& v,
                                const SolveCfg& cfg, SolveOut& out) {
    double tol = cfg.tol, err = 0.0, dummy = 0.0;
    if (!prologue(g, m, v, cfg, out, tol, err, dummy, false)) return;
    const bool diag = cfg.prec == 1;
    T* z2 = v.u1;
    T* q2 = v.v2;
    // shadow r2 = r; z = M^-1 r, z2 = M^-1 r2; rho = (z, r2)
    T a0[1] = {T(0)};
    TF_FOR4(g, m, i) {
        const V4<T> r = ld4(v.r + i);
        V4<T> z = r;
        if (diag) {
            const V4<T> d = ld4(v.D + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) z.a[u] = jacobi(r.a[u], d.a[u]);
        }
        st4(v.r2 + i, r);
        st4(v.z + i, z);
        st4(z2 + i, z);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u < m.n) a0[0] += z.a[u] * r.a[u];
    }
    publish_t<1>(g, SLOT_A, a0);
    if (!grid_sync(g, 60)) { out.exit_kind = EXIT_ABORT; return; }
    double t0[1];
    totals<1>(g, SLOT_A, t0);
    double rho = t0[0], rhoold = 0.0;
    int iter = 1;
    for (; iter <= cfg.maxiter; ++iter) {
        const T beta = T(iter == 1 ? 0.0 : rho / rhoold);
        TF_FOR4(g, m, i) {
            const V4<T> z = ld4(v.z + i), zz = ld4(z2 + i);
            V4<T> p = z, pp = zz;
            if (iter > 1) {
                p = ld4(v.p + i);
                pp = ld4(v.p2 + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    p.a[u] = z.a[u] + beta * p.a[u];
                    pp.a[u] = zz.a[u] + beta * pp.a[u];
                }
            }
            st4(v.p + i, p);
            st4(v.p2 + i, pp);
        }
        if (!grid_sync(g, 61)) { out.exit_kind = EXIT_ABORT; return; }
        T a1[1] = {T(0)};
        for (int s = g.wg; s < m.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const T qi = sell_row(m, s, g.lane, v.p);
            const T q2i = sell_row(mT, s, g.lane, v.p2);
            if (i < m.n) {
                v.q[i] = qi;
                q2[i] = q2i;
                a1[0] += v.p2[i] * qi;
            }
        }
        publish_t<1>(g, SLOT_B, a1);
        if (!grid_sync(g, 62)) { out.exit_kind = EXIT_ABORT; return; }
        double t1[1];
        totals<1>(g, SLOT_B, t1);
        const T alfa = T(rho / t1[0]);
        T a3[2] = {T(0), T(0)};
        TF_FOR4(g, m, i) {
            V4<T> x = ld4(v.x + i), r = ld4(v.r + i), rr = ld4(v.r2 + i);
            const V4<T> p = ld4(v.p + i), q = ld4(v.q + i), qq = ld4(q2 + i);
            V4<T> z, zz, d;
            if (diag) d = ld4(v.D + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                x.a[u] = x.a[u] + alfa * p.a[u];
                r.a[u] = r.a[u] - alfa * q.a[u];
                rr.a[u] = rr.a[u] - alfa * qq.a[u];
                z.a[u] = diag ? jacobi(r.a[u], d.a[u]) : r.a[u];
                zz.a[u] = diag ? jacobi(rr.a[u], d.a[u]) : rr.a[u];
                if (i + u < m.n) {
                    a3[0] += r.a[u] * r.a[u];
                    a3[1] += z.a[u] * rr.a[u];
                }
            }
            st4(v.x + i, x);
            st4(v.r + i, r);
            st4(v.r2 + i, rr);
            st4(v.z + i, z);
            st4(z2 + i, zz);
        }
        publish_t<2>(g, SLOT_C, a3);
        if (!grid_sync(g, 63)) { out.exit_kind = EXIT_ABORT; return; }
        double t3[2];
        totals<2>(g, SLOT_C, t3);
        err = sqrt(t3[0]);
        out.fin_res = err;
        if (err < tol) {
            out.exit_kind = EXIT_CONVERGED;
            out.iterations = iter;
            return;
        }
        if (!finite_val(err)) {
            out.exit_kind = EXIT_NONFINITE;
            out.iterations = cfg.maxiter + 1;
            return;
        }
        rhoold = rho;
        rho = t3[1];
    }
    out.exit_kind = EXIT_MAXITER;
    out.iterations = iter;
}

// ---- mixed precision: FP32 inner Krylov inside FP64 iterative refinement ---------
// Outer loop in FP64: r = b - A x with the FP64 values (exact row order),
// ||r|| and the convergence test; inner solve of A d = r in FP32 (FP32 SELL
// values and vectors, FP64 reductions) by the same CG / CGS code with a
// relative tolerance; x += d in FP64.  The preconditioner setup (Prec1) runs
// once in FP64 and is rounded to FP32.
struct MixedCfg {
    int method;
    int prec;
    int max_ref;
    int maxiter;         // cap on the total number of FP32 iterations
    int restart;         // 1: restarted refinement; 0: reliable updates (CG)
    int inner_maxiter;
    double tol;
    double inner_rtol;
    int tol_is_relative;
    int x_is_zero;
    int ic_sweeps;       // prec 2: 0 exact sweeps, k > 0 Jacobi sweeps
};

struct MixedOut {
    int exit_kind;
    int iterations;   // total inner iterations
    int refinements;
    double ini_res;
    double fin_res;
    double bnrm2;
};

// r64 = b - A x64, r32 = (float) r64, d32 = 0; returns ||r64|| (after a barrier).
__device__ __forceinline__ bool mixed_residual(Grid& g, const Mat<double>& m64, const double* b64,
                                               const double* x64, double* r64, float* r32,
                                               float* d32, bool x_zero, double& err) {
    double a[1] = {0.0};
    for (int s = g.wg; s < m64.nslices; s += g.nw) {
        const int i = s * kWarp + g.lane;
        double ri = i < m64.n ? b64[i] : 0.0;
        if (!x_zero) ri = sell_resid_row(m64, s, g.lane, ri, x64);
        if (i < m64.n) {
            r64[i] = ri;
            r32[i] = (float)ri;
            if (d32) d32[i] = 0.0f;
            a[0] += ri * ri;
        }
    }
    publish<1>(g, SLOT_D + 3, a);
    if (!grid_sync(g, 70)) return false;
    double t[1];
    totals<1>(g, SLOT_D + 3, t);
    err = sqrt(t[0]);
    return true;
}

static __device__ void mixed_solve(Grid& g, const Mat<double>& m64, const Mat<float>& m32, double* x64,
                            double* r64, const double* b64, double* D64, Vecs<float>& v32,
                            const MixedCfg& c, MixedOut& out) {
    out.exit_kind = EXIT_ABORT;
    if (!prec1_phase(g, m64, D64, c.prec)) return;
    // D64 was written in slice order; the next pass reads it four rows per
    // thread, so it must be complete first.
    if (!grid_sync(g, 74)) return;
    double acc[1] = {0.0};
    TF_FOR4(g, m64, i) {
        const V4<double> d = ld4(D64 + i), bb = ld4(b64 + i);
        V4<float> df, wf;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            // FP32 solves hold 1/D for the diagonal preconditioner
            df.a[u] = c.prec == 1 ? (float)(kRecipDiag64 ? d.a[u] : 1.0 / d.a[u])
                                  : (float)d.a[u];
            wf.a[u] = Cell<float>::sentinel();
            if (i + u < m64.n) acc[0] += bb.a[u] * bb.a[u];
        }
        st4(v32.D + i, df);
        st4(v32.w + i, wf);
    }
    publish<1>(g, SLOT_A, acc);
    if (!grid_sync(g, 71)) return;
    // (the residual pass below ends with a barrier before the first apply)
    if (c.prec == 2 && m32.tile.on) tiles_init(g, m32, v32.D);
    double tot[1];
    totals<1>(g, SLOT_A, tot);
    const double bnrm2 = sqrt(tot[0]);
    out.bnrm2 = bnrm2;
    double tol = c.tol_is_relative ? c.tol * bnrm2 : c.tol;
    if (bnrm2 < tol || (c.tol_is_relative && bnrm2 == 0.0)) {
        out.exit_kind = EXIT_BNRM;
        out.iterations = 0;
        return;
    }
    double err;
    if (!mixed_residual(g, m64, b64, x64, r64, v32.r, v32.x, c.x_is_zero != 0, err)) return;
    out.ini_res = err;
    out.fin_res = err;
    if (err < tol) {
        out.exit_kind = EXIT_INIRES;
        out.iterations = 0;
        return;
    }
    SolveCfg ci;
    ci.method = c.method;
    ci.prec = c.prec;
    ci.maxiter = c.inner_maxiter;
    ci.tol = c.inner_rtol;
    ci.x_is_zero = 1;
    ci.do_prec1 = 0;
    ci.tol_is_relative = 1;
    ci.ic_sweeps = c.ic_sweeps;
    int total = 0, stall = 0;
    double prev = err;
    for (int ref = 1; ref <= c.max_ref; ++ref) {
        ci.maxiter = min(c.inner_maxiter, c.maxiter - total);
        if (ci.maxiter <= 0) break;
        SolveOut oi;
        oi.exit_kind = 0;
        oi.iterations = 0;
        oi.fin_res = 0.0;
        if (c.method == 2) cgs_solve<float>(g, m32, v32, ci, oi);
        else cg_solve<float>(g, m32, v32, ci, oi);
        if (oi.exit_kind == EXIT_ABORT) return;
        total += oi.exit_kind == EXIT_MAXITER || oi.exit_kind == EXIT_NONFINITE ? ci.maxiter
                                                                                 : oi.iterations;
        out.iterations = total;
        out.refinements = ref;
        if (!isfinite(oi.fin_res)) {
            out.exit_kind = EXIT_NONFINITE;
            return;
        }
        TF_FOR4(g, m64, i) {
            V4<double> xx = ld4(x64 + i);
            const V4<float> d = ld4(v32.x + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) xx.a[u] = xx.a[u] + (double)d.a[u];
            st4(x64 + i, xx);
        }
        if (!grid_sync(g, 72)) return;
        // r = b - A x; d32 is kept (not cleared) until the step is accepted
        double err_new;
        if (!mixed_residual(g, m64, b64, x64, r64, v32.r, nullptr, false, err_new)) return;
        if (!(err_new <= 10.0 * prev)) {
            // The correction made the true residual grow tenfold (the inner
            // iteration diverged in FP32): take the step back and stop.  (CG
            // minimises the error in the A-norm, so a smaller rise of the
            // residual norm is normal and is kept.)
            TF_FOR4(g, m64, i) {
                V4<double> xx = ld4(x64 + i);
                const V4<float> d = ld4(v32.x + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) xx.a[u] = xx.a[u] - (double)d.a[u];
                st4(x64 + i, xx);
            }
            if (!grid_sync(g, 73)) return;
            if (!mixed_residual(g, m64, b64, x64, r64, v32.r, v32.x, false, err)) return;
            out.fin_res = err;
            out.exit_kind = isfinite(err_new) ? EXIT_MAXITER : EXIT_NONFINITE;
            return;
        }
        err = err_new;
        TF_FOR4(g, m64, i) { st4(v32.x + i, V4<float>{{0.f, 0.f, 0.f, 0.f}}); }
        out.fin_res = err;
        if (err < tol) {
            out.exit_kind = EXIT_CONVERGED;
            return;
        }
        stall = err > 0.9 * prev ? stall + 1 : 0;
        if (stall >= 6) break;
        prev = err;
    }
    out.exit_kind = EXIT_MAXITER;
}

// ---- mixed precision CG with reliable updates ---------------------------------
// Drift between the true and the FP32 recursive residual, relative to the
// latter, above which a reliable update also restarts the search direction.
constexpr double kReliableDrift = 0.3;

// One FP32 preconditioned CG iteration stream (FP32 values and vectors, FP64
// reductions).  Whenever its recursive residual has dropped by `inner_rtol`
// since the last refinement (or below the tolerance), the FP32 correction is
// added to x in FP64, the true residual b - A x is recomputed with the FP64
// values, the convergence test ||r|| < tol is made on it in FP64, and the
// FP32 residual is replaced by it.  Unlike a restarted refinement the search
// direction is kept, so the iteration count stays close to the FP64 solve's.
static __device__ void mixed_cg_reliable(Grid& g, const Mat<double>& m64, const Mat<float>& m32,
                                  double* x64, double* r64, const double* b64, double* D64,
                                  double* xbest, Vecs<float>& v, const MixedCfg& c,
                                  MixedOut& out) {
    out.exit_kind = EXIT_ABORT;
    const int prec = (c.prec == 1 || c.prec == 2) ? c.prec : 0;
    if (!prec1_phase(g, m64, D64, c.prec)) return;
    if (!grid_sync(g, 80)) return;
    double acc[1] = {0.0};
    TF_FOR4(g, m64, i) {
        const V4<double> d = ld4(D64 + i), bb = ld4(b64 + i);
        V4<float> df, wf;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            // FP32 solves hold 1/D for the diagonal preconditioner
            df.a[u] = c.prec == 1 ? (float)(kRecipDiag64 ? d.a[u] : 1.0 / d.a[u])
                                  : (float)d.a[u];
            wf.a[u] = Cell<float>::sentinel();
            if (i + u < m64.n) acc[0] += bb.a[u] * bb.a[u];
        }
        st4(v.D + i, df);
        st4(v.w + i, wf);
    }
    publish<1>(g, SLOT_A, acc);
    if (!grid_sync(g, 81)) return;
    if (c.prec == 2 && m32.tile.on) tiles_init(g, m32, v.D);
    double tot[1];
    totals<1>(g, SLOT_A, tot);
    const double bnrm2 = sqrt(tot[0]);
    out.bnrm2 = bnrm2;
    const double tol = c.tol_is_relative ? c.tol * bnrm2 : c.tol;
    if (bnrm2 < tol || (c.tol_is_relative && bnrm2 == 0.0)) {
        out.exit_kind = EXIT_BNRM;
        out.iterations = 0;
        return;
    }
    const float* z = prec == 0 ? v.r : v.z;
    // r64 = b - A x; r = (float) r64; xl = 0; ||r||; z = M^-1 r (diag) and (r, z)
    // (with `drift`: also ||r_true - r_recursive||^2 into drift, the FP32
    // recursive residual being the one in v.r before it is replaced)
    auto refresh = [&](bool x_zero, double& err, double& rz, double* drift) -> bool {
        double a[3] = {0.0, 0.0, 0.0};
        for (int s = g.wg; s < m64.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            double ri = i < m64.n ? b64[i] : 0.0;
            if (!x_zero) ri = sell_resid_row(m64, s, g.lane, ri, x64);
            if (i < m64.n) {
                r64[i] = ri;
                const float rf = (float)ri;
                if (drift) {
                    const double dr = ri - (double)v.r[i];
                    a[2] += dr * dr;
                }
                v.r[i] = rf;
                v.x[i] = 0.0f;
                a[0] += ri * ri;
                if (prec == 1) {
                    const float zf = rf * v.D[i];
                    v.z[i] = zf;
                    a[1] += double(rf * zf);
                } else if (prec == 0) {
                    a[1] += double(rf * rf);
                }
            }
        }
        publish<3>(g, SLOT_D, a);
        if (!grid_sync(g, 82)) return false;
        double t[3];
        totals<3>(g, SLOT_D, t);
        err = sqrt(t[0]);
        rz = t[1];
        if (drift) *drift = sqrt(t[2]);
        return true;
    };
    auto ic = [&](double& rz) -> bool {
        float a[1] = {0.f};
        const bool ok = ic_precond(g, m32, v, c.ic_sweeps, v.r, v.z, [&](int, float zi, float ri) {
            a[0] += ri * zi;
        });
        publish_t<1>(g, SLOT_A, a);
        if (!grid_sync(g, 83) || !ok) return false;
        double t[1];
        totals<1>(g, SLOT_A, t);
        rz = t[0];
        return true;
    };
    double err, rz;
    if (!refresh(c.x_is_zero != 0, err, rz, nullptr)) return;
    out.ini_res = err;
    out.fin_res = err;
    if (err < tol) {
        out.exit_kind = EXIT_INIRES;
        out.iterations = 0;
        return;
    }
    if (prec == 2 && !ic(rz)) return;
    // best FP64 iterate so far (returned if the iteration later diverges)
    auto keep_best = [&]() {
        TF_FOR4(g, m64, i) { st4(xbest + i, ld4(x64 + i)); }
    };
    keep_best();
    double rho = rz, maxr = err, prev = err, best = err;
    int nref = 0, stall = 0, it = 1;
    bool diverged = false, fresh = false;
    const double delta = c.inner_rtol > 0.0 && c.inner_rtol < 1.0 ? c.inner_rtol : 0.1;
    float beta = 0.0f;
    for (; it <= c.maxiter; ++it) {
        if (it == 1 || fresh) {
            TF_FOR4(g, m32, i) { st4(v.p + i, ld4(z + i)); }
            fresh = false;
        } else {
            TF_FOR4(g, m32, i) {
                const V4<float> zz = ld4(z + i);
                V4<float> pp = ld4(v.p + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) pp.a[u] = zz.a[u] + beta * pp.a[u];
                st4(v.p + i, pp);
            }
        }
        if (!grid_sync(g, 84)) return;
        float a1[1] = {0.f};
        for (int s = g.wg; s < m32.nslices; s += g.nw) {
            const int i = s * kWarp + g.lane;
            const float qi = sell_row(m32, s, g.lane, v.p);
            if (i < m32.n) {
                v.q[i] = qi;
                a1[0] += v.p[i] * qi;
            }
        }
        publish_t<1>(g, SLOT_C, a1);
        if (!grid_sync(g, 85)) return;
        double t1[1];
        totals<1>(g, SLOT_C, t1);
        const float alfa = (float)(rho / t1[0]);
        float a3[2] = {0.f, 0.f};
        TF_FOR4(g, m32, i) {
            V4<float> xx = ld4(v.x + i), rr = ld4(v.r + i), zz;
            const V4<float> pp = ld4(v.p + i), qq = ld4(v.q + i);
            V4<float> dd;
            if (prec == 1) dd = ld4(v.D + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                xx.a[u] = xx.a[u] + alfa * pp.a[u];
                rr.a[u] = rr.a[u] - alfa * qq.a[u];
                if (prec == 1) zz.a[u] = jacobi(rr.a[u], dd.a[u]);
                if (i + u < m32.n) {
                    a3[0] += rr.a[u] * rr.a[u];
                    if (prec == 1) a3[1] += rr.a[u] * zz.a[u];
                }
            }
            st4(v.x + i, xx);
            st4(v.r + i, rr);
            if (prec == 1) st4(v.z + i, zz);
        }
        publish_t<2>(g, SLOT_B, a3);
        if (!grid_sync(g, 86)) return;
        double t3[2];
        totals<2>(g, SLOT_B, t3);
        const double rnorm = sqrt(t3[0]);
        out.iterations = it;
        rz = prec == 1 ? t3[1] : t3[0];
        if (!isfinite(rnorm)) {
            out.exit_kind = EXIT_NONFINITE;
            return;
        }
        if (rnorm < delta * maxr || rnorm < tol) {
            // refinement: x += xl in FP64, true residual, FP64 test
            TF_FOR4(g, m64, i) {
                V4<double> xd = ld4(x64 + i);
                const V4<float> xl = ld4(v.x + i);
#pragma unroll
                for (int u = 0; u < 4; ++u) xd.a[u] = xd.a[u] + (double)xl.a[u];
                st4(x64 + i, xd);
            }
            if (!grid_sync(g, 87)) return;
            double drift = 0.0;
            if (!refresh(false, err, rz, &drift)) return;
            out.fin_res = err;
            out.refinements = ++nref;
            // Keep the search direction only while the recursive residual
            // it was built with is still close to the true one; a larger
            // drift (FP32 recurrences on large, ill-conditioned systems)
            // restarts it from the new preconditioned residual.
            fresh = drift > kReliableDrift * rnorm;
            if (err < tol) {
                out.exit_kind = EXIT_CONVERGED;
                return;
            }
            if (!isfinite(err)) {
                out.exit_kind = EXIT_NONFINITE;
                return;
            }
            if (err < best) {
                best = err;
                keep_best();
            } else if (err > 1e3 * best) {
                diverged = true;
                break;
            }
            stall = err > 0.999 * prev ? stall + 1 : 0;
            if (stall >= 4) break;
            prev = err;
            maxr = err;
        }
        if (prec == 2 && !ic(rz)) return;
        beta = (float)(rz / rho);
        rho = rz;
    }
    // out of iterations: fold the pending correction into x, and fall back
    // to the best iterate if this one is worse
    if (!diverged) {
        TF_FOR4(g, m64, i) {
            V4<double> xd = ld4(x64 + i);
            const V4<float> xl = ld4(v.x + i);
#pragma unroll
            for (int u = 0; u < 4; ++u) xd.a[u] = xd.a[u] + (double)xl.a[u];
            st4(x64 + i, xd);
        }
        if (!grid_sync(g, 88)) return;
        if (!refresh(false, err, rz, nullptr)) return;
    }
    if (diverged || !(err <= best)) {
        TF_FOR4(g, m64, i) { st4(x64 + i, ld4(xbest + i)); }
        if (!grid_sync(g, 89)) return;
        if (!refresh(false, err, rz, nullptr)) return;
    }
    out.fin_res = err;
    out.exit_kind = err < tol ? EXIT_CONVERGED : EXIT_MAXITER;
}

}  // namespace tflows
