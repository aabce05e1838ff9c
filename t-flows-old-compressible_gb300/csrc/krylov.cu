// Kernels and launchers of libtflows_krylov.so.
// Kernels of the reference-arithmetic build (--fmad=false) and the host
// side of every solve, batched launch and plan.
#define TFLOWS_KNS ref
#include "internal.h"
#include "solver_entry.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

namespace tflows {

namespace {

template <typename T>
__global__ void fill_kernel(T* p, long long n, T v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

template <typename T>
__global__ void fill_sentinel_kernel(T* p, long long n) {
    const T v = Cell<T>::sentinel();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void to_double_kernel(const float* __restrict__ a, double* __restrict__ b, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// SELL values from stored-order values: one thread per row.  With `tpos`
// the values of A^T in A's pattern (entry (i,j) <- stored entry (j,i)).
// `s16` receives BF16 bit patterns, rounded to nearest even from FP64.  The
// FP32 copy `s32` holds the row sum (in FP64, rounded) in the diagonal slot:
// its products run in difference form (sell_row).
__global__ void permute_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const long long* __restrict__ soff, const double* __restrict__ val,
                               double* __restrict__ s64, float* __restrict__ s32,
                               unsigned short* __restrict__ s16, const int* __restrict__ tpos) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = rowptr[i], e = rowptr[i + 1];
        const long long base = soff[i >> 5] + (i & 31);
        double rowsum = 0.0;
        for (int j = b; j < e; ++j) {
            const double a = tpos ? val[tpos[j]] : val[j];
            const long long o = base + 32LL * (j - b);
            rowsum += a;
            if (s64) s64[o] = a;
            if (s32) s32[o] = (float)a;
            if (s16) s16[o] = __bfloat16_as_ushort(__double2bfloat16(a));
        }
        if (s32)
            for (int j = b; j < e; ++j)
                if (col[j] == i) s32[base + 32LL * (j - b)] = (float)rowsum;
    }
}

// Coefficient fields of the tiled IC sweeps' step records from the SELL
// values (the same numbers the level-ordered sweeps read: FP64, FP32, or
// BF16 bit patterns).  For the row of thread t of tile k at step s, the
// forward record (k, s) gets its lower coefficients by neighbour (z-1, y-1,
// x-1) and the backward record its upper ones (x+1, y+1, z+1); absent
// neighbours and idle slots hold 0.
template <typename L>
__global__ void tile_permute_kernel(int nx, int ny, int nz, int ty, int ntx, int steps,
                                    long long total, const long long* __restrict__ soff,
                                    const int* __restrict__ meta, const L* __restrict__ sval,
                                    unsigned char* fwd, unsigned char* bwd, unsigned rec_f,
                                    unsigned rec_b) {
    const int B = kTileX * ty;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i % B);
        const long long ks = i / B;
        const int s = (int)(ks % steps), k = (int)(ks / steps);
        const int lx = t % kTileX, ly = t / kTileX;
        const int x = (k % ntx) * kTileX + lx, y = (k / ntx) * ty + ly, z = s - lx - ly;
        L a[6] = {L(0), L(0), L(0), L(0), L(0), L(0)};
        if (x < nx && y < ny && z >= 0 && z < nz) {
            const int row = x + nx * (y + ny * z);
            const long long base = soff[row >> 5] + (row & 31);
            int q = 0;
            if (z > 0) a[0] = sval[base + 32LL * q++];
            if (y > 0) a[1] = sval[base + 32LL * q++];
            if (x > 0) a[2] = sval[base + 32LL * q++];
            q = (meta[row] >> 16) + 1;  // first entry after the diagonal
            if (x < nx - 1) a[3] = sval[base + 32LL * q++];
            if (y < ny - 1) a[4] = sval[base + 32LL * q++];
            if (z < nz - 1) a[5] = sval[base + 32LL * q++];
        }
        L* rf = reinterpret_cast<L*>(fwd + ks * rec_f);
        L* rb = reinterpret_cast<L*>(bwd + ks * rec_b);
        for (int f = 0; f < 3; ++f) {
            rf[f * B + t] = a[f];
            rb[f * B + t] = a[3 + f];
        }
    }
}

// Standalone SELL product (bandwidth measurement and tests).
template <typename T, typename V>
__global__ void __launch_bounds__(kBlock) spmv_kernel(Mat<T> m, const V* __restrict__ x,
                                                      V* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int s = wg; s < m.nslices; s += nw) {
        const T v = sell_row(m, s, lane, x);
        const int i = s * kWarp + lane;
        if (i < m.n) y[i] = V(v);
    }
}

__global__ void __launch_bounds__(kBlock) resid_kernel(Mat<double> m, const double* __restrict__ x,
                                                       double* __restrict__ r) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int s = wg; s < m.nslices; s += nw) {
        const int i = s * kWarp + lane;
        double ri = i < m.n ? r[i] : 0.0;
        ri = sell_resid_row(m, s, lane, ri, x);
        if (i < m.n) r[i] = ri;
    }
}

__global__ void pattern_outer_kernel(int n, const int* __restrict__ rowptr,
                                     const int* __restrict__ col, const double* __restrict__ lam,
                                     const double* __restrict__ x, double* __restrict__ g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double li = lam[i];
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) g[j] = -li * x[col[j]];
    }
}

// Wait limit in SM cycles for `sec` seconds at the device's highest clock.
long long timeout_cycles(double sec) {
    static int khz = 0;
    if (khz == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
        if (khz <= 0) khz = 2100000;
    }
    return (long long)(sec * (double)khz * 1e3);
}

int g_num_sms = 0;
int sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    }
    return g_num_sms;
}

// Longest back-off between polls in the IC sweeps: none (polling back to
// back measured 7-16 % faster on GB300 than any cap from 64 to 1024 ns)
// unless TFLOWS_SWEEP_SLEEP (ns) asks for one.
int sweep_sleep_ns() {
    static const int v = [] {
        const char* e = std::getenv("TFLOWS_SWEEP_SLEEP");
        return e && *e ? std::max(0, std::atoi(e)) : 0;
    }();
    return v;
}

// Gated polling in the IC sweeps (TFLOWS_SWEEP_GATE=0 turns it off).
int sweep_gate_on() {
    static const int v = [] {
        const char* e = std::getenv("TFLOWS_SWEEP_GATE");
        return e && *e ? (std::atoi(e) != 0) : 1;
    }();
    return v;
}

// Column patterns feed the FP64 products and the standalone product; the
// FP32 inner solves keep explicit columns (measured at 256^3: the mixed CG
// 2 % slower with patterns -- its persistent kernel is latency-bound at 50 %
// occupancy and the table lookup lengthens each slice's dependency chain
// more than the saved index bytes shorten it).
template <typename T>
Mat<T> make_mat(const DeviceTopology& t, const T* sval, bool patterns = sizeof(T) == 8) {
    Mat<T> m;
    m.n = t.n;
    m.nslices = t.nslices;
    m.soff = t.soff;
    m.scol = t.scol;
    m.spat = patterns ? t.spat : nullptr;
    m.poff = patterns ? t.poff : nullptr;
    m.sval = sval;
    m.meta = t.meta;
    m.perm_f = t.perm_f;
    m.perm_b = t.perm_b;
    m.lu16 = nullptr;
    m.nchunk_f = t.nchunk_f;
    m.nchunk_b = t.nchunk_b;
    m.wide_f = t.wide_f;
    m.wide_b = t.wide_b;
    m.sweep_mult = 0;
    m.sweep_sleep = sweep_sleep_ns();
    m.sweep_gate = sweep_gate_on();
    return m;
}

// Blocks that give each warp `rows_per_warp` rows (rounded to whole 32-row
// slices; 0 = one slice per warp).
int blocks_for(int nslices, int block = kBlock, int rows_per_warp = 0) {
    const long long per_block = (long long)std::max(1, rows_per_warp / 32) * std::max(1, block / 32);
    return (int)std::max<long long>(1, (nslices + per_block - 1) / per_block);
}

}  // namespace

cudaError_t ensure_workspace(Workspace& ws, const DeviceTopology& t) {
    cudaError_t e = cudaSuccess;
    const size_t vec = (size_t)t.nslices * kWarp + 32;
    if (vec > ws.vec_cap) {
        if (ws.vec64) cudaFree(ws.vec64);
        if (ws.vec32) cudaFree(ws.vec32);
        ws.vec64 = nullptr;
        ws.vec32 = nullptr;
        if ((e = cudaMalloc(&ws.vec64, vec * kVecs * sizeof(double))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&ws.vec32, vec * kVecs * sizeof(float))) != cudaSuccess) return e;
        ws.vec_cap = vec;
    }
    const size_t sl = (size_t)t.sell_len;
    if (sl > ws.sell_cap) {
        if (ws.sval64) cudaFree(ws.sval64);
        if (ws.sval32) cudaFree(ws.sval32);
        if (ws.svalT64) cudaFree(ws.svalT64);
        if (ws.sval16) cudaFree(ws.sval16);
        ws.sval64 = nullptr;
        ws.sval32 = nullptr;
        ws.svalT64 = nullptr;
        ws.sval16 = nullptr;
        if ((e = cudaMalloc(&ws.sval64, sl * sizeof(double))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&ws.sval32, sl * sizeof(float))) != cudaSuccess) return e;
        ws.sell_cap = sl;
    }
    if ((size_t)t.nnz > ws.csr_cap) {
        if (ws.csr_val) cudaFree(ws.csr_val);
        ws.csr_val = nullptr;
        if ((e = cudaMalloc(&ws.csr_val, std::max<size_t>(t.nnz, 1) * sizeof(double))) != cudaSuccess)
            return e;
        ws.csr_cap = t.nnz;
    }
    if (!ws.partials) {
        ws.part_cap = 64 * 1024;
        if ((e = cudaMalloc(&ws.partials, (size_t)NUM_SLOTS * ws.part_cap * sizeof(double))) !=
            cudaSuccess)
            return e;
        if ((e = cudaMalloc(&ws.ctl, sizeof(DevCtl))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&ws.state, sizeof(DevState))) != cudaSuccess) return e;
        cudaEventCreate(&ws.ev0);
        cudaEventCreate(&ws.ev1);
    }
    // SELL padding slots are never read as values, but keep them defined.
    return cudaSuccess;
}

void free_workspace(Workspace& ws) {
    for (void* p : {(void*)ws.sval64, (void*)ws.sval32, (void*)ws.vec64, (void*)ws.vec32,
                    (void*)ws.csr_val, (void*)ws.partials, ws.ctl, ws.state, (void*)ws.svalT64,
                    (void*)ws.sval16, (void*)ws.tile64, (void*)ws.tile32})
        if (p) cudaFree(p);
    if (ws.ev0) cudaEventDestroy(ws.ev0);
    if (ws.ev1) cudaEventDestroy(ws.ev1);
    ws = Workspace();
}

cudaError_t permute_values(const DeviceTopology& t, Workspace& ws, const double* csr_val,
                           bool want64, bool want32, cudaStream_t s, bool want16) {
    if (want16 && !ws.sval16) return cudaErrorInvalidValue;  // ensure_lu16 first
    const int nb = std::min(std::max(1, (t.n + 255) / 256), sms() * 16);
    permute_kernel<<<nb, 256, 0, s>>>(t.n, t.rowptr, t.col, t.soff, csr_val, want64 ? ws.sval64 : nullptr,
                                      want32 ? ws.sval32 : nullptr, want16 ? ws.sval16 : nullptr,
                                      nullptr);
    return cudaGetLastError();
}

cudaError_t ensure_lu16(Workspace& ws) {
    if (ws.sval16) return cudaSuccess;
    return cudaMalloc(&ws.sval16, std::max<size_t>(ws.sell_cap, 1) * sizeof(unsigned short));
}

cudaError_t permute_transposed(const DeviceTopology& t, Workspace& ws, const double* csr_val,
                               cudaStream_t s) {
    if (!t.tpos) return cudaErrorInvalidValue;
    if (!ws.svalT64) {
        cudaError_t e = cudaMalloc(&ws.svalT64, std::max<size_t>(ws.sell_cap, 1) * sizeof(double));
        if (e != cudaSuccess) return e;
    }
    const int nb = std::min(std::max(1, (t.n + 255) / 256), sms() * 16);
    permute_kernel<<<nb, 256, 0, s>>>(t.n, t.rowptr, t.col, t.soff, csr_val, ws.svalT64, nullptr, nullptr,
                                      t.tpos);
    return cudaGetLastError();
}

namespace {

template <typename T>
Vecs<T> carve(T* base, size_t cap, T* x, T* r) {
    Vecs<T> v;
    v.x = x;
    v.r = r;
    v.p = base + 0 * cap;
    v.q = base + 1 * cap;
    v.z = base + 2 * cap;
    v.w = base + 3 * cap;
    v.D = base + 4 * cap;
    v.r2 = base + 5 * cap;
    v.u1 = base + 6 * cap;
    v.u2 = base + 7 * cap;
    v.v2 = base + 8 * cap;
    v.p2 = base + 9 * cap;
    v.t = base + 10 * cap;
    v.s = base + 13 * cap;  // FP32 only (FP64 slot 13 holds b in mixed solves)
    return v;
}

// Lets a persistent kernel take the tiled sweeps' dynamic shared memory
// (once per kernel; a launch without it is unaffected).
void allow_dynamic_smem(const void* kernel, unsigned bytes) {
    if (bytes <= 48u * 1024u) return;
    static std::mutex mu;
    static std::vector<std::pair<const void*, unsigned>> done;
    std::lock_guard<std::mutex> lk(mu);
    for (auto& d : done)
        if (d.first == kernel && d.second >= bytes) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
        cudaSuccess)
        done.emplace_back(kernel, bytes);
}

template <typename K>
int max_coresident(K kernel, int block, unsigned smem = 0) {
    allow_dynamic_smem((const void*)kernel, smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    return std::max(1, per_sm) * sms();
}

template <typename K, typename P>
cudaError_t launch_coop(K kernel, P& params, int grid, int block, cudaStream_t s,
                        unsigned smem = 0) {
    void* args[] = {&params};
    return cudaLaunchCooperativeKernel((const void*)kernel, dim3(grid), dim3(block), args, smem, s);
}

int block_of(const SolveRequest& rq) { return rq.block > 0 ? rq.block : kBlock; }

int choose_grid(const DeviceTopology& t, const SolveRequest& rq, int max_blocks) {
    int g = rq.grid > 0 ? rq.grid : blocks_for(t.nslices, block_of(rq), rq.rows_per_warp);
    return std::max(1, std::min(g, std::min(max_blocks, 64 * 1024)));
}

}  // namespace

int run_prec1(const DeviceTopology& t, Workspace& ws, int prec, double* D, double timeout_s,
              cudaStream_t s, SolveReport& rep) {
    KParams<double> P;
    std::memset(&P, 0, sizeof(P));
    P.m = make_mat<double>(t, ws.sval64);
    P.v = carve<double>(ws.vec64, ws.vec_cap, nullptr, nullptr);
    P.v.D = D;
    P.cfg.prec = prec;
    P.ctl = (DevCtl*)ws.ctl;
    P.state = (DevState*)ws.state;
    P.partials = ws.partials;
    P.timeout_cyc = timeout_cycles(timeout_s);
    P.mode = 1;
    cudaMemsetAsync(ws.ctl, 0, sizeof(DevCtl), s);
    const void* kern = ref_kernel(KernelId::Prec1);
    SolveRequest rq;
    const int grid = choose_grid(t, rq, max_coresident(kern, kBlock));
    cudaError_t e = launch_coop(kern, P, grid, kBlock, s);
    if (e != cudaSuccess) {
        rep.status = ST_CUDA_ERROR;
        rep.message = cudaGetErrorString(e);
        return rep.status;
    }
    DevState st;
    e = cudaMemcpyAsync(&st, ws.state, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rep.status = ST_CUDA_ERROR;
        rep.message = cudaGetErrorString(e);
        return rep.status;
    }
    rep.status = st.status;
    return rep.status;
}

namespace {

// Exact IC(0) on a box-numbered pattern runs the tiled sweeps, unless the
// request asks for the level-ordered ones or TFLOWS_IC_TILED=0 does.
bool tiles_env_on() {
    static const int v = [] {
        const char* e = std::getenv("TFLOWS_IC_TILED");
        return e && *e ? (std::atoi(e) != 0) : 1;
    }();
    return v;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// FP64 CG forms its search direction inside the product only on systems
// whose vectors stay in L2 (measured: config 1, 32^3, 18.0 -> 16.7 us per
// iteration; on 128^3 and 256^3 it was 20-30 % slower, the second gathered
// vector and the per-neighbour z + beta p on the FP64 pipe costing more than
// the update pass it saves).
bool fuse_dir_fp64(const DeviceTopology& t) { return t.n <= (1 << 19); }

struct TileGeom {
    int ty = 0, ntx = 0, nty = 0, steps = 0;
    long long slots = 0;
};

TileGeom tile_geom(const DeviceTopology& t, int block) {
    TileGeom g;
    g.ty = block / kTileX;
    g.ntx = (t.box_nx + kTileX - 1) / kTileX;
    g.nty = (t.box_ny + g.ty - 1) / g.ty;
    g.steps = kTileX + g.ty + t.box_nz - 2;
    g.slots = (long long)g.ntx * g.nty * g.steps * block;
    return g;
}

// Coefficient and value bytes of a request's records.
void tile_elem(const SolveRequest& rq, unsigned& ls, unsigned& sv) {
    if (rq.precision == 1) {
        ls = rq.ic_bf16 ? 2u : 4u;
        sv = 4u;
    } else {
        ls = 8u;
        sv = 8u;
    }
}

// Forward and backward records (three coefficient and at most three value
// fields each) plus the two cell arrays.
size_t tile_buffer_bytes(long long slots, unsigned ls, unsigned sv) {
    return 2 * align256((size_t)slots * (3 * ls + 3 * sv)) + 2 * align256((size_t)slots * sv);
}

}  // namespace

bool tiled_ic(const DeviceTopology& t, const SolveRequest& rq) {
    if (rq.prec != 2 || rq.ic_sweeps > 0 || t.box_nx <= 0 || rq.ic_tiled == 0) return false;
    if (rq.ic_tiled < 0 && !tiles_env_on()) return false;
    const int B = rq.block > 0 ? rq.block : kBlock;
    return B % 32 == 0 && B >= 64 && B <= kMaxBlock;
}

unsigned tile_smem_for(const DeviceTopology& t, const SolveRequest& rq) {
    if (!tiled_ic(t, rq)) return 0;
    unsigned ls, sv;
    tile_elem(rq, ls, sv);
    return tile_smem_bytes(rq.block > 0 ? rq.block : kBlock, ls, sv);
}

cudaError_t ensure_tiles(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq) {
    if (!tiled_ic(t, rq)) return cudaSuccess;
    const TileGeom tg = tile_geom(t, rq.block > 0 ? rq.block : kBlock);
    const bool mixed = rq.precision == 1;
    // the FP32 buffer is sized for FP32 coefficients, which covers BF16 ones
    const size_t need = mixed ? tile_buffer_bytes(tg.slots, 4, 4) : tile_buffer_bytes(tg.slots, 8, 8);
    unsigned char*& buf = mixed ? ws.tile32 : ws.tile64;
    size_t& cap = mixed ? ws.tile_cap32 : ws.tile_cap64;
    if (need <= cap) return cudaSuccess;
    if (buf) cudaFree(buf);
    buf = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&buf, need);
    if (e == cudaSuccess) cap = need;
    return e;
}

namespace {

// The tiled-sweep descriptor of a solve and the coefficient fields of its
// records, queued on stream s from the SELL values (`sval`: FP64, FP32 or
// BF16 bits).
template <typename T, typename L>
cudaError_t fill_tiles(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq,
                       const L* sval, Tiles<T>& tl, cudaStream_t s) {
    std::memset(&tl, 0, sizeof(tl));
    if (!tiled_ic(t, rq)) return cudaSuccess;
    cudaError_t e = ensure_tiles(t, ws, rq);
    if (e != cudaSuccess) return e;
    const int B = rq.block > 0 ? rq.block : kBlock;
    const TileGeom tg = tile_geom(t, B);
    unsigned char* p = sizeof(T) == 8 ? ws.tile64 : ws.tile32;
    // the contracted FP64 build multiplies by 1/(D+TINY) in the middle step
    const int recip = sizeof(T) == 8 && rq.precision == 2 ? 1 : 0;
    const unsigned ls = sizeof(L), sv = sizeof(T);
    const size_t recs = align256((size_t)tg.slots * (3 * ls + 3 * sv));
    tl.on = 1;
    tl.nx = t.box_nx;
    tl.ny = t.box_ny;
    tl.nz = t.box_nz;
    tl.ty = tg.ty;
    tl.ntx = tg.ntx;
    tl.nty = tg.nty;
    tl.steps = tg.steps;
    tl.lu_bf16 = sizeof(L) == 2 ? 1 : 0;
    tl.recip = recip;
    tl.half = tile_half(B, ls, sv);
    tl.rec_f = B * (3 * ls + (recip ? 3 : 2) * sv);
    tl.rec_b = B * (3 * ls + 3 * sv);
    tl.fwd = p;
    tl.bwd = p + recs;
    tl.wt = reinterpret_cast<T*>(p + 2 * recs);
    tl.zt = reinterpret_cast<T*>(p + 2 * recs + align256((size_t)tg.slots * sv));
    const int nb = (int)std::min<long long>(std::max<long long>(1, (tg.slots + 255) / 256), sms() * 16LL);
    tile_permute_kernel<L><<<nb, 256, 0, s>>>(t.box_nx, t.box_ny, t.box_nz, tg.ty, tg.ntx, tg.steps,
                                              tg.slots, t.soff, t.meta, sval, tl.fwd, tl.bwd,
                                              tl.rec_f, tl.rec_b);
    return cudaGetLastError();
}

// Parameters of one FP64 (reference arithmetic) solve; queues the control
// block / counter resets and the IC sentinel fill on stream s.
cudaError_t prepare_fp64(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, double* x,
                         double* r, cudaStream_t s, KParams<double>& P) {
    std::memset(&P, 0, sizeof(P));
    P.m = make_mat<double>(t, ws.sval64);
    P.m.sweep_mult = rq.sweep_mult;
    if (rq.sweep_gate >= 0) P.m.sweep_gate = rq.sweep_gate;
    P.v = carve<double>(ws.vec64, ws.vec_cap, x, r);
    P.cfg.method = rq.method == 2 || rq.method == 3 ? rq.method : 0;
    if (rq.method == 3) P.mT = make_mat<double>(t, ws.svalT64);
    P.cfg.prec = rq.prec;
    P.cfg.maxiter = rq.maxiter;
    P.cfg.tol = rq.tol;
    P.cfg.x_is_zero = rq.x_is_zero;
    P.cfg.do_prec1 = 1;
    P.cfg.tol_is_relative = rq.tol_relative;
    P.ctl = (DevCtl*)ws.ctl;
    P.state = (DevState*)ws.state;
    P.partials = ws.partials;
    P.timeout_cyc = timeout_cycles(rq.timeout_s);
    P.mode = 0;
    P.stall = rq.inject_stall;
    P.cfg.ic_sweeps = rq.prec == 2 ? std::max(rq.ic_sweeps, 0) : 0;
    P.cfg.fuse_dir = fuse_dir_fp64(t) ? 1 : 0;
    cudaError_t e = cudaMemsetAsync(ws.ctl, 0, sizeof(DevCtl), s);
    if (rq.prec == 2) {
        const long long nvec = (long long)t.nslices * kWarp;
        fill_sentinel_kernel<double>
            <<<std::min(1024, (int)((nvec + 255) / 256)), 256, 0, s>>>(P.v.w, nvec);
        if (e == cudaSuccess) e = fill_tiles<double, double>(t, ws, rq, ws.sval64, P.m.tile, s);
    }
    return e;
}

// Parameters of one mixed-precision solve.  b is kept in FP64 workspace slot
// 13 (the residual slot r is rewritten by every refinement).
cudaError_t prepare_mixed(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, double* x,
                          double* r, cudaStream_t s, MixedParams& P) {
    std::memset(&P, 0, sizeof(P));
    P.m64 = make_mat<double>(t, ws.sval64);
    P.m32 = make_mat<float>(t, ws.sval32);
    P.m64.sweep_mult = rq.sweep_mult;
    P.m32.sweep_mult = rq.sweep_mult;
    if (rq.sweep_gate >= 0) P.m64.sweep_gate = P.m32.sweep_gate = rq.sweep_gate;
    P.x64 = x;
    P.r64 = r;
    double* b64 = ws.vec64 + 13 * ws.vec_cap;
    cudaError_t e = cudaSuccess;
    if (b64 != r) e = cudaMemcpyAsync(b64, r, sizeof(double) * t.n, cudaMemcpyDeviceToDevice, s);
    P.b64 = b64;
    P.D64 = ws.vec64 + 4 * ws.vec_cap;
    P.xbest = ws.vec64;
    P.v32 = carve<float>(ws.vec32, ws.vec_cap, ws.vec32 + 11 * ws.vec_cap, ws.vec32 + 12 * ws.vec_cap);
    P.cfg.method = rq.method == 2 ? 2 : 0;
    P.cfg.prec = rq.prec;
    P.cfg.max_ref = rq.max_refinements > 0 ? rq.max_refinements : 30;
    P.cfg.inner_maxiter = rq.inner_maxiter > 0 ? rq.inner_maxiter : 2000;
    P.cfg.maxiter = std::max(rq.maxiter, 0);
    P.cfg.restart = rq.refine_restart;
    P.cfg.tol = rq.tol;
    P.cfg.inner_rtol = rq.inner_rtol > 0 ? rq.inner_rtol : 1e-1;
    P.cfg.tol_is_relative = rq.tol_relative;
    P.cfg.x_is_zero = rq.x_is_zero;
    P.cfg.ic_sweeps = rq.prec == 2 ? std::max(rq.ic_sweeps, 0) : 0;
    if (rq.prec == 2 && rq.ic_bf16) {
        if (!ws.sval16) return cudaErrorInvalidValue;  // filled by permute_values
        P.m32.lu16 = ws.sval16;
    }
    if (e == cudaSuccess && rq.prec == 2)
        e = rq.ic_bf16 ? fill_tiles<float, unsigned short>(t, ws, rq, ws.sval16, P.m32.tile, s)
                       : fill_tiles<float, float>(t, ws, rq, ws.sval32, P.m32.tile, s);
    P.ctl = (DevCtl*)ws.ctl;
    P.state = (DevState*)ws.state;
    P.partials = ws.partials;
    P.timeout_cyc = timeout_cycles(rq.timeout_s);
    P.stall = rq.inject_stall;
    if (e == cudaSuccess) e = cudaMemsetAsync(ws.ctl, 0, sizeof(DevCtl), s);
    return e;
}

// Algorithmic bytes of a finished solve (values + indices of each product,
// each row's x gathered once, plus the vector passes of the schedule).
double solve_bytes(const DeviceTopology& t, const SolveRequest& rq, const DevState& st) {
    const double sl = 8.0 * (t.nslices + 1);
    // column indices of one product: a pattern id per row (FP64 products of
    // a topology with patterns), or 4 bytes per entry
    const double idx64 = t.spat ? (double)t.n : 4.0 * t.nnz;
    const double spmv64 = (double)t.nnz * 8.0 + idx64 + sl + 16.0 * t.n;
    const bool cgs = rq.method == 2;
    // One IC(0) apply: the off-diagonal factor entries (value + index) once,
    // the row metadata, D and the right-hand side read and the result written
    // per triangle.  Jacobi sweeps: each sweep reads one triangle's entries.
    const double offd = (double)std::max(0, t.nnz - t.n);
    // The tiled sweeps read no indices: the factor entries once, and per row
    // D twice, the right-hand side once, w written and read, z written.
    const bool tiled = tiled_ic(t, rq);
    auto ic_bytes = [&](double sv, double sx) {
        if (rq.ic_sweeps > 0)
            return rq.ic_sweeps * (offd * (sv + 4.0) + 2.0 * t.n * (4.0 + 3.0 * sx));
        if (tiled) return offd * sv + 6.0 * t.n * sx;
        return offd * (sv + 4.0) + 2.0 * t.n * (4.0 + 3.0 * sx);
    };
    if (rq.precision == 1) {
        const double spmv32 = (double)t.nnz * 8.0 + sl + 8.0 * t.n;
        const double ic = rq.prec == 2 ? ic_bytes(rq.ic_bf16 ? 2.0 : 4.0, 4.0) : 0.0;
        // restarted CG forms its search direction inside the product (z and
        // p read once, p and q written once), so the product's own vector
        // read and write are part of the 4·N·12 (resp. 10) vector bytes; the
        // reliable-update loop keeps its separate direction pass
        const double cg_fused = !rq.refine_restart ? 8.0 * t.n : 0.0;
        const double inner_it = cgs ? 2 * spmv32 + 4.0 * t.n * 22 + 2 * ic
                                    : spmv32 - 8.0 * t.n + cg_fused +
                                          4.0 * t.n * (rq.prec == 1 ? 12 : 10) + ic;
        return inner_it * st.inner_iters + (spmv64 + 8.0 * t.n * 4) * (st.refinements + 1);
    }
    const int it = std::max(0, std::min(st.iterations, rq.maxiter));
    const double ic = rq.prec == 2 ? ic_bytes(8.0, 8.0) : 0.0;
    // CG on a small system forms its next search direction inside the
    // product (z and the old p read, the new p and q written there, no
    // separate update pass: one vector fewer)
    const double per_it = cgs ? 2 * spmv64 + 8.0 * t.n * 22 + 2 * ic
                              : spmv64 + 8.0 * t.n * ((rq.prec == 1 ? 12 : 10) -
                                                      (fuse_dir_fp64(t) ? 1 : 0)) + ic;
    return per_it * it + spmv64 + 8.0 * t.n * 4;
}

void fill_report(const DeviceTopology& t, const SolveRequest& rq, const DevState& st, double sec,
                 SolveReport& rep) {
    rep.status = st.status;
    rep.exit_kind = st.exit_kind;
    rep.iterations = st.iterations;
    rep.inner_iterations = st.inner_iters;
    rep.refinements = st.refinements;
    rep.ini_res = st.ini_res;
    rep.fin_res = st.fin_res;
    rep.seconds = sec;
    rep.bytes = solve_bytes(t, rq, st);
    if (st.status == ST_TIMEOUT)
        rep.message = "device wait exceeded the timeout (site " + std::to_string(st.timeout_where) + ")";
}

template <typename K, typename P>
int launch_and_report(K kern, P& params, const DeviceTopology& t, Workspace& ws,
                      const SolveRequest& rq, cudaStream_t s, SolveReport& rep, cudaError_t e) {
    const int block = block_of(rq);
    const unsigned smem = tile_smem_for(t, rq);
    const int grid = choose_grid(t, rq, max_coresident(kern, block, smem));
    trace_mark("set-up enqueued");
    cudaEventRecord(ws.ev0, s);
    if (e == cudaSuccess) e = launch_coop(kern, params, grid, block, s, smem);
    rep.block = block;
    rep.grid = grid;
    cudaEventRecord(ws.ev1, s);
    trace_mark("solver launched");
    DevState st;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, ws.state, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    trace_mark("solver finished");
    if (e != cudaSuccess) {
        rep.status = ST_CUDA_ERROR;
        rep.message = std::string("solver: ") + cudaGetErrorString(e);
        return rep.status;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ws.ev0, ws.ev1);
    fill_report(t, rq, st, ms * 1e-3, rep);
    return rep.status;
}

}  // namespace

const void* ref_kernel(KernelId id) {
    switch (id) {
        case KernelId::Cg: return (const void*)ref::krylov_kernel<double, 0>;
        case KernelId::Cgs: return (const void*)ref::krylov_kernel<double, 2>;
        case KernelId::BicgTrue: return (const void*)ref::krylov_kernel<double, 3>;
        case KernelId::Prec1: return (const void*)ref::krylov_kernel<double, 9>;
        case KernelId::IcApply: return (const void*)ref::krylov_kernel<double, 8>;
        case KernelId::BatchFp64: return (const void*)ref::batch_kernel<0>;
        default: return nullptr;  // mixed solves are built with contraction only
    }
}

namespace {

// The kernel a request runs: reference arithmetic for TFLOWS_FP64, the
// contracted build for TFLOWS_FP64_FMA and for the mixed solves.
const void* solver_kernel(const SolveRequest& rq) {
    if (rq.precision == 1)
        return fma_kernel(rq.method == 2 ? KernelId::MixedCgs
                                         : (rq.refine_restart ? KernelId::MixedRestart
                                                              : KernelId::MixedReliable));
    const KernelId id = rq.method == 2 ? KernelId::Cgs
                        : rq.method == 3 ? KernelId::BicgTrue : KernelId::Cg;
    return rq.precision == 2 ? fma_kernel(id) : ref_kernel(id);
}

const void* batch_kernel_for(int precision) {
    return precision == 1 ? fma_kernel(KernelId::BatchMixed)
           : precision == 2 ? fma_kernel(KernelId::BatchFp64) : ref_kernel(KernelId::BatchFp64);
}

}  // namespace

int planned_grid(const DeviceTopology& t, const SolveRequest& rq) {
    return choose_grid(t, rq, max_coresident(solver_kernel(rq), block_of(rq), tile_smem_for(t, rq)));
}

int run_ic_apply(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq0, const double* r,
                 double* z, cudaStream_t s, SolveReport& rep) {
    SolveRequest rq = rq0;
    rq.prec = 2;
    rq.method = 0;
    rq.precision = rq0.precision == 2 ? 2 : 0;
    double* R = ws.vec64 + 12 * ws.vec_cap;
    KParams<double> P;
    cudaError_t e = cudaMemcpyAsync(R, r, sizeof(double) * t.n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = prepare_fp64(t, ws, rq, ws.vec64 + 11 * ws.vec_cap, R, s, P);
    const void* kern = rq.precision == 2 ? fma_kernel(KernelId::IcApply) : ref_kernel(KernelId::IcApply);
    const int st = launch_and_report(kern, P, t, ws, rq, s, rep, e);
    if (st == ST_CUDA_ERROR) return st;
    e = cudaMemcpyAsync(z, P.v.z, sizeof(double) * t.n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rep.status = ST_CUDA_ERROR;
        rep.message = cudaGetErrorString(e);
    }
    rep.bytes = 0.0;
    return rep.status;
}

int run_solve(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, double* x, double* r,
              cudaStream_t s, SolveReport& rep) {
    if (rq.precision == 1) {
        MixedParams P;
        cudaError_t e = prepare_mixed(t, ws, rq, x, r, s, P);
        return launch_and_report(solver_kernel(rq), P, t, ws, rq, s, rep, e);
    }
    KParams<double> P;
    cudaError_t e = prepare_fp64(t, ws, rq, x, r, s, P);
    return launch_and_report(solver_kernel(rq), P, t, ws, rq, s, rep, e);
}

// Persistent launch state of a batched solve: pinned host and device copies
// of the per-system parameters and the block -> system map, and pinned room
// for the per-system result records.  Every stream operation it issues is
// capturable, so a batch can be recorded once into a CUDA graph and replayed.
struct BatchLaunch {
    BatchItem* h_items = nullptr;
    BatchItem* d_items = nullptr;
    int* h_map = nullptr;
    int* d_map = nullptr;
    DevState* h_state = nullptr;
    int item_cap = 0;
    int map_cap = 0;
    int total = 0;
    int block = 0;
};

BatchLaunch* batch_create() { return new BatchLaunch(); }

void batch_destroy(BatchLaunch* L) {
    if (!L) return;
    if (L->h_items) cudaFreeHost(L->h_items);
    if (L->h_map) cudaFreeHost(L->h_map);
    if (L->h_state) cudaFreeHost(L->h_state);
    if (L->d_items) cudaFree(L->d_items);
    if (L->d_map) cudaFree(L->d_map);
    delete L;
}

namespace {

cudaError_t grow(BatchLaunch& L, int count, int total) {
    cudaError_t e = cudaSuccess;
    if (count > L.item_cap) {
        if (L.h_items) cudaFreeHost(L.h_items);
        if (L.d_items) cudaFree(L.d_items);
        if (L.h_state) cudaFreeHost(L.h_state);
        L.h_items = nullptr;
        L.d_items = nullptr;
        L.h_state = nullptr;
        if ((e = cudaMallocHost(&L.h_items, sizeof(BatchItem) * count)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&L.d_items, sizeof(BatchItem) * count)) != cudaSuccess) return e;
        if ((e = cudaMallocHost(&L.h_state, sizeof(DevState) * count)) != cudaSuccess) return e;
        L.item_cap = count;
    }
    if (total > L.map_cap) {
        if (L.h_map) cudaFreeHost(L.h_map);
        if (L.d_map) cudaFree(L.d_map);
        L.h_map = nullptr;
        L.d_map = nullptr;
        if ((e = cudaMallocHost(&L.h_map, sizeof(int) * total)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&L.d_map, sizeof(int) * total)) != cudaSuccess) return e;
        L.map_cap = total;
    }
    return e;
}

void fail_all(std::vector<BatchSpec>& specs, int status, const std::string& msg) {
    for (auto& sp : specs) {
        sp.rep->status = status;
        sp.rep->message = msg;
    }
}

}  // namespace

cudaError_t batch_reserve(BatchLaunch* L, int count, int block) {
    if (block <= 0) block = kBlock;
    int maxb = 1;
    for (int p : {0, 1, 2}) maxb = std::max(maxb, max_coresident(batch_kernel_for(p), block));
    return grow(*L, count, maxb);
}

int batch_enqueue(BatchLaunch* L, std::vector<BatchSpec>& specs, cudaStream_t s) {
    const int count = (int)specs.size();
    if (count == 0) return ST_OK;
    const int precision = specs[0].rq.precision;
    const bool mixed = precision == 1;
    for (auto& sp : specs)
        if (sp.rq.precision != precision) {
            fail_all(specs, ST_BAD_INPUT, "one precision per batched launch");
            return ST_BAD_INPUT;
        }
    const void* kern = batch_kernel_for(precision);
    const int block = block_of(specs[0].rq);
    unsigned smem = 0;
    for (auto& sp : specs) {
        if (block_of(sp.rq) != block) {
            fail_all(specs, ST_BAD_INPUT, "one block size per batched launch");
            return ST_BAD_INPUT;
        }
        smem = std::max(smem, tile_smem_for(*sp.t, sp.rq));
    }
    const int maxb = max_coresident(kern, block, smem);
    if (count > maxb) {
        fail_all(specs, ST_BAD_INPUT,
                 "more systems than co-resident blocks (" + std::to_string(maxb) + ")");
        return ST_BAD_INPUT;
    }
    // Blocks per system: the tuner's group sizes when given, else in
    // proportion to the expected work, N^(4/3) (rows times a CG iteration
    // count growing like the mesh edge), at least one, at most one block per
    // rows_per_warp rows per warp (one slice per warp by default).
    std::vector<double> w(count);
    double wsum = 0.0;
    for (int k = 0; k < count; ++k) {
        w[k] = specs[k].weight > 0.0 ? specs[k].weight : std::pow((double)specs[k].t->n, 4.0 / 3.0);
        wsum += w[k];
    }
    std::vector<int> nb(count);
    int total = 0;
    for (int k = 0; k < count; ++k) {
        const int cap = specs[k].rq.grid > 0
                            ? specs[k].rq.grid
                            : blocks_for(specs[k].t->nslices, block, specs[k].rq.rows_per_warp);
        nb[k] = std::max(1, std::min(cap, (int)std::floor((maxb - count) * w[k] / wsum) + 1));
        total += nb[k];
    }
    while (total > maxb) {
        int big = (int)(std::max_element(nb.begin(), nb.end()) - nb.begin());
        --nb[big];
        --total;
    }
    cudaError_t e = grow(*L, count, total);
    if (e != cudaSuccess) {
        fail_all(specs, ST_CUDA_ERROR, std::string("batch buffers: ") + cudaGetErrorString(e));
        return ST_CUDA_ERROR;
    }
    int b0 = 0;
    for (int k = 0; k < count; ++k) {
        BatchSpec& sp = specs[k];
        BatchItem& it = L->h_items[k];
        std::memset(&it, 0, sizeof(it));
        it.b0 = b0;
        it.nb = nb[k];
        it.method = sp.rq.method == 2 ? 2 : 0;
        it.mixed = mixed;
        cudaError_t ek = mixed ? prepare_mixed(*sp.t, *sp.ws, sp.rq, sp.x, sp.r, s, it.PM)
                               : prepare_fp64(*sp.t, *sp.ws, sp.rq, sp.x, sp.r, s, it.P64);
        if (ek != cudaSuccess) e = ek;
        for (int j = 0; j < nb[k]; ++j) L->h_map[b0 + j] = k;
        b0 += nb[k];
    }
    L->total = total;
    L->block = block;
    for (int k = 0; k < count; ++k) specs[k].rep->grid = nb[k];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(L->d_items, L->h_items, sizeof(BatchItem) * count,
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(L->d_map, L->h_map, sizeof(int) * total, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(total);
        cfg.blockDim = dim3(block);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const BatchItem* di = L->d_items;
        const int* dm = L->d_map;
        void* args[] = {(void*)&di, (void*)&dm};
        e = cudaLaunchKernelExC(&cfg, kern, args);
    }
    for (int k = 0; k < count && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync(L->h_state + k, specs[k].ws->state, sizeof(DevState),
                            cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) {
        fail_all(specs, ST_CUDA_ERROR, std::string("batched solver: ") + cudaGetErrorString(e));
        return ST_CUDA_ERROR;
    }
    return ST_OK;
}

int batch_collect(BatchLaunch* L, std::vector<BatchSpec>& specs, cudaStream_t s, double seconds) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        fail_all(specs, ST_CUDA_ERROR, std::string("batched solver: ") + cudaGetErrorString(e));
        return ST_CUDA_ERROR;
    }
    int worst = ST_OK;
    for (int k = 0; k < (int)specs.size(); ++k) {
        fill_report(*specs[k].t, specs[k].rq, L->h_state[k], seconds, *specs[k].rep);
        specs[k].rep->block = L->block;
        specs[k].rep->group_seconds = L->h_state[k].group_ns * 1e-9;
        worst = std::max(worst, L->h_state[k].status);
    }
    return worst;
}

int run_batch(std::vector<BatchSpec>& specs, cudaStream_t s, double* seconds) {
    if (specs.empty()) return ST_OK;
    BatchLaunch* L = batch_create();
    cudaEvent_t e0 = specs[0].ws->ev0, e1 = specs[0].ws->ev1;
    cudaEventRecord(e0, s);
    int st = batch_enqueue(L, specs, s);
    cudaEventRecord(e1, s);
    if (st == ST_OK) {
        cudaStreamSynchronize(s);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (seconds) *seconds = ms * 1e-3;
        st = batch_collect(L, specs, s, ms * 1e-3);
    } else {
        cudaStreamSynchronize(s);
    }
    batch_destroy(L);
    return st;
}

cudaError_t run_resid(const DeviceTopology& t, Workspace& ws, const double* x, double* r,
                      cudaStream_t s) {
    Mat<double> m = make_mat<double>(t, ws.sval64);
    const int nb = std::min(blocks_for(t.nslices), sms() * 8);
    resid_kernel<<<nb, kBlock, 0, s>>>(m, x, r);
    return cudaGetLastError();
}

cudaError_t run_spmv(const DeviceTopology& t, Workspace& ws, const double* x, double* y, bool fp32,
                     int repeat, cudaStream_t s, float* ms) {
    const int nb = std::min(blocks_for(t.nslices), sms() * 8);
    float* x32 = ws.vec32;
    float* y32 = ws.vec32 + ws.vec_cap;
    if (fp32) {
        to_float_kernel<<<std::min(1024, (t.n + 255) / 256), 256, 0, s>>>(x, x32, t.n);
    }
    cudaEventRecord(ws.ev0, s);
    for (int k = 0; k < std::max(1, repeat); ++k) {
        if (fp32) {
            spmv_kernel<float, float><<<nb, kBlock, 0, s>>>(make_mat<float>(t, ws.sval32, true), x32,
                                                            y32);
        } else {
            spmv_kernel<double, double><<<nb, kBlock, 0, s>>>(make_mat<double>(t, ws.sval64), x, y);
        }
    }
    cudaEventRecord(ws.ev1, s);
    if (fp32) to_double_kernel<<<std::min(1024, (t.n + 255) / 256), 256, 0, s>>>(y32, y, t.n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaEventSynchronize(ws.ev1);
    if (ms) cudaEventElapsedTime(ms, ws.ev0, ws.ev1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

cudaError_t run_pattern_outer(const DeviceTopology& t, const double* lambda, const double* x,
                              double* g, cudaStream_t s) {
    const int nb = std::min(std::max(1, (t.n + 255) / 256), sms() * 16);
    pattern_outer_kernel<<<nb, 256, 0, s>>>(t.n, t.rowptr, t.col, lambda, x, g);
    return cudaGetLastError();
}

}  // namespace tflows
