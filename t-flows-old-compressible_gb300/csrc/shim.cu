// C-ABI shim of libtflows_krylov.so: argument checks, the topology cache,
// host<->device traffic and the reference's output conventions.
//
// Reference interfaces replaced (all in T-FlowS Process/):
//   cg    CG.f90:2-34      bicg  BiCG.f90:2-34     CGS  CGS.f90:2-34
//   Prec1 Prec1.f90:2-18   Resid Resid.f90:2-16
#include "../../include/tflows_krylov.h"
#include "device_common.cuh"
#include "internal.h"

#include <algorithm>
#include <chrono>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

struct tflows_topology {
    tflows::DeviceTopology t;
    tflows::Workspace ws;
    // extra workspaces for batches that solve several systems on this pattern
    std::vector<std::unique_ptr<tflows::Workspace>> extra_ws;
    std::mutex mu;
    // cache key (legacy host path)
    const void* k_acol = nullptr;
    const void* k_arow = nullptr;
    const void* k_adia = nullptr;
    unsigned long long k_hash = 0;
    unsigned long long last_use = 0;
};

namespace {

using namespace tflows;

thread_local int t_status = 0;
thread_local std::string t_error;
thread_local tflows_result t_result{};

struct Context {
    std::mutex mu;
    int device = -1;
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<tflows_topology>> cache;
    unsigned long long clock = 0;
    double error_state = 0.0;  // sol_mod :: error (Library/sol_mod.f90:9)
    tflows_options opts{};
    bool opts_set = false;
};

Context& ctx() {
    static Context* c = new Context();
    return *c;
}

int fail(int status, const std::string& msg) {
    t_status = status;
    t_error = msg;
    return status;
}

void default_opts(tflows_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->precision = TFLOWS_FP64;
    o->tol_mode = TFLOWS_TOL_ABSOLUTE;
    o->inner_rtol = 1e-1;
    o->refine_restart = 0;
    o->inner_maxiter = 2000;
    o->max_refinements = 30;
    o->ic_sweeps = 0;
    o->ic_bf16 = 0;
    o->timeout_s = 5.0;
    o->block_size = 0;
    o->grid_blocks = 0;
    o->autotune = 0;
    o->rows_per_warp = 0;
    o->sweep_warps = 0;
    o->sweep_gate = -1;
    o->ic_tiled = -1;
    o->device = -1;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(TFLOWS_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

// --- topology construction ----------------------------------------------------

// Checks the compressed-row arrays (base 0 or 1) and fills host 0-based copies.
int check_pattern(int n, int nnz, const int* rp, const int* col, const int* dg, int base,
                  DeviceTopology& t, std::string& msg) {
    if (n < 0 || nnz < 0) { msg = "negative N or NONZ"; return TFLOWS_BAD_INPUT; }
    if (!rp || (!col && nnz > 0) || (!dg && n > 0)) { msg = "null CSR array"; return TFLOWS_BAD_INPUT; }
    if (rp[0] != base) { msg = "Acol(1) must be 1"; return TFLOWS_BAD_INPUT; }
    if (rp[n] - base != nnz) { msg = "Acol(N+1) must equal NONZ"; return TFLOWS_BAD_INPUT; }
    t.h_rowptr.resize((size_t)n + 1);
    t.h_col.resize((size_t)nnz);
    t.h_diag.resize((size_t)n);
    bool ic_ok = true;
    int max_len = 0;
    for (int i = 0; i <= n; ++i) t.h_rowptr[i] = rp[i] - base;
    for (int i = 0; i < n; ++i) {
        const int b = t.h_rowptr[i], e = t.h_rowptr[i + 1];
        if (e < b) { msg = "Acol is not non-decreasing at row " + std::to_string(i + 1); return TFLOWS_BAD_INPUT; }
        if (e - b > 65535) { msg = "row longer than 65535 entries"; return TFLOWS_BAD_INPUT; }
        max_len = std::max(max_len, e - b);
        const int d = dg[i] - base;
        if (d < b || d >= e) { msg = "Adia outside its row at row " + std::to_string(i + 1); return TFLOWS_BAD_INPUT; }
        for (int j = b; j < e; ++j) {
            const int c = col[j] - base;
            if (c < 0 || c >= n) { msg = "Arow out of range at position " + std::to_string(j + 1); return TFLOWS_BAD_INPUT; }
            t.h_col[j] = c;
            if (j < d && c >= i) ic_ok = false;
            if (j > d && c <= i) ic_ok = false;
        }
        if (t.h_col[d] != i) { msg = "Arow(Adia(i)) != i at row " + std::to_string(i + 1); return TFLOWS_BAD_INPUT; }
        t.h_diag[i] = d;
    }
    t.n = n;
    t.nnz = nnz;
    t.ic_ok = ic_ok;
    t.max_len = max_len;
    return TFLOWS_OK;
}

template <typename T>
cudaError_t upload(T** dst, const T* src, size_t count) {
    cudaError_t e = cudaMalloc((void**)dst, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (count) e = cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

void free_topology_arrays(DeviceTopology& t) {
    for (void* p : {(void*)t.rowptr, (void*)t.col, (void*)t.soff, (void*)t.scol, (void*)t.meta,
                    (void*)t.perm_f, (void*)t.perm_b, (void*)t.tpos, (void*)t.spat,
                    (void*)t.poff})
        if (p) cudaFree(p);
    t.rowptr = t.col = t.scol = t.meta = t.perm_f = t.perm_b = t.tpos = nullptr;
    t.soff = nullptr;
    t.spat = nullptr;
    t.poff = nullptr;
    t.npat = 0;
}

// Column patterns: when every row has at most 8 stored entries and the rows'
// offset tuples (column - row, in stored order) take at most 255 distinct
// values -- cells of a structured or block-structured mesh repeat a few
// stencils -- each row stores a one-byte pattern id and the products read
// the offsets from an 8-int table, instead of 4 bytes of column index per
// entry.  Turned off by TFLOWS_SELL_PATTERNS=0.
cudaError_t build_patterns(DeviceTopology& t) {
    const char* env = std::getenv("TFLOWS_SELL_PATTERNS");
    if ((env && *env && std::atoi(env) == 0) || t.max_len > 8 || t.n <= 0 || t.n >= (1 << 30))
        return cudaSuccess;
    constexpr int kNoColHost = -(1 << 30);  // i + kNoColHost < 0 for every row
    std::map<std::array<int, 8>, int> ids;
    std::vector<std::array<int, 8>> table;
    std::vector<unsigned char> spat((size_t)t.nslices * 32);
    auto id_of = [&](const std::array<int, 8>& key) -> int {
        auto it = ids.find(key);
        if (it != ids.end()) return it->second;
        if (table.size() >= 255) return -1;
        ids.emplace(key, (int)table.size());
        table.push_back(key);
        return (int)table.size() - 1;
    };
    std::array<int, 8> last;
    int last_id = -1;
    for (size_t i = 0; i < spat.size(); ++i) {
        std::array<int, 8> key;
        key.fill(kNoColHost);
        if ((int)i < t.n) {
            const int b = t.h_rowptr[i], e = t.h_rowptr[i + 1];
            for (int j = b; j < e; ++j) {
                key[j - b] = t.h_col[j] - (int)i;  // |offset| < n < 2^30
            }
        }
        // neighbouring rows mostly share a stencil: look up only on a change
        const int id = last_id >= 0 && key == last ? last_id : id_of(key);
        if (id < 0) return cudaSuccess;  // too many patterns: explicit columns
        spat[i] = (unsigned char)id;
        last = key;
        last_id = id;
    }
    std::vector<int> poff(table.size() * 8);
    for (size_t p = 0; p < table.size(); ++p)
        for (int k = 0; k < 8; ++k) poff[8 * p + k] = table[p][k];
    cudaError_t e;
    if ((e = upload(&t.spat, spat.data(), spat.size())) != cudaSuccess) return e;
    if ((e = upload(&t.poff, poff.data(), poff.size())) != cudaSuccess) return e;
    t.npat = (int)table.size();
    return cudaSuccess;
}

// Box numbering: row 0 holds columns 0, 1, nx, nx*ny; then every row i,
// with x = i mod nx, y = (i / nx) mod ny, z = i / (nx ny), must hold exactly
// its existing neighbours i-nx*ny, i-nx, i-1, i, i+1, i+nx, i+nx*ny in that
// (ascending) order.  Boxes thinner than 2 cells in any direction are left
// to the level-ordered sweeps.
void detect_box(DeviceTopology& t) {
    t.box_nx = t.box_ny = t.box_nz = 0;
    const int n = t.n;
    if (n < 8 || t.h_rowptr[1] - t.h_rowptr[0] != 4) return;
    const int* c0 = t.h_col.data();
    if (c0[0] != 0 || c0[1] != 1) return;
    const long long nx = c0[2], nxy = c0[3];
    if (nx < 2 || nxy <= nx || nxy % nx != 0 || n % nxy != 0) return;
    const long long ny = nxy / nx, nz = n / nxy;
    if (ny < 2 || nz < 2) return;
    for (long long i = 0; i < n; ++i) {
        const long long x = i % nx, y = (i / nx) % ny, z = i / nxy;
        long long want[7];
        int k = 0, dia = 0;
        if (z > 0) want[k++] = i - nxy;
        if (y > 0) want[k++] = i - nx;
        if (x > 0) want[k++] = i - 1;
        dia = k;
        want[k++] = i;
        if (x < nx - 1) want[k++] = i + 1;
        if (y < ny - 1) want[k++] = i + nx;
        if (z < nz - 1) want[k++] = i + nxy;
        const int b = t.h_rowptr[i], e = t.h_rowptr[i + 1];
        if (e - b != k || t.h_diag[i] - b != dia) return;
        for (int j = 0; j < k; ++j)
            if (t.h_col[b + j] != want[j]) return;
    }
    t.box_nx = (int)nx;
    t.box_ny = (int)ny;
    t.box_nz = (int)nz;
}

// SELL-32 layout: slice s holds rows 32s..32s+31, width = longest row.
cudaError_t build_device(DeviceTopology& t) {
    detect_box(t);
    const int n = t.n;
    t.nslices = (n + 31) / 32;
    std::vector<long long> soff((size_t)t.nslices + 1, 0);
    for (int s = 0; s < t.nslices; ++s) {
        int w = 0;
        for (int i = s * 32; i < std::min(n, s * 32 + 32); ++i)
            w = std::max(w, t.h_rowptr[i + 1] - t.h_rowptr[i]);
        soff[s + 1] = soff[s] + 32LL * w;
    }
    t.sell_len = soff[t.nslices];
    std::vector<int> scol((size_t)t.sell_len, -1);
    std::vector<int> meta((size_t)n);
    for (int i = 0; i < n; ++i) {
        const int b = t.h_rowptr[i], e = t.h_rowptr[i + 1];
        const long long base = soff[i >> 5] + (i & 31);
        for (int j = b; j < e; ++j) scol[base + 32LL * (j - b)] = t.h_col[j];
        meta[i] = (e - b) | ((t.h_diag[i] - b) << 16);
    }
    cudaError_t e;
    if ((e = upload(&t.rowptr, t.h_rowptr.data(), t.h_rowptr.size())) != cudaSuccess) return e;
    if ((e = upload(&t.col, t.h_col.data(), t.h_col.size())) != cudaSuccess) return e;
    if ((e = upload(&t.soff, soff.data(), soff.size())) != cudaSuccess) return e;
    if ((e = upload(&t.scol, scol.data(), scol.size())) != cudaSuccess) return e;
    if ((e = upload(&t.meta, meta.data(), meta.size())) != cudaSuccess) return e;
    return build_patterns(t);
}

// Wavefront levels of the forward (lower, in row order) and backward (upper,
// in reverse row order) dependency graphs; each level is padded to a whole
// number of warps so that no warp ever waits on one of its own lanes.
cudaError_t build_levels(DeviceTopology& t) {
    if (t.levels_built) return cudaSuccess;
    const int n = t.n;
    std::vector<int> lev((size_t)n);
    auto make_perm = [&](bool forward, int** out, int* nchunk, int* nlev, int* wide) -> cudaError_t {
        int maxl = -1;
        if (forward) {
            for (int i = 0; i < n; ++i) {
                int l = 0;
                for (int j = t.h_rowptr[i]; j < t.h_diag[i]; ++j) l = std::max(l, lev[t.h_col[j]] + 1);
                lev[i] = l;
                maxl = std::max(maxl, l);
            }
        } else {
            for (int i = n - 1; i >= 0; --i) {
                int l = 0;
                for (int j = t.h_diag[i] + 1; j < t.h_rowptr[i + 1]; ++j)
                    l = std::max(l, lev[t.h_col[j]] + 1);
                lev[i] = l;
                maxl = std::max(maxl, l);
            }
        }
        const int L = maxl + 1;
        std::vector<long long> cnt((size_t)L + 1, 0);
        for (int i = 0; i < n; ++i) cnt[lev[i] + 1]++;
        std::vector<long long> start((size_t)L + 1, 0);
        for (int l = 0; l < L; ++l) start[l + 1] = start[l] + ((cnt[l + 1] + 31) / 32) * 32;
        std::vector<int> perm((size_t)std::max<long long>(start[L], 32), -1);
        std::vector<long long> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < n; ++i) perm[fill[lev[i]]++] = i;
        *nchunk = (int)(start[L] / 32);
        *nlev = L;
        *wide = 0;
        for (int l = 0; l < L; ++l) *wide = std::max(*wide, (int)((start[l + 1] - start[l]) / 32));
        return upload(out, perm.data(), perm.size());
    };
    cudaError_t e = make_perm(true, &t.perm_f, &t.nchunk_f, &t.nlev_f, &t.wide_f);
    if (e != cudaSuccess) return e;
    e = make_perm(false, &t.perm_b, &t.nchunk_b, &t.nlev_b, &t.wide_b);
    if (e != cudaSuccess) return e;
    t.levels_built = true;
    return cudaSuccess;
}

// Transposed-entry positions: for each stored (i,j), where (j,i) is stored
// (-1 where it is not: a structurally unsymmetric pattern).
cudaError_t build_transpose(DeviceTopology& t) {
    if (t.tpos) return cudaSuccess;
    std::vector<int> tp((size_t)t.nnz, -1);
    for (int i = 0; i < t.n; ++i)
        for (int j = t.h_rowptr[i]; j < t.h_rowptr[i + 1]; ++j) {
            const int c = t.h_col[j];
            const int* b = t.h_col.data() + t.h_rowptr[c];
            const int* e = t.h_col.data() + t.h_rowptr[c + 1];
            for (const int* p = b; p != e; ++p)
                if (*p == i) { tp[j] = (int)(p - t.h_col.data()); break; }
        }
    t.tsym = std::find(tp.begin(), tp.end(), -1) == tp.end();
    return upload(&t.tpos, tp.data(), tp.size());
}

unsigned long long mix(unsigned long long h, unsigned long long v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h * 0xBF58476D1CE4E5B9ull;
}

// Hash of the pattern arrays: every element when TFLOWS_TOPOLOGY_CHECK=full,
// otherwise ~8k samples spread over each array plus both ends.
unsigned long long pattern_hash(int n, int nnz, const int* Acol, const int* Arow, const int* Adia) {
    static const bool full = [] {
        const char* v = std::getenv("TFLOWS_TOPOLOGY_CHECK");
        return v && std::strcmp(v, "full") == 0;
    }();
    unsigned long long h = mix(0x1234567ull, (unsigned long long)n * 1000003ull + nnz);
    // About 8k evenly spaced entries per array (every entry with "full"),
    // hashed into four independent chains so that the loads overlap: the
    // check costs tens of microseconds per call, not milliseconds.
    auto sample = [&](const int* a, long long len) {
        if (len <= 0) return;
        const long long step = full ? 1 : std::max(1LL, len / 8192);
        unsigned long long c[4] = {h, h ^ 0x9e37ull, h ^ 0x7f4aull, h ^ 0x3c6eull};
        long long i = 0;
        for (; i + 3 * step < len; i += 4 * step)
            for (int k = 0; k < 4; ++k)
                c[k] = mix(c[k], (unsigned)a[i + k * step] + (unsigned long long)(i + k * step) * 31);
        for (; i < len; i += step) c[0] = mix(c[0], (unsigned)a[i] + (unsigned long long)i * 31);
        h = mix(mix(mix(mix(h, c[0]), c[1]), c[2]), c[3]);
        h = mix(h, (unsigned)a[len - 1]);
    };
    sample(Acol, (long long)n + 1);
    sample(Arow, nnz);
    sample(Adia, n);
    return h;
}

int set_device(Context& c, int want) {
    int dev = want;
    if (dev < 0) {
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return fail(TFLOWS_NO_DEVICE, "no CUDA device");
    if (dev >= count) return fail(TFLOWS_BAD_INPUT, "device ordinal out of range");
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    if (c.device != dev) {
        if (c.stream) cudaStreamDestroy(c.stream);
        c.stream = nullptr;
        c.cache.clear();
        c.device = dev;
    }
    if (!c.stream) {
        e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    }
    return TFLOWS_OK;
}

void destroy_topo(tflows_topology* tp) {
    if (!tp) return;
    free_topology_arrays(tp->t);
    free_workspace(tp->ws);
    for (auto& w : tp->extra_ws) free_workspace(*w);
    tp->extra_ws.clear();
}

struct TopoDeleter {
    void operator()(tflows_topology* p) const {
        destroy_topo(p);
        delete p;
    }
};

// Builds a topology from host arrays; returns status.
int make_topology(tflows_topology** out, int n, int nnz, const int* rp, const int* col,
                  const int* dg, int base) {
    auto tp = std::make_unique<tflows_topology>();
    std::string msg;
    int st = check_pattern(n, nnz, rp, col, dg, base, tp->t, msg);
    if (st != TFLOWS_OK) return fail(st, msg);
    cudaGetDevice(&tp->t.device);
    cudaError_t e = build_device(tp->t);
    if (e != cudaSuccess) {
        destroy_topo(tp.get());
        return cuda_fail(e, "topology upload");
    }
    *out = tp.release();
    return TFLOWS_OK;
}

// Legacy path: find or build the topology for these host arrays.
int cached_topology(Context& c, int N, int NONZ, const int* Acol, const int* Arow, const int* Adia,
                    tflows_topology** out) {
    const unsigned long long h = pattern_hash(N, NONZ - 1, Acol, Arow, Adia);
    for (auto& tp : c.cache) {
        if (tp->t.n == N && tp->t.nnz == NONZ - 1 && tp->k_acol == Acol && tp->k_arow == Arow &&
            tp->k_adia == Adia && tp->k_hash == h) {
            tp->last_use = ++c.clock;
            *out = tp.get();
            return TFLOWS_OK;
        }
    }
    tflows_topology* tp = nullptr;
    int st = make_topology(&tp, N, NONZ - 1, Acol, Arow, Adia, 1);
    if (st != TFLOWS_OK) return st;
    tp->k_acol = Acol;
    tp->k_arow = Arow;
    tp->k_adia = Adia;
    tp->k_hash = h;
    tp->last_use = ++c.clock;
    if (c.cache.size() >= 8) {
        auto it = std::min_element(c.cache.begin(), c.cache.end(),
                                   [](auto& a, auto& b) { return a->last_use < b->last_use; });
        destroy_topo(it->get());
        c.cache.erase(it);
    }
    c.cache.emplace_back(tp);
    *out = tp;
    return TFLOWS_OK;
}

double* ws_vec(tflows_topology* tp, int k) { return tp->ws.vec64 + (size_t)k * tp->ws.vec_cap; }

SolveRequest make_request(const tflows_options& o, int method, int prec, int maxiter, double tol) {
    SolveRequest rq;
    rq.method = method;
    rq.prec = prec;
    rq.precision = o.precision;
    rq.maxiter = maxiter;
    rq.tol = tol;
    rq.tol_relative = o.tol_mode == TFLOWS_TOL_RELATIVE;
    rq.inner_rtol = o.inner_rtol;
    rq.inner_maxiter = o.inner_maxiter;
    rq.max_refinements = o.max_refinements;
    // BF16 factor values exist only in the FP32 inner solves of the mixed
    // mode with IC(0); Jacobi sweeps there and in the contracted FP64 build
    // (the reference-arithmetic build keeps the reference's exact apply).
    const bool mixed_ic = o.precision == TFLOWS_MIXED && prec == 2;
    const bool fma_ic = o.precision == TFLOWS_FP64_FMA && prec == 2;
    rq.ic_sweeps = mixed_ic || fma_ic ? std::max(o.ic_sweeps, 0) : 0;
    rq.ic_bf16 = mixed_ic && o.ic_bf16 ? 1 : 0;
    rq.ic_tiled = o.ic_tiled < 0 ? -1 : (o.ic_tiled != 0);
    rq.refine_restart = o.refine_restart;
    rq.inject_stall = o.inject_stall;
    rq.timeout_s = o.timeout_s > 0 ? o.timeout_s : 5.0;
    rq.block = o.block_size;
    rq.grid = o.grid_blocks;
    rq.rows_per_warp = o.rows_per_warp;
    rq.sweep_mult = o.sweep_warps;
    rq.sweep_gate = o.sweep_gate < 0 ? -1 : (o.sweep_gate != 0);
    rq.autotune = o.autotune && o.block_size == 0 && o.grid_blocks == 0 ? 1 : 0;
    return rq;
}

// Launch-shape options a kernel launch can take.
bool shape_ok(const SolveRequest& rq, std::string& msg) {
    if (rq.precision != TFLOWS_FP64 && rq.precision != TFLOWS_MIXED &&
        rq.precision != TFLOWS_FP64_FMA) {
        msg = "precision must be TFLOWS_FP64, TFLOWS_MIXED or TFLOWS_FP64_FMA";
        return false;
    }
    if (rq.block != 0 && (rq.block % 32 != 0 || rq.block < 64 || rq.block > 512)) {
        msg = "block_size must be 0 or a multiple of 32 in 64..512";
        return false;
    }
    if (rq.grid < 0 || rq.rows_per_warp < 0 || rq.sweep_mult < 0) {
        msg = "grid_blocks, rows_per_warp and sweep_warps must be >= 0";
        return false;
    }
    return true;
}

// The tuned launch shape for this system class: from the table, or timed
// now on the caller's values and right-hand side (device arrays; x0 and b
// are preserved even where they live in the workspace slots the timing
// runs use).
int autotune_on(tflows_topology* tp, SolveRequest& rq, const double* d_b, const double* d_x,
                cudaStream_t s, TuneChoice& ch) {
    if (tune_lookup(tp->t, rq, ch)) {
        tune_apply(ch, rq);
        return TFLOWS_OK;
    }
    const size_t nb = sizeof(double) * tp->t.n;
    double* tmp = nullptr;
    cudaError_t e = cudaMalloc(&tmp, 2 * std::max<size_t>(nb, 8));
    if (e != cudaSuccess) return cuda_fail(e, "tuning buffers");
    double* tb = tmp;
    double* tx = tmp + std::max<size_t>(tp->t.n, 1);
    e = cudaMemcpyAsync(tb, d_b, nb, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && d_x) e = cudaMemcpyAsync(tx, d_x, nb, cudaMemcpyDeviceToDevice, s);
    std::string msg;
    int st = e == cudaSuccess ? tune_solve(tp->t, tp->ws, rq, tb, s, ch, msg) : TFLOWS_CUDA_ERROR;
    if (e == cudaSuccess && d_x) e = cudaMemcpyAsync((double*)d_x, tx, nb, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "tuning");
    if (st != TFLOWS_OK) return fail(st, msg);
    tune_apply(ch, rq);
    return TFLOWS_OK;
}

void record(const SolveReport& rep, tflows_result* res) {
    tflows_result r{};
    r.status = rep.status;
    r.iterations = rep.iterations;
    r.inner_iterations = rep.inner_iterations;
    r.refinements = rep.refinements;
    r.ini_res = rep.ini_res;
    r.fin_res = rep.fin_res;
    r.seconds = rep.seconds;
    r.bytes = rep.bytes;
    r.block_size = rep.block;
    r.grid_blocks = rep.grid;
    r.group_seconds = rep.group_seconds;
    t_result = r;
    if (res) *res = r;
}

// Core of the device-resident solve; b is read from `b` into a workspace
// residual vector.  Caller holds tp->mu.
int solve_on(tflows_topology* tp, const SolveRequest& rq0, const double* d_val, const double* d_b,
             double* d_x, double* d_r_out, cudaStream_t s, SolveReport& rep) {
    SolveRequest rq = rq0;
    if (std::string msg; !shape_ok(rq, msg)) return fail(TFLOWS_BAD_INPUT, msg);
    if (rq.method == TFLOWS_METHOD_BICG_TRUE) {
        if (rq.precision == TFLOWS_MIXED)
            return fail(TFLOWS_UNSUPPORTED, "true BiCG runs in FP64 only (TFLOWS_FP64 or _FP64_FMA)");
        if (rq.prec == 2) return fail(TFLOWS_UNSUPPORTED, "true BiCG takes prec 0 or 1");
        if (cudaError_t e = build_transpose(tp->t); e != cudaSuccess)
            return cuda_fail(e, "transpose map");
        if (!tp->t.tsym)
            return fail(TFLOWS_BAD_INPUT, "true BiCG needs a structurally symmetric pattern");
    }
    if (rq.prec == 2) {
        if (!tp->t.ic_ok)
            return fail(TFLOWS_BAD_INPUT,
                        "IC(0) needs each row's entries before Adia to have smaller column "
                        "indices and those after it larger ones");
        cudaError_t e = build_levels(tp->t);
        if (e != cudaSuccess) return cuda_fail(e, "level sets");
    }
    cudaError_t e = ensure_workspace(tp->ws, tp->t);
    if (e == cudaSuccess && rq.ic_bf16) e = ensure_lu16(tp->ws);
    if (e != cudaSuccess) return cuda_fail(e, "workspace");
    if ((e = permute_values(tp->t, tp->ws, d_val, true, rq.precision == TFLOWS_MIXED, s,
                            rq.ic_bf16 != 0)) != cudaSuccess)
        return cuda_fail(e, "value layout");
    if (rq.method == TFLOWS_METHOD_BICG_TRUE &&
        (e = permute_transposed(tp->t, tp->ws, d_val, s)) != cudaSuccess)
        return cuda_fail(e, "transposed values");
    trace_mark("layout enqueued");
    if (rq.autotune) {
        TuneChoice ch;
        if (int st = autotune_on(tp, rq, d_b, d_x, s, ch); st != TFLOWS_OK) return st;
    }
    trace_mark("launch shape");
    // The kernels work on padded, 16-byte aligned workspace vectors: x and b
    // are staged into workspace slots 11 and 12 unless they already are them.
    const size_t nb = sizeof(double) * tp->t.n;
    double* X = ws_vec(tp, 11);
    double* R = ws_vec(tp, 12);
    if (d_x != X && (e = cudaMemcpyAsync(X, d_x, nb, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy x");
    if ((e = cudaMemcpyAsync(R, d_b, nb, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy b");
    int st = run_solve(tp->t, tp->ws, rq, X, R, s, rep);
    if (st == TFLOWS_CUDA_ERROR) return fail(st, rep.message);
    if (d_x != X && (e = cudaMemcpyAsync(d_x, X, nb, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy x back");
    if (d_r_out && (e = cudaMemcpyAsync(d_r_out, R, nb, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy r");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "sync");
    t_status = st;
    t_error = rep.message;
    return st;
}

}  // namespace

unsigned long long tflows::legacy_pattern_hash(int n, int nnz, const int* Acol, const int* Arow,
                                               const int* Adia) {
    return pattern_hash(n, nnz, Acol, Arow, Adia);
}

// Status and message of the last call on this thread, for the other units.
int tflows::report_status(int status, const std::string& msg) {
    t_status = status;
    t_error = msg;
    return status;
}

namespace {
// TFLOWS_TRACE_LEGACY=1: the legacy calls print the host time at each phase
// (topology lookup, uploads enqueued, solve returned, results copied back).
struct LegacyTrace {
    const bool on = [] {
        const char* v = std::getenv("TFLOWS_TRACE_LEGACY");
        return v && *v && *v != '0';
    }();
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    LegacyTrace();
    ~LegacyTrace();
    void mark(const char* what) const {
        if (!on) return;
        const double ms = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "tflows legacy: %-22s %10.3f ms\n", what, ms);
    }
};
thread_local const LegacyTrace* t_trace = nullptr;
LegacyTrace::LegacyTrace() { if (on) t_trace = this; }
LegacyTrace::~LegacyTrace() { if (t_trace == this) t_trace = nullptr; }
}  // namespace

// Phase marks from inside a traced legacy call (no-op otherwise).
void tflows::trace_mark(const char* what) {
    if (t_trace) t_trace->mark(what);
}

extern "C" {

void tflows_default_options(tflows_options* opt) {
    if (opt) default_opts(opt);
}

int tflows_set_options(const tflows_options* opt) {
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!opt) {
        default_opts(&c.opts);
    } else {
        c.opts = *opt;
    }
    c.opts_set = true;
    return TFLOWS_OK;
}

int tflows_last_status(void) { return t_status; }

const char* tflows_status_string(int s) {
    switch (s) {
        case TFLOWS_OK: return "ok";
        case TFLOWS_NOT_CONVERGED: return "not converged";
        case TFLOWS_BREAKDOWN: return "breakdown";
        case TFLOWS_NONFINITE: return "non-finite residual";
        case TFLOWS_TIMEOUT: return "device wait timed out";
        case TFLOWS_BAD_INPUT: return "bad input";
        case TFLOWS_CUDA_ERROR: return "CUDA error";
        case TFLOWS_NO_DEVICE: return "no CUDA device";
        case TFLOWS_UNSUPPORTED: return "unsupported option";
        case TFLOWS_HALO_ERROR: return "halo callback failed";
        default: return "unknown status";
    }
}

const char* tflows_last_error(void) { return t_error.c_str(); }

void tflows_last_result(tflows_result* res) {
    if (res) *res = t_result;
}

void tflows_forget_topologies(void) {
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.device >= 0) cudaSetDevice(c.device);
    for (auto& tp : c.cache) destroy_topo(tp.get());
    c.cache.clear();
}

void tflows_finalize(void) {
    halo_release();
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    for (auto& tp : c.cache) destroy_topo(tp.get());
    c.cache.clear();
    if (c.stream) cudaStreamDestroy(c.stream);
    c.stream = nullptr;
    c.device = -1;
}


int tflows_solve_ex(int method, const int* N, const int* NB, const int* NONZ, const double* A,
                    const int* Acol, const int* Arow, const int* Adia, const double* Ab, double* x,
                    double* r1, const int* prec, int* niter, const double* tol, double* IniRes,
                    double* FinRes, const tflows_options* opt, tflows_result* res) {
    t_error.clear();
    SolveReport rep;
    if (!N || !NB || !NONZ || !prec || !niter || !tol || !IniRes || !FinRes || !x || !r1) {
        record(rep, res);
        return fail(TFLOWS_BAD_INPUT, "null argument");
    }
    if (method < 0 || method > 3) return fail(TFLOWS_BAD_INPUT, "unknown method");
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    tflows_options o;
    if (opt) o = *opt;
    else if (c.opts_set) o = c.opts;
    else default_opts(&o);
    const int n = *N, nb = *NB, nonz = *NONZ;
    if (n < 0 || nb < 0 || nonz < 1) return fail(TFLOWS_BAD_INPUT, "N, NB must be >= 0 and NONZ >= 1");
    if (n == 0) {
        // Empty system: ||b|| = 0.  The reference exits on bnrm2 < tol with
        // iter = 0 and reports the stale module error; with tol <= 0 it runs
        // the loop on empty sums, which ends at niter+1 with error = 0.
        if (0.0 < *tol) {
            *niter = 0;
            *FinRes = c.error_state;
        } else {
            *IniRes = 0.0;
            c.error_state = 0.0;
            *FinRes = 0.0;
            *niter = std::max(*niter, 0) + 1;
        }
        rep.status = TFLOWS_OK;
        record(rep, res);
        t_status = TFLOWS_OK;
        return TFLOWS_OK;
    }
    if (!A || !Acol || !Arow || !Adia) return fail(TFLOWS_BAD_INPUT, "null matrix array");
    const LegacyTrace trace;
    int st = set_device(c, o.device);
    if (st != TFLOWS_OK) return st;
    if (halo_registered()) {
        // subdomain run: Ab couples the rows to the neighbours' buffer cells
        if (o.precision != TFLOWS_FP64)
            return fail(TFLOWS_UNSUPPORTED, "halo-coupled solves run in FP64 reference arithmetic");
        st = halo_solve(method, n, nb, nonz, A, Acol, Arow, Adia, Ab, x, r1, *prec, niter, *tol,
                        IniRes, FinRes, c.error_state, c.stream, rep);
        record(rep, res);
        t_status = st;
        t_error = rep.message;
        return st;
    }
    // one-domain run (Npro = 0): the subdomain loops are empty and Ab is not read
    tflows_topology* tp = nullptr;
    st = cached_topology(c, n, nonz, Acol, Arow, Adia, &tp);
    if (st != TFLOWS_OK) return st;
    trace.mark("topology");
    cudaError_t e = ensure_workspace(tp->ws, tp->t);
    if (e != cudaSuccess) return cuda_fail(e, "workspace");
    cudaStream_t s = c.stream;
    double* X = ws_vec(tp, 11);
    double* B = ws_vec(tp, 13);
    const size_t nbytes = sizeof(double) * (size_t)n;
    if ((e = cudaMemcpyAsync(tp->ws.csr_val, A, sizeof(double) * (size_t)(nonz - 1),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy A");
    if ((e = cudaMemcpyAsync(X, x + nb + 1, nbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy x");
    if ((e = cudaMemcpyAsync(B, r1, nbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "copy r1");
    if (trace.on) cudaStreamSynchronize(s);
    trace.mark("uploads done");
    SolveRequest rq = make_request(o, method, *prec, *niter, *tol);
    st = solve_on(tp, rq, tp->ws.csr_val, B, X, nullptr, s, rep);
    trace.mark("solve returned");
    if (st == TFLOWS_CUDA_ERROR || st == TFLOWS_BAD_INPUT || st == TFLOWS_UNSUPPORTED) {
        record(rep, res);
        return st;
    }
    const double* R = ws_vec(tp, 12);
    const bool untouched = rep.exit_kind == EXIT_BNRM;
    if (!untouched) {
        if ((e = cudaMemcpyAsync(x + nb + 1, X, nbytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail(e, "copy x back");
        if ((e = cudaMemcpyAsync(r1, R, nbytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail(e, "copy r1 back");
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "sync");
        trace.mark("results copied back");
    }
    *niter = rep.iterations;
    if (untouched) {
        *FinRes = c.error_state;
    } else {
        *IniRes = rep.ini_res;
        *FinRes = rep.fin_res;
        c.error_state = rep.fin_res;
    }
    record(rep, res);
    t_status = st;
    return st;
}

#define TFLOWS_LEGACY(NAME, METHOD)                                                            \
    void NAME(const int* N, const int* NB, const int* NONZ, const double* A, const int* Acol,  \
              const int* Arow, const int* Adia, const double* Ab, double* x, double* r1,      \
              const int* prec, int* niter, const double* tol, double* IniRes, double* FinRes) { \
        tflows_solve_ex(METHOD, N, NB, NONZ, A, Acol, Arow, Adia, Ab, x, r1, prec, niter, tol,  \
                        IniRes, FinRes, nullptr, nullptr);                                     \
    }
TFLOWS_LEGACY(tflows_cg, TFLOWS_METHOD_CG)
TFLOWS_LEGACY(tflows_bicg, TFLOWS_METHOD_BICG)
TFLOWS_LEGACY(tflows_cgs, TFLOWS_METHOD_CGS)
#undef TFLOWS_LEGACY

void tflows_prec1(const int* N, const int* NONZ, const double* A, const int* Acol, const int* Arow,
                  const int* Adia, double* D, const int* prec) {
    t_error.clear();
    if (!N || !NONZ || !D || !prec) { fail(TFLOWS_BAD_INPUT, "null argument"); return; }
    const int n = *N;
    if (n == 0) { t_status = TFLOWS_OK; return; }
    if (*prec != 1 && *prec != 2) {
        for (int i = 0; i < n; ++i) D[i] = 1.0;
        t_status = TFLOWS_OK;
        return;
    }
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    int st = set_device(c, c.opts_set ? c.opts.device : -1);
    if (st != TFLOWS_OK) return;
    tflows_topology* tp = nullptr;
    if ((st = cached_topology(c, n, *NONZ, Acol, Arow, Adia, &tp)) != TFLOWS_OK) return;
    if (*prec == 2) {
        if (!tp->t.ic_ok) { fail(TFLOWS_BAD_INPUT, "IC(0) needs a triangular-ordered pattern"); return; }
        if (cudaError_t e = build_levels(tp->t); e != cudaSuccess) { cuda_fail(e, "levels"); return; }
    }
    cudaError_t e = ensure_workspace(tp->ws, tp->t);
    if (e != cudaSuccess) { cuda_fail(e, "workspace"); return; }
    cudaStream_t s = c.stream;
    if ((e = cudaMemcpyAsync(tp->ws.csr_val, A, sizeof(double) * (size_t)(*NONZ - 1),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess) { cuda_fail(e, "copy A"); return; }
    if ((e = permute_values(tp->t, tp->ws, tp->ws.csr_val, true, false, s)) != cudaSuccess) {
        cuda_fail(e, "layout");
        return;
    }
    double* Dd = ws_vec(tp, 13);
    SolveReport rep;
    const double to = c.opts_set && c.opts.timeout_s > 0 ? c.opts.timeout_s : 5.0;
    st = run_prec1(tp->t, tp->ws, *prec, Dd, to, s, rep);
    if (st != TFLOWS_OK) { fail(st, rep.message); return; }
    if ((e = cudaMemcpyAsync(D, Dd, sizeof(double) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        cuda_fail(e, "copy D");
        return;
    }
    t_status = TFLOWS_OK;
}

void tflows_resid(const int* N, const int* NB, const int* NONZ, const double* A, const int* Acol,
                  const int* Arow, const double* Ab, const double* x, double* r1) {
    t_error.clear();
    if (!N || !NB || !NONZ || !x || !r1) { fail(TFLOWS_BAD_INPUT, "null argument"); return; }
    const int n = *N, nb = *NB;
    if (n == 0) { t_status = TFLOWS_OK; return; }
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    int st = set_device(c, c.opts_set ? c.opts.device : -1);
    if (st != TFLOWS_OK) return;
    if (halo_registered()) {
        // subdomain run: r1(BufInd(k)) -= Ab(k) x(k) after the local rows
        std::string msg;
        if (!A || !Acol || !Arow) { fail(TFLOWS_BAD_INPUT, "null matrix array"); return; }
        st = halo_resid(n, nb, *NONZ, A, Acol, Arow, Ab, x, r1, c.stream, msg);
        if (st != TFLOWS_OK) { fail(st, msg); return; }
        t_status = TFLOWS_OK;
        return;
    }
    // Resid needs no diagonal positions; a pattern without Adia gets a
    // synthesised one so that the cache and layout can be shared.
    tflows_topology* tp = nullptr;
    std::vector<int> fake_dia;
    const int* dia = nullptr;
    {
        fake_dia.resize(n);
        for (int i = 0; i < n; ++i) {
            fake_dia[i] = -1;
            for (int j = Acol[i]; j < Acol[i + 1]; ++j)
                if (Arow[j - 1] == i + 1) { fake_dia[i] = j; break; }
            if (fake_dia[i] < 0) { fail(TFLOWS_BAD_INPUT, "row without a diagonal entry"); return; }
        }
        dia = fake_dia.data();
    }
    if ((st = make_topology(&tp, n, *NONZ - 1, Acol, Arow, dia, 1)) != TFLOWS_OK) return;
    std::unique_ptr<tflows_topology, TopoDeleter> hold(tp);
    cudaError_t e = ensure_workspace(tp->ws, tp->t);
    if (e != cudaSuccess) { cuda_fail(e, "workspace"); return; }
    cudaStream_t s = c.stream;
    double* X = ws_vec(tp, 11);
    double* R = ws_vec(tp, 12);
    e = cudaMemcpyAsync(tp->ws.csr_val, A, sizeof(double) * (size_t)(*NONZ - 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(X, x + nb + 1, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(R, r1, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = permute_values(tp->t, tp->ws, tp->ws.csr_val, true, false, s);
    if (e == cudaSuccess) e = run_resid(tp->t, tp->ws, X, R, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r1, R, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cuda_fail(e, "resid"); return; }
    t_status = TFLOWS_OK;
}

// ---- device-pointer interface --------------------------------------------------

int tflows_topology_create(tflows_topology** out, int n, int nnz, const int* rowptr, const int* col,
                           const int* diag, int index_base, int on_device) {
    t_error.clear();
    if (!out) return fail(TFLOWS_BAD_INPUT, "null output");
    if (index_base != 0 && index_base != 1) return fail(TFLOWS_BAD_INPUT, "index_base must be 0 or 1");
    if (n <= 0 || nnz < 0) return fail(TFLOWS_BAD_INPUT, "n must be > 0");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(TFLOWS_NO_DEVICE, "no CUDA device");
    std::vector<int> hr, hc, hd;
    const int *prp = rowptr, *pc = col, *pd = diag;
    if (on_device) {
        hr.resize((size_t)n + 1);
        hc.resize((size_t)nnz);
        hd.resize((size_t)n);
        cudaError_t e = cudaMemcpy(hr.data(), rowptr, hr.size() * sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && nnz) e = cudaMemcpy(hc.data(), col, hc.size() * sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hd.data(), diag, hd.size() * sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "read pattern");
        prp = hr.data();
        pc = hc.data();
        pd = hd.data();
    }
    int st = make_topology(out, n, nnz, prp, pc, pd, index_base);
    t_status = st;
    return st;
}

void tflows_topology_destroy(tflows_topology* topo) {
    if (!topo) return;
    destroy_topo(topo);
    delete topo;
}

int tflows_topology_patterns(tflows_topology* topo) { return topo ? topo->t.npat : 0; }

const int* tflows_topology_transpose_map(tflows_topology* topo) {
    if (!topo) return nullptr;
    std::lock_guard<std::mutex> lk(topo->mu);
    if (build_transpose(topo->t) != cudaSuccess) return nullptr;
    return topo->t.tpos;
}

int tflows_solve_device(tflows_topology* topo, int method, int prec, const tflows_options* opt,
                        const double* val, const double* b, double* x, double* r_out, int maxiter,
                        double tol, void* stream, tflows_result* res) {
    t_error.clear();
    SolveReport rep;
    if (!topo || !val || !b || !x) {
        record(rep, res);
        return fail(TFLOWS_BAD_INPUT, "null argument");
    }
    tflows_options o;
    if (opt) o = *opt;
    else default_opts(&o);
    std::lock_guard<std::mutex> lk(topo->mu);
    cudaSetDevice(topo->t.device);
    SolveRequest rq = make_request(o, method, prec, maxiter, tol);
    cudaStream_t s = (cudaStream_t)stream;
    int st = solve_on(topo, rq, val, b, x, r_out, s, rep);
    if (!r_out) cudaStreamSynchronize(s);
    record(rep, res);
    return st;
}

int tflows_solve_batched_device(int count, tflows_topology* const* topos, const int* methods,
                                const int* precs, const tflows_options* opt,
                                const double* const* vals, const double* const* bs,
                                double* const* xs, const int* maxiters, const double* tols,
                                void* stream, tflows_result* results) {
    t_error.clear();
    if (count < 0 || (count > 0 && (!topos || !methods || !precs || !vals || !bs || !xs || !maxiters ||
                                    !tols)))
        return fail(TFLOWS_BAD_INPUT, "null argument");
    if (count == 0) return TFLOWS_OK;
    for (int k = 0; k < count; ++k)
        if (!topos[k] || !vals[k] || !bs[k] || !xs[k]) return fail(TFLOWS_BAD_INPUT, "null system");
    tflows_options o;
    if (opt) o = *opt;
    else default_opts(&o);
    std::vector<tflows_topology*> uniq(topos, topos + count);
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    std::vector<std::unique_lock<std::mutex>> locks;
    for (auto* tp : uniq) locks.emplace_back(tp->mu);
    const int dev = topos[0]->t.device;
    for (auto* tp : uniq)
        if (tp->t.device != dev) return fail(TFLOWS_BAD_INPUT, "systems on different devices");
    cudaSetDevice(dev);
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<SolveReport> reps(count);
    std::vector<BatchSpec> specs(count);
    std::vector<std::pair<tflows_topology*, int>> uses;
    for (int k = 0; k < count; ++k) {
        tflows_topology* tp = topos[k];
        int j = 0;
        for (auto& u : uses)
            if (u.first == tp) j = ++u.second;
        if (j == 0) uses.emplace_back(tp, 0);
        while ((int)tp->extra_ws.size() < j) tp->extra_ws.emplace_back(new Workspace());
        Workspace* ws = j == 0 ? &tp->ws : tp->extra_ws[j - 1].get();
        SolveRequest rq = make_request(o, methods[k], precs[k], maxiters[k], tols[k]);
        if (std::string msg; !shape_ok(rq, msg)) return fail(TFLOWS_BAD_INPUT, msg);
        if (rq.method == TFLOWS_METHOD_BICG_TRUE)
            return fail(TFLOWS_UNSUPPORTED, "true BiCG is not available in batched solves");
        if (rq.prec == 2) {
            if (!tp->t.ic_ok) return fail(TFLOWS_BAD_INPUT, "IC(0) needs a triangular-ordered pattern");
            cudaError_t e = build_levels(tp->t);
            if (e != cudaSuccess) return cuda_fail(e, "level sets");
        }
        cudaError_t e = ensure_workspace(*ws, tp->t);
        if (e == cudaSuccess && rq.ic_bf16) e = ensure_lu16(*ws);
        if (e == cudaSuccess)
            e = permute_values(tp->t, *ws, vals[k], true, rq.precision == TFLOWS_MIXED, s,
                               rq.ic_bf16 != 0);
        double* X = ws->vec64 + 11 * ws->vec_cap;
        double* R = ws->vec64 + 12 * ws->vec_cap;
        const size_t nb = sizeof(double) * tp->t.n;
        if (e == cudaSuccess) e = cudaMemcpyAsync(X, xs[k], nb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(R, bs[k], nb, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "batch staging");
        specs[k] = BatchSpec{&tp->t, ws, rq, X, R, &reps[k]};
    }
    double sec = 0.0;
    int worst = run_batch(specs, s, &sec);
    std::string msg;
    for (int k = 0; k < count; ++k)
        if (!reps[k].message.empty()) {
            msg = "system " + std::to_string(k) + ": " + reps[k].message;
            break;
        }
    if (worst == TFLOWS_CUDA_ERROR || worst == TFLOWS_BAD_INPUT) {
        for (int k = 0; k < count; ++k) record(reps[k], results ? results + k : nullptr);
        return fail(worst, msg);
    }
    t_error = msg;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < count && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync(xs[k], specs[k].x, sizeof(double) * specs[k].t->n,
                            cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "batch results");
    for (int k = 0; k < count; ++k) record(reps[k], results ? results + k : nullptr);
    t_status = worst;
    t_error = msg;
    return worst;
}

struct tflows_plan {
    std::vector<tflows_topology*> topos;
    std::vector<std::unique_ptr<Workspace>> ws;
    std::vector<SolveReport> reps;
    std::vector<BatchSpec> specs;
    BatchLaunch* launch = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t last = nullptr;
    int device = 0;
    BatchTuning tuning;
    bool tuned = false;
};

int tflows_plan_create(tflows_plan** out, int count, tflows_topology* const* topos,
                       const int* methods, const int* precs, const tflows_options* opt,
                       const double* const* vals, const double* const* bs, double* const* xs,
                       const int* maxiters, const double* tols) {
    t_error.clear();
    if (!out || count <= 0 || !topos || !methods || !precs || !vals || !bs || !xs || !maxiters ||
        !tols)
        return fail(TFLOWS_BAD_INPUT, "null argument");
    tflows_options o;
    if (opt) o = *opt;
    else default_opts(&o);
    auto plan = std::make_unique<tflows_plan>();
    plan->device = topos[0]->t.device;
    cudaSetDevice(plan->device);
    plan->reps.resize(count);
    plan->specs.resize(count);
    for (int k = 0; k < count; ++k) {
        tflows_topology* tp = topos[k];
        if (!tp || !vals[k] || !bs[k] || !xs[k]) return fail(TFLOWS_BAD_INPUT, "null system");
        if (tp->t.device != plan->device) return fail(TFLOWS_BAD_INPUT, "systems on different devices");
        std::lock_guard<std::mutex> lk(tp->mu);
        SolveRequest rq = make_request(o, methods[k], precs[k], maxiters[k], tols[k]);
        if (std::string msg; !shape_ok(rq, msg)) return fail(TFLOWS_BAD_INPUT, msg);
        if (rq.method == TFLOWS_METHOD_BICG_TRUE)
            return fail(TFLOWS_UNSUPPORTED, "true BiCG is not available in batched solves");
        if (rq.prec == 2) {
            if (!tp->t.ic_ok) return fail(TFLOWS_BAD_INPUT, "IC(0) needs a triangular-ordered pattern");
            if (cudaError_t e = build_levels(tp->t); e != cudaSuccess) return cuda_fail(e, "level sets");
        }
        plan->ws.emplace_back(new Workspace());
        cudaError_t ew = ensure_workspace(*plan->ws.back(), tp->t);
        if (ew == cudaSuccess && rq.ic_bf16) ew = ensure_lu16(*plan->ws.back());
        if (ew != cudaSuccess) return cuda_fail(ew, "workspace");
        Workspace* ws = plan->ws.back().get();
        plan->specs[k] = BatchSpec{&tp->t, ws, rq, ws->vec64 + 11 * ws->vec_cap,
                                   ws->vec64 + 12 * ws->vec_cap, &plan->reps[k]};
        plan->topos.push_back(tp);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&plan->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "plan stream");
    if (o.autotune && o.block_size == 0 && o.grid_blocks == 0) {
        // Block size and group split from timed full batched solves on the
        // caller's data (x0 and b re-staged before every run).
        cudaStream_t ts = plan->cap;
        for (int k = 0; k < count && e == cudaSuccess; ++k) {
            BatchSpec& sp = plan->specs[k];
            e = permute_values(*sp.t, *sp.ws, vals[k], true, sp.rq.precision == TFLOWS_MIXED, ts,
                               sp.rq.ic_bf16 != 0);
        }
        if (e != cudaSuccess) return cuda_fail(e, "plan tuning");
        auto restage = [&]() -> cudaError_t {
            cudaError_t er = cudaSuccess;
            for (int k = 0; k < count && er == cudaSuccess; ++k) {
                BatchSpec& sp = plan->specs[k];
                const size_t nb = sizeof(double) * sp.t->n;
                er = cudaMemcpyAsync(sp.x, xs[k], nb, cudaMemcpyDeviceToDevice, ts);
                if (er == cudaSuccess) er = cudaMemcpyAsync(sp.r, bs[k], nb, cudaMemcpyDeviceToDevice, ts);
            }
            return er;
        };
        std::string msg;
        const int st = tune_batch(plan->specs, restage, ts, plan->tuning, msg);
        if (st != TFLOWS_OK) return fail(st, msg);
        plan->tuned = true;
        for (auto& r : plan->reps) r = SolveReport();
    }
    // records of the tiled IC sweeps for the final launch shape (no
    // allocation may happen inside the capture)
    for (int k = 0; k < count && e == cudaSuccess; ++k)
        e = ensure_tiles(*plan->specs[k].t, *plan->specs[k].ws, plan->specs[k].rq);
    if (e != cudaSuccess) return cuda_fail(e, "tile buffers");
    plan->launch = batch_create();
    if ((e = batch_reserve(plan->launch, count, plan->specs[0].rq.block)) != cudaSuccess) {
        tflows_plan_destroy(plan.release());
        return cuda_fail(e, "plan buffers");
    }
    cudaStream_t s = plan->cap;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "begin capture");
    int st = TFLOWS_OK;
    for (int k = 0; k < count && e == cudaSuccess; ++k) {
        BatchSpec& sp = plan->specs[k];
        const size_t nb = sizeof(double) * sp.t->n;
        e = permute_values(*sp.t, *sp.ws, vals[k], true, sp.rq.precision == TFLOWS_MIXED, s,
                           sp.rq.ic_bf16 != 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(sp.x, xs[k], nb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(sp.r, bs[k], nb, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess) st = batch_enqueue(plan->launch, plan->specs, s);
    for (int k = 0; k < count && e == cudaSuccess && st == TFLOWS_OK; ++k)
        e = cudaMemcpyAsync(xs[k], plan->specs[k].x, sizeof(double) * plan->specs[k].t->n,
                            cudaMemcpyDeviceToDevice, s);
    cudaError_t ee = cudaStreamEndCapture(s, &plan->graph);
    if (e == cudaSuccess) e = ee;
    if (st != TFLOWS_OK) {
        std::string msg = plan->reps[0].message;
        tflows_plan_destroy(plan.release());
        return fail(st, msg);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (e != cudaSuccess) {
        tflows_plan_destroy(plan.release());
        return fail(TFLOWS_UNSUPPORTED, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    *out = plan.release();
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

int tflows_plan_launch(tflows_plan* plan, void* stream) {
    if (!plan || !plan->exec) return fail(TFLOWS_BAD_INPUT, "null plan");
    cudaSetDevice(plan->device);
    cudaError_t e = cudaGraphLaunch(plan->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    plan->last = (cudaStream_t)stream;
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

int tflows_plan_results(tflows_plan* plan, tflows_result* results) {
    if (!plan) return fail(TFLOWS_BAD_INPUT, "null plan");
    cudaSetDevice(plan->device);
    int worst = batch_collect(plan->launch, plan->specs, plan->last, 0.0);
    for (size_t k = 0; k < plan->reps.size(); ++k) record(plan->reps[k], results ? results + k : nullptr);
    t_status = worst;
    return worst;
}

void tflows_plan_destroy(tflows_plan* plan) {
    if (!plan) return;
    cudaSetDevice(plan->device);
    if (plan->last) cudaStreamSynchronize(plan->last);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    if (plan->cap) cudaStreamDestroy(plan->cap);
    if (plan->launch) batch_destroy(plan->launch);
    for (auto& w : plan->ws) free_workspace(*w);
    delete plan;
}

int tflows_plan_tuning(const tflows_plan* plan, tflows_batch_tuning* out) {
    if (!plan || !out) return fail(TFLOWS_BAD_INPUT, "null argument");
    out->block_size = plan->specs.empty() ? 0 : std::max(plan->specs[0].rq.block, 0);
    if (out->block_size == 0) out->block_size = 256;
    out->runs = plan->tuned ? plan->tuning.runs : 0;
    out->default_seconds = plan->tuned ? plan->tuning.default_seconds : 0.0;
    out->tuned_seconds = plan->tuned ? plan->tuning.tuned_seconds : 0.0;
    return TFLOWS_OK;
}

int tflows_autotune(tflows_topology* topo, int method, int prec, const tflows_options* opt,
                    const double* val, const double* b, void* stream, tflows_tuning* out) {
    t_error.clear();
    if (!topo || !val || !b || !out) return fail(TFLOWS_BAD_INPUT, "null argument");
    tflows_options o;
    if (opt) o = *opt;
    else default_opts(&o);
    std::lock_guard<std::mutex> lk(topo->mu);
    cudaSetDevice(topo->t.device);
    SolveRequest rq = make_request(o, method, prec, 1, 0.0);
    if (std::string msg; !shape_ok(rq, msg)) return fail(TFLOWS_BAD_INPUT, msg);
    if (rq.method == TFLOWS_METHOD_BICG_TRUE)
        return fail(TFLOWS_UNSUPPORTED, "the tuner covers CG, BiCG and CGS");
    if (rq.prec == 2) {
        if (!topo->t.ic_ok) return fail(TFLOWS_BAD_INPUT, "IC(0) needs a triangular-ordered pattern");
        if (cudaError_t e = build_levels(topo->t); e != cudaSuccess) return cuda_fail(e, "level sets");
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = ensure_workspace(topo->ws, topo->t);
    if (e == cudaSuccess && rq.ic_bf16) e = ensure_lu16(topo->ws);
    if (e == cudaSuccess)
        e = permute_values(topo->t, topo->ws, val, true, rq.precision == TFLOWS_MIXED, s,
                           rq.ic_bf16 != 0);
    if (e != cudaSuccess) return cuda_fail(e, "tuning setup");
    TuneChoice ch;
    const int st = autotune_on(topo, rq, b, nullptr, s, ch);
    if (st != TFLOWS_OK) return st;
    out->block_size = ch.block;
    out->rows_per_warp = ch.rows_per_warp;
    out->grid_blocks = planned_grid(topo->t, rq);
    out->sweep_warps = ch.sweep_mult;
    out->sweep_gate = ch.sweep_gate;
    out->candidates = ch.candidates;
    out->from_table = ch.from_cache;
    out->us_per_iteration = ch.us_per_iter;
    out->default_us_per_iteration = ch.default_us_per_iter;
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

void tflows_autotune_clear(void) { tune_clear(); }

int tflows_pattern_outer(tflows_topology* topo, const double* lambda, const double* x,
                         double* grad_val, void* stream) {
    if (!topo || !lambda || !x || !grad_val) return fail(TFLOWS_BAD_INPUT, "null argument");
    cudaSetDevice(topo->t.device);
    cudaError_t e = run_pattern_outer(topo->t, lambda, x, grad_val, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "pattern outer");
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

int tflows_ic_apply_device(tflows_topology* topo, const tflows_options* opt, const double* val,
                           const double* r, double* z, void* stream, tflows_result* res) {
    t_error.clear();
    if (!topo || !val || !r || !z) return fail(TFLOWS_BAD_INPUT, "null argument");
    std::lock_guard<std::mutex> lk(topo->mu);
    cudaSetDevice(topo->t.device);
    tflows_options o;
    if (opt) o = *opt;
    else default_opts(&o);
    if (o.precision == TFLOWS_MIXED) return fail(TFLOWS_UNSUPPORTED, "the apply runs in FP64");
    if (!topo->t.ic_ok)
        return fail(TFLOWS_BAD_INPUT, "IC(0) needs a triangular-ordered pattern");
    SolveRequest rq = make_request(o, TFLOWS_METHOD_CG, 2, 0, 0.0);
    if (std::string msg; !shape_ok(rq, msg)) return fail(TFLOWS_BAD_INPUT, msg);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = build_levels(topo->t);
    if (e == cudaSuccess) e = ensure_workspace(topo->ws, topo->t);
    if (e == cudaSuccess) e = permute_values(topo->t, topo->ws, val, true, false, s);
    if (e != cudaSuccess) return cuda_fail(e, "ic apply");
    SolveReport rep;
    const int st = run_ic_apply(topo->t, topo->ws, rq, r, z, s, rep);
    record(rep, res);
    if (st != TFLOWS_OK) return fail(st, rep.message);
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

int tflows_spmv_device(tflows_topology* topo, const double* val, const double* x, double* y,
                       int repeat, int fp32, void* stream, double* sec) {
    if (!topo || !val || !x || !y) return fail(TFLOWS_BAD_INPUT, "null argument");
    std::lock_guard<std::mutex> lk(topo->mu);
    cudaSetDevice(topo->t.device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = ensure_workspace(topo->ws, topo->t);
    if (e == cudaSuccess) e = permute_values(topo->t, topo->ws, val, true, fp32 != 0, s);
    float ms = 0.f;
    if (e == cudaSuccess) e = run_spmv(topo->t, topo->ws, x, y, fp32 != 0, repeat, s, &ms);
    if (e != cudaSuccess) return cuda_fail(e, "spmv");
    if (sec) *sec = ms * 1e-3 / std::max(1, repeat);
    t_status = TFLOWS_OK;
    return TFLOWS_OK;
}

}  // extern "C"
