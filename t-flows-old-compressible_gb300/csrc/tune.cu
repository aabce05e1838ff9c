// Launch-shape autotuner of libtflows_krylov.so.
//
// The persistent solvers have three launch parameters that trade parallelism
// against synchronisation cost and whose best values depend on the system
// size, the method and the precision:
//   * threads per block (128, 256 or 512; the kernels are compiled for up to
//     512 with the register budget of four 256-thread blocks per SM);
//   * rows per warp, which sets the grid: a small system spread over few
//     blocks pays less per grid barrier, a large one wants every SM;
//   * for IC(0), the warps per chunk of the widest wavefront level that take
//     part in the sync-free sweeps.
// tune_solve times candidate shapes on the caller's own system (a capped
// number of iterations from x0 = 0) and keeps the fastest per iteration in a
// process-wide table keyed by device, method, preconditioner, precision
// options and size class; the table can be kept in a text file.  tune_batch
// sizes the block groups of a batched launch from each system's measured
// solve time (the launch ends when its slowest group does).
#include "internal.h"
#include "tflows_krylov.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>

namespace tflows {

namespace {

using Key = std::tuple<std::string, int, int, int, int, int, int, int, int>;

struct Table {
    std::mutex mu;
    std::map<Key, TuneChoice> entries;
    bool loaded = false;
};

Table& table() {
    static Table* t = new Table();
    return *t;
}

// Device name and SM count, looked up once per device (the property query is
// far too slow to repeat on every solve that consults the table).
std::string device_tag(int device) {
    static std::mutex mu;
    static std::map<int, std::string> tags;
    std::lock_guard<std::mutex> lk(mu);
    auto it = tags.find(device);
    if (it != tags.end()) return it->second;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "unknown";
    std::string name = p.name;
    for (char& c : name)
        if (c == ' ') c = '_';
    return tags[device] = name + "/" + std::to_string(p.multiProcessorCount);
}

// Size class: quarter octaves of the row count, half entries per row.
Key make_key(const DeviceTopology& t, const SolveRequest& rq) {
    const int nclass = (int)std::floor(4.0 * std::log2(std::max(1, t.n)));
    const int rclass = (int)std::lround(2.0 * t.nnz / std::max(1, t.n));
    const int method = rq.method == 1 ? 0 : rq.method;
    const int prec = (rq.prec == 1 || rq.prec == 2) ? rq.prec : 0;
    const int variant = (rq.precision == 1 ? (rq.refine_restart ? 1 : 2) + 4 * rq.ic_bf16 : 0) +
                        8 * (tiled_ic(t, rq) ? 1 : 0);
    return Key(device_tag(t.device), rq.precision, method, prec, rq.ic_sweeps, variant, nclass,
               rclass, 0);
}

const char* table_path() {
    const char* p = std::getenv("TFLOWS_TUNE_FILE");
    return p && *p ? p : nullptr;
}

// One line per entry: the key fields, then block rows_per_warp sweep_mult
// sweep_gate and the measured microseconds per iteration.
void load_file(Table& T) {
    T.loaded = true;
    const char* path = table_path();
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char dev[256];
    int a, b, c, d, e, g, h, i, blk, rpw, sm, gate;
    double us;
    while (std::fscanf(f, "%255s %d %d %d %d %d %d %d %d %d %d %d %d %lf", dev, &a, &b, &c, &d,
                       &e, &g, &h, &i, &blk, &rpw, &sm, &gate, &us) == 14) {
        TuneChoice ch;
        ch.block = blk;
        ch.rows_per_warp = rpw;
        ch.sweep_mult = sm;
        ch.sweep_gate = gate;
        ch.us_per_iter = us;
        T.entries[Key(dev, a, b, c, d, e, g, h, i)] = ch;
    }
    std::fclose(f);
}

void append_file(const Key& k, const TuneChoice& ch) {
    const char* path = table_path();
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %d %d %d %d %d %d %d %d %d %d %.6g\n", std::get<0>(k).c_str(),
                 std::get<1>(k), std::get<2>(k), std::get<3>(k), std::get<4>(k), std::get<5>(k),
                 std::get<6>(k), std::get<7>(k), std::get<8>(k), ch.block, ch.rows_per_warp,
                 ch.sweep_mult, ch.sweep_gate, ch.us_per_iter);
    std::fclose(f);
}

// Microseconds per iteration of one capped solve from x0 = 0 (best of two).
int time_shape(const DeviceTopology& t, Workspace& ws, const SolveRequest& base, const double* b,
               int block, int rpw, int sweep_mult, int sweep_gate, cudaStream_t s, double& us,
               int& grid, std::string& msg) {
    SolveRequest rq = base;
    rq.block = block;
    rq.rows_per_warp = rpw;
    rq.grid = 0;
    rq.sweep_mult = sweep_mult;
    rq.sweep_gate = sweep_gate;
    rq.tol = 1e-30;  // relative: never reached within the cap
    rq.tol_relative = 1;
    rq.x_is_zero = 1;
    rq.maxiter = rq.precision == 1 ? 60 : 30;
    rq.inject_stall = 0;
    double* X = ws.vec64 + 11 * ws.vec_cap;
    double* R = ws.vec64 + 12 * ws.vec_cap;
    us = 1e300;
    for (int rep = 0; rep < 2; ++rep) {
        cudaError_t e = cudaMemsetAsync(X, 0, sizeof(double) * t.n, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(R, b, sizeof(double) * t.n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) {
            msg = std::string("tuning: ") + cudaGetErrorString(e);
            return TFLOWS_CUDA_ERROR;
        }
        SolveReport r;
        const int st = run_solve(t, ws, rq, X, R, s, r);
        if (st == TFLOWS_CUDA_ERROR || st == TFLOWS_TIMEOUT || st == TFLOWS_BAD_INPUT) {
            msg = "tuning: " + r.message;
            return st;
        }
        const int its = rq.precision == 1 ? r.inner_iterations : std::min(r.iterations, rq.maxiter);
        us = std::min(us, 1e6 * r.seconds / std::max(1, its));
        grid = r.grid;
    }
    return TFLOWS_OK;
}

}  // namespace

bool tune_lookup(const DeviceTopology& t, const SolveRequest& rq, TuneChoice& out) {
    Table& T = table();
    std::lock_guard<std::mutex> lk(T.mu);
    if (!T.loaded) load_file(T);
    auto it = T.entries.find(make_key(t, rq));
    if (it == T.entries.end()) return false;
    out = it->second;
    out.from_cache = 1;
    return true;
}

void tune_apply(const TuneChoice& ch, SolveRequest& rq) {
    rq.block = ch.block;
    rq.rows_per_warp = ch.rows_per_warp;
    rq.sweep_mult = ch.sweep_mult;
    rq.sweep_gate = ch.sweep_gate;
    rq.grid = 0;
}

int tune_solve(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, const double* b,
               cudaStream_t s, TuneChoice& out, std::string& msg) {
    static const int kBlocks[] = {256, 128, 512};
    static const int kRows[] = {0, 128, 512, 2048};
    TuneChoice best;
    best.us_per_iter = 1e300;
    int count = 0;
    std::vector<std::pair<int, int>> seen;  // (block, grid) already timed
    for (int blk : kBlocks)
        for (int rpw : kRows) {
            // shapes that give the same grid (co-residency clamps large
            // systems) are timed once
            SolveRequest probe = rq;
            probe.block = blk;
            probe.rows_per_warp = rpw;
            probe.grid = 0;
            const int want = planned_grid(t, probe);
            if (std::find(seen.begin(), seen.end(), std::make_pair(blk, want)) != seen.end())
                continue;
            seen.emplace_back(blk, want);
            double us = 0.0;
            int grid = 0;
            const int st = time_shape(t, ws, rq, b, blk, rpw, 0, rq.sweep_gate, s, us, grid, msg);
            if (st != TFLOWS_OK) return st;
            ++count;
            if (blk == 256 && rpw == 0) out.default_us_per_iter = us;
            if (us < best.us_per_iter) {
                best.block = blk;
                best.rows_per_warp = rpw;
                best.grid = grid;
                best.us_per_iter = us;
            }
        }
    if (rq.prec == 2 && rq.ic_sweeps == 0 && !tiled_ic(t, rq)) {
        for (int sm : {2, 8}) {
            double us = 0.0;
            int grid = 0;
            const int st = time_shape(t, ws, rq, b, best.block, best.rows_per_warp, sm,
                                      rq.sweep_gate, s, us, grid, msg);
            if (st != TFLOWS_OK) return st;
            ++count;
            if (us < best.us_per_iter) {
                best.sweep_mult = sm;
                best.us_per_iter = us;
            }
        }
        // gated polling on and off (it pays on large systems, where
        // thousands of warps wait)
        for (int gate : {0, 1}) {
            double us = 0.0;
            int grid = 0;
            const int st = time_shape(t, ws, rq, b, best.block, best.rows_per_warp,
                                      best.sweep_mult, gate, s, us, grid, msg);
            if (st != TFLOWS_OK) return st;
            ++count;
            if (us < best.us_per_iter) {
                best.sweep_gate = gate;
                best.us_per_iter = us;
            }
        }
    }
    best.default_us_per_iter = out.default_us_per_iter;
    best.candidates = count;
    best.from_cache = 0;
    out = best;
    Table& T = table();
    std::lock_guard<std::mutex> lk(T.mu);
    if (!T.loaded) load_file(T);
    const Key k = make_key(t, rq);
    T.entries[k] = best;
    append_file(k, best);
    return TFLOWS_OK;
}

void tune_clear() {
    Table& T = table();
    std::lock_guard<std::mutex> lk(T.mu);
    T.entries.clear();
    T.loaded = false;  // the next lookup reads TFLOWS_TUNE_FILE again
}

int tune_batch(std::vector<BatchSpec>& specs, const std::function<cudaError_t()>& restage,
               cudaStream_t s, BatchTuning& out, std::string& msg) {
    const int count = (int)specs.size();
    std::vector<double> w(count), best_w(count);
    for (int k = 0; k < count; ++k) w[k] = std::pow((double)specs[k].t->n, 4.0 / 3.0);
    out.default_seconds = 0.0;
    out.tuned_seconds = 1e300;
    out.runs = 0;
    int best_block = 256;
    auto run = [&](int block, const std::vector<double>& weights, double& sec) -> int {
        for (int k = 0; k < count; ++k) {
            specs[k].rq.block = block;
            specs[k].rq.grid = 0;
            specs[k].weight = weights[k];
        }
        cudaError_t e = restage();
        if (e != cudaSuccess) {
            msg = std::string("batch tuning: ") + cudaGetErrorString(e);
            return TFLOWS_CUDA_ERROR;
        }
        const int st = run_batch(specs, s, &sec);
        ++out.runs;
        if (st == TFLOWS_CUDA_ERROR || st == TFLOWS_TIMEOUT || st == TFLOWS_BAD_INPUT) {
            for (auto& sp : specs)
                if (!sp.rep->message.empty()) msg = "batch tuning: " + sp.rep->message;
            return st;
        }
        return TFLOWS_OK;
    };
    // 256 threads: the N^(4/3) split, then two rebalancing passes that give
    // each system blocks in proportion to its measured work (its own solve
    // time times the blocks it had).
    for (int pass = 0; pass < 3; ++pass) {
        double sec = 0.0;
        const int st = run(256, w, sec);
        if (st != TFLOWS_OK) return st;
        if (pass == 0) out.default_seconds = sec;
        if (sec < out.tuned_seconds) {
            out.tuned_seconds = sec;
            best_w = w;
        }
        double tot = 0.0;
        for (int k = 0; k < count; ++k) {
            const SolveReport& r = *specs[k].rep;
            w[k] = std::max(r.group_seconds, 1e-7) * std::max(1, r.grid);
            tot += w[k];
        }
        if (tot <= 0.0) break;
    }
    for (int block : {512, 128}) {
        double sec = 0.0;
        const int st = run(block, best_w, sec);
        if (st != TFLOWS_OK) return st;
        if (sec < out.tuned_seconds) {
            out.tuned_seconds = sec;
            best_block = block;
        }
    }
    for (int k = 0; k < count; ++k) {
        specs[k].rq.block = best_block;
        specs[k].rq.grid = 0;
        specs[k].weight = best_w[k];
    }
    out.block = best_block;
    return TFLOWS_OK;
}

}  // namespace tflows
