// Internal host-side interfaces of libtflows_krylov.so (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace tflows {

// A compressed-row pattern resident on one device, in SELL-32 form plus the
// wavefront orders the IC(0) sweeps need.
struct DeviceTopology {
    int device = 0;
    int n = 0;
    int nnz = 0;
    int nslices = 0;
    long long sell_len = 0;
    int max_len = 0;
    bool ic_ok = false;        // lower part = slots before the diagonal, ascending
    bool levels_built = false;
    bool tsym = false;         // every entry has its transpose (valid once tpos exists)
    int nlev_f = 0, nlev_b = 0;
    int nchunk_f = 0, nchunk_b = 0;
    int wide_f = 0, wide_b = 0;  // chunks in the widest level
    // device arrays
    int* rowptr = nullptr;     // 0-based, n + 1
    int* col = nullptr;        // 0-based, nnz
    long long* soff = nullptr; // nslices + 1
    int* scol = nullptr;       // sell_len
    // column patterns (see build_patterns): one id per row (32 * nslices),
    // 8 offsets per pattern; null when the rows have too many patterns
    unsigned char* spat = nullptr;
    int* poff = nullptr;
    int npat = 0;
    int* meta = nullptr;       // n: length | diag slot << 16
    int* perm_f = nullptr;
    int* perm_b = nullptr;
    int* tpos = nullptr;       // transpose map (lazy)
    // box numbering (0 = not a box): row = x + nx (y + ny z), each row holding
    // exactly its 7-point neighbours in ascending order (what TopolM builds
    // for a structured block); enables the tiled IC sweeps
    int box_nx = 0, box_ny = 0, box_nz = 0;
    // host copies (0-based) for lazy derived data
    std::vector<int> h_rowptr, h_col, h_diag;
};

// Device buffers reused across solves of one context.
struct Workspace {
    int device = -1;
    size_t vec_cap = 0;        // elements per vector (padded n)
    size_t sell_cap = 0;       // SELL elements
    int part_cap = 0;          // blocks
    double* sval64 = nullptr;
    float* sval32 = nullptr;
    double* svalT64 = nullptr;  // A^T values (true BiCG), allocated on first use
    unsigned short* sval16 = nullptr;  // BF16 values for the IC sweeps (ensure_lu16)
    double* vec64 = nullptr;   // kVecs vectors of vec_cap doubles
    float* vec32 = nullptr;    // kVecs vectors of vec_cap floats
    double* csr_val = nullptr; // staging for host values (nnz)
    size_t csr_cap = 0;
    double* partials = nullptr;
    void* ctl = nullptr;       // DevCtl
    void* state = nullptr;     // DevState
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // step records and cells of the tiled IC sweeps, per working precision
    unsigned char* tile64 = nullptr;
    unsigned char* tile32 = nullptr;
    size_t tile_cap64 = 0, tile_cap32 = 0;  // bytes
};
constexpr int kVecs = 14;

struct SolveRequest {
    int method = 0;     // 0 CG, 1 BiCG, 2 CGS, 3 true BiCG
    int prec = 0;
    int precision = 0;  // 0 FP64, 1 mixed
    int maxiter = 0;
    double tol = 0.0;
    int tol_relative = 0;
    int x_is_zero = 0;
    double inner_rtol = 1e-4;
    int inner_maxiter = 1000;
    int max_refinements = 30;
    int ic_sweeps = 0;
    int ic_bf16 = 0;
    int refine_restart = 0;
    int inject_stall = 0;
    double timeout_s = 5.0;
    int block = 0;          // threads per block (0 = 256)
    int grid = 0;           // persistent blocks (0 = from rows_per_warp)
    int rows_per_warp = 0;  // rows each warp owns (0 = one 32-row slice)
    int sweep_mult = 0;     // IC sweep warps per chunk of the widest level (0 = 4)
    int sweep_gate = -1;    // IC sweeps: gated polling 1 / 0, -1 = process default
    int autotune = 0;       // take block/rows_per_warp/sweep_mult from the tuner
    int ic_tiled = -1;      // exact IC on a box pattern: 1 tiled sweeps, 0 level
                            // sweeps, -1 tiled unless TFLOWS_IC_TILED=0
};

struct SolveReport {
    int status = 0;
    int exit_kind = 0;
    int iterations = 0;
    int inner_iterations = 0;
    int refinements = 0;
    double ini_res = 0.0;
    double fin_res = 0.0;
    double seconds = 0.0;
    double bytes = 0.0;
    int block = 0;              // launch shape used
    int grid = 0;               // blocks (batched: blocks of this system's group)
    double group_seconds = 0.0; // batched: this system's own solve time
    std::string message;
};

// One system of a batched launch.
struct BatchSpec {
    const DeviceTopology* t;
    Workspace* ws;
    SolveRequest rq;
    double* x;  // workspace x (slot 11), in/out
    double* r;  // workspace residual (slot 12), holds b on entry
    SolveReport* rep;
    double weight = 0.0;  // share of the launch's blocks (0 = N^(4/3))
};

// krylov.cu
cudaError_t ensure_workspace(Workspace& ws, const DeviceTopology& t);
void free_workspace(Workspace& ws);
// Values (nnz FP64, stored order, device) -> SELL values (FP64 and/or FP32).
cudaError_t permute_values(const DeviceTopology& t, Workspace& ws, const double* csr_val,
                           bool want64, bool want32, cudaStream_t s, bool want16 = false);
// The BF16 value array of the IC sweeps (allocated once; call before a capture).
cudaError_t ensure_lu16(Workspace& ws);
// A^T values in A's pattern into ws.svalT64 (needs t.tpos).
cudaError_t permute_transposed(const DeviceTopology& t, Workspace& ws, const double* csr_val,
                               cudaStream_t s);
// Runs a full solve. x (n) and r (n, holds b on entry) are device FP64 arrays.
int run_solve(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, double* x, double* r,
              cudaStream_t s, SolveReport& rep);
// The IC(0) pivots and one apply z = M^-1 r in FP64 (reference or contracted
// arithmetic per rq.precision; tiled or level sweeps per rq.ic_tiled).
int run_ic_apply(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, const double* r,
                 double* z, cudaStream_t s, SolveReport& rep);
// Prec1 only: D (n, device FP64).
int run_prec1(const DeviceTopology& t, Workspace& ws, int prec, double* D, double timeout_s,
              cudaStream_t s, SolveReport& rep);
// r <- r - A x (Resid), device arrays.
// All systems in one cooperative launch (block groups sized by expected work).
int run_batch(std::vector<BatchSpec>& specs, cudaStream_t s, double* seconds);
// The same split into a capturable enqueue (parameters, launch, result
// records into pinned memory) and a collect step (synchronise, reports).
struct BatchLaunch;
BatchLaunch* batch_create();
void batch_destroy(BatchLaunch* L);
// Allocate the launch buffers for `count` systems up front (before a capture).
cudaError_t batch_reserve(BatchLaunch* L, int count, int block = 0);
int batch_enqueue(BatchLaunch* L, std::vector<BatchSpec>& specs, cudaStream_t s);
int batch_collect(BatchLaunch* L, std::vector<BatchSpec>& specs, cudaStream_t s, double seconds);
cudaError_t run_resid(const DeviceTopology& t, Workspace& ws, const double* x, double* r,
                      cudaStream_t s);
// The grid a solve with this request would launch (co-residency included).
int planned_grid(const DeviceTopology& t, const SolveRequest& rq);
// Tiled IC sweeps: whether this request runs them, the dynamic shared memory
// a launch needs for them, and their step records (allocated here, so call
// before a stream capture).
bool tiled_ic(const DeviceTopology& t, const SolveRequest& rq);
unsigned tile_smem_for(const DeviceTopology& t, const SolveRequest& rq);
cudaError_t ensure_tiles(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq);
cudaError_t run_spmv(const DeviceTopology& t, Workspace& ws, const double* x, double* y, bool fp32,
                     int repeat, cudaStream_t s, float* ms);
cudaError_t run_pattern_outer(const DeviceTopology& t, const double* lambda, const double* x,
                              double* g, cudaStream_t s);

// Records the status and message tflows_last_status / tflows_last_error report.
int report_status(int status, const std::string& msg);
// The legacy topology cache's key hash of a 1-based pattern (about 8k
// samples per array; every element with TFLOWS_TOPOLOGY_CHECK=full).
unsigned long long legacy_pattern_hash(int n, int nnz, const int* Acol, const int* Arow,
                                       const int* Adia);
// Host-time phase mark of a legacy call run with TFLOWS_TRACE_LEGACY set.
void trace_mark(const char* what);

// Subdomain-coupled solves (halo.cu): whether a halo is registered, the
// coupled solve of the Fortran-facing entry points and the coupled Resid.
bool halo_registered();
void halo_release();  // frees the coupled solves' buffers, keeps the registration
int halo_solve(int method, int n, int nb, int nonz, const double* A, const int* Acol,
               const int* Arow, const int* Adia, const double* Ab, double* x, double* r1,
               int prec, int* niter, double tol, double* IniRes, double* FinRes,
               double& error_state, cudaStream_t s, SolveReport& rep);
int halo_resid(int n, int nb, int nonz, const double* A, const int* Acol, const int* Arow,
               const double* Ab, const double* x, double* r1, cudaStream_t s, std::string& msg);

// The persistent kernels, built twice: krylov.cu with the reference's
// arithmetic (separate rounded products and sums, dividing diagonal) and
// krylov_fma.cu with fused multiply-adds (TFLOWS_FP64_FMA and mixed solves).
enum class KernelId { Cg, Cgs, BicgTrue, Prec1, IcApply, MixedRestart, MixedReliable, MixedCgs,
                      BatchFp64, BatchMixed };
const void* ref_kernel(KernelId id);
const void* fma_kernel(KernelId id);

// tune.cu: launch-shape autotuner.
struct TuneChoice {
    int block = 256;
    int rows_per_warp = 0;
    int grid = 0;
    int sweep_mult = 0;
    int sweep_gate = -1;
    int candidates = 0;
    int from_cache = 0;
    double us_per_iter = 0.0;
    double default_us_per_iter = 0.0;
};
struct BatchTuning {
    int block = 256;
    int runs = 0;
    double default_seconds = 0.0;
    double tuned_seconds = 0.0;
};
// The table's entry for this system class, if any.
bool tune_lookup(const DeviceTopology& t, const SolveRequest& rq, TuneChoice& out);
void tune_apply(const TuneChoice& ch, SolveRequest& rq);
// Times candidate shapes on this system (values already in ws, b on the
// device); uses workspace slots 11 and 12; stores the winner in the table.
int tune_solve(const DeviceTopology& t, Workspace& ws, const SolveRequest& rq, const double* b,
               cudaStream_t s, TuneChoice& out, std::string& msg);
void tune_clear();
// Block size and group sizes of a batched launch from measured per-system
// times; `restage` re-queues each system's x0 and b before every run.
int tune_batch(std::vector<BatchSpec>& specs, const std::function<cudaError_t()>& restage,
               cudaStream_t s, BatchTuning& out, std::string& msg);

}  // namespace tflows
