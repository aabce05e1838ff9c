// tflows_cg_noalloc: a CG solve (Jacobi or no preconditioning) that
// allocates no device memory.
//
// Who needs it: code that must not call cudaMalloc while it runs -- a time
// loop whose GPU memory is reserved up front by another allocator (for
// example PyTorch's caching allocator holding the whole device), hosts with
// a fixed memory budget that forbid allocation after start-up, or callers
// that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
// imply.  Such callers hand in only their own inputs and outputs; every
// work vector lives in one file-scope __device__ array below.
//
// Limits and sharing rules:
//   * at most kMaxRows (262144) rows, i.e. 64^3 cells; larger systems are
//     rejected with TFLOWS_BAD_INPUT;
//   * the array (about 10.2 MB) exists on every GPU that loads the library
//     until the process exits;
//   * all calls share it and it keeps the last call's contents; calls whose
//     kernels overlap on the GPU (different streams or threads at once)
//     race on it and must not be issued;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before capturing any stream.  The lookup is repeated when the device's
//     context has changed since (after cudaDeviceReset, for example);
//   * every call waits for its stream to finish before it returns (it reads
//     the status record back);
//   * the pattern is checked on the device (row pointers from 0, never
//     decreasing; columns in [0, n); diagonal positions inside their rows):
//     TFLOWS_BAD_INPUT, with nothing written to x or r_out.
#include "../../include/tflows_krylov.h"
#include "device_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <mutex>

namespace tflows {
namespace {

constexpr int kNaBlock = 256;
constexpr int kMaxRows = 262144;
constexpr int kMaxBlocks = 1024;
constexpr int kNaSlots = 8;
constexpr size_t kCtlBytes = 256;    // DevCtl, padded
constexpr size_t kStateBytes = 256;  // DevState, padded
constexpr size_t kPartialBytes = sizeof(double) * kNaSlots * kMaxBlocks;
constexpr int kNaVecs = 5;           // r (when no r_out), p, q, z, D
constexpr size_t kScratchBytes =
    kCtlBytes + kStateBytes + kPartialBytes + sizeof(double) * kNaVecs * (size_t)kMaxRows;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct NaParams {
    int n, prec, maxiter;
    double tol;
    long long timeout_cyc;
    const int* rowptr;
    const int* col;
    const int* diag;
    const double* val;
    const double* b;
    double* x;
    double* r;
    double *p, *q, *z, *D;
    DevCtl* ctl;
    DevState* state;
    double* partials;
};

// CG of Process/CG.f90 on a plain 0-based compressed-row matrix, one thread
// per row, same per-row operation order as the reference loops.
__global__ void __launch_bounds__(kNaBlock) noalloc_cg_kernel(NaParams P) {
    Grid g;
    grid_init(g, P.ctl, P.partials, P.timeout_cyc);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    const int n = P.n;
    const int prec = P.prec == 1 ? 1 : 0;
    int exit_kind = EXIT_ABORT, iterations = 0;
    double ini = 0.0, err = 0.0;

    // The caller's pattern, checked before any vector is indexed through it:
    // row pointers start at 0 and never decrease, every column lies in
    // [0, n), and (prec 1) every diagonal position lies inside its row.  A
    // bad row raises BAD_INPUT and skips the loads that depend on it; the
    // barrier then makes the flag visible to every block before the first
    // gather.  (rowptr[n] itself must not exceed the length of col and val:
    // the call has no way to know that length.)
    for (int i = tid; i < n; i += nt) {
        const int j0 = P.rowptr[i], j1 = P.rowptr[i + 1];
        bool bad = j0 < 0 || j1 < j0 || (i == 0 && j0 != 0);
        for (int j = j0; !bad && j < j1; ++j) {
            const int c = P.col[j];
            bad = c < 0 || c >= n;
        }
        if (!bad && prec == 1) {
            const int d = P.diag[i];
            bad = d < j0 || d >= j1;
        }
        if (bad) raise_abort(P.ctl, ST_BAD_INPUT, 95);
    }
    double a1[1];  // (declared before the jump, initialised after it)
    if (!grid_sync(g, 96)) goto done;

    // Prec1 (diag or 1), r = b, ||b||
    a1[0] = 0.0;
    for (int i = tid; i < n; i += nt) {
        P.D[i] = prec == 1 ? P.val[P.diag[i]] : 1.0;
        const double bi = P.b[i];
        P.r[i] = bi;
        a1[0] += bi * bi;
    }
    publish<1>(g, 0, a1);
    if (!grid_sync(g, 90)) goto done;
    {
        double t[1];
        totals<1>(g, 0, t);
        if (sqrt(t[0]) < P.tol) {
            exit_kind = EXIT_BNRM;
            goto done;
        }
    }
    // Resid: r_i = r_i - a_i1 x_1 - ...; error; z = r/D; rho
    {
        double a2[2] = {0.0, 0.0};
        for (int i = tid; i < n; i += nt) {
            double ri = P.r[i];
            for (int j = P.rowptr[i]; j < P.rowptr[i + 1]; ++j) ri = ri - P.val[j] * P.x[P.col[j]];
            P.r[i] = ri;
            a2[0] += ri * ri;
            if (prec == 1) {
                const double zi = ri / P.D[i];
                P.z[i] = zi;
                a2[1] += ri * zi;
            }
        }
        publish<2>(g, 1, a2);
        if (!grid_sync(g, 91)) goto done;
        double t[2];
        totals<2>(g, 1, t);
        err = sqrt(t[0]);
        ini = err;
        if (err < P.tol) {
            exit_kind = EXIT_INIRES;
            goto done;
        }
        double rho_next = prec == 1 ? t[1] : t[0], rho = 0.0, rhoold = 0.0;
        const double* z = prec == 1 ? P.z : P.r;
        bool nonfinite = false;
        int iter = 1;
        for (; iter <= P.maxiter; ++iter) {
            rho = rho_next;
            if (iter == 1) {
                for (int i = tid; i < n; i += nt) P.p[i] = z[i];
            } else {
                const double beta = rho / rhoold;
                for (int i = tid; i < n; i += nt) P.p[i] = z[i] + beta * P.p[i];
            }
            if (!grid_sync(g, 92)) goto done;
            double a3[1] = {0.0};
            for (int i = tid; i < n; i += nt) {
                double qi = 0.0;
                for (int j = P.rowptr[i]; j < P.rowptr[i + 1]; ++j) qi = qi + P.val[j] * P.p[P.col[j]];
                P.q[i] = qi;
                a3[0] += P.p[i] * qi;
            }
            publish<1>(g, 3, a3);
            if (!grid_sync(g, 93)) goto done;
            double t3[1];
            totals<1>(g, 3, t3);
            const double alfa = rho / t3[0];
            double a4[3] = {0.0, 0.0, 0.0};
            for (int i = tid; i < n; i += nt) {
                const double xi = P.x[i] + alfa * P.p[i];
                const double ri = P.r[i] - alfa * P.q[i];
                P.x[i] = xi;
                P.r[i] = ri;
                a4[0] += ri * ri;
                if (prec == 1) {
                    const double zi = ri / P.D[i];
                    P.z[i] = zi;
                    a4[1] += ri * zi;
                }
                if (nonfinite) a4[2] += (xi == xi ? 1.0 : 0.0) + (ri == ri ? 1.0 : 0.0);
            }
            publish<3>(g, 4, a4);
            if (!grid_sync(g, 94)) goto done;
            double t4[3];
            totals<3>(g, 4, t4);
            err = sqrt(t4[0]);
            if (err < P.tol) {
                exit_kind = EXIT_CONVERGED;
                iterations = iter;
                goto done;
            }
            rho_next = prec == 1 ? t4[1] : t4[0];
            if (!isfinite(err)) {
                if (nonfinite && t4[2] == 0.0) {
                    exit_kind = EXIT_NONFINITE;
                    iterations = P.maxiter + 1;
                    goto done;
                }
                nonfinite = true;
            }
            rhoold = rho;
        }
        exit_kind = EXIT_MAXITER;
        iterations = iter;
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        DevState* s = P.state;
        int st = P.ctl->status;
        if (st == 0) {
            if (exit_kind == EXIT_MAXITER) st = isfinite(err) ? ST_NOT_CONVERGED : ST_NONFINITE;
            else if (exit_kind == EXIT_NONFINITE) st = ST_NONFINITE;
            else if (exit_kind == EXIT_ABORT) st = ST_TIMEOUT;
        }
        s->status = st;
        s->exit_kind = exit_kind;
        s->iterations = iterations;
        s->ini_res = ini;
        s->fin_res = err;
    }
}

// Device address of the scratch array, looked up once per device and
// remembered together with the identity of the context it was looked up in:
// after cudaDeviceReset (or the release of the primary context) the device
// gets a new context with a new copy of the array, and the address is looked
// up again.  The context identity comes from the driver (cuCtxGetCurrent,
// cuCtxGetId), reached through the runtime's entry-point query so the
// library needs no link against libcuda.
struct AddrEntry {
    unsigned long long ctx_id;  // 0: not looked up yet
    void* ptr;
};
std::mutex g_addr_mu;
AddrEntry g_addr[64] = {};
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// Identity of the calling thread's current context (0 when there is none or
// the driver cannot tell).  Call with g_addr_mu held.
unsigned long long current_context_id() {
    if (!g_ctx_fns_tried) {
        g_ctx_fns_tried = true;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&g_ctx_current, 4000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            g_ctx_current = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&g_ctx_id, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            g_ctx_id = nullptr;
    }
    if (!g_ctx_current || !g_ctx_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace
}  // namespace tflows

extern "C" int tflows_cg_noalloc(int n, const int* rowptr, const int* col, const int* diag,
                                 const double* val, const double* b, double* x, double* r_out,
                                 int prec, int maxiter, double tol, void* stream, int* iterations,
                                 double* ini_res, double* fin_res) {
    using namespace tflows;
    if (n < 1 || n > kMaxRows) return TFLOWS_BAD_INPUT;
    if (!rowptr || !col || !val || !b || !x || !iterations || !ini_res || !fin_res)
        return TFLOWS_BAD_INPUT;
    if (prec == 2) return TFLOWS_UNSUPPORTED;
    if (prec == 1 && !diag) return TFLOWS_BAD_INPUT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TFLOWS_NO_DEVICE;
    unsigned char* base = nullptr;
    {
        // Set-up, once per device (and again after that device's context
        // was replaced), with the device current: the host-side name
        // g_noalloc_scratch is not a device address, so the kernel gets the
        // address the runtime reports for it.
        std::lock_guard<std::mutex> lk(g_addr_mu);
        AddrEntry& e = g_addr[dev];
        const unsigned long long id = current_context_id();
        if (!e.ptr || id == 0 || id != e.ctx_id) {
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr)
                return TFLOWS_CUDA_ERROR;
            e.ptr = ptr;
            // the lookup above made the runtime's context current if none was
            e.ctx_id = id != 0 ? id : current_context_id();
        }
        base = static_cast<unsigned char*>(e.ptr);
    }
    NaParams P;
    P.n = n;
    P.prec = prec;
    P.maxiter = maxiter;
    P.tol = tol;
    int khz = 0;
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
    P.timeout_cyc = 5LL * (khz > 0 ? khz : 2100000) * 1000LL;  // 5 s of SM cycles
    P.rowptr = rowptr;
    P.col = col;
    P.diag = diag;
    P.val = val;
    P.b = b;
    P.x = x;
    P.ctl = reinterpret_cast<DevCtl*>(base);
    P.state = reinterpret_cast<DevState*>(base + kCtlBytes);
    P.partials = reinterpret_cast<double*>(base + kCtlBytes + kStateBytes);
    double* vec = reinterpret_cast<double*>(base + kCtlBytes + kStateBytes + kPartialBytes);
    P.p = vec;
    P.q = vec + kMaxRows;
    P.z = vec + 2 * (size_t)kMaxRows;
    P.D = vec + 3 * (size_t)kMaxRows;
    P.r = r_out ? r_out : vec + 4 * (size_t)kMaxRows;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The barrier counter, abort flag and status must start at zero.
    if (cudaMemsetAsync(P.ctl, 0, sizeof(DevCtl), s) != cudaSuccess) return TFLOWS_CUDA_ERROR;
    int per_sm = 0, sm_count = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, noalloc_cg_kernel, kNaBlock, 0);
    cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    int grid = (n + kNaBlock - 1) / kNaBlock;
    grid = std::max(1, std::min({grid, std::max(1, per_sm) * sm_count, kMaxBlocks}));
    void* args[] = {&P};
    if (cudaLaunchCooperativeKernel((const void*)noalloc_cg_kernel, dim3(grid), dim3(kNaBlock),
                                    args, 0, s) != cudaSuccess)
        return TFLOWS_CUDA_ERROR;
    DevState st;
    if (cudaMemcpyAsync(&st, P.state, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TFLOWS_CUDA_ERROR;
    *iterations = st.iterations;
    if (st.exit_kind != EXIT_BNRM) {
        *ini_res = st.ini_res;
        *fin_res = st.fin_res;
    }
    return st.status;
}
