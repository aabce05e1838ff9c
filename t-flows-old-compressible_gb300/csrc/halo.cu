// Subdomain-coupled (halo) solves for the Fortran-facing entry points.
//
// A caller running T-FlowS on several ranks (Npro > 0) solves its own
// subdomain's rows on its GPU; the rows next to another subdomain carry
// couplings Ab(k) to buffer cells k (negative indices of x(-NB:N)) whose
// values live on the neighbouring rank.  The reference couples the ranks in
// three places:
//   * after every product q = A p: Exchng(p) fills p's buffer cells with the
//     neighbours' values (Parallel/Double/Exchng.f90:26-62) and
//     q(BufInd(k)) += Ab(k) p(k) adds them (CG.f90:200-208,
//     BiCG.f90:202-211, CGS.f90:201-208 and :301-308);
//   * after every inner product and norm: glosum sums it over the ranks
//     (Parallel/Double/GloSum.f90);
//   * in Resid: r(BufInd(k)) -= Ab(k) x(k) with x's buffer cells as the
//     caller left them (Resid.f90:36-42, no exchange).
// The transport is the caller's (MPI in T-FlowS): it registers the halo maps
// of par_mod (BufLoa.f90:35-84) and two callbacks with tflows_set_halo.
//
// The solve runs on the device in reference arithmetic (this unit is
// compiled without contraction): the product sums each row in stored order
// from 0.0, the halo terms follow it row by row in the reference's order
// (neighbour ascending, buffer cell descending), the IC(0) apply is the
// library's exact apply (bit-identical to the sequential sweeps), and the
// vector updates round as the reference's statements do.  Local inner
// products are reduced on the device by a fixed tree, then summed over the
// ranks by the caller.  The iteration is driven from the host: every
// exchange and every global sum is a host round trip, which a multi-rank
// solve needs anyway; no kernel waits on another rank.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tflows_krylov.h"
#include "device_common.cuh"
#include "internal.h"

namespace tflows {
namespace {

constexpr int kThreads = 256;
constexpr int kDotBlocks = 1024;

// ---- kernels (reference arithmetic: no fused multiply-add in this unit) -----------

// q(i) = sum_j A(j) p(Arow(j)) in stored order from 0.0 (CG.f90:193-199);
// 1-based acol / arow as the caller stores them.
__global__ void k_spmv(int n, const int* __restrict__ acol, const int* __restrict__ arow,
                       const double* __restrict__ a, const double* __restrict__ p,
                       double* __restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int j = acol[i] - 1; j < acol[i + 1] - 1; ++j) s = s + a[j] * p[arow[j] - 1];
    q[i] = s;
}

// r(i) = r(i) - A(j) x(Arow(j)) in stored order (Resid.f90:29-35).
__global__ void k_resid(int n, const int* __restrict__ acol, const int* __restrict__ arow,
                        const double* __restrict__ a, const double* __restrict__ x,
                        double* __restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = r[i];
    for (int j = acol[i] - 1; j < acol[i + 1] - 1; ++j) s = s - a[j] * x[arow[j] - 1];
    r[i] = s;
}

// The halo terms of the rows that have any, each row's terms in the
// reference's order: v(i) = v(i) +/- Ab(k) phi(k).  ab and phi are indexed
// by NB + k.
__global__ void k_halo(int nrows, const int* __restrict__ rows, const int* __restrict__ ptr,
                       const int* __restrict__ kk, const double* __restrict__ ab,
                       const double* __restrict__ phi, double* __restrict__ v, int minus) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrows) return;
    const int i = rows[t];
    double s = v[i];
    for (int e = ptr[t]; e < ptr[t + 1]; ++e) {
        const double prod = ab[kk[e]] * phi[kk[e]];
        s = minus ? s - prod : s + prod;
    }
    v[i] = s;
}

// Exchng.f90:36-43: every buffer cell takes the value of the cell it mirrors.
__global__ void k_pack(int m, const int* __restrict__ kk, const int* __restrict__ src,
                       const double* __restrict__ p, double* __restrict__ phi) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) phi[kk[t]] = p[src[t]];
}

// Local inner product: per-block partial sums (fixed grid, fixed tree), then
// one block sums the partials in a fixed order.
__global__ void k_dot_partial(int n, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ part) {
    __shared__ double sh[kThreads];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s = s + a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_dot_final(int m, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[kDotBlocks];
    for (int t = threadIdx.x; t < kDotBlocks; t += blockDim.x) sh[t] = t < m ? part[t] : 0.0;
    __syncthreads();
    for (int w = kDotBlocks / 2; w > 0; w >>= 1) {
        for (int t = threadIdx.x; t < w; t += blockDim.x) sh[t] = sh[t] + sh[t + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void k_diag(int n, const int* __restrict__ adia, const double* __restrict__ a,
                       double* __restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = a[adia[i] - 1];
}
// z = r / D (CG.f90:125-127)
__global__ void k_div(int n, const double* __restrict__ r, const double* __restrict__ d,
                      double* __restrict__ z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = r[i] / d[i];
}
// p = z + beta p (CG.f90:183-185)
__global__ void k_xpby(int n, const double* __restrict__ z, double beta, double* __restrict__ p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
}
// x = x + alfa p; r = r - alfa q (CG.f90:226-229)
__global__ void k_update(int n, double alfa, const double* __restrict__ p,
                         const double* __restrict__ q, double* __restrict__ x,
                         double* __restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        x[i] = x[i] + alfa * p[i];
        r[i] = r[i] - alfa * q[i];
    }
}
// CGS: u1 = r1 + beta q1; u2 = u1 + beta (q1 + beta u2) (CGS.f90:131-140)
__global__ void k_cgs_u(int n, double beta, const double* __restrict__ r1,
                        const double* __restrict__ q1, double* __restrict__ u1,
                        double* __restrict__ u2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double a = r1[i] + beta * q1[i];
        u1[i] = a;
        u2[i] = a + beta * (q1[i] + beta * u2[i]);
    }
}
// CGS: q1 = u1 - alfa v2 (CGS.f90:226-228)
__global__ void k_axmy(int n, double alfa, const double* __restrict__ u,
                       const double* __restrict__ v, double* __restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = u[i] - alfa * v[i];
}
// CGS: w = u1 + q1, and with a diagonal p1 = (u1 + q1) / D (CGS.f90:238-280)
__global__ void k_sum(int n, const double* __restrict__ a, const double* __restrict__ b,
                      const double* __restrict__ d, double* __restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = d ? (a[i] + b[i]) / d[i] : a[i] + b[i];
}
// y = y + alfa p (CGS.f90:286-288 and :318-320 with the sign folded into alfa)
__global__ void k_axpy(int n, double alfa, const double* __restrict__ p, double* __restrict__ y,
                       int minus) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = minus ? y[i] - alfa * p[i] : y[i] + alfa * p[i];
}

unsigned blocks_for(int n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---- registration ---------------------------------------------------------------------

struct HaloSolve;

struct HaloState {
    std::mutex mu;
    int npro = 0;
    int nb = 0;
    std::vector<int> nbbs, nbbe, bufind;  // bufind[nb + k] = BufInd(k)
    tflows_exchange_fn exchange = nullptr;
    tflows_glosum_fn glosum = nullptr;
    void* user = nullptr;
    HaloSolve* work = nullptr;  // buffers kept between calls (grow-only)
};
HaloState& state() {
    static HaloState* s = new HaloState();  // outlives every caller, as par_mod does
    return *s;
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t need(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) cap = n;
        return e;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// The device arrays of the coupled solves and the halo lists of the current
// call.  One instance lives in the halo state and is reused by every call
// until the halo is cleared: buffers only grow, and the IC(0) pattern of the
// last prec-2 call stays on the device while the caller passes the same
// arrays (same addresses, sizes and sampled content hash as the legacy
// topology cache).
struct HaloSolve {
    const HaloState& h;
    cudaStream_t s = nullptr;
    int n = 0, nb = 0, nnz = 0;
    DevBuf<int> acol, arow, adia, hrows, hptr, hkk, pkk, psrc;
    DevBuf<double> a, ab, d, phi, part, scal;
    DevBuf<double> vec[12];
    int nhrows = 0, npack = 0;
    double* phi_h = nullptr;
    size_t phi_cap = 0;
    double* scal_h = nullptr;
    tflows_topology* topo = nullptr;
    int topo_n = 0, topo_nnz = 0;
    const int *topo_acol = nullptr, *topo_arow = nullptr, *topo_adia = nullptr;
    unsigned long long topo_hash = 0;
    std::string msg;

    explicit HaloSolve(const HaloState& hs) : h(hs) {}
    ~HaloSolve() {
        if (phi_h) cudaFreeHost(phi_h);
        if (scal_h) cudaFreeHost(scal_h);
        if (topo) tflows_topology_destroy(topo);
    }
    void begin(cudaStream_t st, int rows, int nbuf) {
        s = st;
        n = rows;
        nb = nbuf;
        msg.clear();
    }

    // The IC(0) pattern for these arrays, rebuilt only when they changed.
    int ic_topology(const int* Acol, const int* Arow, const int* Adia) {
        const unsigned long long hsh = legacy_pattern_hash(n, nnz, Acol, Arow, Adia);
        if (topo && topo_n == n && topo_nnz == nnz && topo_acol == Acol && topo_arow == Arow &&
            topo_adia == Adia && topo_hash == hsh)
            return TFLOWS_OK;
        if (topo) tflows_topology_destroy(topo);
        topo = nullptr;
        const int st = tflows_topology_create(&topo, n, nnz, Acol, Arow, Adia, 1, 0);
        if (st != TFLOWS_OK) {
            topo = nullptr;
            msg = std::string("halo: IC(0) pattern: ") + tflows_last_error();
            return st;
        }
        topo_n = n;
        topo_nnz = nnz;
        topo_acol = Acol;
        topo_arow = Arow;
        topo_adia = Adia;
        topo_hash = hsh;
        return TFLOWS_OK;
    }

    // Halo lists for this N: rows with their buffer cells in the reference's
    // order, and the cells to pack.  BAD_INPUT when a map leaves its range.
    int build_lists() {
        std::vector<std::vector<int>> per_row;
        std::vector<int> order;  // rows in first-appearance order
        std::vector<int> slot((size_t)n, -1);
        std::vector<int> pk, ps;
        for (int sub = 1; sub <= h.npro; ++sub) {
            const int s0 = h.nbbs[sub - 1], e0 = h.nbbe[sub - 1];
            if (e0 > s0) continue;  // no connection with this neighbour
            if (e0 < -nb || s0 > -1) {
                msg = "halo: NBBe/NBBs of neighbour " + std::to_string(sub) + " outside -NB..-1";
                return TFLOWS_BAD_INPUT;
            }
            for (int k = s0; k >= e0; --k) {
                const int i = h.bufind[(size_t)(nb + k)];
                if (i < 1 || i > n) {
                    msg = "halo: BufInd(" + std::to_string(k) + ") = " + std::to_string(i) +
                          " outside 1..N";
                    return TFLOWS_BAD_INPUT;
                }
                if (slot[i - 1] < 0) {
                    slot[i - 1] = (int)per_row.size();
                    per_row.emplace_back();
                    order.push_back(i - 1);
                }
                per_row[slot[i - 1]].push_back(nb + k);
                pk.push_back(nb + k);
                ps.push_back(i - 1);
            }
        }
        std::vector<int> ptr(1, 0), kk;
        for (const auto& l : per_row) {
            kk.insert(kk.end(), l.begin(), l.end());
            ptr.push_back((int)kk.size());
        }
        nhrows = (int)order.size();
        npack = (int)pk.size();
        cudaError_t e = hrows.need(order.size());
        if (e == cudaSuccess) e = hptr.need(ptr.size());
        if (e == cudaSuccess) e = hkk.need(kk.size());
        if (e == cudaSuccess) e = pkk.need(pk.size());
        if (e == cudaSuccess) e = psrc.need(ps.size());
        if (e == cudaSuccess && nhrows)
            e = cudaMemcpyAsync(hrows.p, order.data(), order.size() * sizeof(int),
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hptr.p, ptr.data(), ptr.size() * sizeof(int),
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && !kk.empty())
            e = cudaMemcpyAsync(hkk.p, kk.data(), kk.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && npack)
            e = cudaMemcpyAsync(pkk.p, pk.data(), pk.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && npack)
            e = cudaMemcpyAsync(psrc.p, ps.data(), ps.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        // the copies read host vectors that go out of scope here
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e == cudaSuccess ? TFLOWS_OK : cuda(e, "halo lists");
    }

    int cuda(cudaError_t e, const char* what) {
        msg = std::string(what) + ": " + cudaGetErrorString(e);
        return TFLOWS_CUDA_ERROR;
    }

    int upload(const double* A, const int* Acol, const int* Arow, const int* Adia,
               const double* Ab, int nonz) {
        nnz = nonz - 1;
        cudaError_t e = acol.need((size_t)n + 1);
        if (e == cudaSuccess) e = arow.need((size_t)nnz);
        if (e == cudaSuccess) e = a.need((size_t)nnz);
        if (e == cudaSuccess && Adia) e = adia.need((size_t)n);
        if (e == cudaSuccess) e = ab.need((size_t)nb);
        if (e == cudaSuccess) e = phi.need((size_t)nb);
        if (e == cudaSuccess) e = part.need(kDotBlocks);
        if (e == cudaSuccess) e = scal.need(1);
        if (e == cudaSuccess && (size_t)nb > phi_cap) {
            if (phi_h) cudaFreeHost(phi_h);
            phi_h = nullptr;
            phi_cap = 0;
            if ((e = cudaMallocHost(&phi_h, (size_t)nb * sizeof(double))) == cudaSuccess)
                phi_cap = (size_t)nb;
        }
        if (e == cudaSuccess && !scal_h) e = cudaMallocHost(&scal_h, sizeof(double));
        if (e != cudaSuccess) return cuda(e, "halo workspace");
        e = cudaMemcpyAsync(acol.p, Acol, ((size_t)n + 1) * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(arow.p, Arow, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(a.p, A, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && Adia)
            e = cudaMemcpyAsync(adia.p, Adia, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nb && Ab)
            e = cudaMemcpyAsync(ab.p, Ab, (size_t)nb * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nb && !Ab) e = cudaMemsetAsync(ab.p, 0, (size_t)nb * sizeof(double), s);
        return e == cudaSuccess ? TFLOWS_OK : cuda(e, "halo upload");
    }

    // Local inner product, then the caller's sum over the ranks.
    int dot(const double* x, const double* y, double& out) {
        const unsigned g = std::min<unsigned>(kDotBlocks, std::max(1u, blocks_for(n)));
        k_dot_partial<<<g, kThreads, 0, s>>>(n, x, y, part.p);
        k_dot_final<<<1, 1024, 0, s>>>((int)g, part.p, scal.p);
        cudaError_t e = cudaMemcpyAsync(scal_h, scal.p, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda(e, "inner product");
        out = *scal_h;
        return glosum(out);
    }
    int glosum(double& v) {
        if (h.glosum(h.user, &v) != 0) {
            msg = "halo: the global-sum callback failed";
            return TFLOWS_HALO_ERROR;
        }
        return TFLOWS_OK;
    }

    // q = A p, then Exchng(p) and the halo terms (CG.f90:193-208).
    int product(const double* p, double* q) {
        k_spmv<<<blocks_for(n), kThreads, 0, s>>>(n, acol.p, arow.p, a.p, p, q);
        if (nb == 0) return TFLOWS_OK;
        if (npack) k_pack<<<blocks_for(npack), kThreads, 0, s>>>(npack, pkk.p, psrc.p, p, phi.p);
        cudaError_t e = cudaMemcpyAsync(phi_h, phi.p, (size_t)nb * sizeof(double),
                                        cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda(e, "exchange copy");
        if (h.exchange(h.user, phi_h, nb) != 0) {
            msg = "halo: the exchange callback failed";
            return TFLOWS_HALO_ERROR;
        }
        e = cudaMemcpyAsync(phi.p, phi_h, (size_t)nb * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda(e, "exchange copy");
        if (nhrows)
            k_halo<<<blocks_for(nhrows), kThreads, 0, s>>>(nhrows, hrows.p, hptr.p, hkk.p, ab.p,
                                                           phi.p, q, 0);
        return TFLOWS_OK;
    }

    // z = M^-1 r for prec 1 (diagonal), 2 (IC(0)) or other (identity).
    int precondition(int prec, const double* r, double* z) {
        if (prec == 1) {
            k_div<<<blocks_for(n), kThreads, 0, s>>>(n, r, d.p, z);
        } else if (prec == 2) {
            tflows_options o;
            tflows_default_options(&o);
            o.precision = TFLOWS_FP64;
            const int st = tflows_ic_apply_device(topo, &o, a.p, r, z, s, nullptr);
            if (st != TFLOWS_OK) {
                msg = std::string("halo: IC(0) apply: ") + tflows_last_error();
                return st;
            }
        } else {
            cudaError_t e = cudaMemcpyAsync(z, r, (size_t)n * sizeof(double),
                                            cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return cuda(e, "copy");
        }
        return TFLOWS_OK;
    }
};

}  // namespace

void halo_release() {
    HaloState& h = state();
    std::lock_guard<std::mutex> lk(h.mu);
    delete h.work;
    h.work = nullptr;
}

bool halo_registered() {
    HaloState& h = state();
    std::lock_guard<std::mutex> lk(h.mu);
    return h.npro > 0;
}

int halo_solve(int method, int n, int nb, int nonz, const double* A, const int* Acol,
               const int* Arow, const int* Adia, const double* Ab, double* x, double* r1,
               int prec, int* niter, double tol, double* IniRes, double* FinRes,
               double& error_state, cudaStream_t s, SolveReport& rep) {
    HaloState& h = state();
    std::lock_guard<std::mutex> lk(h.mu);
    if (nb != h.nb) {
        rep.message = "halo: the solver's NB differs from the registered NB";
        return rep.status = TFLOWS_BAD_INPUT;
    }
    if (method == TFLOWS_METHOD_BICG_TRUE) {
        rep.message = "halo: the transposed BiCG extension has no halo form";
        return rep.status = TFLOWS_UNSUPPORTED;
    }
    if (!h.work) h.work = new HaloSolve(h);
    HaloSolve& hs = *h.work;
    hs.begin(s, n, nb);
    int st = hs.upload(A, Acol, Arow, Adia, Ab, nonz);
    if (st == TFLOWS_OK) st = hs.build_lists();
    const bool cgs = method == TFLOWS_METHOD_CGS;
    for (int v = 0; v < (cgs ? 12 : 5) && st == TFLOWS_OK; ++v)
        if (cudaError_t e = hs.vec[v].need((size_t)n); e != cudaSuccess) st = hs.cuda(e, "vectors");
    if (st == TFLOWS_OK && prec == 1) {
        if (cudaError_t e = hs.d.need((size_t)n); e != cudaSuccess) st = hs.cuda(e, "D");
        else k_diag<<<blocks_for(n), kThreads, 0, s>>>(n, hs.adia.p, hs.a.p, hs.d.p);
    }
    if (st == TFLOWS_OK && prec == 2) st = hs.ic_topology(Acol, Arow, Adia);
    if (st != TFLOWS_OK) {
        rep.message = hs.msg;
        return rep.status = st;
    }

    double* X = hs.vec[0].p;
    double* R = hs.vec[1].p;
    const size_t nbytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaMemcpyAsync(X, x + nb + 1, nbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(R, r1, nbytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        rep.message = "halo: copy x, r1";
        return rep.status = TFLOWS_CUDA_ERROR;
    }

    // The reference's control flow (CG.f90:55-262, CGS.f90:55-337; BiCG runs
    // CG's recurrence, as its shadow sequence equals the primary one).
    int iter = 0;
    double err = error_state;
    bool touched = false;
    int exit_kind = EXIT_MAXITER;
    auto run = [&]() -> int {
        double bn = 0.0;
        int rc = hs.dot(R, R, bn);
        if (rc != TFLOWS_OK) return rc;
        if (std::sqrt(bn) < tol) {
            exit_kind = EXIT_BNRM;
            return TFLOWS_OK;
        }
        touched = true;
        // Resid with the caller's buffer values of x
        std::vector<double> xb(x, x + nb);
        e = cudaMemcpyAsync(hs.phi.p, xb.data(), (size_t)nb * sizeof(double),
                            cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return hs.cuda(e, "copy x buffers");
        k_resid<<<blocks_for(n), kThreads, 0, s>>>(n, hs.acol.p, hs.arow.p, hs.a.p, X, R);
        if (hs.nhrows)
            k_halo<<<blocks_for(hs.nhrows), kThreads, 0, s>>>(hs.nhrows, hs.hrows.p, hs.hptr.p,
                                                              hs.hkk.p, hs.ab.p, hs.phi.p, R, 1);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return hs.cuda(e, "resid");
        double e2 = 0.0;
        if ((rc = hs.dot(R, R, e2)) != TFLOWS_OK) return rc;
        err = std::sqrt(e2);
        *IniRes = err;
        if (err < tol) {
            exit_kind = EXIT_INIRES;
            return TFLOWS_OK;
        }
        double rho = 0.0, rhoold = 0.0, alfa = 0.0, beta = 0.0;
        if (!cgs) {
            double *Z = hs.vec[2].p, *P = hs.vec[3].p, *Q = hs.vec[4].p;
            for (iter = 1; iter <= *niter; ++iter) {
                if ((rc = hs.precondition(prec, R, Z)) != TFLOWS_OK) return rc;
                if ((rc = hs.dot(R, Z, rho)) != TFLOWS_OK) return rc;
                if (iter == 1) {
                    e = cudaMemcpyAsync(P, Z, nbytes, cudaMemcpyDeviceToDevice, s);
                    if (e != cudaSuccess) return hs.cuda(e, "copy");
                } else {
                    beta = rho / rhoold;
                    k_xpby<<<blocks_for(n), kThreads, 0, s>>>(n, Z, beta, P);
                }
                if ((rc = hs.product(P, Q)) != TFLOWS_OK) return rc;
                double pq = 0.0;
                if ((rc = hs.dot(P, Q, pq)) != TFLOWS_OK) return rc;
                alfa = rho / pq;
                k_update<<<blocks_for(n), kThreads, 0, s>>>(n, alfa, P, Q, X, R);
                if ((rc = hs.dot(R, R, e2)) != TFLOWS_OK) return rc;
                err = std::sqrt(e2);
                if (!std::isfinite(err)) {
                    exit_kind = EXIT_NONFINITE;
                    return TFLOWS_NONFINITE;
                }
                if (err < tol) {
                    exit_kind = EXIT_CONVERGED;
                    return TFLOWS_OK;
                }
                rhoold = rho;
            }
            return TFLOWS_NOT_CONVERGED;
        }
        double *R2 = hs.vec[2].p, *U1 = hs.vec[3].p, *U2 = hs.vec[4].p, *P1 = hs.vec[5].p,
               *P2 = hs.vec[6].p, *V2 = hs.vec[7].p, *Q1 = hs.vec[8].p, *Q2 = hs.vec[9].p,
               *W = hs.vec[10].p;
        if ((e = cudaMemcpyAsync(R2, R, nbytes, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return hs.cuda(e, "copy");
        for (iter = 1; iter <= *niter; ++iter) {
            if ((rc = hs.dot(R, R2, rho)) != TFLOWS_OK) return rc;
            if (iter == 1) {
                e = cudaMemcpyAsync(U1, R, nbytes, cudaMemcpyDeviceToDevice, s);
                if (e == cudaSuccess) e = cudaMemcpyAsync(U2, R, nbytes, cudaMemcpyDeviceToDevice, s);
                if (e != cudaSuccess) return hs.cuda(e, "copy");
            } else {
                beta = rho / rhoold;
                k_cgs_u<<<blocks_for(n), kThreads, 0, s>>>(n, beta, R, Q1, U1, U2);
            }
            if ((rc = hs.precondition(prec, U2, P2)) != TFLOWS_OK) return rc;
            if ((rc = hs.product(P2, V2)) != TFLOWS_OK) return rc;
            double rv = 0.0;
            if ((rc = hs.dot(R2, V2, rv)) != TFLOWS_OK) return rc;
            alfa = rho / rv;
            k_axmy<<<blocks_for(n), kThreads, 0, s>>>(n, alfa, U1, V2, Q1);
            if (prec == 1) {
                k_sum<<<blocks_for(n), kThreads, 0, s>>>(n, U1, Q1, hs.d.p, P1);
            } else {
                k_sum<<<blocks_for(n), kThreads, 0, s>>>(n, U1, Q1, nullptr, W);
                if ((rc = hs.precondition(prec, W, P1)) != TFLOWS_OK) return rc;
            }
            k_axpy<<<blocks_for(n), kThreads, 0, s>>>(n, alfa, P1, X, 0);
            if ((rc = hs.product(P1, Q2)) != TFLOWS_OK) return rc;
            k_axpy<<<blocks_for(n), kThreads, 0, s>>>(n, alfa, Q2, R, 1);
            if ((rc = hs.dot(R, R, e2)) != TFLOWS_OK) return rc;
            err = std::sqrt(e2);
            if (!std::isfinite(err)) {
                exit_kind = EXIT_NONFINITE;
                return TFLOWS_NONFINITE;
            }
            if (err < tol) {
                exit_kind = EXIT_CONVERGED;
                return TFLOWS_OK;
            }
            rhoold = rho;
        }
        return TFLOWS_NOT_CONVERGED;
    };
    st = run();
    rep.exit_kind = exit_kind;
    if (st != TFLOWS_OK && st != TFLOWS_NOT_CONVERGED && st != TFLOWS_NONFINITE) {
        rep.message = hs.msg;
        return rep.status = st;
    }
    if (exit_kind == EXIT_BNRM) {
        *niter = 0;
        *FinRes = error_state;
    } else {
        if (exit_kind == EXIT_INIRES) iter = 0;
        *niter = iter;  // niter + 1 when the loop ran out, as the Fortran DO leaves it
        *FinRes = err;
        error_state = err;
    }
    if (touched) {
        e = cudaMemcpyAsync(x + nb + 1, X, nbytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(r1, R, nbytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rep.message = "halo: copy x, r1 back";
            return rep.status = TFLOWS_CUDA_ERROR;
        }
    }
    rep.iterations = *niter;
    rep.ini_res = touched ? *IniRes : 0.0;
    rep.fin_res = *FinRes;
    if (st == TFLOWS_NONFINITE) rep.message = "non-finite residual";
    return rep.status = st;
}

int halo_resid(int n, int nb, int nonz, const double* A, const int* Acol, const int* Arow,
               const double* Ab, const double* x, double* r1, cudaStream_t s, std::string& msg) {
    HaloState& h = state();
    std::lock_guard<std::mutex> lk(h.mu);
    if (nb != h.nb) {
        msg = "halo: the NB of Resid differs from the registered NB";
        return TFLOWS_BAD_INPUT;
    }
    if (!h.work) h.work = new HaloSolve(h);
    HaloSolve& hs = *h.work;
    hs.begin(s, n, nb);
    int st = hs.upload(A, Acol, Arow, nullptr, Ab, nonz);
    if (st == TFLOWS_OK) st = hs.build_lists();
    for (int v = 0; v < 2 && st == TFLOWS_OK; ++v)
        if (cudaError_t e = hs.vec[v].need((size_t)n); e != cudaSuccess) st = hs.cuda(e, "vectors");
    if (st != TFLOWS_OK) {
        msg = hs.msg;
        return st;
    }
    const size_t nbytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaMemcpyAsync(hs.vec[0].p, x + nb + 1, nbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hs.vec[1].p, r1, nbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nb)
        e = cudaMemcpyAsync(hs.phi.p, x, (size_t)nb * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_resid<<<blocks_for(n), kThreads, 0, s>>>(n, hs.acol.p, hs.arow.p, hs.a.p, hs.vec[0].p,
                                                   hs.vec[1].p);
        if (hs.nhrows)
            k_halo<<<blocks_for(hs.nhrows), kThreads, 0, s>>>(hs.nhrows, hs.hrows.p, hs.hptr.p,
                                                              hs.hkk.p, hs.ab.p, hs.phi.p,
                                                              hs.vec[1].p, 1);
        e = cudaMemcpyAsync(r1, hs.vec[1].p, nbytes, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        msg = std::string("halo resid: ") + cudaGetErrorString(e);
        return TFLOWS_CUDA_ERROR;
    }
    return TFLOWS_OK;
}

}  // namespace tflows

extern "C" {

int tflows_set_halo(int Npro, int NB, const int* NBBs, const int* NBBe, const int* BufInd,
                    tflows_exchange_fn exchange, tflows_glosum_fn glosum, void* user) {
    using namespace tflows;
    HaloState& h = state();
    std::lock_guard<std::mutex> lk(h.mu);
    if (Npro <= 0) {
        delete h.work;  // frees the device and pinned buffers
        h.work = nullptr;
        h.npro = 0;
        h.nb = 0;
        h.nbbs.clear();
        h.nbbe.clear();
        h.bufind.clear();
        h.exchange = nullptr;
        h.glosum = nullptr;
        h.user = nullptr;
        return report_status(TFLOWS_OK, "");
    }
    if (NB < 0 || !NBBs || !NBBe || !exchange || !glosum || (NB > 0 && !BufInd))
        return report_status(TFLOWS_BAD_INPUT, "halo: null map or callback, or NB < 0");
    std::vector<int> bs(NBBs, NBBs + Npro), be(NBBe, NBBe + Npro);
    for (int sub = 0; sub < Npro; ++sub)
        if (be[sub] <= bs[sub] && (be[sub] < -NB || bs[sub] > -1))
            return report_status(TFLOWS_BAD_INPUT, "halo: NBBe/NBBs outside -NB..-1");
    h.npro = Npro;
    h.nb = NB;
    h.nbbs.swap(bs);
    h.nbbe.swap(be);
    h.bufind.assign(BufInd, BufInd + NB);
    h.exchange = exchange;
    h.glosum = glosum;
    h.user = user;
    return report_status(TFLOWS_OK, "");
}

void tflows_clear_halo(void) { tflows_set_halo(0, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr); }

}  // extern "C"
