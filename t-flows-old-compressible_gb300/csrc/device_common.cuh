// Device-side building blocks shared by the Krylov kernels (sm_103a).
//
// * memory-model helpers (relaxed / acquire / release accesses at gpu scope)
// * a grid barrier for persistent cooperative launches whose every wait is
//   bounded by the SM cycle counter and by a shared abort flag
// * value-as-flag cells for the sync-free triangular sweeps: a cell holds a
//   signalling-NaN sentinel until its producer stores the computed value
//   (arithmetic never yields a signalling NaN, so a stored result can never
//   be mistaken for the sentinel)
// * deterministic block and grid reductions (fixed summation tree)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tflows {

constexpr int kWarp = 32;

// ---- status codes (mirror include/tflows_krylov.h) -------------------------
enum : int {
    ST_OK = 0, ST_NOT_CONVERGED = 1, ST_BREAKDOWN = 2, ST_NONFINITE = 3,
    ST_TIMEOUT = 4, ST_BAD_INPUT = 5, ST_CUDA_ERROR = 6
};

// Exit kinds of the reference control flow (Process/CG.f90:69-72,105-108,255).
enum : int { EXIT_BNRM = 1, EXIT_INIRES = 2, EXIT_CONVERGED = 3, EXIT_MAXITER = 4,
             EXIT_ABORT = 5, EXIT_NONFINITE = 6 };

// Per-solve device record (one per system), written by block 0.
struct DevState {
    int status;
    int exit_kind;
    int iterations;      // reference-visible iteration count
    int inner_iters;     // mixed mode: total inner iterations
    int refinements;     // mixed mode: refinement steps
    int timeout_where;   // which wait timed out (diagnostics)
    double ini_res;
    double fin_res;
    double bnrm2;
    double group_ns;     // batched launches: the system's own solve time
    double pad[2];
};

// Nanosecond clock shared by all SMs (measurement only; waits use clock64).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Control block shared by all blocks of one persistent launch.
struct DevCtl {
    unsigned long long bar;  // monotonically increasing arrival counter
    int abort;               // set by whoever gives up; every wait checks it
    int status;              // first error status raised
    int where;
    int pad;
};

// Wait limits are measured in SM clock cycles (clock64: monotonic and local
// to the SM, unlike the host-synchronised %globaltimer); the host converts
// the limit in seconds with the device's highest SM clock, so the real limit
// is never shorter than requested.

__device__ __forceinline__ long long ld_relaxed_s64(const long long* p) {
    long long v;
    asm volatile("ld.relaxed.gpu.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_s64(long long* p, long long v) {
    asm volatile("st.relaxed.gpu.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_s32(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Raise an abort: first status wins; everyone polling `abort` leaves.
__device__ __forceinline__ void raise_abort(DevCtl* c, int status, int where) {
    if (atomicCAS(&c->status, 0, status) == 0) c->where = where;
    atomicExch(&c->abort, 1);
}

// ---- shared-memory staging with bulk async copies --------------------------------
// The tiled IC sweeps stream each wavefront step's record (contiguous in its
// step-major layout) into a ring of shared-memory slots with the bulk copy
// engine (cp.async.bulk, global -> shared), one mbarrier per slot: the
// issuing thread announces the byte count (arrive.expect_tx), the copy
// completes the transaction, and the consumers wait on the slot's phase
// parity.  Sizes are multiples of 16 bytes and both addresses 16-byte
// aligned (the host sizes the layout so).
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
// Makes the initialised barriers visible to the async proxy (the bulk copies).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// `bytes` from global `src` into this CTA's shared `dst`, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Explicit shared-memory accesses at 32-bit shared addresses (the tiled
// sweeps' ring and neighbour exchange): ld.shared / st.shared rather than
// generic accesses, which the compiler emits when the address space of a
// pointer carried through structures is not known and which wait on the
// long scoreboard.  Volatile, so they stay ordered after the barrier waits.
template <typename T> __device__ __forceinline__ T lds(unsigned a);
template <> __device__ __forceinline__ double lds<double>(unsigned a) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(a));
    return v;
}
template <> __device__ __forceinline__ float lds<float>(unsigned a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
template <> __device__ __forceinline__ unsigned short lds<unsigned short>(unsigned a) {
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ void sts(unsigned a, double v) {
    asm volatile("st.shared.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ void sts(unsigned a, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// Orders this thread's earlier generic-proxy accesses before its later
// async-proxy accesses: in shared memory (the block's reads of a ring slot
// before the bulk copy that refills it; cheap, issued every step) or in
// global memory (words written before a barrier that bulk copies read after
// it; once per sweep or tile, as it waits for this thread's global accesses).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// ---- value-as-flag cells ------------------------------------------------------
template <typename T> struct Cell;
template <> struct Cell<double> {
    using bits_t = long long;
    static constexpr long long kSentinel = 0x7FF4242424242424LL;  // signalling NaN
    __device__ static __forceinline__ bits_t bits(double v) { return __double_as_longlong(v); }
    __device__ static __forceinline__ double value(bits_t b) { return __longlong_as_double(b); }
    __device__ static __forceinline__ bits_t load(const double* p) {
        return ld_relaxed_s64(reinterpret_cast<const long long*>(p));
    }
    __device__ static __forceinline__ void store(double* p, double v) {
        st_relaxed_s64(reinterpret_cast<long long*>(p), __double_as_longlong(v));
    }
    __device__ static __forceinline__ double sentinel() { return __longlong_as_double(kSentinel); }
};
template <> struct Cell<float> {
    using bits_t = int;
    static constexpr int kSentinel = 0x7FA42424;  // signalling NaN
    __device__ static __forceinline__ bits_t bits(float v) { return __float_as_int(v); }
    __device__ static __forceinline__ float value(bits_t b) { return __int_as_float(b); }
    __device__ static __forceinline__ bits_t load(const float* p) {
        return ld_relaxed_s32(reinterpret_cast<const int*>(p));
    }
    __device__ static __forceinline__ void store(float* p, float v) {
        st_relaxed_s32(reinterpret_cast<int*>(p), __float_as_int(v));
    }
    __device__ static __forceinline__ float sentinel() { return __int_as_float(kSentinel); }
};

// ---- reductions ---------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum K per-thread values over the block; thread 0 writes them to out[k].
// `sm` must hold K * (blockDim.x / 32) doubles.
template <int K>
__device__ __forceinline__ void block_sums(const double (&v)[K], double* sm, double* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) sm[k * nw + warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = lane < nw ? sm[k * nw + lane] : 0.0;
            s = warp_sum(s);
            if (lane == 0) out[k] = s;
        }
    }
    __syncthreads();
}

// Persistent-launch context kept in registers / shared memory of each block.
struct Grid {
    DevCtl* ctl;
    double* partials;   // [slots][nblocks]
    long long timeout_cyc;
    unsigned long long target;  // thread 0 only
    int nblocks;
    int wg;   // global warp index
    int nw;   // warps in the grid
    int lane;
    int tid;  // thread index within the group of blocks solving one system
    int nt;   // threads in the group
    int bid;  // block index within the group
    unsigned ep_f;  // forward / backward level-sweep epochs (counter targets)
    unsigned ep_b;
    int stall;      // test hook: block 0 skips its first barrier arrival
};

// A "grid" here is the group of `nb` blocks (starting at block `b0` of the
// launch) that solves one system: barriers, partial sums and work
// distribution are all relative to the group, so one launch can carry many
// independent solves.
__device__ __forceinline__ void grid_init_group(Grid& g, DevCtl* ctl, double* partials,
                                                long long timeout_cyc, int b0, int nb) {
    g.ctl = ctl;
    g.partials = partials;
    g.timeout_cyc = timeout_cyc;
    g.target = 0;
    g.nblocks = nb;
    g.bid = blockIdx.x - b0;
    g.lane = threadIdx.x & 31;
    g.tid = g.bid * blockDim.x + threadIdx.x;
    g.nt = nb * blockDim.x;
    g.wg = g.tid >> 5;
    g.nw = g.nt >> 5;
    g.ep_f = 0;
    g.ep_b = 0;
    g.stall = 0;
}

__device__ __forceinline__ void grid_init(Grid& g, DevCtl* ctl, double* partials,
                                          long long timeout_cyc) {
    grid_init_group(g, ctl, partials, timeout_cyc, 0, gridDim.x);
}

// Grid-wide barrier with release/acquire ordering (every write before the
// barrier is visible to every read after it).  Returns false when the
// launch was aborted (timeout or error raised anywhere).  The block's
// threads meet at __syncthreads, then thread 0 arrives with a release add
// and waits with acquire loads; the release is cumulative over the writes
// the block barrier ordered before it and the acquire orders every read
// after the closing block barrier, so no separate fence is needed (a fence
// on each side cost 0.9 us of a 6.6 us barrier with 304 blocks).
__device__ __forceinline__ bool grid_sync(Grid& g, int where) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        g.target += (unsigned long long)g.nblocks;
        if (g.stall && g.bid == 0) g.stall = 0;  // withheld: the barrier cannot complete
        else red_release_add_u64(&g.ctl->bar, 1ull);
        int ok = 1;
        long long t0 = 0;
        unsigned spins = 0;
        while (ld_acquire_u64(&g.ctl->bar) < g.target) {
            if ((++spins & 255u) == 0u) {
                if (ld_relaxed_s32(&g.ctl->abort)) { ok = 0; break; }
                long long t = clock64();
                if (t0 == 0) t0 = t;
                else if (t - t0 > g.timeout_cyc) {
                    raise_abort(g.ctl, ST_TIMEOUT, where);
                    ok = 0;
                    break;
                }
            }
        }
        if (ld_relaxed_s32(&g.ctl->abort)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Publish this block's K partial sums into slot range [slot, slot+K): the
// sums of block_sums, stored by thread 0, which forms them (the grid_sync
// that follows every publish orders the stores before its arrival).
template <int K>
__device__ __forceinline__ void publish(Grid& g, int slot, const double (&v)[K]) {
    __shared__ double sm[K * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double s = warp_sum(v[k]);
        if (lane == 0) sm[k * nw + warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const double s = warp_sum(lane < nw ? sm[k * nw + lane] : 0.0);
            if (lane == 0) g.partials[(size_t)(slot + k) * g.nblocks + g.bid] = s;
        }
    }
}

// After a grid_sync: every block computes the same K totals in the same
// order (deterministic), broadcast through shared memory.
template <int K>
__device__ __forceinline__ void totals(Grid& g, int slot, double (&res)[K]) {
    __shared__ double s_tot[K];
    if ((threadIdx.x >> 5) == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const long long* src =
                reinterpret_cast<const long long*>(g.partials + (size_t)(slot + k) * g.nblocks);
            // each lane's partials in increasing block order, loads issued
            // eight at a time ahead of their sums
            double s = 0.0;
            for (int b0 = g.lane; b0 < g.nblocks; b0 += 32 * 8) {
                long long w[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    w[u] = b0 + 32 * u < g.nblocks ? ld_relaxed_s64(src + b0 + 32 * u) : 0;
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (b0 + 32 * u < g.nblocks) s += __longlong_as_double(w[u]);
            }
            s = warp_sum(s);
            if (g.lane == 0) s_tot[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) res[k] = s_tot[k];
    // no closing block barrier: the next write of s_tot comes after the
    // next grid_sync, whose opening __syncthreads every thread reaches after
    // reading these totals
}

}  // namespace tflows
