// Kernels of the contracted build: the same solver code as krylov.cu,
// compiled with fused multiply-adds (--fmad=true) and a reciprocal diagonal
// for the Jacobi preconditioner.  It serves two kinds of solves:
//   * TFLOWS_FP64_FMA: the reference's recurrences in FP64 with about half
//     the FP64 instructions (GB300's FP64 pipe, not its memory, bounds the
//     reference-arithmetic build); results differ from the reference's only
//     by rounding;
//   * the mixed-precision solves (FP32 inner iterations, FP64 refinement),
//     which make no bitwise claim.
#define TFLOWS_KNS fma
#define TFLOWS_FP64_RECIP_DIAG 1
#include "internal.h"
#include "solver_entry.cuh"

namespace tflows {

const void* fma_kernel(KernelId id) {
    switch (id) {
        case KernelId::Cg: return (const void*)fma::krylov_kernel<double, 0>;
        case KernelId::Cgs: return (const void*)fma::krylov_kernel<double, 2>;
        case KernelId::BicgTrue: return (const void*)fma::krylov_kernel<double, 3>;
        case KernelId::IcApply: return (const void*)fma::krylov_kernel<double, 8>;
        case KernelId::MixedRestart: return (const void*)fma::mixed_kernel<0>;
        case KernelId::MixedReliable: return (const void*)fma::mixed_kernel<1>;
        case KernelId::MixedCgs: return (const void*)fma::mixed_kernel<2>;
        case KernelId::BatchFp64: return (const void*)fma::batch_kernel<0>;
        case KernelId::BatchMixed: return (const void*)fma::batch_kernel<1>;
        default: return nullptr;  // Prec1 (TFLOWS_FP64 semantics) lives in krylov.cu only
    }
}

}  // namespace tflows
