// Momentum assembly on the GPU for one component Ui of rho*u
// (Process/NewUVW.f90:138-499, with the blended face values of
// Process/ConvScheme.f90 and the bounds of Process/CalMinMax.f90).
//
// The reference runs two sequential face loops that scatter into the sums of
// each face's two cells (convection C and the upwind X, then the cross
// diffusion X, the diagonal and off-diagonal entries of Aval, b on boundary
// faces and Abou) and then cell loops for the explicit, inertial, pressure
// and under-relaxation terms.  Here:
//   bounds pass  one thread per cell: rhoUi = Rho%n * Ui%n and, when a
//                material blends, PHImax/PHImin over the cell's faces
//                (CalMinMax), in increasing face order;
//   face pass    one thread per face: the face value rhoUiS (central, or
//                ConvScheme's), the products Flux_u*rhoUiS and
//                Flux_u*rhoUi(upwind), Fex, Fim, A12, A21, D12, D21 and the
//                boundary term, into one record per face;
//   cell pass    one thread per cell: its faces' records in increasing face
//                order, exactly as the reference's loops add them, then the
//                per-cell terms; it also owns its row's off-diagonal entries
//                of Aval (a face adds to the entry of each of its two rows),
//                so two faces between the same cells add in face order too.
// Every sum sees the reference's operands in the reference's order (built
// with --fmad=false), so Aval, b, Abou and Asave are bit-identical to it.
#include "assembly_internal.h"
#include "internal.h"
#include "tflows_krylov.h"

#include <algorithm>
#include <string>

namespace {

// Process/IniPar.f90:22-49
enum : int {
    kCN = 2, kFI = 3, kLIN = 4, kPAR = 5, kYES = 10, kNO = 11, kCDS = 20, kQUICK = 21,
    kLUDS = 22, kMINMOD = 23, kSMART = 24, kAVL_SMART = 25, kSUPERBEE = 26, kGAMMA = 27
};

// input errors the kernels find (bits of *mom_err)
enum : int { kErrBlend = 1, kErrMaterial = 2 };

// what the cell pass does with a face (MomRec::flags)
enum : int {
    kUpwind = 1,       // the upwind sums X include this face (BLEND_TEM)
    kMatrix = 2,       // DIFFUS is CN or FI: Aval, b, Abou terms
    kShift = 2,        // boundary class in bits 2..4:
    kInterior = 0,     //   both cells interior
    kWallLike = 1,     //   WALL, CONVECT, INFLOW, WALLFL: diagonal + A21 + D21, b term
    kOutflowB = 2,     //   OUTFLOW: diagonal + A21, b term
    kBufferB = 3,      //   BUFFER: diagonal + A21 + D21 (Abou by the boundary cell)
    kOtherB = 4        //   anything else: no matrix term
};

struct __align__(16) MomRec {
    double t;         // Flux_u * rhoUiS
    double u;         // Flux_u * rhoUi(upwind cell)
    double fex, fim;  // exact and implicit diffusive flux of the cross terms
    double a12, a21, d12, d21;
    double bv;        // b(c1) term of a boundary face
    int flags;
    int pad;
};

struct MomCells {  // over cells -NbC..NC, element c at [c + NbC]
    const int* material;
    const double *rho_n, *rho_o, *rho_oo, *ui_n, *ui_o, *ui_oo;
    const double *duidi, *duidj, *duidk, *dujdi, *dukdi, *dujdj, *dukdk;
    const double *pi, *source, *vol;
    const int* type;
};

struct MomFaces {
    const double *flux_u, *flux, *ff, *scoef, *f, *omf;
    const double *si, *sj, *sk, *di, *dj, *dk;
};

struct MomMats {
    const int *blend, *blend_tem;
    const double* urfc;
    int nmat;
};

struct MomScalars {
    int var, moin, convec, cross, diffus, inert;
    double visc, dt, urf;
};

// MIN / MAX: the first argument unless a later one is strictly smaller /
// larger, as the statement-by-statement execution of the reference's text
// gives (Fortran leaves equal signed zeros and NaN to the compiler).
__device__ __forceinline__ double min2(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double max2(double a, double b) { return b > a ? b : a; }

__device__ __forceinline__ int material_code(const int* tab, int nmat, int m, int* err) {
    if (m < 1 || m > nmat) {
        atomicOr(err, kErrMaterial);
        return kNO;
    }
    return tab[m - 1];
}

// ConvScheme.f90:52-135 for face i (0-based); phi, dphid* over cells at
// [c + NbC].  Returns false for a code the routine does not handle.
__device__ bool conv_scheme(double& phis, int i, int c1, int c2, int NbC, const MomFaces& F,
                            const MomCells& K, const double* __restrict__ phi,
                            const double* __restrict__ pmax, const double* __restrict__ pmin,
                            int blenda) {
    double fj, sign;
    int C, D;
    const double fl = F.flux[i];
    if (fl > 0.0) {
        fj = 1.0 - F.f[i];
        C = c1;
        D = c2;
        sign = +1.0;
    } else {
        fj = F.f[i];
        C = c2;
        D = c1;
        sign = -1.0;
    }
    const int kc = C + NbC, kd = D + NbC;
    const double grad = K.duidi[kc] * F.di[i] + K.duidj[kc] * F.dj[i] + K.duidk[kc] * F.dk[i];
    const double phiC = phi[kc], phiD = phi[kd];
    if (blenda == kGAMMA) {
        // the value ConvScheme forms before its GAMMA block is overwritten
        // in every branch of it (:111-133)
        const double Beta = 0.1;
        const double den = 2.0 * grad;
        const double PhiUstar = fl > 0.0 ? 1.0 - (phiD - phiC) / den : 1.0 + (phiD - phiC) / den;
        const double GammaC = PhiUstar / Beta;
        if (PhiUstar < Beta && PhiUstar > 0.0)
            phis = (1.0 - GammaC * (1.0 - F.f[i])) * phiC + GammaC * (1.0 - F.f[i]) * phiD;
        else if (PhiUstar < 1.0 && PhiUstar >= Beta)
            phis = F.f[i] * phiC + (1.0 - F.f[i]) * phiD;
        else
            phis = phiC;
        return true;
    }
    if (blenda == kYES) return true;
    const double PhiUstar = fl > 0.0 ? phiD - 2.0 * grad : phiD + 2.0 * grad;
    const double PhiU = max2(pmin[kc], min2(PhiUstar, pmax[kc]));
    double rj = (phiC - PhiU) / (phiD - phiC + 1.0e-16);
    const double gD = 0.5 * fj * (1.0 + fj);
    const double gU = 0.5 * fj * (1.0 - fj);
    double Phij;
    switch (blenda) {
        case kCDS:
            Phij = fj;
            break;
        case kQUICK: {
            rj = (phiC - PhiU) / (phiD - phiC + 1.0e-12);
            const double alfa = 0.0;
            Phij = (gD - alfa) + (gU + alfa) * rj;
            break;
        }
        case kLUDS: {
            const double alfa = 0.5 * fj * (1.0 + fj);
            Phij = (gD - alfa) + (gU + alfa) * rj;
            break;
        }
        case kMINMOD:
            Phij = fj * max2(0.0, min2(rj, 1.0));
            break;
        case kSMART: {
            const double beta1 = 3.0, beta2 = 1.0;
            Phij = max2(0.0, min2(min2((beta1 - 1.0) * rj, gD + gU * rj), beta2));
            break;
        }
        case kAVL_SMART: {
            const double beta1 = 1.0 + fj * (2.0 + fj);
            const double beta2 = fj * (2.0 - fj);
            Phij = max2(0.0, min2(min2((beta1 - 1.0) * rj, gD + gU * rj), beta2));
            break;
        }
        case kSUPERBEE:
            Phij = 0.5 * max2(max2(0.0, min2(2.0 * rj, 1.0)), min2(rj, 2.0));
            break;
        default:
            return false;
    }
    phis = phiC + Phij * sign * (phi[c2 + NbC] - phi[c1 + NbC]);
    return true;
}

// rhoUi over all cells, and CalMinMax (CalMinMax.f90:20-36) when any
// material blends.
__global__ void __launch_bounds__(kAsmBlock) mom_bounds_kernel(
    int NC, int NbC, const int* __restrict__ c1s, const int* __restrict__ c2s,
    const int* __restrict__ cf_ptr, const int* __restrict__ slot_face,
    const int* __restrict__ bnd_ptr, const int* __restrict__ bnd_face, MomCells K, MomMats Mt,
    double* __restrict__ rhoui, double* __restrict__ pmax, double* __restrict__ pmin) {
    bool blends = false;
    for (int m = 0; m < Mt.nmat; ++m) blends |= Mt.blend[m] != kNO;
    const int ncell = NbC + NC + 1;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
        const double own = K.rho_n[k] * K.ui_n[k];
        rhoui[k] = own;
        if (!blends) continue;
        double hi = own, lo = own;
        if (k > NbC) {  // interior cell: every face with an interior or BUFFER neighbour
            for (int e = cf_ptr[k - NbC - 1]; e < cf_ptr[k - NbC]; ++e) {
                const int sf = slot_face[e];
                const int s = sf >= 0 ? sf : ~sf;
                const int c2 = c2s[s];
                if (c2 > 0 || K.type[c2 + NbC] == kBuffer) {
                    const int o = (sf >= 0 ? c2 : c1s[s]) + NbC;
                    const double v = K.rho_n[o] * K.ui_n[o];
                    hi = max2(hi, v);
                    lo = min2(lo, v);
                }
            }
        } else if (k < NbC && K.type[k] == kBuffer) {
            for (int e = bnd_ptr[k]; e < bnd_ptr[k + 1]; ++e) {
                const int o = c1s[bnd_face[e]] + NbC;
                const double v = K.rho_n[o] * K.ui_n[o];
                hi = max2(hi, v);
                lo = min2(lo, v);
            }
        }
        pmax[k] = hi;
        pmin[k] = lo;
    }
}

// One thread per face s = i + 1: NewUVW.f90:205-236 and 276-416.
__global__ void __launch_bounds__(kAsmBlock) mom_face_kernel(
    int NS, int NbC, const int* __restrict__ c1s, const int* __restrict__ c2s, MomFaces F,
    MomCells K, MomMats Mt, MomScalars P, const double* __restrict__ rhoui,
    const double* __restrict__ pmax, const double* __restrict__ pmin, MomRec* __restrict__ rec,
    int* __restrict__ err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NS; i += gridDim.x * blockDim.x) {
        const int c1 = c1s[i], c2 = c2s[i];
        const int k1 = c1 + NbC, k2 = c2 + NbC;
        const int m1 = K.material[k1], m2 = K.material[k2];
        const int bl1 = material_code(Mt.blend, Mt.nmat, m1, err);
        const int bl2 = material_code(Mt.blend, Mt.nmat, m2, err);
        const int bt1 = material_code(Mt.blend_tem, Mt.nmat, m1, err);
        const int bt2 = material_code(Mt.blend_tem, Mt.nmat, m2, err);
        MomRec r;
        int flags = 0;
        // convection (:208-235)
        double rhoUiS = F.f[i] * rhoui[k1] + F.omf[i] * rhoui[k2];
        const bool blend = bl1 != kNO || bl2 != kNO;
        if (blend && !conv_scheme(rhoUiS, i, c1, c2, NbC, F, K, rhoui, pmax, pmin,
                                  bl1 > bl2 ? bl1 : bl2))
            atomicOr(err, kErrBlend);
        const double fu = F.flux_u[i];
        r.t = fu * rhoUiS;
        r.u = 0.0;
        if (bt1 != kNO || bt2 != kNO) {
            flags |= kUpwind;
            r.u = fu < 0 ? fu * rhoui[k2] : fu * rhoui[k1];
        }
        // diffusion (:277-331)
        const double ff = F.ff[i], omff = 1.0 - F.ff[i];
        const double RhoS = ff * K.rho_n[k1] + omff * K.rho_n[k2];
        const double VISeff = P.moin == 4 ? P.visc * RhoS : P.visc;
        const double dUidiS = ff * K.duidi[k1] + omff * K.duidi[k2];
        const double dUidjS = ff * K.duidj[k1] + omff * K.duidj[k2];
        const double dUidkS = ff * K.duidk[k1] + omff * K.duidk[k2];
        const double dUjdiS = ff * K.dujdi[k1] + omff * K.dujdi[k2];
        const double dUkdiS = ff * K.dukdi[k1] + omff * K.dukdi[k2];
        const double dUjdjS = ff * K.dujdj[k1] + omff * K.dujdj[k2];
        const double dUkdkS = ff * K.dukdk[k1] + omff * K.dukdk[k2];
        r.fex = VISeff * (4.0 / 3.0 * dUidiS * F.si[i] + (dUidjS + dUjdiS) * F.sj[i] +
                          (dUidkS + dUkdiS) * F.sk[i] - 2.0 / 3.0 * (dUjdjS + dUkdkS) * F.si[i]);
        const double A0 = VISeff * F.scoef[i];
        r.fim = A0 * (dUidiS * F.di[i] + dUidjS * F.dj[i] + dUidkS * F.dk[i]);
        // matrix coefficients (:347-414)
        double A12 = 0.0, A21 = 0.0, D12 = 0.0, D21 = 0.0;
        r.bv = 0.0;
        if (P.diffus == kCN || P.diffus == kFI) {
            flags |= kMatrix;
            if (P.diffus == kFI) {
                D12 = D12 + A0 / K.rho_n[k2];
                D21 = D21 + A0 / K.rho_n[k1];
            }
            if (blend) {
                A12 = A12 - min2(fu, 0.0);
                A21 = A21 + max2(fu, 0.0);
            }
            int cls = kInterior;
            if (c2 < 0) {
                const int t = K.type[k2];
                if (t == kWall || t == kConvect || t == kInflow || t == kWallfl) {
                    cls = kWallLike;
                    r.bv = (A12 + D12) * rhoui[k2];
                } else if (t == kOutflow) {
                    cls = kOutflowB;
                    r.bv = (A12)*rhoui[k2];
                } else if (t == kBuffer) {
                    cls = kBufferB;
                } else {
                    cls = kOtherB;
                }
            }
            flags |= cls << kShift;
        }
        r.a12 = A12;
        r.a21 = A21;
        r.d12 = D12;
        r.d21 = D21;
        r.flags = flags;
        r.pad = 0;
        rec[i] = r;
    }
}

// One thread per cell: interior cell c = k - NbC takes its faces' records in
// increasing face order (NewUVW.f90:205-499); boundary cell k < NbC sets
// Abou from its last BUFFER face (:405), 0 otherwise (:146).
__global__ void __launch_bounds__(kAsmBlock) mom_cell_kernel(
    int NC, int NbC, const int* __restrict__ cf_ptr, const int* __restrict__ slot_face,
    const int* __restrict__ bnd_ptr, const int* __restrict__ bnd_face,
    const int* __restrict__ sid1, const int* __restrict__ sid2, const int* __restrict__ adia,
    const MomRec* __restrict__ rec, MomCells K, MomMats Mt, MomScalars P,
    const double* __restrict__ rhoui, double* __restrict__ aval, double* __restrict__ b,
    double* __restrict__ abou, double* __restrict__ asave, int* __restrict__ err) {
    const int ncell = NbC + NC + 1;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
        if (k < NbC) {
            double ab = 0.0;
            if (K.type[k] == kBuffer)
                for (int e = bnd_ptr[k]; e < bnd_ptr[k + 1]; ++e) {
                    const MomRec& r = rec[bnd_face[e]];
                    if (r.flags & kMatrix) ab = -r.a12 - r.d12;
                }
            abou[k] = ab;
            continue;
        }
        if (k == NbC) continue;  // there is no cell 0
        const int i = k - NbC - 1;
        const int e0 = cf_ptr[i], e1 = cf_ptr[i + 1];
        // convection and upwind sums (:205-236)
        double C = 0.0, X = 0.0;
        for (int e = e0; e < e1; ++e) {
            const int sf = slot_face[e];
            const MomRec& r = rec[sf >= 0 ? sf : ~sf];
            if (sf >= 0) {
                C = C - r.t;
                if (r.flags & kUpwind) X = X - r.u;
            } else {
                C = C + r.t;
                if (r.flags & kUpwind) X = X + r.u;
            }
        }
        double bb = 0.0;
        if (P.convec == kFI) {
            const int m = K.material[k];
            double urfc = 0.0;
            if (m < 1 || m > Mt.nmat)
                atomicOr(err, kErrMaterial);
            else
                urfc = Mt.urfc[m - 1];
            bb = bb + urfc * (C - X);
        }
        // cross diffusion, Aval and boundary b terms (:276-416)
        X = 0.0;
        double d = 0.0;
        for (int e = e0; e < e1; ++e) {
            const int sf = slot_face[e];
            const int s = sf >= 0 ? sf : ~sf;
            const MomRec& r = rec[s];
            if (sf >= 0) {
                X = X + r.fex - r.fim;
                if (r.flags & kMatrix) {
                    const int cls = (r.flags >> kShift) & 7;
                    if (cls == kInterior) {
                        d = d + r.a21 + r.d21;
                        const int o = sid1[s];
                        aval[o] = aval[o] - r.a12 - r.d12;
                    } else if (cls == kWallLike) {
                        d = d + r.a21 + r.d21;
                        bb = bb + r.bv;
                    } else if (cls == kOutflowB) {
                        d = d + r.a21;
                        bb = bb + r.bv;
                    } else if (cls == kBufferB) {
                        d = d + r.a21 + r.d21;
                    }
                }
            } else {
                X = X - r.fex + r.fim;
                if (r.flags & kMatrix) {
                    d = d + r.a12 + r.d12;
                    const int o = sid2[s];
                    aval[o] = aval[o] - r.a21 - r.d21;
                }
            }
        }
        if (P.cross == kFI) bb = bb + X;
        // inertial terms (:451-460)
        const double vol = K.vol[k];
        if (P.inert == kLIN) {
            d = d + vol / P.dt;
            bb = bb + vol / P.dt * K.rho_o[k] * K.ui_o[k] + K.source[k] * vol;
        } else if (P.inert == kPAR) {
            d = d + 1.5 * vol / P.dt;
            bb = bb + 2.0 * vol / P.dt * K.rho_o[k] * K.ui_o[k] -
                 0.5 * vol / P.dt * K.rho_oo[k] * K.ui_oo[k] + K.source[k] * vol;
        }
        bb = bb - K.pi[k] * vol;  // :488
        // under-relaxation (:497-499)
        if (P.var == 1 && asave) asave[i] = d;
        bb = bb + d * (1.0 - P.urf) * rhoui[k] / P.urf;
        aval[adia[i]] = d / P.urf;
        b[i] = bb;
    }
}

int mom_fail(int status, const std::string& msg) { return tflows::report_status(status, msg); }

}  // namespace

extern "C" int tflows_newuvw_assemble_device(tflows_assembly* a, const tflows_newuvw_params* p,
                                             const tflows_newuvw_fields* in, double* aval,
                                             double* b, double* abou, double* asave,
                                             double* rhoui, void* stream, double* seconds) {
    if (!a || !p || !in || !aval || !b || (a->NbC > 0 && !abou))
        return mom_fail(TFLOWS_BAD_INPUT, "null argument");
    if (p->var < 1 || p->var > 3) return mom_fail(TFLOWS_BAD_INPUT, "var must be 1, 2 or 3");
    if (p->nmat < 1) return mom_fail(TFLOWS_BAD_INPUT, "nmat must be >= 1");
    const void* req[] = {in->material, in->rho_n, in->rho_o, in->ui_n, in->ui_o, in->duidi,
                         in->duidj, in->duidk, in->dujdi, in->dukdi, in->dujdj, in->dukdk,
                         in->pi, in->source, in->flux_u, in->flux, in->ff, in->blend,
                         in->blend_tem, in->urfc};
    for (const void* q : req)
        if (!q) return mom_fail(TFLOWS_BAD_INPUT, "null field");
    if (p->inert == kPAR && (!in->rho_oo || !in->ui_oo))
        return mom_fail(TFLOWS_BAD_INPUT, "three time levels need Rho % oo and Ui % oo");
    cudaSetDevice(a->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int ncell = a->NbC + a->NC + 1;
    cudaError_t e = cudaSuccess;
    if (!a->mom_rec) {
        e = cudaMalloc(&a->mom_rec, sizeof(MomRec) * (size_t)std::max(a->NS, 1));
        if (e == cudaSuccess) e = cudaMalloc(&a->mom_cells, sizeof(double) * 3 * (size_t)ncell);
        if (e == cudaSuccess) e = cudaMalloc(&a->mom_err, sizeof(int));
        if (e != cudaSuccess) {
            for (void** q : {&a->mom_rec, (void**)&a->mom_cells, (void**)&a->mom_err})
                if (*q) {
                    cudaFree(*q);
                    *q = nullptr;
                }
            return mom_fail(TFLOWS_CUDA_ERROR, std::string("momentum set-up: ") + cudaGetErrorString(e));
        }
    }
    const size_t ns = a->NS;
    const double* G = a->geom;
    // Processor.f90:314-340: (Si, Sj, Sk, Di, Dj, Dk) of each component
    static const int perm[3][6] = {{0, 1, 2, 3, 4, 5}, {1, 0, 2, 4, 3, 5}, {2, 0, 1, 5, 3, 4}};
    const int* q = perm[p->var - 1];
    MomFaces F{in->flux_u,  in->flux,    in->ff,      in->scoef ? in->scoef : G + 7 * ns,
               G + 6 * ns,  G + 8 * ns,  G + q[0] * ns, G + q[1] * ns,
               G + q[2] * ns, G + q[3] * ns, G + q[4] * ns, G + q[5] * ns};
    MomCells K{in->material, in->rho_n, in->rho_o,  in->rho_oo, in->ui_n,  in->ui_o,
               in->ui_oo,    in->duidi, in->duidj,  in->duidk,  in->dujdi, in->dukdi,
               in->dujdj,    in->dukdk, in->pi,     in->source, a->vol,    a->type};
    // the three-level arrays are read only with INERT == PAR
    if (!K.rho_oo) K.rho_oo = K.rho_o;
    if (!K.ui_oo) K.ui_oo = K.ui_o;
    MomMats Mt{in->blend, in->blend_tem, in->urfc, p->nmat};
    MomScalars P{p->var, p->moin_problem, p->convec, p->cross, p->diffus, p->inert,
                 p->visc, p->dt, p->urf};
    double* ru = rhoui ? rhoui : a->mom_cells;
    double* pmax = a->mom_cells + ncell;
    double* pmin = a->mom_cells + 2 * (size_t)ncell;
    auto* rec = (MomRec*)a->mom_rec;
    const int cb = std::max(1, std::min((ncell + kAsmBlock - 1) / kAsmBlock, 65535));
    const int fb = std::max(1, std::min((a->NS + kAsmBlock - 1) / kAsmBlock, 65535));
    cudaEventRecord(a->ev0, s);
    e = cudaMemsetAsync(aval, 0, sizeof(double) * a->NONZ, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->mom_err, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        mom_bounds_kernel<<<cb, kAsmBlock, 0, s>>>(a->NC, a->NbC, a->c1, a->c2, a->cf_ptr,
                                                   a->slot_face, a->bnd_ptr, a->bnd_face, K, Mt,
                                                   ru, pmax, pmin);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && a->NS > 0) {
        mom_face_kernel<<<fb, kAsmBlock, 0, s>>>(a->NS, a->NbC, a->c1, a->c2, F, K, Mt, P, ru,
                                                 pmax, pmin, rec, a->mom_err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        mom_cell_kernel<<<cb, kAsmBlock, 0, s>>>(a->NC, a->NbC, a->cf_ptr, a->slot_face,
                                                 a->bnd_ptr, a->bnd_face, a->sid1, a->sid2,
                                                 a->adia, rec, K, Mt, P, ru, aval, b, abou,
                                                 asave, a->mom_err);
        e = cudaGetLastError();
    }
    cudaEventRecord(a->ev1, s);
    int bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, a->mom_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return mom_fail(TFLOWS_CUDA_ERROR, std::string("momentum assembly: ") + cudaGetErrorString(e));
    if (bad & kErrMaterial) return mom_fail(TFLOWS_BAD_INPUT, "material index outside 1..nmat");
    if (bad & kErrBlend)
        return mom_fail(TFLOWS_BAD_INPUT,
                        "a face joins a material blending with YES and one with NO: ConvScheme "
                        "has no value for that code");
    if (seconds) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a->ev0, a->ev1);
        *seconds = ms * 1e-3;
    }
    return mom_fail(TFLOWS_OK, "");
}
