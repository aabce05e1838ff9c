// Pressure-correction assembly on the GPU (Process/CalcPS.f90:49-202): the
// face loop that fills Aval through SidAij and Adia, Abou and the face mass
// fluxes, the right-hand side b, the density time-derivative source and the
// removal of the volume-weighted mean of b.
//
// The reference runs one sequential loop over faces that scatters into the
// diagonal and b of each face's two cells.  Here one thread per face computes
// everything that depends on the face alone (A12, the flux, the off-diagonal
// entries, Abou) and one thread per cell then adds its faces' contributions
// in increasing face order (repeating the whole sequence Nmat times, as the
// reference's `do m = 1, Nmat` does), from 0 as Aval(:) = 0 and b(:) = 0 do:
// every cell sees the same operands in the same order, so Aval, Abou, the
// fluxes and b before the mean removal are bit-identical to the sequential
// loop (built with --fmad=false).  The mean sum_c b(c) volume(c) /
// sum_c volume(c) is a deterministic tree reduction, not the reference's
// left-to-right sum, so b differs from the reference by the rounding of that
// one scalar.
#include "assembly_internal.h"
#include "internal.h"
#include "tflows_krylov.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace {

// What a face adds to its cells (set by the face pass, read by the cell pass).
enum : unsigned char { kDiag1 = 1, kB1 = 2, kCell2 = 4 };

struct FaceGeom {
    const double* sx;
    const double* sy;
    const double* sz;
    const double* dx;
    const double* dy;
    const double* dz;
    const double* f;
    const double* smdpn;  // |S|^2 / (S.d), fixed with the mesh
    const double* omf;    // 1.0 - f
};

struct CellFields {  // all over cells -NbC..NC, element c at [c + NbC]
    const double* vol;
    const double* vdiva;  // volume / Asave of this call
    const double* asave;
    const double* rho_n;
    const double* rho_o;
    const double* rho_oo;
    const double* u;
    const double* v;
    const double* w;
    const double* p;
    const double* px;
    const double* py;
    const double* pz;
    const int* type;
};

// Quantities the face loop recomputes per face although they depend on the
// mesh only (SMDPN, 1 - f) or on one cell only (volume / Asave) are formed
// once, with the same operations, so the face pass is bit-identical to the
// reference's and does a third of its FP64 work (the divides dominate).
__global__ void __launch_bounds__(kAsmBlock) geom_kernel(int NS, const double* __restrict__ sx,
                                                         const double* __restrict__ sy,
                                                         const double* __restrict__ sz,
                                                         const double* __restrict__ dx,
                                                         const double* __restrict__ dy,
                                                         const double* __restrict__ dz,
                                                         const double* __restrict__ f,
                                                         double* __restrict__ smdpn,
                                                         double* __restrict__ omf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NS; i += gridDim.x * blockDim.x) {
        smdpn[i] = (sx[i] * sx[i] + sy[i] * sy[i] + sz[i] * sz[i]) /
                   (sx[i] * dx[i] + sy[i] * dy[i] + sz[i] * dz[i]);
        omf[i] = 1.0 - f[i];
    }
}

__global__ void __launch_bounds__(kAsmBlock) vdiva_kernel(int n, const double* __restrict__ vol,
                                                          const double* __restrict__ asave,
                                                          double* __restrict__ q) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        q[i] = vol[i] / asave[i];
}

// One thread per face: CalcPS.f90:71-164 for face s = i + 1.
__global__ void __launch_bounds__(kAsmBlock) face_kernel(int NS, int NbC, const int* __restrict__ c1s,
                                                         const int* __restrict__ c2s,
                                                         const int* __restrict__ pos1,
                                                         const int* __restrict__ pos2, FaceGeom g,
                                                         CellFields F, double* __restrict__ abou,
                                                         double* __restrict__ flux,
                                                         double* __restrict__ slot_a,
                                                         double* __restrict__ slot_f,
                                                         unsigned char* __restrict__ slot_k) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NS; i += gridDim.x * blockDim.x) {
        const int c1 = c1s[i] + NbC, c2 = c2s[i];
        const int k2 = c2 + NbC;
        const double f = g.f[i], omf = g.omf[i];
        double A12 = 0.0, fl = 0.0;
        unsigned char kd = 0;
        const int t2 = c2 < 0 ? F.type[k2] : 0;
        if (c2 > 0 || (c2 < 0 && t2 == kBuffer)) {
            const double S = g.smdpn[i];
            const double Urs = f * F.rho_n[c1] * F.u[c1] + omf * F.rho_n[k2] * F.u[k2];
            const double Vrs = f * F.rho_n[c1] * F.v[c1] + omf * F.rho_n[k2] * F.v[k2];
            const double Wrs = f * F.rho_n[c1] * F.w[c1] + omf * F.rho_n[k2] * F.w[k2];
            A12 = 0.5 * S * (F.vdiva[c1] + F.vdiva[k2]);
            if (c2 > 0) {
                kd = kDiag1 | kB1 | kCell2;  // the cell pass sets Aval(SidAij(:, s)) = -A12
            } else {
                abou[k2] = -A12;
                kd = kDiag1 | kB1;
            }
            const double dPxi = .5 * (F.px[c1] + F.px[k2]) * g.dx[i];
            const double dPyi = .5 * (F.py[c1] + F.py[k2]) * g.dy[i];
            const double dPzi = .5 * (F.pz[c1] + F.pz[k2]) * g.dz[i];
            fl = (Urs * g.sx[i] + Vrs * g.sy[i] + Wrs * g.sz[i]) + A12 * (F.p[c1] - F.p[k2]) +
                 A12 * (dPxi + dPyi + dPzi);
        } else if (t2 == kInflow || t2 == kOutflow || t2 == kConvect) {
            const double Urs = f * F.rho_n[c1] * F.u[c1] + omf * F.rho_n[k2] * F.u[k2];
            const double Vrs = f * F.rho_n[c1] * F.v[c1] + omf * F.rho_n[k2] * F.v[k2];
            const double Wrs = f * F.rho_n[c1] * F.w[c1] + omf * F.rho_n[k2] * F.w[k2];
            fl = (Urs * g.sx[i] + Vrs * g.sy[i] + Wrs * g.sz[i]);
            kd = kB1;
            if (t2 != kInflow) {  // OUTFLOW / CONVECT add A12 to the diagonal
                // SMDPN * volume(c1) / Asave(c1): a product then a divide
                A12 = g.smdpn[i] * F.vol[c1] / F.asave[c1];
                kd |= kDiag1;
            }
        } else if (t2 == kPressure) {
            const double Urs = F.rho_n[c1] * F.u[c1];
            const double Vrs = F.rho_n[c1] * F.v[c1];
            const double Wrs = F.rho_n[c1] * F.w[c1];
            fl = (Urs * g.sx[i] + Vrs * g.sy[i] + Wrs * g.sz[i]);
            A12 = g.smdpn[i] * F.vol[c1] / F.asave[c1];
            kd = kB1 | kDiag1;
        }  // every other type (walls, symmetry): Flux(s) = 0, nothing added
        flux[i] = fl;
        // the face's entries in its cells' contribution lists
        const int p1 = pos1[i];
        slot_a[p1] = A12;
        slot_f[p1] = fl;
        slot_k[p1] = kd & (kDiag1 | kB1);
        if (c2 > 0) {
            const int p2 = pos2[i];
            slot_a[p2] = A12;
            slot_f[p2] = fl;
            slot_k[p2] = kCell2;
        }
    }
}

// One thread per cell c = i + 1: its faces' contributions in face order,
// Nmat times (CalcPS.f90:69-167), errmax (171-174), then the source
// (186-193) and this cell's terms of the two sums of the mean.  The face
// pass left each contribution in the cell's own list (entries cf_ptr[i] ..
// cf_ptr[i+1]-1, faces in increasing order), so the reads are contiguous.
// The cell also sets its row's off-diagonal entries Aval(SidAij) = -A12 in
// face order, so where two faces join the same cells (one entry) the later
// face's value stays, as in the reference.
__global__ void __launch_bounds__(kAsmBlock) cell_kernel(
    int NC, int NbC, int Nmat, double dt, const int* __restrict__ cf_ptr,
    const int* __restrict__ slot_face, const int* __restrict__ sid1,
    const int* __restrict__ sid2, const int* __restrict__ adia, const double* __restrict__ slot_a,
    const double* __restrict__ slot_f, const unsigned char* __restrict__ slot_k, CellFields F,
    double* __restrict__ aval, double* __restrict__ b, double* __restrict__ part_sum,
    double* __restrict__ part_vol, unsigned long long* __restrict__ errmax_bits) {
    __shared__ double s_sum[kAsmBlock / 32], s_vol[kAsmBlock / 32];
    double my_sum = 0.0, my_vol = 0.0;
    unsigned long long my_max = 0ull;
    for (int base = blockIdx.x * blockDim.x; base < NC; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        if (i < NC) {
            const int e0 = cf_ptr[i], e1 = cf_ptr[i + 1];
            double d = 0.0, bb = 0.0;
            bool diag = false;
            for (int m = 0; m < Nmat; ++m)
                for (int e = e0; e < e1; ++e) {
                    const unsigned char kd = slot_k[e];
                    if (kd & kCell2) {  // this cell is the face's c2
                        d = d + slot_a[e];
                        bb = bb + slot_f[e];
                        diag = true;
                    } else {
                        if (kd & kDiag1) {
                            d = d + slot_a[e];
                            diag = true;
                        }
                        if (kd & kB1) bb = bb - slot_f[e];
                    }
                }
            if (diag) aval[adia[i]] = d;
            for (int e = e0; e < e1; ++e) {
                const int sf = slot_face[e];
                const int o = sf >= 0 ? sid1[sf] : sid2[~sf];
                if (o >= 0) aval[o] = -slot_a[e];
            }
            my_max = max(my_max, (unsigned long long)__double_as_longlong(fabs(bb)));
            const int c = i + 1 + NbC;
            for (int m = 0; m < Nmat; ++m) {
                bb = bb - F.vol[c] / dt * (1.5 * F.rho_n[c] - 2.0 * F.rho_o[c] + 0.5 * F.rho_oo[c]);
                my_sum = my_sum + bb * F.vol[c];
                my_vol = my_vol + F.vol[c];
            }
            b[i] = bb;
        }
    }
    // block partial sums in a fixed order (deterministic)
    for (int o = 16; o > 0; o >>= 1) {
        my_sum += __shfl_down_sync(0xffffffffu, my_sum, o);
        my_vol += __shfl_down_sync(0xffffffffu, my_vol, o);
        my_max = max(my_max, __shfl_down_sync(0xffffffffu, my_max, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_sum[warp] = my_sum;
        s_vol[warp] = my_vol;
        atomicMax(errmax_bits, my_max);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += s_sum[w];
            v += s_vol[w];
        }
        part_sum[blockIdx.x] = a;
        part_vol[blockIdx.x] = v;
    }
}

// b(c) = b(c) - bc_sum / vol (CalcPS.f90:199-202); every thread sums the
// block partials in the same order.
__global__ void __launch_bounds__(kAsmBlock) mean_kernel(int NC, int nparts,
                                                         const double* __restrict__ part_sum,
                                                         const double* __restrict__ part_vol,
                                                         double* __restrict__ b,
                                                         double* __restrict__ sums) {
    __shared__ double s_shift;
    if (threadIdx.x == 0) {
        double a = 0.0, v = 0.0;
        for (int k = 0; k < nparts; ++k) {
            a += part_sum[k];
            v += part_vol[k];
        }
        s_shift = a / v;
        if (blockIdx.x == 0) {
            sums[0] = a;
            sums[1] = v;
        }
    }
    __syncthreads();
    const double shift = s_shift;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NC; i += gridDim.x * blockDim.x)
        b[i] = b[i] - shift;
}

template <typename T>
cudaError_t upload(T** dst, const T* src, size_t count) {
    cudaError_t e = cudaMalloc((void**)dst, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess && count)
        e = cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

int asm_fail(int status, const std::string& msg) { return tflows::report_status(status, msg); }

}  // namespace

extern "C" {

void tflows_assembly_destroy(tflows_assembly* a) {
    if (!a) return;
    cudaSetDevice(a->device);
    for (void* p : {(void*)a->c1, (void*)a->c2, (void*)a->sid1, (void*)a->sid2, (void*)a->adia,
                    (void*)a->type, (void*)a->cf_ptr, (void*)a->pos1, (void*)a->pos2,
                    (void*)a->geom, (void*)a->vol, (void*)a->slot_a, (void*)a->slot_f,
                    (void*)a->slot_k, (void*)a->parts, (void*)a->errmax, (void*)a->vdiva,
                    (void*)a->slot_face, (void*)a->bnd_ptr, (void*)a->bnd_face,
                    a->mom_rec, (void*)a->mom_cells, (void*)a->mom_err})
        if (p) cudaFree(p);
    if (a->ev0) cudaEventDestroy(a->ev0);
    if (a->ev1) cudaEventDestroy(a->ev1);
    delete a;
}

int tflows_assembly_create(tflows_assembly** out, int NC, int NbC, int NS, int NONZ,
                           const int* SideC, const int* SidAij, const int* Adia,
                           const int* TypeBC, const double* Sx, const double* Sy,
                           const double* Sz, const double* Dx, const double* Dy,
                           const double* Dz, const double* f, const double* volume, int device) {
    if (!out || NC <= 0 || NbC < 0 || NS < 0 || NONZ < 1 || !SideC || !SidAij || !Adia ||
        !TypeBC || !Sx || !Sy || !Sz || !Dx || !Dy || !Dz || !f || !volume)
        return asm_fail(TFLOWS_BAD_INPUT, "null argument or bad size");
    // host-side checks: every index the kernels follow stays in range
    std::vector<int> c1(NS), c2(NS), s1(NS), s2(NS);
    std::vector<int> deg(NC + 1, 0);
    for (int s = 0; s < NS; ++s) {
        c1[s] = SideC[3 * s + 1];
        c2[s] = SideC[3 * s + 2];
        if (c1[s] < 1 || c1[s] > NC || c2[s] == 0 || c2[s] > NC || c2[s] < -NbC)
            return asm_fail(TFLOWS_BAD_INPUT, "SideC out of range at face " + std::to_string(s + 1));
        if (c2[s] > 0) {
            s1[s] = SidAij[2 * s] - 1;
            s2[s] = SidAij[2 * s + 1] - 1;
            if (s1[s] < 0 || s1[s] >= NONZ || s2[s] < 0 || s2[s] >= NONZ)
                return asm_fail(TFLOWS_BAD_INPUT, "SidAij out of range at face " + std::to_string(s + 1));
            deg[c2[s]] += 1;
        } else {
            s1[s] = s2[s] = -1;
        }
        deg[c1[s]] += 1;
    }
    std::vector<int> adia(NC);
    for (int c = 0; c < NC; ++c) {
        adia[c] = Adia[c] - 1;
        if (adia[c] < 0 || adia[c] >= NONZ) return asm_fail(TFLOWS_BAD_INPUT, "Adia out of range");
    }
    // each cell's faces in increasing face order: the entry of face s in the
    // list of its c1 (pos1) and of its c2 (pos2, interior faces)
    std::vector<int> ptr(NC + 1, 0);
    for (int c = 1; c <= NC; ++c) ptr[c] = ptr[c - 1] + deg[c];
    std::vector<int> pos1(std::max(NS, 1)), pos2(std::max(NS, 1), -1);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    std::vector<int> slot_face(std::max(ptr[NC], 1));
    for (int s = 0; s < NS; ++s) {
        pos1[s] = fill[c1[s] - 1]++;
        slot_face[pos1[s]] = s;
        if (c2[s] > 0) {
            pos2[s] = fill[c2[s] - 1]++;
            slot_face[pos2[s]] = ~s;
        }
    }
    // each boundary cell's faces in increasing order
    std::vector<int> bptr(NbC + 1, 0);
    for (int s = 0; s < NS; ++s)
        if (c2[s] < 0) ++bptr[c2[s] + NbC + 1];
    for (int j = 0; j < NbC; ++j) bptr[j + 1] += bptr[j];
    std::vector<int> bface(std::max(bptr[NbC], 1));
    {
        std::vector<int> bf(bptr.begin(), bptr.end() - 1);
        for (int s = 0; s < NS; ++s)
            if (c2[s] < 0) bface[bf[c2[s] + NbC]++] = s;
    }
    const size_t nslot = std::max(ptr[NC], 1);
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess)
        return asm_fail(TFLOWS_NO_DEVICE, "cudaSetDevice failed");
    auto* a = new tflows_assembly();
    cudaGetDevice(&a->device);
    a->NC = NC;
    a->NbC = NbC;
    a->NS = NS;
    a->NONZ = NONZ;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, a->device);
    a->nblocks = std::max(1, std::min((NC + kAsmBlock - 1) / kAsmBlock, 8 * std::max(sms, 1)));
    std::vector<double> geom((size_t)9 * NS);
    const double* src[7] = {Sx, Sy, Sz, Dx, Dy, Dz, f};
    for (int k = 0; k < 7; ++k) std::memcpy(geom.data() + (size_t)k * NS, src[k], sizeof(double) * NS);
    cudaError_t e = upload(&a->c1, c1.data(), NS);
    if (e == cudaSuccess) e = upload(&a->c2, c2.data(), NS);
    if (e == cudaSuccess) e = upload(&a->sid1, s1.data(), NS);
    if (e == cudaSuccess) e = upload(&a->sid2, s2.data(), NS);
    if (e == cudaSuccess) e = upload(&a->adia, adia.data(), NC);
    if (e == cudaSuccess) e = upload(&a->type, TypeBC, (size_t)NbC + NC + 1);
    if (e == cudaSuccess) e = upload(&a->cf_ptr, ptr.data(), ptr.size());
    if (e == cudaSuccess) e = upload(&a->pos1, pos1.data(), pos1.size());
    if (e == cudaSuccess) e = upload(&a->pos2, pos2.data(), pos2.size());
    if (e == cudaSuccess) e = upload(&a->slot_face, slot_face.data(), slot_face.size());
    if (e == cudaSuccess) e = upload(&a->bnd_ptr, bptr.data(), bptr.size());
    if (e == cudaSuccess) e = upload(&a->bnd_face, bface.data(), bface.size());
    if (e == cudaSuccess) e = upload(&a->geom, geom.data(), geom.size());
    if (e == cudaSuccess) e = upload(&a->vol, volume, (size_t)NbC + NC + 1);
    if (e == cudaSuccess && NS > 0) {
        double* G = a->geom;
        const size_t ns = NS;
        geom_kernel<<<std::max(1, std::min((NS + kAsmBlock - 1) / kAsmBlock, 65535)), kAsmBlock>>>(
            NS, G, G + ns, G + 2 * ns, G + 3 * ns, G + 4 * ns, G + 5 * ns, G + 6 * ns, G + 7 * ns,
            G + 8 * ns);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaMalloc(&a->vdiva, sizeof(double) * ((size_t)NbC + NC + 1));
    if (e == cudaSuccess) e = cudaMalloc(&a->slot_a, sizeof(double) * nslot);
    if (e == cudaSuccess) e = cudaMalloc(&a->slot_f, sizeof(double) * nslot);
    if (e == cudaSuccess) e = cudaMalloc(&a->slot_k, nslot);
    if (e == cudaSuccess) e = cudaMalloc(&a->parts, sizeof(double) * (2 * a->nblocks + 2));
    if (e == cudaSuccess) e = cudaMalloc(&a->errmax, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreate(&a->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&a->ev1);
    if (e != cudaSuccess) {
        tflows_assembly_destroy(a);
        return asm_fail(TFLOWS_CUDA_ERROR, std::string("assembly set-up: ") + cudaGetErrorString(e));
    }
    *out = a;
    return asm_fail(TFLOWS_OK, "");
}

int tflows_calcps_assemble_device(tflows_assembly* a, int Nmat, double dt,
                                  const tflows_calcps_fields* in, double* aval, double* b,
                                  double* abou, double* flux, double* errmax, void* stream,
                                  double* seconds) {
    if (!a || !in || !aval || !b || !flux || (a->NbC > 0 && !abou))
        return asm_fail(TFLOWS_BAD_INPUT, "null argument");
    if (Nmat < 1) return asm_fail(TFLOWS_BAD_INPUT, "Nmat must be >= 1");
    const double* fl[11] = {in->rho_n, in->rho_o, in->rho_oo, in->u, in->v, in->w,
                            in->p, in->px, in->py, in->pz, in->asave};
    for (const double* p : fl)
        if (!p) return asm_fail(TFLOWS_BAD_INPUT, "null field");
    cudaSetDevice(a->device);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t ns = a->NS;
    FaceGeom g{a->geom,          a->geom + ns,     a->geom + 2 * ns,
               a->geom + 3 * ns, a->geom + 4 * ns, a->geom + 5 * ns,
               a->geom + 6 * ns, a->geom + 7 * ns, a->geom + 8 * ns};
    CellFields F{a->vol, a->vdiva, in->asave, in->rho_n, in->rho_o, in->rho_oo, in->u, in->v,
                 in->w, in->p, in->px, in->py, in->pz, a->type};
    cudaEventRecord(a->ev0, s);
    cudaError_t e = cudaMemsetAsync(aval, 0, sizeof(double) * a->NONZ, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->errmax, 0, sizeof(unsigned long long), s);
    const int ncell = a->NbC + a->NC + 1;
    if (e == cudaSuccess) {
        vdiva_kernel<<<std::max(1, std::min((ncell + kAsmBlock - 1) / kAsmBlock, 65535)), kAsmBlock,
                       0, s>>>(ncell, a->vol, in->asave, a->vdiva);
        e = cudaGetLastError();
    }
    const int fb = std::max(1, std::min((a->NS + kAsmBlock - 1) / kAsmBlock, 65535));
    if (e == cudaSuccess && a->NS > 0) {
        face_kernel<<<fb, kAsmBlock, 0, s>>>(a->NS, a->NbC, a->c1, a->c2, a->pos1, a->pos2, g,
                                             F, abou, flux, a->slot_a, a->slot_f, a->slot_k);
        e = cudaGetLastError();
    }
    double* ps = a->parts;
    double* pv = a->parts + a->nblocks;
    double* tot = a->parts + 2 * a->nblocks;
    if (e == cudaSuccess) {
        cell_kernel<<<a->nblocks, kAsmBlock, 0, s>>>(a->NC, a->NbC, Nmat, dt, a->cf_ptr,
                                                     a->slot_face, a->sid1, a->sid2, a->adia,
                                                     a->slot_a, a->slot_f, a->slot_k, F, aval, b,
                                                     ps, pv, a->errmax);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        mean_kernel<<<a->nblocks, kAsmBlock, 0, s>>>(a->NC, a->nblocks, ps, pv, b, tot);
        e = cudaGetLastError();
    }
    cudaEventRecord(a->ev1, s);
    unsigned long long bits = 0;
    if (e == cudaSuccess && errmax)
        e = cudaMemcpyAsync(&bits, a->errmax, sizeof(bits), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && (errmax || seconds)) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return asm_fail(TFLOWS_CUDA_ERROR, std::string("assembly: ") + cudaGetErrorString(e));
    if (errmax) std::memcpy(errmax, &bits, sizeof(double));
    if (seconds) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a->ev0, a->ev1);
        *seconds = ms * 1e-3;
    }
    return asm_fail(TFLOWS_OK, "");
}

}  // extern "C"
