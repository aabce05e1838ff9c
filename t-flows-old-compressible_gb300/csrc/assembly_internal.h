// Device-resident mesh data shared by the pressure-correction assembly
// (assembly.cu) and the momentum assembly (momentum.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

constexpr int kAsmBlock = 256;

// Library/allp_mod.f90:16-24
enum : int {
    kInflow = 1,
    kWall = 2,
    kOutflow = 3,
    kConvect = 5,
    kWallfl = 6,
    kBuffer = 11,
    kPressure = 12
};

struct tflows_assembly {
    int device = 0;
    int NC = 0, NbC = 0, NS = 0, NONZ = 0;
    int nblocks = 0;
    int *c1 = nullptr, *c2 = nullptr, *sid1 = nullptr, *sid2 = nullptr;
    int *adia = nullptr, *type = nullptr, *cf_ptr = nullptr, *pos1 = nullptr, *pos2 = nullptr;
    // each interior cell's faces in increasing order: entry e holds the face
    // (0-based) where the cell is the face's c1, its complement ~s where it
    // is the face's c2 (entries cf_ptr[i] .. cf_ptr[i+1]-1 of cell i + 1)
    int* slot_face = nullptr;
    // each boundary cell's faces in increasing order (cell c = j - NbC at
    // bnd_ptr[j] .. bnd_ptr[j+1]-1)
    int *bnd_ptr = nullptr, *bnd_face = nullptr;
    double* geom = nullptr;  // Sx Sy Sz Dx Dy Dz f SMDPN (1-f), NS each
    double* vol = nullptr;   // -NbC..NC
    double* vdiva = nullptr; // volume / Asave of the current call, -NbC..NC
    double* slot_a = nullptr;  // per (cell, face): A12 and the flux the face adds
    double* slot_f = nullptr;
    unsigned char* slot_k = nullptr;
    double* parts = nullptr;  // 2 * nblocks partial sums, then the two totals
    unsigned long long* errmax = nullptr;
    // momentum assembly, allocated on its first call
    void* mom_rec = nullptr;        // one record per face
    double* mom_cells = nullptr;    // rhoUi, PHImax, PHImin over -NbC..NC
    int* mom_err = nullptr;         // input errors found on the device
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace tflows {
int report_status(int status, const std::string& msg);
}
