// T-FlowS mesh files and the compressed-row layout built from them.
//
// tflows_mesh_read loads the two unformatted Fortran files the solver reads
// at start-up, NAME.cns (Process/CnsLoa.f90: sizes, materials, the face list
// SideC, boundary marks, copy cells) and NAME.geo (Library/GeoLoa.f90: cell
// centres, volumes, face vectors Sx..Sz, centre-to-centre vectors Dx..Dz,
// interpolation factors f, face centres), record by record in the order
// those subroutines read them.  The files are written by gfortran's
// sequential unformatted I/O: each record is framed by a 4-byte length
// before and after it, a record over 2 GiB is split into subrecords whose
// leading length is negative while more follow; INTEGER is 4 bytes and REAL
// 8 bytes (-fdefault-real-8, Process/Makefile), native byte order.
//
// tflows_topolm builds the solver's matrix layout from the face list as
// Process/TopolM.f90:24-98 does: one row per cell holding the cell and its
// face neighbours, columns ascending, the diagonal position Adia and, per
// interior face, the positions SidAij of its two off-diagonal entries.
#include "tflows_krylov.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace tflows {
int report_status(int status, const std::string& msg);
}

namespace {

struct Reader {
    FILE* f = nullptr;
    std::string path;
    std::string err;

    bool open(const char* p) {
        path = p;
        f = std::fopen(p, "rb");
        if (!f) err = "cannot open " + path;
        return f != nullptr;
    }
    ~Reader() {
        if (f) std::fclose(f);
    }
    // One logical record (all its subrecords) into `out`.
    bool record(std::vector<char>& out) {
        out.clear();
        while (true) {
            int32_t head = 0, tail = 0;
            if (std::fread(&head, 4, 1, f) != 1) {
                err = path + ": unexpected end of file";
                return false;
            }
            const bool more = head < 0;
            const int64_t len = more ? -(int64_t)head : head;
            const size_t at = out.size();
            out.resize(at + (size_t)len);
            if (len && std::fread(out.data() + at, 1, (size_t)len, f) != (size_t)len) {
                err = path + ": truncated record";
                return false;
            }
            if (std::fread(&tail, 4, 1, f) != 1 || (tail != head && tail != -head && -tail != head)) {
                err = path + ": record length markers disagree";
                return false;
            }
            if (!more) return true;
        }
    }
    template <typename T>
    bool array(T* dst, int64_t count, const char* what) {
        std::vector<char> buf;
        if (!record(buf)) return false;
        if ((int64_t)buf.size() != count * (int64_t)sizeof(T)) {
            err = path + ": record '" + what + "' holds " + std::to_string(buf.size()) +
                  " bytes, expected " + std::to_string(count * (int64_t)sizeof(T));
            return false;
        }
        if (count) std::memcpy(dst, buf.data(), buf.size());
        return true;
    }
    bool scalar(int* v, const char* what) { return array(v, 1, what); }
    // a record written as (a(c), c=-1,-n,-1): element -k at dst[n - k]
    template <typename T>
    bool reversed(T* dst_at_minus_n, int n, const char* what) {
        std::vector<T> tmp((size_t)std::max(n, 0));
        if (!array(tmp.data(), n, what)) return false;
        for (int k = 1; k <= n; ++k) dst_at_minus_n[n - k] = tmp[k - 1];
        return true;
    }
};

void free_mesh(tflows_mesh* m) {
    if (!m) return;
    for (void* p : {(void*)m->material, (void*)m->SideC, (void*)m->bcmark, (void*)m->CopyC,
                    (void*)m->xc, (void*)m->yc, (void*)m->zc, (void*)m->volume, (void*)m->delta,
                    (void*)m->WallDs, (void*)m->Sx, (void*)m->Sy, (void*)m->Sz, (void*)m->Dx,
                    (void*)m->Dy, (void*)m->Dz, (void*)m->f, (void*)m->xsp, (void*)m->ysp,
                    (void*)m->zsp})
        std::free(p);
    std::free(m);
}

template <typename T>
T* alloc(int64_t n) {
    return (T*)std::calloc((size_t)std::max<int64_t>(n, 1), sizeof(T));
}

}  // namespace

extern "C" {

void tflows_mesh_free(tflows_mesh* m) { free_mesh(m); }

int tflows_mesh_read(const char* cns_path, const char* geo_path, tflows_mesh** out) {
    using tflows::report_status;
    if (!cns_path || !out) return report_status(TFLOWS_BAD_INPUT, "null argument");
    *out = nullptr;
    Reader r;
    if (!r.open(cns_path)) return report_status(TFLOWS_BAD_INPUT, r.err);
    auto* m = (tflows_mesh*)std::calloc(1, sizeof(tflows_mesh));
    auto bad = [&](const std::string& msg) {
        free_mesh(m);
        return report_status(TFLOWS_BAD_INPUT, msg);
    };
    // Process/CnsLoa.f90:22-45
    if (!r.scalar(&m->NC, "NC") || !r.scalar(&m->NbC, "NbC") || !r.scalar(&m->NS, "NS") ||
        !r.scalar(&m->NSsh, "NSsh") || !r.scalar(&m->Nmat, "Nmat"))
        return bad(r.err);
    const int NC = m->NC, NbC = m->NbC, NS = m->NS;
    if (NC < 0 || NbC < 0 || NS < 0) return bad(std::string(cns_path) + ": negative sizes");
    m->material = alloc<int>((int64_t)NbC + NC + 1);
    m->SideC = alloc<int>(3 * (int64_t)NS);
    m->bcmark = alloc<int>(NbC);
    m->CopyC = alloc<int>(NbC);
    std::vector<int> side((size_t)std::max(NS, 1));
    bool ok = r.array(m->material + NbC + 1, NC, "material(1:NC)") &&
              r.reversed(m->material, NbC, "material(-1:-NbC)");
    for (int k = 0; k < 3 && ok; ++k) {
        ok = r.array(side.data(), NS, "SideC");
        for (int s = 0; s < NS && ok; ++s) m->SideC[3 * s + k] = side[s];
    }
    ok = ok && r.reversed(m->bcmark, NbC, "bcmark") && r.reversed(m->CopyC, NbC, "CopyC");
    if (!ok) return bad(r.err);
    for (int s = 0; s < NS; ++s) {
        const int c1 = m->SideC[3 * s + 1], c2 = m->SideC[3 * s + 2];
        if (c1 < 1 || c1 > NC || c2 == 0 || c2 > NC || c2 < -NbC)
            return bad(std::string(cns_path) + ": SideC out of range at face " + std::to_string(s + 1));
    }
    if (geo_path) {
        // Library/GeoLoa.f90:14-38
        Reader g;
        if (!g.open(geo_path)) return bad(g.err);
        m->xc = alloc<double>((int64_t)NbC + NC + 1);
        m->yc = alloc<double>((int64_t)NbC + NC + 1);
        m->zc = alloc<double>((int64_t)NbC + NC + 1);
        m->volume = alloc<double>(NC);
        m->delta = alloc<double>(NC);
        m->WallDs = alloc<double>(NC);
        double** face[10] = {&m->Sx, &m->Sy, &m->Sz, &m->Dx, &m->Dy,
                             &m->Dz, &m->f,  &m->xsp, &m->ysp, &m->zsp};
        for (double** p : face) *p = alloc<double>(NS);
        ok = g.array(m->xc + NbC + 1, NC, "xc") && g.array(m->yc + NbC + 1, NC, "yc") &&
             g.array(m->zc + NbC + 1, NC, "zc") && g.reversed(m->xc, NbC, "xc(-1:-NbC)") &&
             g.reversed(m->yc, NbC, "yc(-1:-NbC)") && g.reversed(m->zc, NbC, "zc(-1:-NbC)") &&
             g.array(m->volume, NC, "volume") && g.array(m->delta, NC, "delta") &&
             g.array(m->WallDs, NC, "WallDs");
        static const char* names[10] = {"Sx", "Sy", "Sz", "Dx", "Dy", "Dz", "f", "xsp", "ysp", "zsp"};
        for (int k = 0; k < 10 && ok; ++k) ok = g.array(*face[k], NS, names[k]);
        if (!ok) return bad(g.err);
    }
    *out = m;
    return report_status(TFLOWS_OK, "");
}

int tflows_topolm(int NC, int NS, const int* SideC, int* Acol, int* Arow, int* Adia, int* SidAij,
                  int* NONZ) {
    using tflows::report_status;
    if (NC < 0 || NS < 0 || !SideC || !NONZ) return report_status(TFLOWS_BAD_INPUT, "null argument");
    // stencil width per cell: itself plus its interior faces (TopolM.f90:24-38)
    std::vector<int> w((size_t)NC + 1, 1);
    for (int s = 0; s < NS; ++s) {
        const int c1 = SideC[3 * s + 1], c2 = SideC[3 * s + 2];
        if (c1 < 1 || c1 > NC || c2 > NC)
            return report_status(TFLOWS_BAD_INPUT, "SideC out of range at face " + std::to_string(s + 1));
        if (c2 > 0) {
            ++w[c1];
            ++w[c2];
        }
    }
    int64_t n = 0;
    for (int c = 1; c <= NC; ++c) n += w[c];
    if (n + 1 > INT32_MAX) return report_status(TFLOWS_BAD_INPUT, "too many stored entries");
    *NONZ = (int)(n + 1);
    if (!Acol || !Arow || !Adia) return report_status(TFLOWS_OK, "");  // size query
    // rows: the cell first, then neighbours in face order, then sorted
    Acol[0] = 1;
    for (int c = 1; c <= NC; ++c) Acol[c] = Acol[c - 1] + w[c];
    std::fill(Arow, Arow + n + 1, 0);
    std::vector<int> fillp((size_t)NC + 1);
    for (int c = 1; c <= NC; ++c) {
        Arow[Acol[c - 1] - 1] = c;
        fillp[c] = 1;
    }
    for (int s = 0; s < NS; ++s) {
        const int c1 = SideC[3 * s + 1], c2 = SideC[3 * s + 2];
        if (c2 > 0) {
            Arow[Acol[c1 - 1] - 1 + fillp[c1]++] = c2;
            Arow[Acol[c2 - 1] - 1 + fillp[c2]++] = c1;
        }
    }
    for (int c = 1; c <= NC; ++c) {
        int* row = Arow + Acol[c - 1] - 1;
        const int len = Acol[c] - Acol[c - 1];
        std::sort(row, row + len);
        for (int j = 0; j < len; ++j)
            if (row[j] == c) Adia[c - 1] = Acol[c - 1] + j;
    }
    if (SidAij) {
        for (int s = 0; s < NS; ++s) {
            const int c1 = SideC[3 * s + 1], c2 = SideC[3 * s + 2];
            SidAij[2 * s] = SidAij[2 * s + 1] = 0;
            if (c2 > 0) {
                const int* r1 = Arow + Acol[c1 - 1] - 1;
                const int* r2 = Arow + Acol[c2 - 1] - 1;
                const int l1 = Acol[c1] - Acol[c1 - 1], l2 = Acol[c2] - Acol[c2 - 1];
                // the last matching position, as the reference's search keeps
                const int* p = std::upper_bound(r1, r1 + l1, c2) - 1;
                const int* q = std::upper_bound(r2, r2 + l2, c1) - 1;
                SidAij[2 * s] = (int)(p - Arow) + 1;
                SidAij[2 * s + 1] = (int)(q - Arow) + 1;
            }
        }
    }
    return report_status(TFLOWS_OK, "");
}

}  // extern "C"
