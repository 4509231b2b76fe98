// cns_io.cpp -- the reference's text formats and a binary snapshot for checkpoint/resume.
//
//  * general_input: whitespace-separated "ng nc ncells lo[3] hi[3] dx[3] cfl eta alam nsteps dt"
//    with the derived fields of read_configurations (cpu/helper_functions.cpp:38-83);
//  * component files as read_3D reads them (cpu/helper_functions.cpp:166-175): per component,
//    values with i fastest, then j, then k (the Fortran order of the original dumps);
//  * print_4D dumps (cpu/helper_functions.cpp:85-98), "%.17e\t" per value, a newline per j row,
//    a blank line per k plane and per component, optionally preceded by cpu/main.cpp:36-40's
//    header lines (ncomp, then the three dims).
// Arrays are the reference's host layout [i][j][k][l].
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/cns_gb300.h"

namespace cns {
int set_error(int code, const char* msg);  // cns_capi.cu: the thread's cns_last_error() text
}

namespace {
int io_fail(int code, const std::string& msg) { return cns::set_error(code, msg.c_str()); }
inline size_t at(const int d[3], int nc, int i, int j, int k, int l) {
    return (((size_t)i * d[1] + j) * d[2] + k) * nc + l;
}
struct File {
    FILE* f;
    explicit File(FILE* p) : f(p) {}
    ~File() {
        if (f) fclose(f);
    }
};
}  // namespace

extern "C" int cns_read_general_input(const char* path, cns_global_const_t* h) {
    if (!path || !h) return io_fail(CNS_ERR_INVALID, "null argument");
    File in(fopen(path, "r"));
    if (!in.f) return io_fail(CNS_ERR_INVALID, std::string("cannot open ") + path + ": " + strerror(errno));
    memset(h, 0, sizeof *h);
    int ok = fscanf(in.f, "%d %d %d", &h->ng, &h->nc, &h->ncells) == 3;
    ok = ok && fscanf(in.f, "%d %d %d", &h->lo[0], &h->lo[1], &h->lo[2]) == 3;
    ok = ok && fscanf(in.f, "%d %d %d", &h->hi[0], &h->hi[1], &h->hi[2]) == 3;
    ok = ok && fscanf(in.f, "%le %le %le", &h->dx[0], &h->dx[1], &h->dx[2]) == 3;
    ok = ok && fscanf(in.f, "%le %le %le", &h->cfl, &h->eta, &h->alam) == 3;
    ok = ok && fscanf(in.f, "%d %le", &h->nsteps, &h->dt) == 2;
    if (!ok) return io_fail(CNS_ERR_INVALID, std::string("malformed general_input: ") + path);
    for (int a = 0; a < 3; a++) {
        h->dim[a] = h->hi[a] - h->lo[a] + 1;
        h->dim_g[a] = h->dim[a] + 2 * h->ng;
        h->dxinv[a] = 1.0E0 / h->dx[a];
    }
    h->comp_offset_g = h->dim_g[0] * h->dim_g[1] * h->dim_g[2];
    h->comp_offset = h->dim[0] * h->dim[1] * h->dim[2];
    h->plane_offset_g = h->dim_g[1] * h->dim_g[2];
    h->plane_offset = h->dim[1] * h->dim[2];
    h->ALP = 0.8E0;
    h->BET = -0.2E0;
    h->GAM = 4.0E0 / 105.0E0;
    h->DEL = -1.0E0 / 280.0E0;
    h->OneThird = 1.0E0 / 3.0E0;
    h->TwoThirds = 2.0E0 / 3.0E0;
    h->FourThirds = 4.0E0 / 3.0E0;
    h->OneQuarter = 1.E0 / 4.E0;
    h->ThreeQuarters = 3.E0 / 4.E0;
    h->CENTER = -205.0E0 / 72.0E0;
    h->OFF1 = 8.0E0 / 5.0E0;
    h->OFF2 = -0.2E0;
    h->OFF3 = 8.0E0 / 315.0E0;
    h->OFF4 = -1.0E0 / 560.0E0;
    return CNS_OK;
}

extern "C" int cns_write_general_input(const char* path, const cns_global_const_t* h) {
    if (!path || !h) return io_fail(CNS_ERR_INVALID, "null argument");
    File out(fopen(path, "w"));
    if (!out.f) return io_fail(CNS_ERR_INVALID, std::string("cannot create ") + path);
    fprintf(out.f, "%d\n%d\n%d\n", h->ng, h->nc, h->ncells);
    fprintf(out.f, "%d %d %d\n%d %d %d\n", h->lo[0], h->lo[1], h->lo[2], h->hi[0], h->hi[1], h->hi[2]);
    fprintf(out.f, "%.17e %.17e %.17e\n", h->dx[0], h->dx[1], h->dx[2]);
    fprintf(out.f, "%.17e\n%.17e\n%.17e\n%d\n%.17e\n", h->cfl, h->eta, h->alam, h->nsteps, h->dt);
    return ferror(out.f) ? io_fail(CNS_ERR_INVALID, "write failed") : CNS_OK;
}

extern "C" int cns_read_3d(const char* path, double* a, const int dims[3], int ncomp) {
    if (!path || !a || !dims || ncomp <= 0) return io_fail(CNS_ERR_INVALID, "bad argument");
    File in(fopen(path, "r"));
    if (!in.f) return io_fail(CNS_ERR_INVALID, std::string("cannot open ") + path);
    for (int l = 0; l < ncomp; l++)
        for (int k = 0; k < dims[2]; k++)
            for (int j = 0; j < dims[1]; j++)
                for (int i = 0; i < dims[0]; i++)
                    if (fscanf(in.f, "%le", &a[at(dims, ncomp, i, j, k, l)]) != 1)
                        return io_fail(CNS_ERR_INVALID, std::string("short component file: ") + path);
    return CNS_OK;
}

extern "C" int cns_write_3d(const char* path, const double* a, const int dims[3], int ncomp) {
    if (!path || !a || !dims || ncomp <= 0) return io_fail(CNS_ERR_INVALID, "bad argument");
    File out(fopen(path, "w"));
    if (!out.f) return io_fail(CNS_ERR_INVALID, std::string("cannot create ") + path);
    for (int l = 0; l < ncomp; l++)
        for (int k = 0; k < dims[2]; k++)
            for (int j = 0; j < dims[1]; j++) {
                for (int i = 0; i < dims[0]; i++) fprintf(out.f, "%.17e ", a[at(dims, ncomp, i, j, k, l)]);
                fputc('\n', out.f);
            }
    return ferror(out.f) ? io_fail(CNS_ERR_INVALID, "write failed") : CNS_OK;
}

extern "C" int cns_print_4d(const char* path, const double* a, const int dims[3], int ncomp, int with_header) {
    if (!path || !a || !dims || ncomp <= 0) return io_fail(CNS_ERR_INVALID, "bad argument");
    File out(fopen(path, "w"));
    if (!out.f) return io_fail(CNS_ERR_INVALID, std::string("cannot create ") + path);
    if (with_header) fprintf(out.f, "%d\n%d %d %d\n", ncomp, dims[0], dims[1], dims[2]);
    for (int l = 0; l < ncomp; l++) {
        for (int k = 0; k < dims[2]; k++) {
            for (int j = 0; j < dims[1]; j++) {
                for (int i = 0; i < dims[0]; i++) fprintf(out.f, "%.17e\t", a[at(dims, ncomp, i, j, k, l)]);
                fputc('\n', out.f);
            }
            fputc('\n', out.f);
        }
        fputc('\n', out.f);
    }
    return ferror(out.f) ? io_fail(CNS_ERR_INVALID, "write failed") : CNS_OK;
}

extern "C" int cns_read_4d(const char* path, double* a, const int dims[3], int ncomp, int with_header) {
    if (!path || !a || !dims || ncomp <= 0) return io_fail(CNS_ERR_INVALID, "bad argument");
    File in(fopen(path, "r"));
    if (!in.f) return io_fail(CNS_ERR_INVALID, std::string("cannot open ") + path);
    if (with_header) {
        int nc, d0, d1, d2;
        if (fscanf(in.f, "%d %d %d %d", &nc, &d0, &d1, &d2) != 4 || nc != ncomp || d0 != dims[0] || d1 != dims[1] ||
            d2 != dims[2])
            return io_fail(CNS_ERR_INVALID, std::string("header does not match the requested shape: ") + path);
    }
    for (int l = 0; l < ncomp; l++)
        for (int k = 0; k < dims[2]; k++)
            for (int j = 0; j < dims[1]; j++)
                for (int i = 0; i < dims[0]; i++)
                    if (fscanf(in.f, "%le", &a[at(dims, ncomp, i, j, k, l)]) != 1)
                        return io_fail(CNS_ERR_INVALID, std::string("short print_4D file: ") + path);
    return CNS_OK;
}
