// ref_harness.cpp -- C entry points over the reference's own cpu/ implementation.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with the unmodified
// reference sources (cpu/ctoprim.cpp, cpu/hypterm.cpp, cpu/diffterm.cpp,
// cpu/helper_functions.cpp, cpu/advance.cpp) into oracle/_ref/libcnsref.so.  It replaces the
// reference's file-driven cpu/main.cpp:9-57: it defines the globals that main.cpp defines
// (h_const and the three operator timers, cpu/main.cpp:4-7), fills h_const the way
// read_configurations does (cpu/helper_functions.cpp:38-83) from arguments instead of
// ../testcases/general_input, and wraps caller-owned flat arrays in the double**** pointer
// trees that the reference functions take (the allocate_4D layout,
// cpu/helper_functions.cpp:100-122).
#include <cstdlib>
#include <cstring>
#include "header.h"
#include "helper_functions.h"

global_const_t h_const;
double ctoprim_time = 0.0;
double diffterm_time = 0.0;
double hypterm_time = 0.0;

namespace {

// A pointer tree [d0][d1][d2] -> &base[((i*d1+j)*d2+k)*dl] over an existing flat block.
struct Tree4 {
    double ****p = nullptr;
    int d0 = 0, d1 = 0;
    Tree4(double *base, int a, int b, int c, int dl) : d0(a), d1(b) {
        p = (double ****)malloc(sizeof(double ***) * a);
        for (int i = 0; i < a; i++) {
            p[i] = (double ***)malloc(sizeof(double **) * b);
            for (int j = 0; j < b; j++) {
                p[i][j] = (double **)malloc(sizeof(double *) * c);
                for (int k = 0; k < c; k++) p[i][j][k] = base + (((size_t)i * b + j) * c + k) * dl;
            }
        }
    }
    ~Tree4() {
        for (int i = 0; i < d0; i++) {
            for (int j = 0; j < d1; j++) free(p[i][j]);
            free(p[i]);
        }
        free(p);
    }
};

void set_const(int n0, int n1, int n2, const double dx[3], double cfl, double eta, double alam) {
    memset(&h_const, 0, sizeof(h_const));
    h_const.ng = NG;
    h_const.nc = NC;
    h_const.ncells = n0;
    int n[3] = {n0, n1, n2};
    for (int i = 0; i < 3; i++) {
        h_const.lo[i] = 0;
        h_const.hi[i] = n[i] - 1;
        h_const.dim[i] = n[i];
        h_const.dim_g[i] = n[i] + 2 * NG;
        h_const.dx[i] = dx[i];
        h_const.dxinv[i] = 1.0E0 / dx[i];
    }
    h_const.comp_offset_g = h_const.dim_g[0] * h_const.dim_g[1] * h_const.dim_g[2];
    h_const.comp_offset = n0 * n1 * n2;
    h_const.plane_offset_g = h_const.dim_g[1] * h_const.dim_g[2];
    h_const.plane_offset = n1 * n2;
    h_const.cfl = cfl;
    h_const.eta = eta;
    h_const.alam = alam;
    h_const.ALP = 0.8E0;
    h_const.BET = -0.2E0;
    h_const.GAM = 4.0E0 / 105.0E0;
    h_const.DEL = -1.0E0 / 280.0E0;
    h_const.OneThird = 1.0E0 / 3.0E0;
    h_const.TwoThirds = 2.0E0 / 3.0E0;
    h_const.FourThirds = 4.0E0 / 3.0E0;
    h_const.OneQuarter = 1.E0 / 4.E0;
    h_const.ThreeQuarters = 3.E0 / 4.E0;
    h_const.CENTER = -205.0E0 / 72.0E0;
    h_const.OFF1 = 8.0E0 / 5.0E0;
    h_const.OFF2 = -0.2E0;
    h_const.OFF3 = 8.0E0 / 315.0E0;
    h_const.OFF4 = -1.0E0 / 560.0E0;
}

}  // namespace

extern "C" {

// nsteps calls of the reference new_advance on a cubic box (cpu/advance.cpp:13-154).
// U: ghost-inclusive [n+8]^3 x 5, updated in place.  dt_hist (nullable) gets each step's dt.
int ref_new_advance(double *U, int n, const double dx[3], double cfl, double eta, double alam, int nsteps,
                    double *dt_hist) {
    set_const(n, n, n, dx, cfl, eta, alam);
    const int g = n + 2 * NG;
    Tree4 u(U, g, g, g, NC);
    int dim[3] = {n, n, n}, dim_g[3] = {g, g, g};
    double ****Q, ****D, ****F;
    allocate_4D(Q, dim_g, NC + 1);
    allocate_4D(D, dim, NC);
    allocate_4D(F, dim, NC);
    double *unew_blk = (double *)calloc((size_t)g * g * g * NC, sizeof(double));
    Tree4 un(unew_blk, g, g, g, NC);
    for (int s = 0; s < nsteps; s++) {
        double dt = 0.0;
        new_advance(u.p, un.p, Q, D, F, dt);
        if (dt_hist) dt_hist[s] = dt;
    }
    free_4D(Q, dim_g);
    free_4D(D, dim);
    free_4D(F, dim);
    free(unew_blk);
    return 0;
}

// cpu/helper_functions.cpp:226-262 on a ghost-inclusive [dim+8] x 5 block.
int ref_fill_boundary(double *U, const int dim[3]) {
    int d[3] = {dim[0], dim[1], dim[2]}, dg[3] = {dim[0] + 2 * NG, dim[1] + 2 * NG, dim[2] + 2 * NG};
    Tree4 u(U, dg[0], dg[1], dg[2], NC);
    fill_boundary(u.p, d, dg);
    return 0;
}

// cpu/ctoprim.cpp:11-70 (courno != nullptr) or 72-105 (courno == nullptr).
int ref_ctoprim(const int lo_in[3], const int hi_in[3], double *u, double *q, const double dx_in[3], int ng,
                double *courno) {
    int lo[3], hi[3], dg[3];
    double dx[3];
    for (int i = 0; i < 3; i++) {
        lo[i] = lo_in[i];
        hi[i] = hi_in[i];
        dx[i] = dx_in[i];
        dg[i] = hi[i] - lo[i] + 1 + 2 * ng;
    }
    Tree4 tu(u, dg[0], dg[1], dg[2], 5), tq(q, dg[0], dg[1], dg[2], 6);
    if (courno)
        ctoprim(lo, hi, tu.p, tq.p, dx, ng, *courno);
    else
        ctoprim(lo, hi, tu.p, tq.p, dx, ng);
    return 0;
}

// cpu/hypterm.cpp:11-209.
int ref_hypterm(const int lo_in[3], const int hi_in[3], int ng, const double dx_in[3], double *cons, double *q,
                double *flux) {
    int lo[3], hi[3], dg[3], di[3];
    double dx[3];
    for (int i = 0; i < 3; i++) {
        lo[i] = lo_in[i];
        hi[i] = hi_in[i];
        dx[i] = dx_in[i];
        di[i] = hi[i] - lo[i] + 1;
        dg[i] = di[i] + 2 * ng;
    }
    Tree4 tc(cons, dg[0], dg[1], dg[2], 5), tq(q, dg[0], dg[1], dg[2], 6), tf(flux, di[0], di[1], di[2], 5);
    hypterm(lo, hi, ng, dx, tc.p, tq.p, tf.p);
    return 0;
}

// cpu/diffterm.cpp:22-320.
int ref_diffterm(const int lo_in[3], const int hi_in[3], int ng, const double dx_in[3], double *q, double *difflux,
                 double eta, double alam) {
    int lo[3], hi[3], dg[3], di[3];
    double dx[3];
    for (int i = 0; i < 3; i++) {
        lo[i] = lo_in[i];
        hi[i] = hi_in[i];
        dx[i] = dx_in[i];
        di[i] = hi[i] - lo[i] + 1;
        dg[i] = di[i] + 2 * ng;
    }
    Tree4 tq(q, dg[0], dg[1], dg[2], 6), td(difflux, di[0], di[1], di[2], 5);
    diffterm(lo, hi, ng, dx, tq.p, td.p, eta, alam);
    return 0;
}

}  // extern "C"

extern "C" {

// cpu/helper_functions.cpp:85-98 print_4D into a file (dims as given, dl components).
int ref_print_4D(const char *path, double *A, const int dims[3], int dl) {
    FILE *f = fopen(path, "w");
    if (!f) return 1;
    int d[3] = {dims[0], dims[1], dims[2]};
    Tree4 t(A, d[0], d[1], d[2], dl);
    print_4D(f, t.p, d, dl);
    fclose(f);
    return 0;
}

// cpu/helper_functions.cpp:166-175 read_3D of dl components from a file.
int ref_read_3D(const char *path, double *A, const int dims[3], int dl) {
    FILE *f = fopen(path, "r");
    if (!f) return 1;
    int d[3] = {dims[0], dims[1], dims[2]};
    Tree4 t(A, d[0], d[1], d[2], dl);
    for (int l = 0; l < dl; l++) read_3D(f, t.p, d, l);
    fclose(f);
    return 0;
}

// cpu/helper_functions.cpp:38-83 read_configurations, which opens ../testcases/general_input
// relative to the working directory; the caller chdirs accordingly.  Copies h_const out.
int ref_read_configurations(void *out, int out_size) {
    if (out_size != (int)sizeof(global_const_t)) return 1;
    read_configurations(h_const);
    memcpy(out, &h_const, sizeof(global_const_t));
    return 0;
}

}  // extern "C"
