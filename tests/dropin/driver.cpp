// Drives the drop-in (advance_gb300.cpp) through the reference's signatures, the way
// cpu/main.cpp:9-57 does: pointer trees over contiguous blocks, h_const, new_advance per step.
//   driver advance <n> <nsteps> <in.bin> <out.bin>       U: (n+8)^3 x 5 doubles
//   driver ops <n0> <n1> <n2> <U.bin> <out.bin>          writes Q (ghosts x6), courno, F, D
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "header.h"

global_const_t h_const;

static double ****tree(double *base, int a, int b, int c, int dl) {
    double ****p = (double ****)malloc(sizeof(double ***) * a);
    for (int i = 0; i < a; i++) {
        p[i] = (double ***)malloc(sizeof(double **) * b);
        for (int j = 0; j < b; j++) {
            p[i][j] = (double **)malloc(sizeof(double *) * c);
            for (int k = 0; k < c; k++) p[i][j][k] = base + (((size_t)i * b + j) * c + k) * dl;
        }
    }
    return p;
}

static std::vector<double> load(const char *f, size_t n) {
    std::vector<double> v(n);
    FILE *fp = fopen(f, "rb");
    if (!fp || fread(v.data(), sizeof(double), n, fp) != n) { fprintf(stderr, "read %s\n", f); exit(2); }
    fclose(fp);
    return v;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const double eta = 1.8e-4, alam = 1.5e2, cfl = 0.5;
    if (!strcmp(argv[1], "advance")) {
        int n = atoi(argv[2]), steps = atoi(argv[3]), g = n + 8;
        memset(&h_const, 0, sizeof h_const);
        h_const.ng = 4; h_const.nc = 5; h_const.ncells = n;
        for (int a = 0; a < 3; a++) {
            h_const.lo[a] = 0; h_const.hi[a] = n - 1; h_const.dim[a] = n; h_const.dim_g[a] = g;
            h_const.dx[a] = 1.0 / n; h_const.dxinv[a] = n;
        }
        h_const.cfl = cfl; h_const.eta = eta; h_const.alam = alam;
        std::vector<double> U = load(argv[4], (size_t)g * g * g * 5);
        double ****u = tree(U.data(), g, g, g, 5);
        double dt = 0;
        for (int s = 0; s < steps; s++) new_advance(u, nullptr, nullptr, nullptr, nullptr, dt);
        FILE *fo = fopen(argv[5], "wb");
        fwrite(U.data(), sizeof(double), U.size(), fo);
        fwrite(&dt, sizeof(double), 1, fo);
        fclose(fo);
        return 0;
    }
    if (!strcmp(argv[1], "ops")) {
        int n[3] = {atoi(argv[2]), atoi(argv[3]), atoi(argv[4])}, g[3], lo[3], hi[3];
        double dx[3];
        size_t ng3 = 1, ni3 = 1;
        for (int a = 0; a < 3; a++) {
            g[a] = n[a] + 8; lo[a] = 4; hi[a] = n[a] + 3; dx[a] = 1.0 / n[a];
            ng3 *= g[a]; ni3 *= n[a];
        }
        std::vector<double> U = load(argv[5], ng3 * 5), Q(ng3 * 6), F(ni3 * 5), D(ni3 * 5);
        double ****u = tree(U.data(), g[0], g[1], g[2], 5), ****q = tree(Q.data(), g[0], g[1], g[2], 6);
        double ****f = tree(F.data(), n[0], n[1], n[2], 5), ****d = tree(D.data(), n[0], n[1], n[2], 5);
        double courno = 1.0e-50;
        ctoprim(lo, hi, u, q, dx, 4, courno);
        hypterm(lo, hi, 4, dx, u, q, f);
        diffterm(lo, hi, 4, dx, q, d, eta, alam);
        FILE *fo = fopen(argv[6], "wb");
        fwrite(Q.data(), sizeof(double), Q.size(), fo);
        fwrite(&courno, sizeof(double), 1, fo);
        fwrite(F.data(), sizeof(double), F.size(), fo);
        fwrite(D.data(), sizeof(double), D.size(), fo);
        fclose(fo);
        return 0;
    }
    return 2;
}
