// advance_gb300.cpp -- drop-in replacement for the reference's cpu/advance.cpp,
// cpu/ctoprim.cpp, cpu/hypterm.cpp and cpu/diffterm.cpp.
//
// Same names and signatures as the reference (cpu/header.h:98-156), same argument meaning
// (ghost-offset lo/hi, [i][j][k][l] pointer trees from allocate_4D, interior-indexed flux and
// difflux, parameters from the global h_const), implemented by libcns_gb300.so on the GPU.
// Build it in place of those four files against the reference's own headers and link the
// library:
//
//   g++ -O2 -I<reference>/cpu -I<this repo>/include -c advance_gb300.cpp
//   g++ -o cpu main.o helper_functions.o advance_gb300.o -L<lib dir> -lcns_gb300
//
// The reference has no error path on these functions; a failure here prints the library's
// message and exits with status 1, as the reference's own checks do
// (cpu/helper_functions.cpp:177-224).
#include <cstdio>
#include <cstdlib>

#include "cns_gb300.h"
#include "header.h"

extern global_const_t h_const;

static_assert(sizeof(global_const_t) == sizeof(cns_global_const_t),
              "cns_global_const_t must mirror global_const_t (cpu/header.h:47-86)");

static void die_on(int rc, const char* what) {
    if (rc != CNS_OK) {
        fprintf(stderr, "%s: %s\n", what, cns_last_error());
        exit(1);
    }
}

void ctoprim(int lo[], int hi[], double**** u, double**** q, double dx[], int ng, double& courno) {
    die_on(cns_ctoprim(lo, hi, &u[0][0][0][0], &q[0][0][0][0], dx, ng, &courno), "ctoprim");
}

void ctoprim(int lo[], int hi[], double**** u, double**** q, double dx[], int ng) {
    die_on(cns_ctoprim(lo, hi, &u[0][0][0][0], &q[0][0][0][0], dx, ng, nullptr), "ctoprim");
}

void hypterm(int lo[], int hi[], int ng, double dx[], double**** cons, double**** q, double**** flux) {
    die_on(cns_hypterm(lo, hi, ng, dx, &cons[0][0][0][0], &q[0][0][0][0], &flux[0][0][0][0]), "hypterm");
}

void diffterm(int lo[], int hi[], int ng, double dx[], double**** q, double**** difflux, double eta, double alam) {
    die_on(cns_diffterm(lo, hi, ng, dx, &q[0][0][0][0], &difflux[0][0][0][0], eta, alam), "diffterm");
}

void new_advance(double**** U, double**** Unew, double**** Q, double**** D, double**** F, double& dt) {
    (void)Unew, (void)Q, (void)D, (void)F;
    die_on(cns_new_advance(reinterpret_cast<const cns_global_const_t*>(&h_const), &U[0][0][0][0], nullptr, nullptr,
                           nullptr, nullptr, &dt),
           "new_advance");
    printf("dt, courno = %le, %le\n", dt, h_const.cfl / dt);  // the reference's per-step line (cpu/advance.cpp:59)
}
