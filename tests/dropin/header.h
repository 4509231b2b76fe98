// Test stand-in for the reference's cpu/header.h, for machines without the reference tree.
// It declares the same parameter struct (field for field, so the layout matches
// global_const_t, cpu/header.h:47-86) and the same operator signatures (cpu/header.h:98-156)
// that advance_gb300.cpp implements.  The real header is used wherever it exists.
#ifndef HEADER_INCLUDED
#define HEADER_INCLUDED
#define NG 4
#define NC 5
typedef struct global_const {
    int ng, nc, ncells;
    int lo[3], hi[3], dim[3], dim_g[3];
    int comp_offset_g, comp_offset, plane_offset_g, plane_offset;
    int nsteps;
    double dt;
    double dx[3], dxinv[3];
    double cfl, eta, alam;
    double *temp[27];
    double ALP, BET, GAM, DEL;
    double OneThird, TwoThirds, FourThirds, OneQuarter, ThreeQuarters;
    double CENTER, OFF1, OFF2, OFF3, OFF4;
} global_const_t;
extern void ctoprim(int lo[], int hi[], double ****u, double ****q, double dx[], int ng, double &courno);
extern void ctoprim(int lo[], int hi[], double ****u, double ****q, double dx[], int ng);
extern void hypterm(int lo[], int hi[], int ng, double dx[], double ****cons, double ****q, double ****flux);
extern void diffterm(int lo[], int hi[], int ng, double dx[], double ****q, double ****difflux, double eta,
                     double alam);
extern void new_advance(double ****U, double ****Unew, double ****Q, double ****D, double ****F, double &dt);
#endif
