// cns_common.cuh -- shared device definitions for the GB300 CNS_NoSpec RK3 advance.
//
// Device layout of one periodic box (n0 x n1 x n2 interior cells, NG = 4 ghost cells a side):
// structure of arrays, one field after another; inside a field the reference's spatial order
// (i slowest, k fastest, cpu/helper_functions.cpp:100-122) with each k row padded to `pk`
// elements (a multiple of 8: 64-byte rows for FP64, 32-byte for FP32; TMA-legal strides).
//   elem(f, i, j, k) = f*fs + i*si + j*sj + k      (i, j, k ghost-inclusive, 0..n+7)
// i pairs with dx[0], j with dx[1], k with dx[2], exactly as in the reference.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CNS_NG 4
#define CNS_NC 5

namespace cns {

// ---- physics and stencil constants (cpu/ctoprim.cpp:23-24, cpu/header.h:88-91,
//      cpu/diffterm.cpp:48-52) -------------------------------------------------------------
constexpr double kGamma = 1.4;
constexpr double kGm1 = kGamma - 1.0;  // the reference forms (GAMMA-1.0) the same way
constexpr double kCv = 8.3333333333e6;
constexpr double kAlp = 0.8, kBet = -0.2, kGam = 4.0 / 105.0, kDel = -1.0 / 280.0;
constexpr double kCenter = -205.0 / 72.0, kOff1 = 8.0 / 5.0, kOff2 = -0.2, kOff3 = 8.0 / 315.0,
                 kOff4 = -1.0 / 560.0;
// The same operators as integer weights over a common denominator (ALP..DEL = 672, -168, 32,
// -3 over 840; OFF1..OFF4 = 8064, -1008, 128, -9 over 5040), for the exact stencil sums.
constexpr double kD1Den = 840.0, kD2Den = 5040.0;

// ---- field indices ----------------------------------------------------------------------
// Conserved state (FP64 always): rho, rho u, rho v, rho w, rho E  (cpu/header.h:20-26).
enum { URHO = 0, UMX, UMY, UMZ, UENE };
// Primitive/flux set P (precision R): what the stencils read.  Each is produced once per
// cell by the epilogue of the previous stage (ctoprim fused there) with its periodic ghost
// images, so no stencil ever recomputes a neighbour's primitive.
enum {
    PU = 0, PV, PW, PT,        // velocities, and c_v T = e for the heat conduction (diffterm; its
                               // coefficients carry alam / c_v, so T itself is never formed)
    PMX, PMY, PMZ,             // rho u, rho v, rho w  (density flux)
    PFUU, PFVV, PFWW,          // rho u u + p, rho v v + p, rho w w + p
    PFUV, PFUW, PFVW,          // rho u v, rho u w, rho v w
    PHU, PHV, PHW,             // (rho E + p) u, (rho E + p) v, (rho E + p) w
    NPF
};
// Derivative set S (precision R), made by the derivative pass.
enum { SX = 0,   // v_y + w_z  (differenced along x for the mixed terms of the x momentum)
       SY,       // u_x + w_z  (along y)
       SZ,       // u_x + v_y  (along z)
       SPHI,     // eta * viscous dissipation
       NSF };

// Per-box coefficient table, folded with 1/dx and the transport coefficients so that every
// stencil tap is one fused multiply-add.  Kept in FP64 (plain form) and FP32 (mixed form).
template <class R>
struct CoefT {
    // Each stencil row holds its four coefficients (weight x factor) and, at [4], the factor
    // over the weights' denominator (840 or 5040) for the exact sums of the plain form.
    R da[3][5];     // first derivative along d: a_m / dx_d
    R ha[3][5];     // convective flux divergence: -a_m / dx_d
    R mx[3][5];     // mixed viscous term: (eta/3) a_m / dx_d
    R vl[3][3][5];  // viscous Laplacian of velocity c along d: eta (4/3 if c==d) b_m / dx_d^2
    R vc[3];        // its centre weight: eta c0 sum_d (4/3 if c==d) / dx_d^2
    R tl[3][5];     // heat conduction along d: (alam / c_v) b_m / dx_d^2, applied to e = c_v T
    R tc;           // (alam / c_v) c0 sum_d 1/dx_d^2
    R cour[3];      // 1/dx_d (Courant number)
    R eta;          // viscosity
};

// Device scalars of one box (written by kernels only).
struct BoxScalars {
    unsigned long long courno_bits;  // running max of the Courant number (bits of a positive double)
    double dt;                       // dt of the step in progress (or the next one, between steps)
    double dt_last;                  // dt of the last completed step
    int pbase;                       // which P set holds the primitives of the step's start state
    int nsteps_done;
    int status;                      // HEALTH_* bits, sticky
    int pad;
    // Reference values of the mixed form, fixed at upload from one cell of the state (FP64):
    // the FP32 stencil fields carry p - p_ref, e - e_ref and (E + p) - H_ref, whose rounding
    // is ~10-30x smaller than that of p, T, E + p themselves.  Every difference operator
    // annihilates a constant, and the energy flux splits exactly as
    // d((E+p) u)/dx = H_ref du/dx + d(((E+p) - H_ref) u)/dx.
    double p_ref, e_ref, E_ref, H_ref;
    // The plain form's fixed-point copies of the P sets (cns_exact.cuh): fx_bad[s] != 0 when the
    // copy of P[s] is unusable (not written, or a value did not fit its exponent), fx_e[s][f] the
    // exponent of field f in it; fx_prev[f] / fx_cur[f] the largest biased exponent field of P
    // field f over the previous step's tracked writes / those since (the direct kernels track
    // stage 3's writes, the TMA kernel every stage's; an upload, the uploaded set).  fx_restore: the box was just
    // restored with its exponents (the conversion after the upload keeps fx_e, and fx_prev stays).
    // fx_fresh: the copy was made from an upload (not written by a step) and the step after it
    // has not ended; that step's first derivative pass reads the FP64 fields, as the upload fused
    // with that pass (host arrays read in place) does, so both routes give the same bits.
    int fx_bad[2];
    int fx_restore;
    int fx_fresh;
    int fx_e[2][NPF];
    int fx_prev[NPF];
    int fx_cur[NPF];
};

constexpr int DTLOG_CAP = 1024;

// HEALTH_TIMEOUT: a bounded wait inside a kernel gave up (the kernel returned early).
enum { HEALTH_OK = 0, HEALTH_NONPOS_RHO = 1, HEALTH_NONFINITE = 2, HEALTH_NONPOS_EINT = 4, HEALTH_TIMEOUT = 8 };

// Everything a kernel needs about one box.  Kept in device memory (one entry per box) so
// that a batched launch can walk tiles of many boxes.
struct BoxView {
    int n[3];               // interior dims
    int pk;                 // padded k row (elements)
    long long sj, si, fs;   // strides (elements)
    double* U;              // 5 fields, FP64: state at the start of the step
    double* Us;             // 5 fields, FP64: stage state
    void* P[2];             // NPF fields each, precision R
    void* S;                // NSF fields, precision R
    BoxScalars* sc;
    double* dtlog;          // dt of completed steps, ring of DTLOG_CAP entries
    double* host_out;       // when set (only around the last step of a host-array call): the
                            // device address of the caller's page-locked host array; stage 3
                            // also stores each cell's new state there, in the reference layout
    const void* tma;        // mixed boxes: device copy of the TMA tensor maps of P[0], P[1], S
    double cfl;
    int precision;          // 0 = plain FP64, 1 = mixed
    int tlog[3];            // tile shape of this box: log2 of its (i, j, k) extent; the three sum to 8
                            // (256 threads, one cell each, k fastest across a warp)
    CoefT<double> c64;
    CoefT<float> c32;
    long long* X[2];        // plain FP64 boxes: fixed-point copies of the first `fx` fields of P[0],
                            // P[1] (the P sets' geometry, fields fs apart)
    int fx;                 // fields with copies: 0 (none), kFxFields (CNS_ASSEMBLE_FX) or NPF
                            // (CNS_ASSEMBLE_TMA_FX)
    int lap_merge;          // the Laplacians' factors are equal where the merged sums need it
                            // (cubic cells: v_yy's and w_zz's 4/3 apart)
};
// The fields the direct kernels keep fixed-point copies of: u, v, w, e (the derivative pass's and
// the Laplacians' taps; PU..PT).
constexpr int kFxFields = 4;

// A unit of work: one tile of one box, with origin (i0, j0, k0); its shape is the box's tlog.
struct Tile {
    int box, i0, j0, k0;
};

constexpr int kTileThreads = 256;

// The cell of this thread inside a tile of shape tlog (k fastest, then j, then i).
__device__ __forceinline__ void tile_cell(const int tlog[3], int t, int* ti, int* tj, int* tk) {
    const int lk = tlog[2], lj = tlog[1];
    *tk = t & ((1 << lk) - 1);
    *tj = (t >> lk) & ((1 << lj) - 1);
    *ti = t >> (lk + lj);
}

// A box whose tlog[0] is kLinearTile uses linear tiles: tile T is the 256 consecutive cells
// 256 * T.k0 ... of the box's interior in its own order (i slowest, k fastest), so no box shape
// pads a tile; a warp still covers 32 consecutive k cells except where a k row ends.
constexpr int kLinearTile = -1;

// The cell of thread t of tile T (i >= n[0] past the end of a box: the caller skips it).
__device__ __forceinline__ void tile_pos(const BoxView& b, const Tile& T, int t, int* i, int* j, int* k) {
    if (b.tlog[0] == kLinearTile) {
        const long long p = (long long)T.k0 * kTileThreads + t;
        const long long row = p / b.n[2];
        *k = (int)(p - row * b.n[2]);
        *j = (int)(row % b.n[1]);
        *i = (int)(row / b.n[1]);
    } else {
        int ti, tj, tk;
        tile_cell(b.tlog, t, &ti, &tj, &tk);
        *i = T.i0 + ti;
        *j = T.j0 + tj;
        *k = T.k0 + tk;
    }
}

__host__ __device__ inline long long cell_off(const BoxView& b, int i, int j, int k) {
    // (i, j, k) interior indices, 0-based; returns the element offset inside one field
    return (long long)(i + CNS_NG) * b.si + (long long)(j + CNS_NG) * b.sj + (k + CNS_NG);
}

// Positive doubles order like their bit patterns; the Courant max uses integer atomics.
__device__ inline unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

// Reciprocal for FP64: the PTX approximate reciprocal (rcp.approx.ftz.f64, special-function
// unit) as the seed, refined by one third-order Newton-series step r <- r (1 + e + e^2),
// e = 1 - x r (Householder's method of order 3 for 1/x).  The seed's relative error e0 (a
// single-precision-level approximation) becomes ~e0^3, so the result is within a few ulp of
// 1/x.  Costs three FP64 FMAs instead of a full IEEE division, and no FP32<->FP64 conversion
// (those issue to the FP64 pipe).
__device__ inline double rcp_nr(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

}  // namespace cns
