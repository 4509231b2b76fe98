// cns_fused.cuh -- the fused RK3 stage kernels (plain FP64 and mixed FP32/FP64).
//
// One RK3 step of the reference (new_advance, cpu/advance.cpp:13-154) is, per box:
//
//   k_prim       (once, after an upload)  ctoprim + flux functions of U -> P[pbase], Courant
//   k_stepend    dt = cfl / max(courno, 1e-50)          (cpu/advance.cpp:52-58)
//   stage s = 1, 2, 3:
//     k_deriv     first derivatives of (u,v,w) -> S = (v_y+w_z, u_x+w_z, u_x+v_y, eta*Phi)
//     k_assemble  diffterm + hypterm from P and S, RK stage combine in FP64
//                 (cpu/advance.cpp:78-85, 110-119, 144-153), then, fused into the
//                 write-back, ctoprim + flux functions of the new stage state -> the other P
//                 set with its periodic ghost images (fill_boundary fused,
//                 cpu/helper_functions.cpp:226-262); stage 3 also folds the Courant number
//                 of U^{n+1} (cpu/ctoprim.cpp:50-69) into the box's running max.
//   k_stepend    flip the P set, next dt.
//
// GB300's FP64 rate is 1/67 of its FP32 rate, so the plain form is bound by the FP64 pipe,
// not by HBM: the kernels are arranged so that every FP64 quantity is computed exactly once
// per cell (no halo recomputation of primitives or derivatives) and every stencil tap is one
// FMA with a coefficient pre-folded with 1/dx, eta or alam.  Part of the stencils (chosen per
// family and axis, cns_exact.cuh) are instead summed exactly on the integer pipes and cost one
// FP64 instruction each, so that the integer and FP64 pipes share the work.
//
// Algebraic regrouping against the reference (same discrete operators; rounding differs at
// the level of a few ulp):
//   * hypterm's products cons*u at each neighbour become per-cell flux functions
//     (rho u u + p, rho u v, ..., (rho E + p) u) differenced by the same 8-point stencil
//     (cpu/hypterm.cpp:43-204);
//   * diffterm's vyx + wzx, uxy + wzy, uxz + vyz become one stencil each on the per-cell sums
//     v_y + w_z, u_x + w_z, u_x + v_y (cpu/diffterm.cpp:177-265);
//   * the three second differences of each Laplacian share one centre tap.
#pragma once
#include "cns_common.cuh"
#include "cns_exact.cuh"

namespace cns {

template <class R>
__device__ __forceinline__ const CoefT<R>& coefs(const BoxView& b);
template <>
__device__ __forceinline__ const CoefT<double>& coefs<double>(const BoxView& b) { return b.c64; }
template <>
__device__ __forceinline__ const CoefT<float>& coefs<float>(const BoxView& b) { return b.c32; }

// Loads of stencil taps: through the read-only path (NC, for data no thread of the launch
// writes), or from L2 past L1 (for data other blocks of the same launch write: L1 is not kept
// coherent, and a 128-byte line can hold bytes of a row that is not written yet; and for the S
// set in the assembly, whose taps reach L1 to no use: the L2 path measured 1 % faster there).
template <bool NC, class R>
__device__ __forceinline__ R ld_tap(const R* p) {
    if (NC) return __ldg(p);
    return __ldcg(p);
}
// acc + sum_m a_m (p[m s] - p[-m s]); in the plain form (R = double) the exact sum (cns_exact.cuh)
// where X.  NB (no branch): the exact sum without its FP64 fallback, *xf set where the fallback
// is needed (the caller then evaluates the cell again with NB = false; cns_exact.cuh).
template <bool X, class R, bool NB = false, bool NC = true>
__device__ __forceinline__ R d1acc(R acc, const R* __restrict__ p, long long s, const R* a, bool* xf = nullptr) {
    if constexpr (sizeof(R) == 8 && X) {
        if constexpr (NB) return xd1acc_nb(acc, XTaps<NC ? 0 : 1>{p, s}, a, xf);
        else return xd1acc(acc, XTaps<NC ? 0 : 1>{p, s}, a);
    }
    acc = fma(a[0], ld_tap<NC>(p + s) - ld_tap<NC>(p - s), acc);
    acc = fma(a[1], ld_tap<NC>(p + 2 * s) - ld_tap<NC>(p - 2 * s), acc);
    acc = fma(a[2], ld_tap<NC>(p + 3 * s) - ld_tap<NC>(p - 3 * s), acc);
    acc = fma(a[3], ld_tap<NC>(p + 4 * s) - ld_tap<NC>(p - 4 * s), acc);
    return acc;
}
template <bool X, class R, bool NC = true, bool NB = false>
__device__ __forceinline__ R d1(const R* __restrict__ p, long long s, const R* a, bool* xf = nullptr) {
    if constexpr (sizeof(R) == 8 && X) {
        if constexpr (NB) return xd1acc_nb(0.0, XTaps<NC ? 0 : 1>{p, s}, a, xf);
        else return xd1acc(0.0, XTaps<NC ? 0 : 1>{p, s}, a);
    }
    R acc = a[0] * (ld_tap<NC>(p + s) - ld_tap<NC>(p - s));
    acc = fma(a[1], ld_tap<NC>(p + 2 * s) - ld_tap<NC>(p - 2 * s), acc);
    acc = fma(a[2], ld_tap<NC>(p + 3 * s) - ld_tap<NC>(p - 3 * s), acc);
    acc = fma(a[3], ld_tap<NC>(p + 4 * s) - ld_tap<NC>(p - 4 * s), acc);
    return acc;
}
// acc + sum_m b_m (p[m s] + p[-m s])
template <bool X, class R, bool NB = false>
__device__ __forceinline__ R d2acc(R acc, const R* __restrict__ p, long long s, const R* b, bool* xf = nullptr) {
    if constexpr (sizeof(R) == 8 && X) {
        if constexpr (NB) return xd2acc_nb(acc, XTaps<0>{p, s}, b, xf);
        else return xd2acc(acc, XTaps<0>{p, s}, b);
    }
    acc = fma(b[0], __ldg(p + s) + __ldg(p - s), acc);
    acc = fma(b[1], __ldg(p + 2 * s) + __ldg(p - 2 * s), acc);
    acc = fma(b[2], __ldg(p + 3 * s) + __ldg(p - 3 * s), acc);
    acc = fma(b[3], __ldg(p + 4 * s) + __ldg(p - 4 * s), acc);
    return acc;
}

// ---- stencils on fixed-point taps (FP64 boxes that keep a fixed-point copy of the P set) -----
// A tap of the copy costs two wide integer multiply-adds (cns_exact.cuh), against ~20 integer
// instructions to place an FP64 tap's significand for an exact sum.  The direct kernels keep
// copies of the first kFxFields fields of the P set (u, v, w, e: the derivative pass's and the
// Laplacians' taps); per family and axis, the masks choose the stencils they evaluate on the
// copies.  The others stay the FP64 form's (kExact* above).  Copies of the twelve flux fields as
// well (kFxFields = NPF) with the flux divergences on them measured 5-7 % slower per 256^3 step:
// writing twelve more copies costs more than their stencils save.
constexpr int kFxDeriv = 0b111, kFxFlux = 0, kFxLap = 0b111;
static_assert(kFxFlux == 0 || kFxFields == NPF, "flux stencils on copies need copies of every field");
static_assert(PU < kFxFields && PV < kFxFields && PW < kFxFields && PT < kFxFields, "u, v, w, e have copies");

// 64-bit words of a field's copy at offsets m * s, through the read-only path.
struct XWords {
    const long long* p;
    long long s;
    __device__ __forceinline__ long long operator()(int m) const { return __ldg(p + m * s); }
};
// d1acc / d1 / d2acc of a field whose taps are p (FP64) or, where FXA, x (its copy, exponent E).
template <bool FXA, bool XA, class R, bool NB>
__device__ __forceinline__ R tap_d1acc(R acc, const R* p, const long long* x, int E, long long s, const R* a,
                                       bool* xf) {
    if constexpr (FXA) return fx_d1acc(acc, XWords{x, s}, E, a, xf);
    else return d1acc<XA, R, NB>(acc, p, s, a, xf);
}
template <bool FXA, bool XA, class R, bool NB>
__device__ __forceinline__ R tap_d1(const R* p, const long long* x, int E, long long s, const R* a, bool* xf) {
    if constexpr (FXA) return fx_d1acc(0.0, XWords{x, s}, E, a, xf);
    else return d1<XA, R, true, NB>(p, s, a, xf);
}
template <bool FXA, bool XA, class R, bool NB>
__device__ __forceinline__ R tap_d2acc(R acc, const R* p, const long long* x, int E, long long s, const R* b,
                                       bool* xf) {
    if constexpr (FXA) return fx_d2acc(acc, XWords{x, s}, E, b, xf);
    else return d2acc<XA, R, NB>(acc, p, s, b, xf);
}

// Store a value and its periodic face images along the axes in `mask` (1 = i, 2 = j, 4 = k).
template <class R>
__device__ __forceinline__ void store_img(R* __restrict__ f, const BoxView& b, long long c, int i, int j, int k,
                                          R v, int mask) {
    f[c] = v;
    if (mask & 1) {
        if (i < CNS_NG) f[c + (long long)b.n[0] * b.si] = v;
        if (i >= b.n[0] - CNS_NG) f[c - (long long)b.n[0] * b.si] = v;
    }
    if (mask & 2) {
        if (j < CNS_NG) f[c + (long long)b.n[1] * b.sj] = v;
        if (j >= b.n[1] - CNS_NG) f[c - (long long)b.n[1] * b.sj] = v;
    }
    if (mask & 4) {
        if (k < CNS_NG) f[c + b.n[2]] = v;
        if (k >= b.n[2] - CNS_NG) f[c - b.n[2]] = v;
    }
}

// The axes along which each P field's stencils difference it (1 = i, 2 = j, 4 = k): the
// periodic face images it needs.
__host__ __device__ constexpr int pimg(int f) {
    return f <= PT ? 7 : (f == PFUV ? 3 : (f == PFUW ? 5 : (f == PFVW ? 6 : 1 << ((f - PMX) % 3))));
}

// Store the 16 P fields of cell (i, j, k), then the face images of those that need them.  Most
// cells need none; i and j are the same across a warp (so those branches do not diverge), and
// only the lanes within 4 cells of a k face take the k branch.  The same stores as store_img
// field by field; images lie in the ghost layers, so the order does not matter.
template <class R>
__device__ __forceinline__ void store_pset(R* __restrict__ Pw, const BoxView& b, long long c, int i, int j, int k,
                                           const R (&v)[NPF]) {
    const long long fs = b.fs;
#pragma unroll
    for (int f = 0; f < NPF; f++) Pw[f * fs + c] = v[f];
    auto images = [&](int axis, long long d) {
#pragma unroll
        for (int f = 0; f < NPF; f++)
            if (pimg(f) & axis) Pw[f * fs + c + d] = v[f];
    };
    if (i < CNS_NG) images(1, (long long)b.n[0] * b.si);
    if (i >= b.n[0] - CNS_NG) images(1, -(long long)b.n[0] * b.si);
    if (j < CNS_NG) images(2, (long long)b.n[1] * b.sj);
    if (j >= b.n[1] - CNS_NG) images(2, -(long long)b.n[1] * b.sj);
    if (k < CNS_NG) images(4, b.n[2]);
    if (k >= b.n[2] - CNS_NG) images(4, -b.n[2]);
}

// Stage 3 of a step whose result goes straight to the caller's page-locked host array
// (BoxView::host_out): the cell's new state at U[i+4][j+4][k+4][0..4] of the reference layout,
// written over the CPU-GPU link while the kernel computes.
__device__ __forceinline__ void store_host(const BoxView& b, int i, int j, int k, const double un[5]) {
    const long long g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    double* h = b.host_out + (((long long)(i + CNS_NG) * g1 + (j + CNS_NG)) * g2 + (k + CNS_NG)) * CNS_NC;
#pragma unroll
    for (int l = 0; l < CNS_NC; l++) h[l] = un[l];
}

// The S sums and the viscous dissipation of one cell from its nine first derivatives
// (cpu/diffterm.cpp:294-304).  The reference's tau_xx u_x + tau_yy v_y + tau_zz w_z, with
// tau_ii = 2 u_i,i - (2/3) d, is the same polynomial as 2 (u_x^2 + v_y^2 + w_z^2) - (2/3) d^2,
// and d = u_x + (v_y + w_z) reuses the S sum: 16 operations instead of 18 (on the FP64 pipe in
// the plain form).  k_deriv and k_deriv_tma share it, so they give the same bits.
template <class R>
__device__ __forceinline__ void dissipation(R ux, R uy, R uz, R vx, R vy, R vz, R wx, R wy, R wz, R* sx, R* sy, R* sz,
                                            R* phi) {
    *sx = vy + wz;
    *sy = ux + wz;
    *sz = ux + vy;
    const R d = ux + *sx;
    const R q = fma(ux, ux, fma(vy, vy, wz * wz));
    R f = fma((R)(-2.0 / 3.0) * d, d, q + q);
    const R txy = uy + vx, txz = uz + wx, tyz = vz + wy;
    f = fma(txy, txy, f);
    f = fma(txz, txz, f);
    f = fma(tyz, tyz, f);
    *phi = f;
}

// The nine first derivatives of (u, v, w) at one cell (cpu/diffterm.cpp:73-151); NB as in d1.
template <class R, bool NC, bool NB>
__device__ __forceinline__ void deriv9(const R* pu, const R* pv, const R* pw, long long si, long long sj,
                                       const CoefT<R>& cf, R (&d)[9], bool* xf) {
    constexpr bool X0 = xon(kExactDeriv, 0), X1 = xon(kExactDeriv, 1), X2 = xon(kExactDeriv, 2);
    d[0] = d1<X0, R, NC, NB>(pu, si, cf.da[0], xf);
    d[1] = d1<X1, R, NC, NB>(pu, sj, cf.da[1], xf);
    d[2] = d1<X2, R, NC, NB>(pu, 1, cf.da[2], xf);
    d[3] = d1<X0, R, NC, NB>(pv, si, cf.da[0], xf);
    d[4] = d1<X1, R, NC, NB>(pv, sj, cf.da[1], xf);
    d[5] = d1<X2, R, NC, NB>(pv, 1, cf.da[2], xf);
    d[6] = d1<X0, R, NC, NB>(pw, si, cf.da[0], xf);
    d[7] = d1<X1, R, NC, NB>(pw, sj, cf.da[1], xf);
    d[8] = d1<X2, R, NC, NB>(pw, 1, cf.da[2], xf);
}
// deriv9 of the plain form with the kFxDeriv axes on the fixed-point copy xu, xv, xw (exponents
// E); no branch, *xf set where a sum leaves FP64's normal range.
__device__ __forceinline__ void deriv9_fx(const double* pu, const double* pv, const double* pw, const long long* xu,
                                          const long long* xv, const long long* xw, const int* E, long long si,
                                          long long sj, const CoefT<double>& cf, double (&d)[9], bool* xf) {
    constexpr bool F0 = xon(kFxDeriv, 0), F1 = xon(kFxDeriv, 1), F2 = xon(kFxDeriv, 2);
    constexpr bool X0 = xon(kExactDeriv, 0), X1 = xon(kExactDeriv, 1), X2 = xon(kExactDeriv, 2);
    const int eu = E[PU], ev = E[PV], ew = E[PW];
    d[0] = tap_d1<F0, X0, double, true>(pu, xu, eu, si, cf.da[0], xf);
    d[1] = tap_d1<F1, X1, double, true>(pu, xu, eu, sj, cf.da[1], xf);
    d[2] = tap_d1<F2, X2, double, true>(pu, xu, eu, 1, cf.da[2], xf);
    d[3] = tap_d1<F0, X0, double, true>(pv, xv, ev, si, cf.da[0], xf);
    d[4] = tap_d1<F1, X1, double, true>(pv, xv, ev, sj, cf.da[1], xf);
    d[5] = tap_d1<F2, X2, double, true>(pv, xv, ev, 1, cf.da[2], xf);
    d[6] = tap_d1<F0, X0, double, true>(pw, xw, ew, si, cf.da[0], xf);
    d[7] = tap_d1<F1, X1, double, true>(pw, xw, ew, sj, cf.da[1], xf);
    d[8] = tap_d1<F2, X2, double, true>(pw, xw, ew, 1, cf.da[2], xf);
}

// deriv9 with the exact sums' fallbacks, out of line (as assemble_terms_fallback).
template <class R, bool NC>
__device__ __noinline__ void deriv9_fallback(const R* pu, const R* pv, const R* pw, long long si, long long sj,
                                             const CoefT<R>& cf, R* d) {
    R g[9];
    deriv9<R, NC, false>(pu, pv, pw, si, sj, cf, g, nullptr);
#pragma unroll
    for (int l = 0; l < 9; l++) d[l] = g[l];
}

// k_deriv's work at cell (i, j, k) of stage `stage`: the nine first derivatives of (u, v, w)
// into the S sums and the viscous dissipation (cpu/diffterm.cpp:294-304).  The plain form
// evaluates the derivatives with no branch between its exact sums and again with their
// fallbacks in the rare cell that needs one (the same bits either way).
// NC = false reads the P set from L2 (ld_tap), for a launch whose other blocks write it.
// FXT: a box that keeps a fixed-point copy of the P set (the kFxDeriv axes read the copy where it
// is usable and the step did not start from an upload; the FP64 evaluation otherwise).
template <class R, bool NC = true, bool FXT = false>
__device__ __forceinline__ void deriv_cell(const BoxView& b, int i, int j, int k, int stage) {
    const int pr = b.sc->pbase ^ ((stage - 1) & 1);
    const R* P = (const R*)b.P[pr];
    R* S = (R*)b.S;
    const long long c = cell_off(b, i, j, k), fs = b.fs, si = b.si, sj = b.sj;
    const CoefT<R>& cf = coefs<R>(b);
    const R* pu = P + PU * fs + c;
    const R* pv = P + PV * fs + c;
    const R* pw = P + PW * fs + c;
    R d[9];
    if constexpr (sizeof(R) == 8 && FXT) {
        // the first stage after an upload reads the FP64 fields (fx_fresh)
        const bool usable = !b.sc->fx_bad[pr] && !(stage == 1 && b.sc->fx_fresh);
        bool xf = !usable;
        if (usable) {
            const long long* X = b.X[pr];
            deriv9_fx(pu, pv, pw, X + PU * fs + c, X + PV * fs + c, X + PW * fs + c, b.sc->fx_e[pr], si, sj, cf, d,
                      &xf);
        }
        if (xf) deriv9_fallback<R, NC>(pu, pv, pw, si, sj, cf, d);
    } else if constexpr (sizeof(R) == 8) {
        bool xf = false;
        deriv9<R, NC, true>(pu, pv, pw, si, sj, cf, d, &xf);
        if (xf) deriv9_fallback<R, NC>(pu, pv, pw, si, sj, cf, d);
    } else {
        deriv9<R, NC, false>(pu, pv, pw, si, sj, cf, d, nullptr);
    }
    R sx, sy, sz, phi;
    dissipation(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], &sx, &sy, &sz, &phi);
    store_img(S + SX * fs, b, c, i, j, k, sx, 1);
    store_img(S + SY * fs, b, c, i, j, k, sy, 2);
    store_img(S + SZ * fs, b, c, i, j, k, sz, 4);
    S[SPHI * fs + c] = cf.eta * phi;
}

// diffterm + hypterm of one cell (cpu/diffterm.cpp:155-311, cpu/hypterm.cpp:29-208) from the P set
// Pr and the S set at element c: f[l] = D[l] + F[l].  NB as in d1.
// FXL / FXF: masks of the Laplacian / flux-divergence axes read from the fixed-point copy Xr of
// the P set (exponents XE); 0 without a copy.  MRG (FXL = all axes, a box whose Laplacian factors
// are equal on the axes merged, lap_merge): the second differences of a field that share a
// factor form one exact sum and one rounding (u: j + k; v: i + k; w: i + j; e: all three).
template <class R, bool NB, int FXL = 0, int FXF = 0, bool MRG = false>
__device__ __forceinline__ void assemble_terms(const BoxView& b, const R* __restrict__ Pr, const R* __restrict__ S,
                                               long long c, R u0, R v0, R w0, R t0, R (&f)[5], bool* xf,
                                               const long long* Xr = nullptr, const int* XE = nullptr) {
    const long long fs = b.fs, si = b.si, sj = b.sj;
    const CoefT<R>& cf = coefs<R>(b);
    const R* pu = Pr + PU * fs + c;
    const R* pv = Pr + PV * fs + c;
    const R* pw = Pr + PW * fs + c;
    const R* pt = Pr + PT * fs + c;
    constexpr bool XL = FXL != 0, XF = FXF != 0;
    // the copy's fields at this cell, and their exponents (unused without a copy)
    auto xat = [&](int f) -> const long long* { return (XL || XF) ? Xr + f * fs + c : nullptr; };
    auto xe = [&](int f) -> int { return (XL || XF) ? XE[f] : 0; };
    // diffterm momentum components (cpu/diffterm.cpp:155-269)
    R dmx = cf.vc[0] * u0, dmy = cf.vc[1] * v0, dmz = cf.vc[2] * w0;
    R de = fma(cf.tc, t0, __ldcg(S + SPHI * fs + c));
    if constexpr (MRG) {
        static_assert(FXL == 0b111, "merged sums read every axis from the copy");
        const XWords ui{xat(PU), si}, uj{xat(PU), sj}, uk{xat(PU), 1};
        dmx = fx_d2acc(dmx, ui, xe(PU), cf.vl[0][0], xf);
        dmx = fx_d2acc2(dmx, uj, uk, xe(PU), cf.vl[0][1], xf);
        const XWords vi{xat(PV), si}, vj{xat(PV), sj}, vk{xat(PV), 1};
        dmy = fx_d2acc(dmy, vj, xe(PV), cf.vl[1][1], xf);
        dmy = fx_d2acc2(dmy, vi, vk, xe(PV), cf.vl[1][0], xf);
        const XWords wi{xat(PW), si}, wj{xat(PW), sj}, wk{xat(PW), 1};
        dmz = fx_d2acc(dmz, wk, xe(PW), cf.vl[2][2], xf);
        dmz = fx_d2acc2(dmz, wi, wj, xe(PW), cf.vl[2][0], xf);
        const XWords ti{xat(PT), si}, tj{xat(PT), sj}, tk{xat(PT), 1};
        de = fx_d2acc3(de, ti, tj, tk, xe(PT), cf.tl[0], xf);
    } else {
        dmx = tap_d2acc<xon(FXL, 0), xon(kExactLap, 0), R, NB>(dmx, pu, xat(PU), xe(PU), si, cf.vl[0][0], xf);
        dmx = tap_d2acc<xon(FXL, 1), xon(kExactLap, 1), R, NB>(dmx, pu, xat(PU), xe(PU), sj, cf.vl[0][1], xf);
        dmx = tap_d2acc<xon(FXL, 2), xon(kExactLap, 2), R, NB>(dmx, pu, xat(PU), xe(PU), 1, cf.vl[0][2], xf);
        dmy = tap_d2acc<xon(FXL, 0), xon(kExactLap, 0), R, NB>(dmy, pv, xat(PV), xe(PV), si, cf.vl[1][0], xf);
        dmy = tap_d2acc<xon(FXL, 1), xon(kExactLap, 1), R, NB>(dmy, pv, xat(PV), xe(PV), sj, cf.vl[1][1], xf);
        dmy = tap_d2acc<xon(FXL, 2), xon(kExactLap, 2), R, NB>(dmy, pv, xat(PV), xe(PV), 1, cf.vl[1][2], xf);
        dmz = tap_d2acc<xon(FXL, 0), xon(kExactLap, 0), R, NB>(dmz, pw, xat(PW), xe(PW), si, cf.vl[2][0], xf);
        dmz = tap_d2acc<xon(FXL, 1), xon(kExactLap, 1), R, NB>(dmz, pw, xat(PW), xe(PW), sj, cf.vl[2][1], xf);
        dmz = tap_d2acc<xon(FXL, 2), xon(kExactLap, 2), R, NB>(dmz, pw, xat(PW), xe(PW), 1, cf.vl[2][2], xf);
        // diffterm energy component (cpu/diffterm.cpp:272-311)
        de = tap_d2acc<xon(FXL, 0), xon(kExactLap, 0), R, NB>(de, pt, xat(PT), xe(PT), si, cf.tl[0], xf);
        de = tap_d2acc<xon(FXL, 1), xon(kExactLap, 1), R, NB>(de, pt, xat(PT), xe(PT), sj, cf.tl[1], xf);
        de = tap_d2acc<xon(FXL, 2), xon(kExactLap, 2), R, NB>(de, pt, xat(PT), xe(PT), 1, cf.tl[2], xf);
    }
    // the mixed viscous terms (cpu/diffterm.cpp:177-265)
    dmx = d1acc<xon(kExactMixed, 0), R, NB, false>(dmx, S + SX * fs + c, si, cf.mx[0], xf);
    dmy = d1acc<xon(kExactMixed, 1), R, NB, false>(dmy, S + SY * fs + c, sj, cf.mx[1], xf);
    dmz = d1acc<xon(kExactMixed, 2), R, NB, false>(dmz, S + SZ * fs + c, 1, cf.mx[2], xf);
    de = fma(dmx, u0, de);
    de = fma(dmy, v0, de);
    de = fma(dmz, w0, de);
    // hypterm (cpu/hypterm.cpp:29-208), added to D
    f[0] = tap_d1<xon(FXF, 0), xon(kExactFlux, 0), R, NB>(Pr + PMX * fs + c, xat(PMX), xe(PMX), si, cf.ha[0], xf);
    f[0] = tap_d1acc<xon(FXF, 1), xon(kExactFlux, 1), R, NB>(f[0], Pr + PMY * fs + c, xat(PMY), xe(PMY), sj,
                                                                  cf.ha[1], xf);
    f[0] = tap_d1acc<xon(FXF, 2), xon(kExactFlux, 2), R, NB>(f[0], Pr + PMZ * fs + c, xat(PMZ), xe(PMZ), 1,
                                                                  cf.ha[2], xf);
    f[1] = tap_d1acc<xon(FXF, 0), xon(kExactFlux, 0), R, NB>(dmx, Pr + PFUU * fs + c, xat(PFUU), xe(PFUU), si,
                                                                  cf.ha[0], xf);
    f[1] = tap_d1acc<xon(FXF, 1), xon(kExactFlux, 1), R, NB>(f[1], Pr + PFUV * fs + c, xat(PFUV), xe(PFUV), sj,
                                                                  cf.ha[1], xf);
    f[1] = tap_d1acc<xon(FXF, 2), xon(kExactFlux, 2), R, NB>(f[1], Pr + PFUW * fs + c, xat(PFUW), xe(PFUW), 1,
                                                                  cf.ha[2], xf);
    f[2] = tap_d1acc<xon(FXF, 0), xon(kExactFlux, 0), R, NB>(dmy, Pr + PFUV * fs + c, xat(PFUV), xe(PFUV), si,
                                                                  cf.ha[0], xf);
    f[2] = tap_d1acc<xon(FXF, 1), xon(kExactFlux, 1), R, NB>(f[2], Pr + PFVV * fs + c, xat(PFVV), xe(PFVV), sj,
                                                                  cf.ha[1], xf);
    f[2] = tap_d1acc<xon(FXF, 2), xon(kExactFlux, 2), R, NB>(f[2], Pr + PFVW * fs + c, xat(PFVW), xe(PFVW), 1,
                                                                  cf.ha[2], xf);
    f[3] = tap_d1acc<xon(FXF, 0), xon(kExactFlux, 0), R, NB>(dmz, Pr + PFUW * fs + c, xat(PFUW), xe(PFUW), si,
                                                                  cf.ha[0], xf);
    f[3] = tap_d1acc<xon(FXF, 1), xon(kExactFlux, 1), R, NB>(f[3], Pr + PFVW * fs + c, xat(PFVW), xe(PFVW), sj,
                                                                  cf.ha[1], xf);
    f[3] = tap_d1acc<xon(FXF, 2), xon(kExactFlux, 2), R, NB>(f[3], Pr + PFWW * fs + c, xat(PFWW), xe(PFWW), 1,
                                                                  cf.ha[2], xf);
    f[4] = tap_d1acc<xon(FXF, 0), xon(kExactFlux, 0), R, NB>(de, Pr + PHU * fs + c, xat(PHU), xe(PHU), si,
                                                                  cf.ha[0], xf);
    f[4] = tap_d1acc<xon(FXF, 1), xon(kExactFlux, 1), R, NB>(f[4], Pr + PHV * fs + c, xat(PHV), xe(PHV), sj,
                                                                  cf.ha[1], xf);
    f[4] = tap_d1acc<xon(FXF, 2), xon(kExactFlux, 2), R, NB>(f[4], Pr + PHW * fs + c, xat(PHW), xe(PHW), 1,
                                                                  cf.ha[2], xf);
}

// assemble_terms with the exact sums' fallbacks, out of line: the rare cell that needs one takes
// a call, and the fast path's registers are allocated without this copy of the code beside it.
template <class R>
__device__ __noinline__ void assemble_terms_fallback(const BoxView& b, const R* __restrict__ Pr,
                                                     const R* __restrict__ S, long long c, R u0, R v0, R w0, R t0,
                                                     R* f) {
    R g[5];
    assemble_terms<R, false>(b, Pr, S, c, u0, v0, w0, t0, g, nullptr);
#pragma unroll
    for (int l = 0; l < 5; l++) f[l] = g[l];
}
// Health bits from raw IEEE fields (integer ops only; no FP64 pipe work).
__device__ __forceinline__ int health_bits(double rho, double eint) {
    unsigned long long rb = dbits(rho), eb = dbits(eint);
    int h = 0;
    if ((rb >> 63) || rb == 0ull) h |= HEALTH_NONPOS_RHO;
    if (((rb >> 52) & 0x7FF) == 0x7FF || ((eb >> 52) & 0x7FF) == 0x7FF) h |= HEALTH_NONFINITE;
    if ((eb >> 63) || eb == 0ull) h |= HEALTH_NONPOS_EINT;
    return h;
}

// ---- the plain form's fixed-point copies (cns_exact.cuh) ------------------------------------
// Largest exponent field of each P field over a block's writes: a warp maximum, folded into the
// block's shared slot by the lowest active lane (the callers run in divergent code).
__device__ __forceinline__ void fx_track(int* slot, int efield) {
    const unsigned mask = __activemask();
    const int m = (int)__reduce_max_sync(mask, (unsigned)efield);
    if ((mask & ((1u << (threadIdx.x & 31)) - 1u)) == 0) atomicMax(slot, m);
}

// Where the plain form's write-back also puts the fixed-point copy of the P set it writes: the
// copy, its exponents, the block's shared maxima, and whether a value did not fit.
struct FxSink {
    long long* X;
    const int* E;
    int* s_emax;
    bool bad;
    int nf;      // fields with a copy: the first nf of the set
    bool track;  // fold the written values into the block's maxima
};
__device__ __forceinline__ void fx_store(FxSink& fx, const BoxView& b, long long c, int i, int j, int k, int f,
                                         double v, int mask) {
    const long long w = fx_word(v, fx.E[f], &fx.bad);
    store_img(fx.X + f * b.fs, b, c, i, j, k, w, mask);
    if (fx.track) fx_track(fx.s_emax + f, fx_efield(v));
}

// The block's maxima and overflow for box `bx` (set W written) into the box's scalars, and the
// slots cleared.  Every thread of the block calls it (block barriers).
__device__ __forceinline__ void fx_flush(const BoxView* boxes, int bx, int W, int* s_emax, bool bad) {
    const int any_bad = __syncthreads_or(bad ? 1 : 0);
    if (bx >= 0) {
        BoxScalars* sc = boxes[bx].sc;
        if (threadIdx.x < NPF && s_emax[threadIdx.x] > 0) atomicMax(&sc->fx_cur[threadIdx.x], s_emax[threadIdx.x]);
        if (threadIdx.x == 0 && any_bad) atomicOr(&sc->fx_bad[W], 1);
    }
    __syncthreads();
    if (threadIdx.x < NPF) s_emax[threadIdx.x] = 0;
    __syncthreads();
}

// Prepares the write of set W by the next kernel (the assembly after a derivative pass): its
// exponents from the previous step's maxima, usable unless a value overflows (boxes whose
// assembly reads the FP64 fields: never usable).  Threads 0..NPF of the caller store (the same
// values from every block).
// The same from one thread (k_stepend).
__device__ __forceinline__ void fx_prepare_one(const BoxView& b, int W) {
    BoxScalars* sc = b.sc;
    for (int f = 0; f < NPF; f++) sc->fx_e[W][f] = fx_exponent(sc->fx_prev[f]);
    sc->fx_bad[W] = b.fx ? 0 : 1;
}
__device__ __forceinline__ void fx_prepare(const BoxView& b, int W) {
    BoxScalars* sc = b.sc;
    if (threadIdx.x < NPF) sc->fx_e[W][threadIdx.x] = fx_exponent(sc->fx_prev[threadIdx.x]);
    if (threadIdx.x == NPF) sc->fx_bad[W] = b.fx ? 0 : 1;
}

// ctoprim + flux functions of one cell's FP64 conserved state, written to the P set `Pw`
// with the periodic face images each field's stencils need.  Returns the cell's Courant
// number (only formed when `want_cour`).  Plain form: everything in FP64 (reciprocal by
// rcp_nr).  Mixed form: E/rho, the subtraction e = E/rho - |u|^2/2 and the offsets
// p - p_ref, e - e_ref, E - E_ref in FP64; the rest in FP32 (see BoxScalars).  Both store e
// (= c_v T) for the heat conduction, whose coefficients carry 1 / c_v.
template <class R>
__device__ __forceinline__ double epilogue(const BoxView& b, R* __restrict__ Pw, long long c, int i, int j, int k,
                                           const double un[5], bool want_cour, int* health);

// What the plain form's Courant number of a cell is formed from (cpu/ctoprim.cpp:50-69).
struct CourantInput64 {
    double p, rinv, u, v, w;
};
__device__ __forceinline__ double courant_plain(const BoxView& b, const CourantInput64& q) {
    const double cs = sqrt((kGamma * q.p) * q.rinv);
    const double cx = (cs + fabs(q.u)) * b.c64.cour[0];
    const double cy = (cs + fabs(q.v)) * b.c64.cour[1];
    const double cz = (cs + fabs(q.w)) * b.c64.cour[2];
    return fmax(fmax(cx, cy), cz);
}
// A double cut to FP32 on the integer pipes: its sign, exponent and top 20 mantissa bits
// (relative error below 2^-20, toward zero); zero stays zero, and anything else outside the
// normal FP32 range becomes NaN.  Hardware conversions would issue to the FP64 pipe, the bound
// of the plain kernels.
__device__ __forceinline__ float f32_cut(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    if (((hi >> 20) & 0x7FFu) - 897u < 254u)
        return __uint_as_float((hi & 0x80000000u) | (((hi & 0x7FFFFFFFu) << 3) - 0xC0000000u));
    return __uint_as_float((((hi & 0x7FFFFFFFu) | lo) == 0u) ? (hi & 0x80000000u) : 0x7FC00000u);
}
// The box's running Courant maximum (the exact FP64 numbers folded in so far), cut to FP32 on
// the integer pipes: a lower bound.  Read by lane 0 and broadcast; all lanes call it.
__device__ __forceinline__ float courant_running_max(const BoxView& b) {
    unsigned long long bits = 0;
    if ((threadIdx.x & 31) == 0) bits = *(volatile const unsigned long long*)&b.sc->courno_bits;
    return f32_cut(__longlong_as_double((long long)__shfl_sync(0xffffffffu, bits, 0)));
}
// A cell whose FP32 Courant estimate, widened by a bound on its error (2^-18, over the
// estimates' ~1.4 * 2^-20), stays below that running maximum cannot be the maximum: its exact
// number is below a value some cell already has.  Tiny or NaN estimates never pass this test.
__device__ __forceinline__ bool courant_below(float est, float running) {
    return est > 1e-30f && est * (1.0f + 0x1p-18f) < running;
}
// An FP32 estimate of courant_plain from those cut inputs: counting 2^-20 per cut input and
// 2^-24 per FP32 rounding (1.4, two products, sqrt, the sum, 1/dx, the last product) it lies
// within ~1.4 * 2^-20 of it (courant_eps is 2^-18) for states whose values are normal FP32
// numbers; outside that range it is NaN.
constexpr float kCourantPlainEps = 0x1p-18f;
__device__ __forceinline__ float courant_plain_est(const BoxView& b, const CourantInput64& q) {
    const float cs = sqrtf(1.4f * f32_cut(q.p) * f32_cut(q.rinv));
    const float cx = (cs + fabsf(f32_cut(q.u))) * b.c32.cour[0];
    const float cy = (cs + fabsf(f32_cut(q.v))) * b.c32.cour[1];
    const float cz = (cs + fabsf(f32_cut(q.w))) * b.c32.cour[2];
    return fmaxf(fmaxf(cx, cy), cz);
}

// The plain form's epilogue without the Courant number, whose inputs it leaves in *q; with `fx`,
// also the fixed-point copy of the P set it writes.
__device__ __forceinline__ void epilogue_plain(const BoxView& b, double* __restrict__ Pw, long long c, int i, int j,
                                               int k, const double un[5], int* health, CourantInput64* q,
                                               FxSink* fx = nullptr);
template <>
__device__ __forceinline__ double epilogue<double>(const BoxView& b, double* __restrict__ Pw, long long c, int i,
                                                   int j, int k, const double un[5], bool want_cour, int* health) {
    CourantInput64 q;
    epilogue_plain(b, Pw, c, i, j, k, un, health, &q);
    return want_cour ? courant_plain(b, q) : 0.0;
}
__device__ __forceinline__ void epilogue_plain(const BoxView& b, double* __restrict__ Pw, long long c, int i, int j,
                                               int k, const double un[5], int* health, CourantInput64* q,
                                               FxSink* fx) {
    const long long fs = b.fs;
    const double rho = un[0], mx = un[1], my = un[2], mz = un[3], E = un[4];
    const double rinv = rcp_nr(rho);
    const double u = mx * rinv, v = my * rinv, w = mz * rinv;
    // rho e = E - (rho u u + rho v v + rho w w) / 2 (cpu/ctoprim.cpp's E/rho - |u|^2/2, times rho);
    // p = (gamma - 1) rho e and e = rho e / rho: one operation fewer than forming E/rho and |u|^2
    const double re = fma(-0.5, fma(mx, u, fma(my, v, mz * w)), E);
    const double p = kGm1 * re;
    const double eint = re * rinv;
    const double H = E + p;
    *health |= health_bits(rho, eint);
    // Field by field, not store_pset: its 16 live FP64 values would cost the upload kernels
    // occupancy, and the FP64-bound kernels gain nothing from fewer store instructions.
    auto put = [&](int f, double val, int mask) {
        store_img(Pw + f * fs, b, c, i, j, k, val, mask);
        if (fx && f < fx->nf) fx_store(*fx, b, c, i, j, k, f, val, mask);
    };
    put(PU, u, 7);
    put(PV, v, 7);
    put(PW, w, 7);
    put(PT, eint, 7);
    put(PMX, mx, 1);
    put(PMY, my, 2);
    put(PMZ, mz, 4);
    put(PFUU, fma(mx, u, p), 1);
    put(PFVV, fma(my, v, p), 2);
    put(PFWW, fma(mz, w, p), 4);
    put(PFUV, mx * v, 3);
    put(PFUW, mx * w, 5);
    put(PFVW, my * w, 6);
    put(PHU, H * u, 1);
    put(PHV, H * v, 2);
    put(PHW, H * w, 4);
    *q = CourantInput64{p, rinv, u, v, w};
}

// The mixed form's reference values (fixed per box).  A loop over cells loads them once: read
// through the box's scalar block after each store, the compiler would have to reload them.
struct MixedRefs {
    double p, e, E;
};
__device__ __forceinline__ MixedRefs mixed_refs(const BoxView& b) {
    const BoxScalars& sc = *b.sc;
    return {sc.p_ref, sc.e_ref, sc.E_ref};
}

// The mixed form's Courant number of a cell, in FP64: it sets dt, and an FP32 dt would advance
// the mixed form by a different time each step (a drift of ~1e-7 dt per step that dominated
// its error against FP64).  1/rho by one Newton step from the FP32 reciprocal (~1e-14).
__device__ __forceinline__ double courant_mixed(const BoxView& b, double rho, double mx, double my, double mz,
                                                double p) {
    const double r64 = (double)(1.0f / (float)rho);
    const double rinv = fma(r64, fma(-rho, r64, 1.0), r64);
    const double cs = sqrt((kGamma * p) * rinv);
    const double cx = (cs + fabs(mx) * rinv) * b.c64.cour[0];
    const double cy = (cs + fabs(my) * rinv) * b.c64.cour[1];
    const double cz = (cs + fabs(mz) * rinv) * b.c64.cour[2];
    return fmax(fmax(cx, cy), cz);
}

// An FP32 estimate of courant_mixed from the FP32 reciprocal rf = 1/(float)rho, the FP32
// velocities u = (float)m * rf and p32 = (float)p.  Counting 2^-24 per rounding (rho, 1/rho,
// 1.4, p, two products, sqrt, |u|, the sum, 1/dx, the last product), its relative distance from
// courant_mixed is at most ~7 * 2^-24 for states whose values are normal FP32 numbers.
__device__ __forceinline__ float courant_mixed_est(const BoxView& b, float rf, float u, float v, float w, float p32) {
    const float cs = sqrtf(1.4f * p32 * rf);
    const float cx = (cs + fabsf(u)) * b.c32.cour[0];
    const float cy = (cs + fabsf(v)) * b.c32.cour[1];
    const float cz = (cs + fabsf(w)) * b.c32.cour[2];
    return fmaxf(fmaxf(cx, cy), cz);
}

// What a write-back that defers the FP64 Courant number keeps of a cell: the estimate and
// p - p_ref (the FP64 number is formed from p = (p - p_ref) + p_ref only for candidates).
struct CourantInput {
    float est;
    double pd;
};

__device__ __forceinline__ double epilogue_mixed(const BoxView& b, float* __restrict__ Pw, long long c, int i, int j,
                                                 int k, const double un[5], bool want_cour, int* health,
                                                 const MixedRefs& sc, CourantInput* ci = nullptr);
template <>
__device__ __forceinline__ double epilogue<float>(const BoxView& b, float* __restrict__ Pw, long long c, int i,
                                                  int j, int k, const double un[5], bool want_cour, int* health) {
    return epilogue_mixed(b, Pw, c, i, j, k, un, want_cour, health, mixed_refs(b));
}
__device__ __forceinline__ double epilogue_mixed(const BoxView& b, float* __restrict__ Pw, long long c, int i, int j,
                                                 int k, const double un[5], bool want_cour, int* health,
                                                 const MixedRefs& sc, CourantInput* ci) {
    const double rho = un[0], E = un[4];
    const float rhof = (float)rho;
    const float rf = 1.0f / rhof;
    const float mx = (float)un[1], my = (float)un[2], mz = (float)un[3];
    const float u = mx * rf, v = my * rf, w = mz * rf;
    // rho e = E - rho |u|^2 / 2: the cancelling subtraction in FP64, with the kinetic energy
    // density rho |u|^2 / 2 formed in FP32 (cpu/ctoprim.cpp's E/rho - |u|^2/2, times rho)
    const float kd = 0.5f * fmaf(mx, u, fmaf(my, v, mz * w));
    const double re = E - (double)kd;
    // offsets from the box's reference values, formed in FP64 before rounding to FP32:
    // p - p_ref = (gamma - 1) rho e - p_ref, and e - e_ref (= c_v (T - T_ref)) as
    // (rho e - rho e_ref) / rho, the difference in FP64 and the division in FP32
    const double pd = fma(kGm1, re, -sc.p);
    const float dp = (float)pd;
    const float dT = (float)fma(-rho, sc.e, re) * rf;
    const float dH = (float)(E - sc.E) + dp;  // (E + p) - H_ref
    // rho e has the sign and finiteness of e where rho > 0 (elsewhere rho's own bit is set)
    *health |= health_bits(rho, re);
    const float pv[NPF] = {u, v, w, dT, mx, my, mz, fmaf(mx, u, dp), fmaf(my, v, dp), fmaf(mz, w, dp),
                           mx * v, mx * w, my * w, dH * u, dH * v, dH * w};
    store_pset(Pw, b, c, i, j, k, pv);
    if (ci) {
        // the estimate's p in FP32 as (p - p_ref) + p_ref: within 5 * 2^-24 of p while p >= p_ref / 2
        // (three roundings of at most 2p each), which keeps the estimate's bound; cells below
        // that are left to the FP64 number (a NaN estimate always makes a cell a candidate)
        const float pref = (float)sc.p;
        ci->pd = pd;
        ci->est = dp >= -0.5f * pref ? courant_mixed_est(b, rf, u, v, w, dp + pref) : __int_as_float(0x7FC00000);
    }
    if (!want_cour) return 0.0;
    return courant_mixed(b, rho, un[1], un[2], un[3], pd + sc.p);
}

// Warp max of positive doubles via their bit patterns; lane 0 folds it into the box max.
__device__ __forceinline__ void courant_fold(const BoxView& b, double cour) {
    unsigned long long v = dbits(cour);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(&b.sc->courno_bits, v);
}

}  // namespace cns
