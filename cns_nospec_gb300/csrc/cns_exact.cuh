// Exact 8-tap stencil sums for the plain FP64 form, on the integer pipes.
//
// On GB300 an FP64 instruction holds the FP64 pipe about 64 times longer than an FP32 or
// integer one, and the plain kernels are bound by that pipe.  The stencils of the 8th-order
// operators have small integer weights over a common denominator:
//   first derivative  (ALP, BET, GAM, DEL)     = ( 672, -168,  32, -3) / 840
//   second derivative (OFF1, OFF2, OFF3, OFF4) = (8064, -1008, 128, -9) / 5040
// (cpu/header.h:88-91, cpu/diffterm.cpp:48-52), so sum_m w_m (f[+m] -+ f[-m]) can be formed
// in integers: each tap's 53-bit significand is placed 9 bits below the ulp of the largest tap
// (the bits of a tap that lie below 2^-62 of the largest one are truncated), split into two
// 31-bit halves, multiplied by its signed weight and summed in two 64-bit accumulators (one
// wide multiply-add per half) without any rounding, then rounded once to FP64, to nearest even.
// The result is therefore within half an ulp of itself plus sum|w| * 2^(emax - 1084) of the
// true sum (emax the largest tap's biased exponent field): a few ulp of the largest tap.  Where
// the taps lie within 9 binades of one another nothing is truncated and the result is the
// correctly rounded sum; where the largest taps cancel (f[+1] = f[-1] in a first derivative)
// the truncation can leave fewer good bits than the FP64 chain, whose f[+1] - f[-1] is exact.
// The caller scales the sum by its per-axis factor (coefficient / 840 or / 5040) in one FP64
// FMA: one FP64 instruction per stencil instead of eight.  Taps that are not finite, and nonzero sums outside
// FP64's normal range (|sum| below 2^-1022 or at least 2^1023), report failure; the caller then
// takes the FP64 chain, so every input gives what FP64 arithmetic gives.
#pragma once
#include <cstring>

#include "cns_common.cuh"

namespace cns {

__host__ __device__ __forceinline__ int xhi(double v) {
#ifdef __CUDA_ARCH__
    return __double2hiint(v);
#else
    unsigned long long u;
    memcpy(&u, &v, 8);
    return (int)(u >> 32);
#endif
}
__host__ __device__ __forceinline__ unsigned xlo(double v) {
#ifdef __CUDA_ARCH__
    return (unsigned)__double2loint(v);
#else
    unsigned long long u;
    memcpy(&u, &v, 8);
    return (unsigned)u;
#endif
}
__host__ __device__ __forceinline__ double xbits(unsigned long long u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double v;
    memcpy(&v, &u, 8);
    return v;
#endif
}
__host__ __device__ __forceinline__ int xclz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// x / 4, exactly, on the integer pipes (the exponent field lowered by two) for normal x of
// exponent field >= 3; infinities and NaNs stay as they are and values below 2^-1020 become a
// zero of their sign.  Both forms keep the first RK3 stage as U1 / 4, so that the second stage's
// 0.25 (U1 + dt L) is one FMA, fma(dt / 4, L, U1 / 4), with the same bits.  The mixed form keeps
// its second stage as (2/3) U2, so that the third stage's (2/3) (U2 + dt L) is
// fma(2 dt / 3, L, (2/3) U2): the multiply moves from stage 3, whose write-back also forms the
// Courant maximum, to stage 2.
__host__ __device__ __forceinline__ double quarter(double x) {
    const unsigned long long bits = ((unsigned long long)(unsigned)xhi(x) << 32) | xlo(x);
    const unsigned ef = (unsigned)(bits >> 52) & 0x7FFu;
    return xbits(ef >= 3u ? (ef == 0x7FFu ? bits : bits - (2ull << 52)) : (bits & (1ull << 63)));
}

constexpr int kXGuard = 9;  // guard bits below the largest tap's ulp

// Which stencils of the plain form take the exact sums (the others the FP64 chain), as masks
// over the axes (bit d: along d): the first derivatives of the derivative pass, those of the
// flux divergence, those of the mixed viscous terms, the Laplacian second differences.  The
// integer and FP64 pipes work side by side, so the best split keeps both busy.
constexpr int kExactDeriv = 0b110, kExactFlux = 0b100, kExactMixed = 0b100, kExactLap = 0b110;
constexpr bool xon(int mask, int axis) { return (mask >> axis) & 1; }

// The exponent field (bits 20-30 of the high word) of the largest of a set of taps, at least 1
// (zeros and subnormals share the scale of exponent 1).
__host__ __device__ __forceinline__ int xfield(double v) { return xhi(v) & 0x7FF00000; }
__host__ __device__ __forceinline__ int xmax(int a, int b) { return a > b ? a : b; }

// One tap of weight w into the accumulators, at the scale of exponent emax.
__host__ __device__ __forceinline__ void xtap(long long& L, long long& H, double v, int emax, int w) {
    const int hi = xhi(v);
    const int e = (hi >> 20) & 0x7FF;
    const unsigned mh = ((unsigned)hi & 0xFFFFFu) | (e ? 0x100000u : 0u);
    int sh = emax - (e > 1 ? e : 1);
    sh = sh < 63 ? sh : 63;
    const unsigned long long t = ((((unsigned long long)mh << 32) | xlo(v)) << kXGuard) >> sh;  // < 2^62
    const int s = hi >> 31;
    const int ws = (w ^ s) - s;  // the weight of the tap's value, sign included
    L += (long long)ws * (int)((unsigned)t & 0x7FFFFFFFu);
    H += (long long)ws * (int)(t >> 31);
}

// (H * 2^31 + L) * 2^e2 rounded to nearest even; false when outside the normal range.  *out is
// written in every case (with an unspecified value when false), so that callers need no branch.
__host__ __device__ __forceinline__ bool xround(long long H, long long L, int e2, double* out) {
    H += L >> 31;
    const unsigned l = (unsigned)L & 0x7FFFFFFFu;  // S = H 2^31 + l, 0 <= l < 2^31
    const bool neg = H < 0;
    // |S| = mh 2^31 + ml with ml < 2^31
    const unsigned long long mh = !neg ? (unsigned long long)H : (l ? (unsigned long long)~H : (unsigned long long)-H);
    const unsigned ml = !neg ? l : (l ? 0x80000000u - l : 0u);
    const bool zero = (mh | ml) == 0;
    unsigned long long top;  // |S| with its leading bit at 63
    bool sticky = false;
    int p;  // position of the leading bit of |S|
    if (mh) {
        const int z = xclz64(mh);  // >= 15: |H| < 2^49
        p = 94 - z;
        if (z <= 31) {
            const int r = 31 - z;
            top = (mh << z) | ((unsigned long long)ml >> r);
            sticky = (ml & ((1u << r) - 1u)) != 0;
        } else {
            top = (mh << z) | ((unsigned long long)ml << (z - 31));
        }
    } else {
        const unsigned long long m1 = zero ? 1ull : (unsigned long long)ml;  // no clz of 0
        const int z = xclz64(m1);  // >= 33
        p = 63 - z;
        top = m1 << z;
    }
    unsigned long long q = top >> 11;
    const unsigned rem = (unsigned)top & 0x7FFu;
    q += (rem > 0x400u || (rem == 0x400u && (sticky || (q & 1ull)))) ? 1ull : 0ull;
    const int be = p + e2 + 1023;
    const unsigned long long bits =
        ((unsigned long long)(be - 1) << 52) + q | (neg ? 0x8000000000000000ull : 0ull);
    *out = zero ? 0.0 : xbits(bits);
    return zero || (be >= 1 && be <= 2045);
}

// sum_{m=1..4} w_m (ld(m) + SGN ld(-m)), exactly, rounded once; false for taps that are not
// finite or a sum outside the normal range (*out is then written with an unspecified value).
// ld(m) returns the tap at offset m; SGN = -1 for first derivatives, +1 for the off-centre part
// of second derivatives.
template <int W1, int W2, int W3, int W4, int SGN, class Ld>
__host__ __device__ __forceinline__ bool xsum8(const Ld& ld, double* out) {
    const double a1 = ld(1), a2 = ld(2), a3 = ld(3), a4 = ld(4);
    const double b1 = ld(-1), b2 = ld(-2), b3 = ld(-3), b4 = ld(-4);
    int f = 0x00100000;
    f = xmax(f, xfield(a1));
    f = xmax(f, xfield(b1));
    f = xmax(f, xfield(a2));
    f = xmax(f, xfield(b2));
    f = xmax(f, xfield(a3));
    f = xmax(f, xfield(b3));
    f = xmax(f, xfield(a4));
    f = xmax(f, xfield(b4));
    const int emax = f >> 20;
    long long L = 0, H = 0;
    xtap(L, H, a1, emax, W1);
    xtap(L, H, b1, emax, SGN * W1);
    xtap(L, H, a2, emax, W2);
    xtap(L, H, b2, emax, SGN * W2);
    xtap(L, H, a3, emax, W3);
    xtap(L, H, b3, emax, SGN * W3);
    xtap(L, H, a4, emax, W4);
    xtap(L, H, b4, emax, SGN * W4);
    const bool ok = xround(H, L, emax - 1075 - kXGuard, out);
    return ok && emax != 0x7FF;
}

// The exact stencils with their FP64 fallbacks.  a[0..3] are the chain's coefficients
// (weights / denominator x factor), a[4] = factor / denominator.
template <class Ld>
__host__ __device__ __forceinline__ double xd1acc(double acc, const Ld& ld, const double* a) {
    double x;
    if (xsum8<672, -168, 32, -3, -1>(ld, &x)) return fma(a[4], x, acc);
    acc = fma(a[0], ld(1) - ld(-1), acc);
    acc = fma(a[1], ld(2) - ld(-2), acc);
    acc = fma(a[2], ld(3) - ld(-3), acc);
    return fma(a[3], ld(4) - ld(-4), acc);
}
template <class Ld>
__host__ __device__ __forceinline__ double xd2acc(double acc, const Ld& ld, const double* b) {
    double x;
    if (xsum8<8064, -1008, 128, -9, 1>(ld, &x)) return fma(b[4], x, acc);
    acc = fma(b[0], ld(1) + ld(-1), acc);
    acc = fma(b[1], ld(2) + ld(-2), acc);
    acc = fma(b[2], ld(3) + ld(-3), acc);
    return fma(b[3], ld(4) + ld(-4), acc);
}
// The same without the fallback branch: the exact result whatever the taps, and *fail set where
// xd1acc / xd2acc would have taken the FP64 chain.  A caller evaluates a whole cell this way,
// with no branch between its stencils, and evaluates the cell again with xd1acc / xd2acc when
// *fail is set; every stencil then gives the bits xd1acc / xd2acc give.
template <class Ld>
__host__ __device__ __forceinline__ double xd1acc_nb(double acc, const Ld& ld, const double* a, bool* fail) {
    double x;
    *fail |= !xsum8<672, -168, 32, -3, -1>(ld, &x);
    return fma(a[4], x, acc);
}
template <class Ld>
__host__ __device__ __forceinline__ double xd2acc_nb(double acc, const Ld& ld, const double* b, bool* fail) {
    double x;
    *fail |= !xsum8<8064, -1008, 128, -9, 1>(ld, &x);
    return fma(b[4], x, acc);
}

// ---- fixed-point copies of the stencil fields ------------------------------------------------
// The integer sums above place each tap's significand for every stencil that reads it (~20
// integer instructions a tap).  The plain form's default kernels (the derivative pass and the
// Laplacians: copies of u, v, w, e) and its TMA-staged fixed-point assembly (copies of every
// field) instead read a fixed-point copy of the field: X = trunc(v * 2^-E), one exponent E per
// field and box, chosen so that |X| < 2^62, stored as two 31-bit chunks in one 64-bit word (low
// word X mod 2^31, in [0, 2^31); high word X >> 31, signed).  A stencil is then two wide integer
// multiply-adds per tap, with no placement, and S = sum_m w_m X_m is exact in two 64-bit
// accumulators (|w| sums to at most 18418 < 2^15 a stencil, 3 x 18418 < 2^16 for three merged
// second differences); it is rounded once to FP64 (xround) as S * 2^E.  Against the exact sum
// sum_m w_m v_m the result is within half an ulp of itself plus sum|w| * 2^E: with E set from the
// field's largest magnitude M (M < 2^(E + 60)), within sum|w| * 2^-60 M.  The producer of a field
// writes its copy; values that do not fit (|v| >= 2^(E + 62) by the exponent test, or not finite)
// are reported, and the assembly then reads the FP64 fields instead.
constexpr int kFxHeadroom = 1082;  // E = (biased exponent field of M) - 1082: M < 2^(E + 60)

// E for a field whose largest biased exponent field was emax (0 when every value was zero).
__host__ __device__ __forceinline__ int fx_exponent(int emax) { return (emax > 0 ? emax : 1) - kFxHeadroom; }

// The fixed-point word of v at exponent E; *bad set when it does not fit.
__host__ __device__ __forceinline__ long long fx_word(double v, int E, bool* bad) {
    const int hi = xhi(v);
    const int e = (hi >> 20) & 0x7FF;
    const unsigned long long m = ((unsigned long long)(((unsigned)hi & 0xFFFFFu) | (e ? 0x100000u : 0u)) << 32) | xlo(v);
    const int sh = (e > 1 ? e : 1) - 1075 - E;  // X = m * 2^sh, truncated toward zero
    *bad |= (e == 0x7FF) | (sh > 9);
    const int r = -sh < 63 ? -sh : 63;
    const unsigned long long x = sh >= 0 ? (m << (sh & 15)) : (m >> r);  // < 2^62 unless bad
    const long long X = (hi < 0) ? -(long long)x : (long long)x;
    return (long long)(((unsigned long long)(unsigned)(int)(X >> 31) << 32) | (unsigned long long)(X & 0x7FFFFFFFll));
}

// Exponent field of |v| (bits 20-30 of its high word) for the producers' maxima.
__host__ __device__ __forceinline__ int fx_efield(double v) { return (xhi(v) >> 20) & 0x7FF; }

// One tap of weight wt into the accumulators.
__host__ __device__ __forceinline__ void fx_tap(long long& L, long long& H, long long w, int wt) {
    L += (long long)wt * (long long)(int)(unsigned)(w & 0xFFFFFFFFll);
    H += (long long)wt * (long long)(int)(w >> 32);
}

// sum_{m=1..4} w_m (X(m) + SGN X(-m)) of fixed-point words, rounded once to FP64 and scaled by
// 2^E; false when the result is outside FP64's normal range (then *out is unspecified).
template <int W1, int W2, int W3, int W4, int SGN, class Ld>
__host__ __device__ __forceinline__ void fx_taps8(long long& L, long long& H, const Ld& ld) {
    fx_tap(L, H, ld(1), W1);
    fx_tap(L, H, ld(-1), SGN * W1);
    fx_tap(L, H, ld(2), W2);
    fx_tap(L, H, ld(-2), SGN * W2);
    fx_tap(L, H, ld(3), W3);
    fx_tap(L, H, ld(-3), SGN * W3);
    fx_tap(L, H, ld(4), W4);
    fx_tap(L, H, ld(-4), SGN * W4);
}
template <int W1, int W2, int W3, int W4, int SGN, class Ld>
__host__ __device__ __forceinline__ bool fx_sum8(const Ld& ld, int E, double* out) {
    long long L = 0, H = 0;
    fx_taps8<W1, W2, W3, W4, SGN>(L, H, ld);
    return xround(H, L, E, out);
}

// First / second derivative stencils on fixed-point words: acc + a[4] * sum, *fail where the sum
// is outside FP64's normal range.
template <class Ld>
__host__ __device__ __forceinline__ double fx_d1acc(double acc, const Ld& ld, int E, const double* a, bool* fail) {
    double x;
    *fail |= !fx_sum8<672, -168, 32, -3, -1>(ld, E, &x);
    return fma(a[4], x, acc);
}
// Second differences of one field along two or three axes whose factors are equal (cubic
// cells): the sum over all their taps formed exactly and rounded once (|S| < 2^(62+16)).
template <class L1, class L2>
__host__ __device__ __forceinline__ double fx_d2acc2(double acc, const L1& l1, const L2& l2, int E, const double* b,
                                                     bool* fail) {
    long long L = 0, H = 0;
    fx_taps8<8064, -1008, 128, -9, 1>(L, H, l1);
    fx_taps8<8064, -1008, 128, -9, 1>(L, H, l2);
    double x;
    *fail |= !xround(H, L, E, &x);
    return fma(b[4], x, acc);
}
template <class L1, class L2, class L3>
__host__ __device__ __forceinline__ double fx_d2acc3(double acc, const L1& l1, const L2& l2, const L3& l3, int E,
                                                     const double* b, bool* fail) {
    long long L = 0, H = 0;
    fx_taps8<8064, -1008, 128, -9, 1>(L, H, l1);
    fx_taps8<8064, -1008, 128, -9, 1>(L, H, l2);
    fx_taps8<8064, -1008, 128, -9, 1>(L, H, l3);
    double x;
    *fail |= !xround(H, L, E, &x);
    return fma(b[4], x, acc);
}
template <class Ld>
__host__ __device__ __forceinline__ double fx_d2acc(double acc, const Ld& ld, int E, const double* b, bool* fail) {
    double x;
    *fail |= !fx_sum8<8064, -1008, 128, -9, 1>(ld, E, &x);
    return fma(b[4], x, acc);
}

// Tap loaders: a strided array (global memory through a chosen load, or shared memory) and a
// register column.
template <int MODE>  // 0: read-only path, 1: L2 (data written during the launch), 2: plain
struct XTaps {
    const double* p;
    long long s;
    __device__ __forceinline__ double operator()(int m) const {
        if (MODE == 0) return __ldg(p + m * s);
        if (MODE == 1) return __ldcg(p + m * s);
        return p[m * s];
    }
};

}  // namespace cns
