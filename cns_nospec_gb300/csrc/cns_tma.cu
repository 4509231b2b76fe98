// cns_tma.cu -- k_assemble of the mixed form with its stencil tiles staged by TMA.
//
// Tile: 8 (i) x 8 (j) x 32 (k) cells; 256 threads = 32 (k) x 8 (j), each thread owns the 8
// cells of its (j, k) column along i.  The 20 FP32 fields the assembly reads are brought into
// shared memory one after another as 3-D boxes of the tile plus a 4-cell halo only along the
// axes that field is differenced on (a full 40x16x16 box for u, v, w, T; 32x8x16 for an
// x-only field; ...), by cp.async.bulk.tensor.4d (a 4-D tensor map over (k, j, i, field) of
// the box's P or S set), double-buffered: the copy of field g+1 is in flight while field g is
// consumed.  i-direction taps come from a 16-deep register column, j/k taps from shared
// memory with compile-time offsets.  The arithmetic is done in exactly the order of the
// direct-load kernel (cns_fused.cu), so both give the same bits.
//
// Every mbarrier wait is bounded (about one second of global time); on expiry the block sets
// HEALTH_TIMEOUT in the box's status, waits (bounded again) for its own copies and returns.
#include <cuda.h>

#include "cns_fused.cuh"
#include "cns_internal.h"

namespace cns {

constexpr int XI = 8, XJ = 8, XK = 32;

// The boxes: halo axes -> extents (k, j, i).
enum { BX_FULL = 0, BX_I, BX_J, BX_K, BX_IJ, BX_IK, BX_JK, BX_C, BX_COUNT };
__host__ __device__ constexpr int box_k(int s) { return (s == BX_FULL || s == BX_K || s == BX_IK || s == BX_JK) ? XK + 8 : XK; }
__host__ __device__ constexpr int box_j(int s) { return (s == BX_FULL || s == BX_J || s == BX_IJ || s == BX_JK) ? XJ + 8 : XJ; }
__host__ __device__ constexpr int box_i(int s) { return (s == BX_FULL || s == BX_I || s == BX_IJ || s == BX_IK) ? XI + 8 : XI; }
__host__ __device__ constexpr int box_elems(int s) { return box_k(s) * box_j(s) * box_i(s); }
constexpr int kBufElems = box_elems(BX_FULL);  // 10240 floats, the largest box

// Tensor maps of one mixed box: P sets (7 shapes each) and the S set (I, J, K, C boxes).
struct TmaMaps {
    CUtensorMap p[2][7];
    CUtensorMap s[4];
    CUtensorMap x[2][7];  // plain FP64 boxes: the fixed-point copies of P[0], P[1] (64-bit words)
};
static_assert(sizeof(CUtensorMap) == 128, "CUtensorMap is 128 bytes");

// The 20 loads of a tile, in consumption order: (set 0 = P / 1 = S, field, box shape).
struct Load {
    unsigned char set, field, shape;
};
#define CNS_TMA_SCHED                                                                       \
    {{1, SPHI, BX_C},  {0, PT, BX_FULL},   {0, PU, BX_FULL},   {1, SX, BX_I},   {0, PV, BX_FULL}, \
     {1, SY, BX_J},    {0, PW, BX_FULL},   {1, SZ, BX_K},      {0, PMX, BX_I},  {0, PMY, BX_J},   \
     {0, PMZ, BX_K},   {0, PFUU, BX_I},    {0, PFUV, BX_IJ},   {0, PFUW, BX_IK}, {0, PFVV, BX_J}, \
     {0, PFVW, BX_JK}, {0, PFWW, BX_K},    {0, PHU, BX_I},     {0, PHV, BX_J},  {0, PHW, BX_K}}
__constant__ Load kSched[20] = CNS_TMA_SCHED;
constexpr Load kSchedPlan[20] = CNS_TMA_SCHED;  // the same list, for compile-time planning
constexpr int kLoads = 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_init_n(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase with the given parity, giving up after ~1 s of global time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > 1000000000ull) return false;
    return true;
}
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// Issue the copy of `L` for tile `tile` into `buf`, completing on `bar` (R: float for mixed
// boxes, double for FP64 boxes, whose tensor maps are FP64).
template <class R, bool FX = false>
__device__ __forceinline__ void issue_load(const BoxView* boxes, const Tile* tiles, int tile, const Load L, int flip,
                                           R* buf, uint64_t* bar) {
    const Tile T = tiles[tile];
    const BoxView& b = boxes[T.box];
    const TmaMaps* maps = (const TmaMaps*)b.tma;
    const CUtensorMap* map;
    if (L.set == 0) {
        // stage s reads P[pbase ^ ((s-1)&1)] (FX: its fixed-point copy)
        map = FX ? &maps->x[b.sc->pbase ^ flip][L.shape] : &maps->p[b.sc->pbase ^ flip][L.shape];
    } else {
        const int si = L.shape == BX_I ? 0 : L.shape == BX_J ? 1 : L.shape == BX_K ? 2 : 3;
        map = &maps->s[si];
    }
    const int hk = box_k(L.shape) == XK ? 0 : 4, hj = box_j(L.shape) == XJ ? 0 : 4, hi = box_i(L.shape) == XI ? 0 : 4;
    mbar_expect_tx(bar, (uint32_t)(box_elems(L.shape) * sizeof(R)));
    tma_load(buf, map, T.k0 + CNS_NG - hk, T.j0 + CNS_NG - hj, T.i0 + CNS_NG - hi, L.field, bar);
}
// Load number g of this block in kSched (tile g / 20, entry g % 20).
template <class R, bool FX = false>
__device__ __forceinline__ void issue(const BoxView* boxes, const Tile* tiles, int tile, int entry, int flip,
                                      R* buf, uint64_t* bar) {
    issue_load<R, FX>(boxes, tiles, tile, kSched[entry], flip, buf, bar);
}

// ---- per-field consumers (compile-time box extents) ----------------------------------------
// Offsets below are in elements of the box in shared memory: (ii, jj, kk) -> (ii*BJ + jj)*BK + kk.
template <int S>
struct Bx {
    static constexpr int K = box_k(S), J = box_j(S), I = box_i(S);
    static constexpr int HK = K == XK ? 0 : 4, HJ = J == XJ ? 0 : 4, HI = I == XI ? 0 : 4;
    __device__ static __forceinline__ int at(int ii, int jj, int kk) { return (ii * J + jj) * K + kk; }
};

// acc + sum_m a_m (p[+m s] - p[-m s]) on shared memory, offsets s in elements
// Ask the copy engine to bring the FP64 state rows this tile's write-back will read into L2
// (a hint; no data moves to the SM).  One row = the tile's k extent of one (field, i, j) line:
// 32 doubles from element (k0 + 4), which is 16-byte aligned (rows are padded to 8 elements),
// rounded up to an even count (16-byte size), which stays inside the padded row.
__device__ __forceinline__ void prefetch_state_l2(const BoxView& b, const Tile& T, int stage, int tid) {
    const int ni = min(XI, b.n[0] - T.i0), nj = min(XJ, b.n[1] - T.j0), nk = min(XK, b.n[2] - T.k0);
    const uint32_t bytes = (uint32_t)((nk + 1) & ~1) * 8u;
    const int rows = CNS_NC * XI * XJ;
    for (int r = tid; r < (stage == 1 ? rows : 2 * rows); r += kTileThreads) {
        const int rr = r % rows, l = rr / (XI * XJ), i = (rr / XJ) % XI, j = rr % XJ;
        if (i >= ni || j >= nj) continue;
        const double* base = r < rows ? b.U : b.Us;
        const double* p = base + l * b.fs + cell_off(b, T.i0 + i, T.j0 + j, T.k0);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
    }
}

template <bool X, class R>
__device__ __forceinline__ R sd1acc(R acc, const R* p, int s, const R* a) {
    if constexpr (sizeof(R) == 8 && X) return xd1acc(acc, XTaps<2>{p, s}, a);
    acc = fma(a[0], p[s] - p[-s], acc);
    acc = fma(a[1], p[2 * s] - p[-2 * s], acc);
    acc = fma(a[2], p[3 * s] - p[-3 * s], acc);
    acc = fma(a[3], p[4 * s] - p[-4 * s], acc);
    return acc;
}
template <bool X, class R>
__device__ __forceinline__ R sd1(const R* p, int s, const R* a) {
    if constexpr (sizeof(R) == 8 && X) return xd1acc(0.0, XTaps<2>{p, s}, a);
    R acc = a[0] * (p[s] - p[-s]);
    acc = fma(a[1], p[2 * s] - p[-2 * s], acc);
    acc = fma(a[2], p[3 * s] - p[-3 * s], acc);
    acc = fma(a[3], p[4 * s] - p[-4 * s], acc);
    return acc;
}
template <bool X, class R>
__device__ __forceinline__ R sd2acc(R acc, const R* p, int s, const R* b) {
    if constexpr (sizeof(R) == 8 && X) return xd2acc(acc, XTaps<2>{p, s}, b);
    acc = fma(b[0], p[s] + p[-s], acc);
    acc = fma(b[1], p[2 * s] + p[-2 * s], acc);
    acc = fma(b[2], p[3 * s] + p[-3 * s], acc);
    acc = fma(b[3], p[4 * s] + p[-4 * s], acc);
    return acc;
}
// the same on a register column (i direction), centre index c
template <bool X, class R>
__device__ __forceinline__ R cd1acc(R acc, const R* col, int c, const R* a) {
    if constexpr (sizeof(R) == 8 && X) return xd1acc(acc, [&](int m) { return col[c + m]; }, a);
    acc = fma(a[0], col[c + 1] - col[c - 1], acc);
    acc = fma(a[1], col[c + 2] - col[c - 2], acc);
    acc = fma(a[2], col[c + 3] - col[c - 3], acc);
    acc = fma(a[3], col[c + 4] - col[c - 4], acc);
    return acc;
}
template <bool X, class R>
__device__ __forceinline__ R cd1(const R* col, int c, const R* a) {
    if constexpr (sizeof(R) == 8 && X) return xd1acc(0.0, [&](int m) { return col[c + m]; }, a);
    R acc = a[0] * (col[c + 1] - col[c - 1]);
    acc = fma(a[1], col[c + 2] - col[c - 2], acc);
    acc = fma(a[2], col[c + 3] - col[c - 3], acc);
    acc = fma(a[3], col[c + 4] - col[c - 4], acc);
    return acc;
}
template <bool X, class R>
__device__ __forceinline__ R cd2acc(R acc, const R* col, int c, const R* b) {
    if constexpr (sizeof(R) == 8 && X) return xd2acc(acc, [&](int m) { return col[c + m]; }, b);
    acc = fma(b[0], col[c + 1] + col[c - 1], acc);
    acc = fma(b[1], col[c + 2] + col[c - 2], acc);
    acc = fma(b[2], col[c + 3] + col[c - 3], acc);
    acc = fma(b[3], col[c + 4] + col[c - 4], acc);
    return acc;
}

// The full-box (u, v, w or T) pass: centre weight, then the i, j, k second differences.
template <class R>
__device__ __forceinline__ void lap_full(const R* s, int tj, int tk, R cw, const R* wi, const R* wj, const R* wk,
                                         R* acc, R* ctr, bool init_from_acc) {
    using B = Bx<BX_FULL>;
    R col[16];
#pragma unroll
    for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj + 4, tk + 4)];
#pragma unroll
    for (int i = 0; i < XI; i++) {
        const R c0 = col[i + 4];
        ctr[i] = c0;
        R a = init_from_acc ? fma(cw, c0, acc[i]) : cw * c0;
        a = cd2acc<xon(kExactLap, 0)>(a, col, i + 4, wi);
        const R* p = s + B::at(i + 4, tj + 4, tk + 4);
        a = sd2acc<xon(kExactLap, 1)>(a, p, B::K, wj);
        a = sd2acc<xon(kExactLap, 2)>(a, p, 1, wk);
        acc[i] = a;
    }
}

// The sums of one tile, per thread (its 8 cells along i): f0..f4 of the five conserved
// variables (f1..f4 accumulate in dmx, dmy, dmz, de) and the centre velocity c0.

// Field e of a tile's 20 loads (schedule kSched), staged at s, folded into the sums.
template <class R>
__device__ __forceinline__ void consume_field(int e, const R* s, const Tile& T, const BoxView& b, const CoefT<R>& cf,
                                              int tj, int tk, R* dmx, R* dmy, R* dmz, R* de, R* f0, R* c0) {
    switch (e) {
        case 0: {  // SPHI: de starts from eta * Phi
            using B = Bx<BX_C>;
#pragma unroll
            for (int i = 0; i < XI; i++) de[i] = s[B::at(i, tj, tk)];
            break;
        }
        case 1: {  // PT: de = tc T0 + phi, then the x, y, z second differences
            R t0[XI];
            lap_full(s, tj, tk, cf.tc, cf.tl[0], cf.tl[1], cf.tl[2], de, t0, true);
            break;
        }
        case 2:  // PU: dmx = vc0 u0 + x, y, z second differences
            lap_full(s, tj, tk, cf.vc[0], cf.vl[0][0], cf.vl[0][1], cf.vl[0][2], dmx, c0, false);
            break;
        case 3: {  // SX: dmx += (eta/3) d/dx (v_y + w_z); then the work term dmx u0
            using B = Bx<BX_I>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj, tk)];
#pragma unroll
            for (int i = 0; i < XI; i++) {
                dmx[i] = cd1acc<xon(kExactMixed, 0)>(dmx[i], col, i + 4, cf.mx[0]);
                de[i] = fma(dmx[i], c0[i], de[i]);
            }
            break;
        }
        case 4:
            lap_full(s, tj, tk, cf.vc[1], cf.vl[1][0], cf.vl[1][1], cf.vl[1][2], dmy, c0, false);
            break;
        case 5: {  // SY
            using B = Bx<BX_J>;
#pragma unroll
            for (int i = 0; i < XI; i++) {
                dmy[i] = sd1acc<xon(kExactMixed, 1)>(dmy[i], s + B::at(i, tj + 4, tk), B::K, cf.mx[1]);
                de[i] = fma(dmy[i], c0[i], de[i]);
            }
            break;
        }
        case 6:
            lap_full(s, tj, tk, cf.vc[2], cf.vl[2][0], cf.vl[2][1], cf.vl[2][2], dmz, c0, false);
            break;
        case 7: {  // SZ
            using B = Bx<BX_K>;
#pragma unroll
            for (int i = 0; i < XI; i++) {
                dmz[i] = sd1acc<xon(kExactMixed, 2)>(dmz[i], s + B::at(i, tj, tk + 4), 1, cf.mx[2]);
                de[i] = fma(dmz[i], c0[i], de[i]);
            }
            break;
        }
        case 8: {  // PMX: f0 = -d(rho u)/dx
            using B = Bx<BX_I>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj, tk)];
#pragma unroll
            for (int i = 0; i < XI; i++) f0[i] = cd1<xon(kExactFlux, 0)>(col, i + 4, cf.ha[0]);
            break;
        }
        case 9: {  // PMY
            using B = Bx<BX_J>;
#pragma unroll
            for (int i = 0; i < XI; i++) f0[i] = sd1acc<xon(kExactFlux, 1)>(f0[i], s + B::at(i, tj + 4, tk), B::K, cf.ha[1]);
            break;
        }
        case 10: {  // PMZ
            using B = Bx<BX_K>;
#pragma unroll
            for (int i = 0; i < XI; i++) f0[i] = sd1acc<xon(kExactFlux, 2)>(f0[i], s + B::at(i, tj, tk + 4), 1, cf.ha[2]);
            break;
        }
        case 11: {  // PFUU along x -> f1 (in dmx)
            using B = Bx<BX_I>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj, tk)];
#pragma unroll
            for (int i = 0; i < XI; i++) dmx[i] = cd1acc<xon(kExactFlux, 0)>(dmx[i], col, i + 4, cf.ha[0]);
            break;
        }
        case 12: {  // PFUV: along y -> f1, along x -> f2 (in dmy)
            using B = Bx<BX_IJ>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj + 4, tk)];
#pragma unroll
            for (int i = 0; i < XI; i++) {
                dmx[i] = sd1acc<xon(kExactFlux, 1)>(dmx[i], s + B::at(i + 4, tj + 4, tk), B::K, cf.ha[1]);
                dmy[i] = cd1acc<xon(kExactFlux, 0)>(dmy[i], col, i + 4, cf.ha[0]);
            }
            break;
        }
        case 13: {  // PFUW: along z -> f1, along x -> f3 (in dmz)
            using B = Bx<BX_IK>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj, tk + 4)];
#pragma unroll
            for (int i = 0; i < XI; i++) {
                dmx[i] = sd1acc<xon(kExactFlux, 2)>(dmx[i], s + B::at(i + 4, tj, tk + 4), 1, cf.ha[2]);
                dmz[i] = cd1acc<xon(kExactFlux, 0)>(dmz[i], col, i + 4, cf.ha[0]);
            }
            break;
        }
        case 14: {  // PFVV along y -> f2
            using B = Bx<BX_J>;
#pragma unroll
            for (int i = 0; i < XI; i++) dmy[i] = sd1acc<xon(kExactFlux, 1)>(dmy[i], s + B::at(i, tj + 4, tk), B::K, cf.ha[1]);
            break;
        }
        case 15: {  // PFVW: along z -> f2, along y -> f3
            using B = Bx<BX_JK>;
#pragma unroll
            for (int i = 0; i < XI; i++) {
                const R* p = s + B::at(i, tj + 4, tk + 4);
                dmy[i] = sd1acc<xon(kExactFlux, 2)>(dmy[i], p, 1, cf.ha[2]);
                dmz[i] = sd1acc<xon(kExactFlux, 1)>(dmz[i], p, B::K, cf.ha[1]);
            }
            break;
        }
        case 16: {  // PFWW along z -> f3
            using B = Bx<BX_K>;
#pragma unroll
            for (int i = 0; i < XI; i++) dmz[i] = sd1acc<xon(kExactFlux, 2)>(dmz[i], s + B::at(i, tj, tk + 4), 1, cf.ha[2]);
            break;
        }
        case 17: {  // PHU along x -> f4 (in de)
            using B = Bx<BX_I>;
            R col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj, tk)];
#pragma unroll
            for (int i = 0; i < XI; i++) de[i] = cd1acc<xon(kExactFlux, 0)>(de[i], col, i + 4, cf.ha[0]);
            break;
        }
        case 18: {  // PHV
            using B = Bx<BX_J>;
#pragma unroll
            for (int i = 0; i < XI; i++) de[i] = sd1acc<xon(kExactFlux, 1)>(de[i], s + B::at(i, tj + 4, tk), B::K, cf.ha[1]);
            break;
        }
        default: {  // 19, PHW; for mixed boxes then -H_ref div(u) (their P set holds
                   // ((E+p) - H_ref) u), with div(u) = (S_x + S_y + S_z) / 2 read at the cell (S is
                   // L2-resident)
            using B = Bx<BX_K>;
            if constexpr (sizeof(R) == 4) {
                const float href = -(float)b.sc->H_ref;
                const float* S = (const float*)b.S;
                const int j = min(T.j0 + tj, b.n[1] - 1), k = min(T.k0 + tk, b.n[2] - 1);
#pragma unroll
                for (int i = 0; i < XI; i++) {
                    const long long c = cell_off(b, min(T.i0 + i, b.n[0] - 1), j, k);
                    const float hsum = __ldg(S + SX * b.fs + c) + __ldg(S + SY * b.fs + c) + __ldg(S + SZ * b.fs + c);
                    const float a = sd1acc<xon(kExactFlux, 2)>(de[i], s + B::at(i, tj, tk + 4), 1, cf.ha[2]);
                    de[i] = fmaf(href, 0.5f * hsum, a);
                }
            } else {
#pragma unroll
                for (int i = 0; i < XI; i++) de[i] = sd1acc<xon(kExactFlux, 2)>(de[i], s + B::at(i, tj, tk + 4), 1, cf.ha[2]);
            }
            break;
        }
    }
}

// Park the five sums of a thread's 8 cells at column `col` of a 40 KB stash; the write-back
// reads them back as stash[(i * 5 + l) * 256 + col].
template <class R>
__device__ __forceinline__ void park_sums(R* stash, int col, const R* f0, const R* dmx, const R* dmy, const R* dmz,
                                          const R* de) {
#pragma unroll
    for (int i = 0; i < XI; i++) {
        stash[(i * 5 + 0) * kTileThreads + col] = f0[i];
        stash[(i * 5 + 1) * kTileThreads + col] = dmx[i];
        stash[(i * 5 + 2) * kTileThreads + col] = dmy[i];
        stash[(i * 5 + 3) * kTileThreads + col] = dmz[i];
        stash[(i * 5 + 4) * kTileThreads + col] = de[i];
    }
}

// RK3 stage combine (FP64) and the fused write-back, as in k_assemble, of the 8 cells of
// column `col` = (tj, tk) of tile T whose sums are parked in `stash`; health bits and (stage 3)
// the Courant number folded into the box's scalars.  Every lane of the calling warp takes part.
template <int STAGE>
__device__ __forceinline__ void write_back(const BoxView& b, const Tile& T, float* stash, int col, int tj,
                                           int tk) {
    const int pr = b.sc->pbase ^ ((STAGE - 1) & 1);
    float* Pw = (float*)b.P[pr ^ 1];
    const double dt = b.sc->dt, dt4 = 0.25 * dt, dt23 = (2.0 / 3.0) * dt;
    const MixedRefs refs = mixed_refs(b);
    const int j = T.j0 + tj, k = T.k0 + tk;
    const int jc = min(j, b.n[1] - 1), kc = min(k, b.n[2] - 1);
    const long long fs = b.fs;
    double cmax = 0.0;
    float m32 = 0.0f;  // stage 3: the largest FP32 Courant estimate of this thread's cells
    int health = 0;
    // Software-pipelined: the state of cell i + 1 is loaded while cell i is computed (the
    // loads of cells outside the box are clamped to a cell inside it and never used).
    double nu[5], ns[5];
    {
        const long long c = cell_off(b, min(T.i0, b.n[0] - 1), jc, kc);
#pragma unroll
        for (int l = 0; l < 5; l++) {
            nu[l] = b.U[c + l * fs];
            ns[l] = STAGE == 1 ? 0.0 : b.Us[c + l * fs];
        }
    }
#pragma unroll 2
    for (int i = 0; i < XI; i++) {
        double u0[5], us[5];
#pragma unroll
        for (int l = 0; l < 5; l++) {
            u0[l] = nu[l];
            us[l] = ns[l];
        }
        if (i + 1 < XI) {
            const long long c1 = cell_off(b, min(T.i0 + i + 1, b.n[0] - 1), jc, kc);
#pragma unroll
            for (int l = 0; l < 5; l++) {
                nu[l] = b.U[c1 + l * fs];
                ns[l] = STAGE == 1 ? 0.0 : b.Us[c1 + l * fs];
            }
        }
        const int ic = T.i0 + i;
        if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
        const long long c = cell_off(b, ic, j, k);
        float f[5];
#pragma unroll
        for (int l = 0; l < 5; l++) f[l] = stash[(i * 5 + l) * kTileThreads + col];
        double un[5];
#pragma unroll
        for (int l = 0; l < 5; l++) {
            const long long e = c + l * fs;
            const double r = (double)f[l];
            if (STAGE == 1) {
                un[l] = fma(dt, r, u0[l]);
                b.Us[e] = quarter(un[l]);  // U1 / 4
            } else if (STAGE == 2) {
                un[l] = fma(0.75, u0[l], fma(dt4, r, us[l]));  // = fma(0.75, U0, 0.25 * fma(dt, L, U1))
                b.Us[e] = (2.0 / 3.0) * un[l];  // (2/3) U2
            } else {
                un[l] = fma(1.0 / 3.0, u0[l], fma(dt23, r, us[l]));  // U0 / 3 + (2/3) (U2 + dt L)
                b.U[e] = un[l];
            }
        }
        if (STAGE == 3) {
            if (b.host_out) store_host(b, ic, j, k, un);
            // park the FP32 Courant estimate and p - p_ref (FP64, as two words) over the cell's sums
            CourantInput ci;
            epilogue_mixed(b, Pw, c, ic, j, k, un, false, &health, refs, &ci);
            stash[(i * 5 + 0) * kTileThreads + col] = ci.est;
            stash[(i * 5 + 1) * kTileThreads + col] = __int_as_float(__double2hiint(ci.pd));
            stash[(i * 5 + 2) * kTileThreads + col] = __int_as_float(__double2loint(ci.pd));
            m32 = fmaxf(m32, ci.est);
        } else {
            epilogue_mixed(b, Pw, c, ic, j, k, un, false, &health, refs);
        }
    }
    if (health) atomicOr(&b.sc->status, health);
    if (STAGE == 3) {
        // The FP64 Courant number only of the cells that can hold this thread's maximum: with
        // |est - exact| <= eps * exact (eps = 2^-20, over twice the estimate's ~7 * 2^-24), a cell
        // whose estimate is below (1 - 2 eps) of the largest estimate is below that cell's exact
        // value, so the maximum over the candidates is the maximum over all cells, bit for bit.
        // NaN or tiny estimates (outside the bound's range) are always candidates, and all cells
        // are when an estimate overflowed.  The warp runs the FP64 code once per round of
        // candidates (mostly one), not once per cell.
        // Cells whose estimate, widened by its bound, stays below the box's running maximum
        // (the exact FP64 numbers earlier tiles folded in) cannot be the maximum either.
        const float thr = m32 * (1.0f - 0x1p-18f);
        const bool all = !(m32 <= 3.0e38f);
        const float gcut = courant_running_max(b);
        unsigned cand = 0;
#pragma unroll
        for (int i = 0; i < XI; i++) {
            const float est = stash[(i * 5 + 0) * kTileThreads + col];
            const bool inside = T.i0 + i < b.n[0] && j < b.n[1] && k < b.n[2];
            if (inside && !courant_below(est, gcut) && (all || !(est < thr) || !(est > 1e-30f))) cand |= 1u << i;
        }
        while (__any_sync(0xffffffffu, cand != 0)) {
            if (cand) {
                const int i = __ffs(cand) - 1;
                cand &= cand - 1;
                const long long c = cell_off(b, T.i0 + i, j, k);
                const double p = __hiloint2double(__float_as_int(stash[(i * 5 + 1) * kTileThreads + col]),
                                                  __float_as_int(stash[(i * 5 + 2) * kTileThreads + col])) +
                                 refs.p;
                const double cour = courant_mixed(b, b.U[c], b.U[c + fs], b.U[c + 2 * fs], b.U[c + 3 * fs], p);
                cmax = cour > cmax ? cour : cmax;
            }
        }
        courant_fold(b, cmax);
    }
}

// The FP64 box's write-back of the 8 cells of column `col` = (tj, tk) of tile T from the FP64
// sums parked in `stash`: the RK3 combine, the host array (stage 3), ctoprim and fluxes as in
// k_assemble<double> (same operations, same bits), and at stage 3 the Courant maximum through
// FP32 candidates over the whole tile (each cell's estimate and p parked over its sums, a block
// maximum, the FP64 number only where it can be the largest).  All threads of the block take
// part (block barriers at stage 3).
template <int STAGE>
__device__ __forceinline__ void write_back_plain(const BoxView& b, const Tile& T, double* stash, int col, int tj,
                                                 int tk, FxSink* fx = nullptr) {
    const int pr = b.sc->pbase ^ ((STAGE - 1) & 1);
    double* Pw = (double*)b.P[pr ^ 1];
    const double dt = b.sc->dt;
    const int j = T.j0 + tj, k = T.k0 + tk;
    const long long fs = b.fs;
    float m32 = -1.0f;
    int health = 0;
#pragma unroll 1
    for (int i = 0; i < XI; i++) {
        const int ic = T.i0 + i;
        if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
        const long long c = cell_off(b, ic, j, k);
        double un[5];
#pragma unroll
        for (int l = 0; l < 5; l++) {
            const long long e = c + l * fs;
            const double r = stash[(i * 5 + l) * kTileThreads + col];
            if (STAGE == 1) {
                un[l] = fma(dt, r, b.U[e]);
                b.Us[e] = quarter(un[l]);  // U1 / 4
            } else if (STAGE == 2) {
                un[l] = fma(0.75, b.U[e], fma(0.25 * dt, r, b.Us[e]));
                b.Us[e] = un[l];
            } else {
                un[l] = fma(1.0 / 3.0, b.U[e], (2.0 / 3.0) * fma(dt, r, b.Us[e]));
                b.U[e] = un[l];
            }
        }
        if (STAGE == 3 && b.host_out) store_host(b, ic, j, k, un);
        CourantInput64 q;
        epilogue_plain(b, Pw, c, ic, j, k, un, &health, &q, fx);
        if (STAGE == 3) {
            const float est = courant_plain_est(b, q);
            reinterpret_cast<float*>(stash + (i * 5 + 0) * kTileThreads + col)[0] = est;
            stash[(i * 5 + 1) * kTileThreads + col] = q.p;
            m32 = fmaxf(m32, est);
        }
    }
    if (health) atomicOr(&b.sc->status, health);
    if (STAGE == 3) {
        __shared__ float s_max[kTileThreads / 32];
        float m = m32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
        __syncthreads();
        m = s_max[0];
#pragma unroll
        for (int w = 1; w < kTileThreads / 32; w++) m = fmaxf(m, s_max[w]);
        __syncthreads();  // s_max is rewritten for the next tile
        const float thr = m * (1.0f - 4.0f * kCourantPlainEps);
        const float gcut = courant_running_max(b);
        double cmax = 0.0;
#pragma unroll 1
        for (int i = 0; i < XI; i++) {
            const int ic = T.i0 + i;
            if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
            const float est = reinterpret_cast<const float*>(stash + (i * 5 + 0) * kTileThreads + col)[0];
            if ((m <= 3.0e38f && est < thr && est > 1e-30f) || courant_below(est, gcut)) continue;
            // the cell's Courant number from its new state, as epilogue_plain formed it
            const long long c = cell_off(b, ic, j, k);
            const double rho = b.U[c], rinv = rcp_nr(rho);
            const CourantInput64 q{stash[(i * 5 + 1) * kTileThreads + col], rinv, b.U[c + fs] * rinv,
                                   b.U[c + 2 * fs] * rinv, b.U[c + 3 * fs] * rinv};
            const double cour = courant_plain(b, q);
            cmax = cour > cmax ? cour : cmax;
        }
        courant_fold(b, cmax);
    }
}

// R = float: mixed boxes, two blocks per SM (80 KB of shared memory each); R = double: FP64
// boxes, one block per SM (160 KB), with up to 255 registers for the 8 cells' FP64 sums.
template <class R, int STAGE>
__global__ void __launch_bounds__(kTileThreads, sizeof(R) == 4 ? 2 : 1) k_assemble_tma(const BoxView* __restrict__ boxes,
                                                                                   const Tile* __restrict__ tiles,
                                                                                   int ntiles) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    R* buf[2] = {(R*)smem_raw, (R*)smem_raw + kBufElems};
    uint64_t* bar = (uint64_t*)(smem_raw + 2 * kBufElems * sizeof(R));
    const int tid = threadIdx.x, tk = tid & (XK - 1), tj = tid >> 5;
    const int my_tiles = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (my_tiles <= 0) return;
    const int total = my_tiles * kLoads;
    if (tid == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    constexpr int flip = (STAGE - 1) & 1;
    if (tid == 0) issue(boxes, tiles, blockIdx.x, 0, flip, buf[0], &bar[0]);

    R dmx[XI], dmy[XI], dmz[XI], de[XI], f0[XI], c0[XI];
    int g = 0;
    for (int it = 0; it < my_tiles; it++) {
        const int tile = blockIdx.x + it * gridDim.x;
        const Tile T = tiles[tile];
        const BoxView& b = boxes[T.box];
        const CoefT<R>& cf = coefs<R>(b);
        prefetch_state_l2(b, T, STAGE, tid);
        // Every sum is first written, not accumulated, by its first load; clearing them here
        // only tells the compiler that the last tile's values are dead once they are parked.
#pragma unroll
        for (int i = 0; i < XI; i++) dmx[i] = dmy[i] = dmz[i] = de[i] = f0[i] = c0[i] = R(0);
        for (int e = 0; e < kLoads; e++, g++) {
            if (tid == 0 && g + 1 < total) {
                const int nt = blockIdx.x + ((g + 1) / kLoads) * gridDim.x;
                issue(boxes, tiles, nt, (g + 1) % kLoads, flip, buf[(g + 1) & 1], &bar[(g + 1) & 1]);
            }
            const bool ok = mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicOr(&b.sc->status, HEALTH_TIMEOUT);
                    // let the copies this block started finish (bounded) before returning
                    mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
                    if (g + 1 < total) mbar_wait_bounded(&bar[(g + 1) & 1], (uint32_t)(((g + 1) >> 1) & 1));
                }
                return;
            }
            consume_field(e, buf[g & 1], T, b, cf, tj, tk, dmx, dmy, dmz, de, f0, c0);
            __syncthreads();  // buffer g & 1 is free for load g + 2
        }
        // The sums are parked in the buffer the last field used (free: every thread passed the
        // barrier after consuming it; each thread reads back only its own entries), so the
        // write-back runs as a rolled loop and its code exists once, not 8x.
        R* stash = buf[(g - 1) & 1];
        park_sums(stash, tid, f0, dmx, dmy, dmz, de);
        if constexpr (sizeof(R) == 4)
            write_back<STAGE>(b, T, stash, tid, tj, tk);
        else
            write_back_plain<STAGE>(b, T, stash, tid, tj, tk);
        __syncthreads();  // the stash buffer receives load g + 1, issued at the top of the next tile
    }
}

// ---- the plain form on its fixed-point copies (CNS_ASSEMBLE_TMA_FX) -------------------------
// k_assemble_tma's tiles, schedule and FP64 write-back, with the P fields staged as the 64-bit
// fixed-point words of the stage's copy (cns_exact.cuh) instead of FP64: every Laplacian and
// flux-divergence stencil is an exact integer sum, rounded once, and one FP64 FMA (the FP64
// form's other stencils cost eight FP64 operations, or ~20 integer operations a tap).  The S set
// stays FP64 (the mixed viscous terms as in k_assemble_tma<double>); the centre values of the
// Laplacians and of the work terms are the FP64 fields, read from global memory.
struct FxCtx {
    const int* E;      // exponents of the copy read, field by field
    const double* Pr;  // the FP64 P set read (centre values)
    long long c;       // element of cell (T.i0, jc, kc) inside a field
    long long si, fs;
    int ni;            // cells of the tile inside the box along i (the rest read the last one)
    bool xf;           // a sum left FP64's normal range
    int i0, i1;        // the thread's cells of its column: [i0, i1)
};
__device__ __forceinline__ double fx_centre(const FxCtx& x, int field, int i) {
    return __ldg(x.Pr + field * x.fs + x.c + (long long)min(i, x.ni - 1) * x.si);
}

// The full-box (u, v, w or e) pass: FP64 centre weight, then the i, j, k second differences.  The
// cells of a thread's column are walked by a rolled loop (one copy of the stencil code: eight
// unrolled copies of 27 fixed-point stencils overflow the instruction cache), taps from shared
// memory along every axis.
__device__ __forceinline__ void lap_full_fx(const long long* s, int tj, int tk, double cw, const double* wi,
                                            const double* wj, const double* wk, double* acc, double* ctr,
                                            bool init_from_acc, int field, FxCtx& x) {
    using B = Bx<BX_FULL>;
    const int E = __ldg(x.E + field);
#pragma unroll 1
    for (int i = x.i0; i < x.i1; i++) {
        const double c0 = fx_centre(x, field, i);
        ctr[i] = c0;
        double a = init_from_acc ? fma(cw, c0, acc[i]) : cw * c0;
        const long long* p = s + B::at(i + 4, tj + 4, tk + 4);
        a = fx_d2acc(a, [&](int m) { return p[m * (B::J * B::K)]; }, E, wi, &x.xf);
        a = fx_d2acc(a, [&](int m) { return p[m * B::K]; }, E, wj, &x.xf);
        a = fx_d2acc(a, [&](int m) { return p[m]; }, E, wk, &x.xf);
        acc[i] = a;
    }
}

// A flux field staged in box shape S, differenced along `axis` (0 = i, 1 = j, 2 = k) into acc
// (first: acc starts at 0).
template <int S, int AXIS>
__device__ __forceinline__ void flux_fx(const long long* s, int tj, int tk, int field, const double* a, double* acc,
                                        bool first, FxCtx& x) {
    using B = Bx<S>;
    const int E = __ldg(x.E + field);
    constexpr int st = AXIS == 0 ? B::J * B::K : (AXIS == 1 ? B::K : 1);
#pragma unroll 1
    for (int i = x.i0; i < x.i1; i++) {
        const long long* p = s + B::at(i + B::HI, tj + B::HJ, tk + B::HK);
        acc[i] = fx_d1acc(first ? 0.0 : acc[i], [&](int m) { return p[m * st]; }, E, a, &x.xf);
    }
}

// Field e of a tile's 20 loads (kSched) folded into the sums; P fields as fixed-point words, S
// fields as FP64 (the same arithmetic as consume_field<double> for those).
__device__ __forceinline__ void consume_field_fx(int e, const void* buf, const CoefT<double>& cf, int tj, int tk,
                                                 FxCtx& x, double* dmx, double* dmy, double* dmz, double* de,
                                                 double* f0, double* c0) {
    const long long* s = (const long long*)buf;
    const double* d = (const double*)buf;
    switch (e) {
        case 0: {  // SPHI: de starts from eta * Phi
            using B = Bx<BX_C>;
#pragma unroll 1
            for (int i = x.i0; i < x.i1; i++) de[i] = d[B::at(i, tj, tk)];
            break;
        }
        case 1: {  // PT: de = tc e0 + phi, then the x, y, z second differences
            double t0[XI];
            lap_full_fx(s, tj, tk, cf.tc, cf.tl[0], cf.tl[1], cf.tl[2], de, t0, true, PT, x);
            break;
        }
        case 2:
            lap_full_fx(s, tj, tk, cf.vc[0], cf.vl[0][0], cf.vl[0][1], cf.vl[0][2], dmx, c0, false, PU, x);
            break;
        case 3: {  // SX: dmx += (eta/3) d/dx (v_y + w_z); then the work term dmx u0
            using B = Bx<BX_I>;
#pragma unroll 1
            for (int i = x.i0; i < x.i1; i++) {
                dmx[i] = sd1acc<xon(kExactMixed, 0)>(dmx[i], d + B::at(i + 4, tj, tk), B::J * B::K, cf.mx[0]);
                de[i] = fma(dmx[i], c0[i], de[i]);
            }
            break;
        }
        case 4:
            lap_full_fx(s, tj, tk, cf.vc[1], cf.vl[1][0], cf.vl[1][1], cf.vl[1][2], dmy, c0, false, PV, x);
            break;
        case 5: {  // SY
            using B = Bx<BX_J>;
#pragma unroll 1
            for (int i = x.i0; i < x.i1; i++) {
                dmy[i] = sd1acc<xon(kExactMixed, 1)>(dmy[i], d + B::at(i, tj + 4, tk), B::K, cf.mx[1]);
                de[i] = fma(dmy[i], c0[i], de[i]);
            }
            break;
        }
        case 6:
            lap_full_fx(s, tj, tk, cf.vc[2], cf.vl[2][0], cf.vl[2][1], cf.vl[2][2], dmz, c0, false, PW, x);
            break;
        case 7: {  // SZ
            using B = Bx<BX_K>;
#pragma unroll 1
            for (int i = x.i0; i < x.i1; i++) {
                dmz[i] = sd1acc<xon(kExactMixed, 2)>(dmz[i], d + B::at(i, tj, tk + 4), 1, cf.mx[2]);
                de[i] = fma(dmz[i], c0[i], de[i]);
            }
            break;
        }
        case 8: flux_fx<BX_I, 0>(s, tj, tk, PMX, cf.ha[0], f0, true, x); break;
        case 9: flux_fx<BX_J, 1>(s, tj, tk, PMY, cf.ha[1], f0, false, x); break;
        case 10: flux_fx<BX_K, 2>(s, tj, tk, PMZ, cf.ha[2], f0, false, x); break;
        case 11: flux_fx<BX_I, 0>(s, tj, tk, PFUU, cf.ha[0], dmx, false, x); break;
        case 12:  // PFUV: along y -> f1, along x -> f2
            flux_fx<BX_IJ, 1>(s, tj, tk, PFUV, cf.ha[1], dmx, false, x);
            flux_fx<BX_IJ, 0>(s, tj, tk, PFUV, cf.ha[0], dmy, false, x);
            break;
        case 13:  // PFUW: along z -> f1, along x -> f3
            flux_fx<BX_IK, 2>(s, tj, tk, PFUW, cf.ha[2], dmx, false, x);
            flux_fx<BX_IK, 0>(s, tj, tk, PFUW, cf.ha[0], dmz, false, x);
            break;
        case 14: flux_fx<BX_J, 1>(s, tj, tk, PFVV, cf.ha[1], dmy, false, x); break;
        case 15:  // PFVW: along z -> f2, along y -> f3
            flux_fx<BX_JK, 2>(s, tj, tk, PFVW, cf.ha[2], dmy, false, x);
            flux_fx<BX_JK, 1>(s, tj, tk, PFVW, cf.ha[1], dmz, false, x);
            break;
        case 16: flux_fx<BX_K, 2>(s, tj, tk, PFWW, cf.ha[2], dmz, false, x); break;
        case 17: flux_fx<BX_I, 0>(s, tj, tk, PHU, cf.ha[0], de, false, x); break;
        case 18: flux_fx<BX_J, 1>(s, tj, tk, PHV, cf.ha[1], de, false, x); break;
        default: flux_fx<BX_K, 2>(s, tj, tk, PHW, cf.ha[2], de, false, x); break;
    }
}

// A thread's 8 cells on the FP64 fields (a copy that is unusable, or a sum outside FP64's normal
// range): the direct kernel's arithmetic, parked over the thread's sums in the stash.
__device__ __noinline__ void assemble_column_fp64(const BoxView& b, const Tile& T, int j, int k, int stage,
                                                  double* stash, int col, int i0, int i1) {
    const int pr = b.sc->pbase ^ ((stage - 1) & 1);
    const double* Pr = (const double*)b.P[pr];
    const double* S = (const double*)b.S;
    for (int i = i0; i < i1; i++) {
        const int ic = T.i0 + i;
        if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
        const long long c = cell_off(b, ic, j, k), fs = b.fs;
        double f[5];
        assemble_terms_fallback<double>(b, Pr, S, c, __ldg(Pr + PU * fs + c), __ldg(Pr + PV * fs + c),
                                        __ldg(Pr + PW * fs + c), __ldg(Pr + PT * fs + c), f);
        for (int l = 0; l < 5; l++) stash[(i * 5 + l) * kTileThreads + col] = f[l];
    }
}

// write_back_plain for 512-thread blocks: the cells [i0, i1) of column `col`, the stage-3 block
// maximum over 16 warps.
template <int STAGE>
__device__ __forceinline__ void write_back_fx(const BoxView& b, const Tile& T, double* stash, int col, int tj, int tk,
                                              int i0, int i1, FxSink* fx) {
    const int pr = b.sc->pbase ^ ((STAGE - 1) & 1);
    double* Pw = (double*)b.P[pr ^ 1];
    const double dt = b.sc->dt;
    const int j = T.j0 + tj, k = T.k0 + tk;
    const long long fs = b.fs;
    float m32 = -1.0f;
    int health = 0;
#pragma unroll 1
    for (int i = i0; i < i1; i++) {
        const int ic = T.i0 + i;
        if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
        const long long c = cell_off(b, ic, j, k);
        double un[5];
#pragma unroll
        for (int l = 0; l < 5; l++) {
            const long long e = c + l * fs;
            const double r = stash[(i * 5 + l) * kTileThreads + col];
            if (STAGE == 1) {
                un[l] = fma(dt, r, b.U[e]);
                b.Us[e] = quarter(un[l]);  // U1 / 4
            } else if (STAGE == 2) {
                un[l] = fma(0.75, b.U[e], fma(0.25 * dt, r, b.Us[e]));
                b.Us[e] = un[l];
            } else {
                un[l] = fma(1.0 / 3.0, b.U[e], (2.0 / 3.0) * fma(dt, r, b.Us[e]));
                b.U[e] = un[l];
            }
        }
        if (STAGE == 3 && b.host_out) store_host(b, ic, j, k, un);
        CourantInput64 q;
        epilogue_plain(b, Pw, c, ic, j, k, un, &health, &q, fx);
        if (STAGE == 3) {
            const float est = courant_plain_est(b, q);
            reinterpret_cast<float*>(stash + (i * 5 + 0) * kTileThreads + col)[0] = est;
            stash[(i * 5 + 1) * kTileThreads + col] = q.p;
            m32 = fmaxf(m32, est);
        }
    }
    if (health) atomicOr(&b.sc->status, health);
    if (STAGE == 3) {
        constexpr int kW = 2 * kTileThreads / 32;
        __shared__ float s_max[kW];
        float m = m32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
        __syncthreads();
        m = s_max[0];
#pragma unroll
        for (int w = 1; w < kW; w++) m = fmaxf(m, s_max[w]);
        __syncthreads();
        const float thr = m * (1.0f - 4.0f * kCourantPlainEps);
        const float gcut = courant_running_max(b);
        double cmax = 0.0;
#pragma unroll 1
        for (int i = i0; i < i1; i++) {
            const int ic = T.i0 + i;
            if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
            const float est = reinterpret_cast<const float*>(stash + (i * 5 + 0) * kTileThreads + col)[0];
            if ((m <= 3.0e38f && est < thr && est > 1e-30f) || courant_below(est, gcut)) continue;
            const long long c = cell_off(b, ic, j, k);
            const double rho = b.U[c], rinv = rcp_nr(rho);
            const CourantInput64 q{stash[(i * 5 + 1) * kTileThreads + col], rinv, b.U[c + fs] * rinv,
                                   b.U[c + 2 * fs] * rinv, b.U[c + 3 * fs] * rinv};
            const double cour = courant_plain(b, q);
            cmax = cour > cmax ? cour : cmax;
        }
        courant_fold(b, cmax);
    }
}

// One block per SM (160 KB of shared memory: two 64-bit field buffers), as k_assemble_tma<double>.
// The write-back also writes the fixed-point copy of the P set it writes; the block's maxima of the
// written fields go to the box's scalars when the block moves to another box and at its end.
template <int STAGE>
__global__ void __launch_bounds__(2 * kTileThreads, 1) k_assemble_fx(const BoxView* __restrict__ boxes,
                                                              const Tile* __restrict__ tiles, int ntiles) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    double* buf[2] = {(double*)smem_raw, (double*)smem_raw + kBufElems};
    uint64_t* bar = (uint64_t*)(smem_raw + 2 * kBufElems * sizeof(double));
    __shared__ int s_emax[NPF];
    // two threads per (j, k) column, four cells of it each
    const int tid = threadIdx.x & (kTileThreads - 1), half = threadIdx.x >> 8, tk = tid & (XK - 1), tj = tid >> 5;
    const int ci0 = half * (XI / 2), ci1 = ci0 + XI / 2;
    const int my_tiles = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (my_tiles <= 0) return;
    const int total = my_tiles * kLoads;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < NPF) s_emax[threadIdx.x] = 0;
    __syncthreads();
    constexpr int flip = (STAGE - 1) & 1;
    if (threadIdx.x == 0) issue<double, true>(boxes, tiles, blockIdx.x, 0, flip, buf[0], &bar[0]);

    double dmx[XI], dmy[XI], dmz[XI], de[XI], f0[XI], c0[XI];
    int g = 0, fx_box = -1, fx_set = 0;
    bool fx_bad = false;
    for (int it = 0; it < my_tiles; it++) {
        const int tile = blockIdx.x + it * gridDim.x;
        const Tile T = tiles[tile];
        const BoxView& b = boxes[T.box];
        const int pr = b.sc->pbase ^ flip;
        if (T.box != fx_box) {
            fx_flush(boxes, fx_box, fx_set, s_emax, fx_bad);
            fx_bad = false;
            fx_box = T.box;
            fx_set = pr ^ 1;
        }
        if (half == 0) prefetch_state_l2(b, T, STAGE, tid);
        const bool usable = !b.sc->fx_bad[pr];
        const int j = T.j0 + tj, k = T.k0 + tk;
        FxCtx x{b.sc->fx_e[pr], (const double*)b.P[pr],
                cell_off(b, T.i0, min(j, b.n[1] - 1), min(k, b.n[2] - 1)), b.si, b.fs, min(XI, b.n[0] - T.i0), false,
                ci0, ci1};
#pragma unroll
        for (int i = 0; i < XI; i++) dmx[i] = dmy[i] = dmz[i] = de[i] = f0[i] = c0[i] = 0.0;
        for (int e = 0; e < kLoads; e++, g++) {
            if (threadIdx.x == 0 && g + 1 < total) {
                const int nt = blockIdx.x + ((g + 1) / kLoads) * gridDim.x;
                issue<double, true>(boxes, tiles, nt, (g + 1) % kLoads, flip, buf[(g + 1) & 1], &bar[(g + 1) & 1]);
            }
            const bool ok = mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) {
                    atomicOr(&b.sc->status, HEALTH_TIMEOUT);
                    mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
                    if (g + 1 < total) mbar_wait_bounded(&bar[(g + 1) & 1], (uint32_t)(((g + 1) >> 1) & 1));
                }
                return;
            }
            if (usable) consume_field_fx(e, buf[g & 1], b.c64, tj, tk, x, dmx, dmy, dmz, de, f0, c0);
            __syncthreads();  // buffer g & 1 is free for load g + 2
        }
        double* stash = buf[(g - 1) & 1];
#pragma unroll 1
        for (int i = ci0; i < ci1; i++) {
            stash[(i * 5 + 0) * kTileThreads + tid] = f0[i];
            stash[(i * 5 + 1) * kTileThreads + tid] = dmx[i];
            stash[(i * 5 + 2) * kTileThreads + tid] = dmy[i];
            stash[(i * 5 + 3) * kTileThreads + tid] = dmz[i];
            stash[(i * 5 + 4) * kTileThreads + tid] = de[i];
        }
        if (!usable || x.xf) assemble_column_fp64(b, T, j, k, STAGE, stash, tid, ci0, ci1);
        FxSink sink{b.X[pr ^ 1], b.sc->fx_e[pr ^ 1], s_emax, false, NPF, true};
        write_back_fx<STAGE>(b, T, stash, tid, tj, tk, ci0, ci1, &sink);
        fx_bad |= sink.bad;
        __syncthreads();  // the stash buffer receives load g + 1, issued at the top of the next tile
    }
    fx_flush(boxes, fx_box, fx_set, s_emax, fx_bad);
}

// ---- warp-specialised variant ------------------------------------------------------------
// One 512-thread block per SM: warps 0-7 (the stencil group) run the 20 TMA-fed field phases of
// tile t while warps 8-15 (the write-back group) run the FP64 write-back of tile t-1, so the
// FP32 stencils and the FP64 write-back overlap instead of alternating.  The fields are
// staged in an 80 KB ring (below), and the sums move between the groups through one 40 KB stash
// slot: full (256 stencil arrivals) hands it to the write-back group, empty (256 write-back
// arrivals) hands it back.  120 KB of shared memory leave the most L1 for the write-back's state
// loads: a second slot (160 KB) measured 0.5-1 % slower, and a third 40 KB field buffer with two
// slots (200 KB) 10-15 % slower; the code takes any kWsSlots.  The stencil group
// synchronises on named barrier 1 only (once per field); the write-back group needs no barrier.
// Every wait is bounded.  A stencil thread whose wait gives up stops waiting and computing but
// keeps taking part in the barrier and the hand-over, so no thread is ever left waiting on it;
// it reports HEALTH_TIMEOUT at the end, after thread 0 has waited (bounded) for the copies it
// issued.  A write-back warp whose wait gives up reports and returns.  Same arithmetic as
// k_assemble_tma, same bits.
constexpr int kWsThreads = 2 * kTileThreads;
constexpr int kStashElems = 5 * XI * kTileThreads;  // 10240 floats
static_assert(kStashElems == kBufElems, "a stash slot is one field buffer in size");

constexpr int kWsSlots = 1;  // stash slots
__device__ __forceinline__ void group_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// The stencil group's field buffers are one ring of 80 KB in which each of a tile's 20 loads has
// a fixed place (`off`, in floats, 512-byte aligned), the same in every tile.  A load is
// issued as soon as the last earlier load whose place overlaps its own (counting back through
// the previous tile's loads) has been consumed: `dep` loads back.  The two full-halo boxes take
// the two halves, as two plain buffers would, but the small boxes (10-32 KB) share a half and
// their copies start two to three phases ahead instead of one.  Each load has its own mbarrier,
// which completes once per tile.
constexpr int kRingElems = 2 * kBufElems;
struct RingPlan {
    int off[kLoads];
    int dep[kLoads];
    bool ok;
};
constexpr RingPlan ring_plan() {
    RingPlan r{{0, 10240, 0, 10240, 0, 10240, 0, 10240, 12800, 0, 4096, 6656, 10752, 0, 5120, 9216, 14336, 0, 4096, 8192},
               {},
               true};
    for (int e = 0; e < kLoads; e++) {
        const int a0 = r.off[e], a1 = a0 + box_elems(kSchedPlan[e].shape);
        if (a0 < 0 || a0 % 128 != 0 || a1 > kRingElems) r.ok = false;
        r.dep[e] = kLoads;  // a load always overlaps its own place in the previous tile
        for (int back = kLoads - 1; back >= 1; back--) {
            const int q = (e - back + kLoads) % kLoads;
            const int b0 = r.off[q], b1 = b0 + box_elems(kSchedPlan[q].shape);
            if (b0 < a1 && a0 < b1) r.dep[e] = back;
        }
    }
    return r;
}
static_assert(ring_plan().ok, "every load lies inside the ring at a 512-byte boundary");
__constant__ RingPlan kRing = ring_plan();

template <int STAGE>
__global__ void __launch_bounds__(kWsThreads, 1) k_assemble_ws(const BoxView* __restrict__ boxes,
                                                            const Tile* __restrict__ tiles, int ntiles) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* buf = (float*)smem_raw;                                // the field ring
    float* stash = buf + kRingElems;                              // kWsSlots stash slots
    uint64_t* bar = (uint64_t*)(stash + kWsSlots * kStashElems);  // TMA[kLoads], full[kWsSlots], empty[kWsSlots]
    uint64_t* full = bar + kLoads;
    uint64_t* empty = full + kWsSlots;
    const int my_tiles = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (my_tiles <= 0) return;
    if (threadIdx.x == 0) {
        for (int q = 0; q < kLoads; q++) mbar_init(&bar[q]);
        for (int q = 0; q < kWsSlots; q++) {
            mbar_init_n(&full[q], kTileThreads);
            mbar_init_n(&empty[q], kTileThreads);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    constexpr int flip = (STAGE - 1) & 1;

    if (threadIdx.x >= kTileThreads) {  // ---- write-back group
        const int wt = threadIdx.x - kTileThreads, tk = wt & (XK - 1), tj = wt >> 5;
        for (int it = 0; it < my_tiles; it++) {
            const Tile T = tiles[blockIdx.x + it * gridDim.x];
            const BoxView& b = boxes[T.box];
            const int slot = it % kWsSlots;
            const bool ok = mbar_wait_bounded(&full[slot], (uint32_t)((it / kWsSlots) & 1));
            if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform, so the shuffles below stay whole
                if ((wt & 31) == 0) atomicOr(&b.sc->status, HEALTH_TIMEOUT);
                return;
            }
            write_back<STAGE>(b, T, stash + slot * kStashElems, wt, tj, tk);
            mbar_arrive(&empty[slot]);
        }
        return;
    }

    // ---- stencil group
    const int tid = threadIdx.x, tk = tid & (XK - 1), tj = tid >> 5;
    const int total = my_tiles * kLoads;
    // thread 0: issue, in order, every load whose place in the ring is free once the loads up to
    // `consumed` have been consumed
    int issued = 0;  // loads issued so far
    auto issue_ready = [&](int consumed) {
        for (; issued < total && issued - kRing.dep[issued % kLoads] <= consumed; issued++) {
            const int e = issued % kLoads, nt = blockIdx.x + (issued / kLoads) * gridDim.x;
            issue(boxes, tiles, nt, e, flip, buf + kRing.off[e], &bar[e]);
        }
    };
    if (tid == 0) issue_ready(-1);
    bool bad = false;
    int* bad_status = nullptr;  // the status word of the box whose wait gave up
    int g = 0;
    float dmx[XI], dmy[XI], dmz[XI], de[XI], f0[XI], c0[XI];
    for (int it = 0; it < my_tiles; it++) {
        const Tile T = tiles[blockIdx.x + it * gridDim.x];
        const BoxView& b = boxes[T.box];
        const CoefT<float>& cf = b.c32;
        // No prefetch_state_l2 here: its 1-3 bulk prefetches per thread queue in the copy engine
        // ahead of the field copies (measured 5 % slower at 128^3, 10 % at 256^3), and the
        // write-back group's own loads are hidden by the stencil group's work.
#pragma unroll
        for (int i = 0; i < XI; i++) dmx[i] = dmy[i] = dmz[i] = de[i] = f0[i] = c0[i] = 0.f;
        for (int e = 0; e < kLoads; e++, g++) {
            // loads up to g - 1 were consumed before the last barrier
            if (tid == 0 && !bad) issue_ready(g - 1);
            if (!bad && !mbar_wait_bounded(&bar[e], (uint32_t)(it & 1))) {
                bad = true;
                bad_status = &b.sc->status;
            }
            if (!bad) consume_field(e, buf + kRing.off[e], T, b, cf, tj, tk, dmx, dmy, dmz, de, f0, c0);
            group_sync();  // load g's place in the ring is free
        }
        // hand the sums over: slot it % kWsSlots, once the write-back of tile it - kWsSlots has released it
        const int slot = it % kWsSlots;
        if (it >= kWsSlots && !bad && !mbar_wait_bounded(&empty[slot], (uint32_t)(((it / kWsSlots) - 1) & 1))) {
            bad = true;
            bad_status = &b.sc->status;
        }
        park_sums(stash + slot * kStashElems, tid, f0, dmx, dmy, dmz, de);
        mbar_arrive(&full[slot]);
    }
    if (bad) {
        atomicOr(bad_status, HEALTH_TIMEOUT);
        if (tid == 0)  // the copies still in flight are among the last kLoads issued
            for (int l = max(0, issued - kLoads); l < issued; l++)
                mbar_wait_bounded(&bar[l % kLoads], (uint32_t)((l / kLoads) & 1));
    }
}

// ---- the mixed form's derivative pass, TMA-staged -------------------------------------------
// Same tiles as the assembly; u, v, w of the stage's P set arrive as full-halo boxes,
// double-buffered; the nine first derivatives come from shared memory with the operations of
// k_deriv (cns_fused.cu) in the same order, and the S fields are stored as k_deriv stores them,
// so the two give the same bits.  Waits bounded as in k_assemble_tma.
__global__ void __launch_bounds__(kTileThreads, 2) k_deriv_tma(const BoxView* __restrict__ boxes,
                                                            const Tile* __restrict__ tiles, int ntiles, int stage) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* buf[2] = {(float*)smem_raw, (float*)smem_raw + kBufElems};
    uint64_t* bar = (uint64_t*)(smem_raw + 2 * kBufElems * sizeof(float));
    const int tid = threadIdx.x, tk = tid & (XK - 1), tj = tid >> 5;
    const int my_tiles = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (my_tiles <= 0) return;
    const int total = my_tiles * 3;
    if (tid == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int flip = (stage - 1) & 1;
    auto load_of = [](int e) { return Load{0, (unsigned char)(PU + e), BX_FULL}; };  // u, v, w
    if (tid == 0) issue_load(boxes, tiles, blockIdx.x, load_of(0), flip, buf[0], &bar[0]);
    float d[3][3][XI];  // d[field][axis][cell]: u_x u_y u_z, v_x ..., w_x ...
    int g = 0;
    for (int it = 0; it < my_tiles; it++) {
        const Tile T = tiles[blockIdx.x + it * gridDim.x];
        const BoxView& b = boxes[T.box];
        const CoefT<float>& cf = b.c32;
#pragma unroll
        for (int e = 0; e < 3; e++, g++) {
            if (tid == 0 && g + 1 < total)
                issue_load(boxes, tiles, blockIdx.x + ((g + 1) / 3) * gridDim.x, load_of((g + 1) % 3), flip,
                           buf[(g + 1) & 1], &bar[(g + 1) & 1]);
            const bool ok = mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicOr(&b.sc->status, HEALTH_TIMEOUT);
                    mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
                    if (g + 1 < total) mbar_wait_bounded(&bar[(g + 1) & 1], (uint32_t)(((g + 1) >> 1) & 1));
                }
                return;
            }
            using B = Bx<BX_FULL>;
            const float* s = buf[g & 1];
            float col[16];
#pragma unroll
            for (int ii = 0; ii < 16; ii++) col[ii] = s[B::at(ii, tj + 4, tk + 4)];
#pragma unroll
            for (int i = 0; i < XI; i++) {
                const float* p = s + B::at(i + 4, tj + 4, tk + 4);
                d[e][0][i] = cd1<xon(kExactDeriv, 0)>(col, i + 4, cf.da[0]);
                d[e][1][i] = sd1<xon(kExactDeriv, 1)>(p, B::K, cf.da[1]);
                d[e][2][i] = sd1<xon(kExactDeriv, 2)>(p, 1, cf.da[2]);
            }
            __syncthreads();  // buffer g & 1 is free for load g + 2
        }
        // cpu/diffterm.cpp:294-304, as in k_deriv
        const int j = T.j0 + tj, k = T.k0 + tk;
        float* S = (float*)b.S;
        const long long fs = b.fs;
#pragma unroll
        for (int i = 0; i < XI; i++) {
            const int ic = T.i0 + i;
            if (ic >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
            const float ux = d[0][0][i], uy = d[0][1][i], uz = d[0][2][i];
            const float vx = d[1][0][i], vy = d[1][1][i], vz = d[1][2][i];
            const float wx = d[2][0][i], wy = d[2][1][i], wz = d[2][2][i];
            float sx, sy, sz, phi;
            dissipation(ux, uy, uz, vx, vy, vz, wx, wy, wz, &sx, &sy, &sz, &phi);
            const long long c = cell_off(b, ic, j, k);
            store_img(S + SX * fs, b, c, ic, j, k, sx, 1);
            store_img(S + SY * fs, b, c, ic, j, k, sy, 2);
            store_img(S + SZ * fs, b, c, ic, j, k, sz, 4);
            S[SPHI * fs + c] = cf.eta * phi;
        }
    }
}

// Self-test of the bounded wait: an mbarrier nothing ever arrives on.  The wait must give up
// after its limit and the block must report HEALTH_TIMEOUT and return normally.
__global__ void k_bounded_wait_selftest(int* out) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0u);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) *out = HEALTH_TIMEOUT;
}

cudaError_t bounded_wait_selftest(int* status) {
    int* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_bounded_wait_selftest<<<1, 32>>>(d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

// Self-test of the exact stencil sums (cns_exact.cuh) as the device computes them: set q has the
// taps taps[8q .. 8q+7] = f[+1..+4], f[-1..-4]; sums[2q] and sums[2q+1] get the sums with the
// first- and the second-derivative weights, ok[2q] and ok[2q+1] are 0 where a sum takes the
// FP64 fallback instead.
__global__ void k_exact_sums_selftest(const double* __restrict__ taps, int n, double* __restrict__ sums,
                                      int* __restrict__ ok) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const double* t = taps + 8LL * q;
        auto ld = [&](int m) { return m > 0 ? t[m - 1] : t[3 - m]; };  // m = 1..4, -1..-4
        double x1 = 0.0, x2 = 0.0;
        ok[2 * q] = xsum8<672, -168, 32, -3, -1>(ld, &x1) ? 1 : 0;
        ok[2 * q + 1] = xsum8<8064, -1008, 128, -9, 1>(ld, &x2) ? 1 : 0;
        sums[2 * q] = x1;
        sums[2 * q + 1] = x2;
    }
}

cudaError_t exact_sums_selftest(const double* taps, int n, double* sums, int* ok) {
    if (n <= 0) return cudaSuccess;
    double *dt = nullptr, *ds = nullptr;
    int* dk = nullptr;
    cudaError_t e = cudaMalloc(&dt, sizeof(double) * 8 * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&ds, sizeof(double) * 2 * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&dk, sizeof(int) * 2 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dt, taps, sizeof(double) * 8 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
        k_exact_sums_selftest<<<grid, 256>>>(dt, n, ds, dk);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(sums, ds, sizeof(double) * 2 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ok, dk, sizeof(int) * 2 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(dt);
    cudaFree(ds);
    cudaFree(dk);
    return e;
}

// ---- host side -------------------------------------------------------------------------------
constexpr size_t kTmaSmem = 2 * kBufElems * sizeof(float) + 2 * sizeof(uint64_t);

void tma_tile_shape(int* ti, int* tj, int* tk) {
    *ti = XI;
    *tj = XJ;
    *tk = XK;
}
size_t tma_maps_bytes() { return sizeof(TmaMaps); }

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encoder() {
    static const EncodeTiledFn fn = [] {  // looked up once, thread-safely
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (EncodeTiledFn)p;
        return (EncodeTiledFn) nullptr;
    }();
    return fn;
}

// Encode the tensor maps of a mixed box into host memory `out` (sizeof(TmaMaps) bytes).
cudaError_t tma_encode_maps(const BoxView& v, void* out) {
    EncodeTiledFn enc = encoder();
    if (!enc) return cudaErrorNotSupported;
    TmaMaps* m = (TmaMaps*)out;
    const cuuint64_t g0 = v.n[0] + 2 * CNS_NG, g1 = v.n[1] + 2 * CNS_NG, g2 = v.n[2] + 2 * CNS_NG;
    const bool fp64 = v.precision == 0;  // FP64 boxes: P and S sets in double
    const cuuint64_t es_bytes = fp64 ? 8 : 4;
    auto one = [&](CUtensorMap* map, void* base, int nfields, int shape) -> bool {
        const cuuint64_t dims[4] = {g2, g1, g0, (cuuint64_t)nfields};
        const cuuint64_t strides[3] = {(cuuint64_t)v.sj * es_bytes, (cuuint64_t)v.si * es_bytes, (cuuint64_t)v.fs * es_bytes};
        const cuuint32_t box[4] = {(cuuint32_t)box_k(shape), (cuuint32_t)box_j(shape), (cuuint32_t)box_i(shape), 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        return enc(map, fp64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides,
                   box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    for (int set = 0; set < 2; set++)
        for (int sh = 0; sh < 7; sh++)
            if (!one(&m->p[set][sh], v.P[set], NPF, sh)) return cudaErrorInvalidValue;
    const int sshape[4] = {BX_I, BX_J, BX_K, BX_C};
    for (int q = 0; q < 4; q++)
        if (!one(&m->s[q], v.S, NSF, sshape[q])) return cudaErrorInvalidValue;
    // the fixed-point copies of every field (CNS_ASSEMBLE_TMA_FX): the P sets' geometry, 64-bit
    // integer words
    for (int set = 0; set < 2 && fp64 && v.X[0] && v.fx == NPF; set++)
        for (int sh = 0; sh < 7; sh++) {
            const cuuint64_t dims[4] = {g2, g1, g0, (cuuint64_t)NPF};
            const cuuint64_t strides[3] = {(cuuint64_t)v.sj * 8, (cuuint64_t)v.si * 8, (cuuint64_t)v.fs * 8};
            const cuuint32_t box[4] = {(cuuint32_t)box_k(sh), (cuuint32_t)box_j(sh), (cuuint32_t)box_i(sh), 1};
            const cuuint32_t es[4] = {1, 1, 1, 1};
            if (enc(&m->x[set][sh], CU_TENSOR_MAP_DATA_TYPE_INT64, 4, v.X[set], dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return cudaErrorInvalidValue;
        }
    return cudaSuccess;
}

template <class R, int STAGE>
static cudaError_t launch_tma_stage(const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    auto fn = k_assemble_tma<R, STAGE>;
    constexpr size_t smem = 2 * kBufElems * sizeof(R) + 2 * sizeof(uint64_t);
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)fn, kTileThreads, smem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    const int grid = ntiles < nsm * per ? ntiles : nsm * per;
    return launch_step(fn, grid, kTileThreads, smem, st, boxes, tiles, ntiles);
}

cudaError_t launch_assemble_tma(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (stage == 1) return launch_tma_stage<float, 1>(boxes, tiles, ntiles, st);
    if (stage == 2) return launch_tma_stage<float, 2>(boxes, tiles, ntiles, st);
    return launch_tma_stage<float, 3>(boxes, tiles, ntiles, st);
}

cudaError_t launch_assemble_tma64(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (stage == 1) return launch_tma_stage<double, 1>(boxes, tiles, ntiles, st);
    if (stage == 2) return launch_tma_stage<double, 2>(boxes, tiles, ntiles, st);
    return launch_tma_stage<double, 3>(boxes, tiles, ntiles, st);
}

template <int STAGE>
static cudaError_t launch_fx_stage(const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    auto fn = k_assemble_fx<STAGE>;
    constexpr size_t smem = 2 * kBufElems * sizeof(double) + 2 * sizeof(uint64_t);
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)fn, 2 * kTileThreads, smem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    const int grid = ntiles < nsm * per ? ntiles : nsm * per;
    return launch_step(fn, grid, 2 * kTileThreads, smem, st, boxes, tiles, ntiles);
}

cudaError_t launch_assemble_fx(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (stage == 1) return launch_fx_stage<1>(boxes, tiles, ntiles, st);
    if (stage == 2) return launch_fx_stage<2>(boxes, tiles, ntiles, st);
    return launch_fx_stage<3>(boxes, tiles, ntiles, st);
}

template <class Fn>
static cudaError_t launch_tma_grid(Fn fn, int nthreads, size_t smem, int ntiles, int* grid) {
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)fn, nthreads, smem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    *grid = ntiles < nsm * per ? ntiles : nsm * per;
    return cudaSuccess;
}

cudaError_t launch_deriv_tma(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    int grid = 0;
    cudaError_t e = launch_tma_grid(k_deriv_tma, kTileThreads, kTmaSmem, ntiles, &grid);
    if (e != cudaSuccess) return e;
    return launch_step(k_deriv_tma, grid, kTileThreads, kTmaSmem, st, boxes, tiles, ntiles, stage);
}

constexpr size_t kWsSmem =
    (kRingElems + kWsSlots * kStashElems) * sizeof(float) + (kLoads + 2 * kWsSlots) * sizeof(uint64_t);

template <int STAGE>
static cudaError_t launch_ws_stage(const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    auto fn = k_assemble_ws<STAGE>;
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWsSmem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)fn, kWsThreads, kWsSmem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;  // 512 threads x 128 registers and kWsSmem must fit
    const int grid = ntiles < nsm * per ? ntiles : nsm * per;
    return launch_step(fn, grid, kWsThreads, kWsSmem, st, boxes, tiles, ntiles);
}

bool assemble_ws_fits() {
    int per = 0;
    if (cudaFuncSetAttribute((const void*)k_assemble_ws<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWsSmem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)k_assemble_ws<3>, kWsThreads, kWsSmem) !=
            cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return per >= 1;
}

cudaError_t launch_assemble_ws(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (stage == 1) return launch_ws_stage<1>(boxes, tiles, ntiles, st);
    if (stage == 2) return launch_ws_stage<2>(boxes, tiles, ntiles, st);
    return launch_ws_stage<3>(boxes, tiles, ntiles, st);
}

}  // namespace cns
