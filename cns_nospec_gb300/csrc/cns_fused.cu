// cns_fused.cu -- persistent tile-walking kernels for the RK3 stages (see cns_fused.cuh).
//
// Every kernel walks a work list of tiles (box, i0, j0, k0); one launch covers every box of a
// batch.  A tile is 256 cells, one per thread, in the shape its box carries (tlog), so boxes
// with different tile shapes share a launch.
#include "cns_fused.cuh"
#include "cns_internal.h"

namespace cns {

template <class R>
__device__ __forceinline__ R ld(const R* p) { return __ldg(p); }

// ---- k_prim: primitives + flux functions + Courant of the uploaded state -------------------
template <class R>
__global__ void __launch_bounds__(kTileThreads) k_prim(const BoxView* __restrict__ boxes, const Tile* __restrict__ tiles,
                                                     int ntiles) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile T = tiles[t];
        const BoxView& b = boxes[T.box];
        int i, j, k;
        tile_pos(b, T, threadIdx.x, &i, &j, &k);
        double cour = 0.0;
        int health = 0;
        if (i < b.n[0] && j < b.n[1] && k < b.n[2]) {
            const long long c = cell_off(b, i, j, k);
            double un[5];
#pragma unroll
            for (int l = 0; l < 5; l++) un[l] = b.U[c + l * b.fs];
            R* Pw = (R*)b.P[b.sc->pbase];
            cour = epilogue<R>(b, Pw, c, i, j, k, un, true, &health);
        }
        if (health) atomicOr(&b.sc->status, health);
        courant_fold(b, cour);
    }
}

// ---- k_deriv: first derivatives of (u,v,w) -> mixed-term sums and viscous dissipation -------
// FXT: FP64 boxes that keep a fixed-point copy of the P set (deriv_cell).
template <class R, bool FXT>
__global__ void __launch_bounds__(kTileThreads, 3) k_deriv(const BoxView* __restrict__ boxes, const Tile* __restrict__ tiles,
                                                      int ntiles, int stage) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile T = tiles[t];
        const BoxView& b = boxes[T.box];
        // a box on the fixed-point assembly: the assembly after this kernel writes the other P set's
        // copy; prepared once per box, by the block holding the box's first tile (a store from every
        // tile, all to the same few words, measured 5 % of this kernel's time)
        if (sizeof(R) == 8 && b.fx && (t == 0 || tiles[t - 1].box != T.box))
            fx_prepare(b, b.sc->pbase ^ ((stage - 1) & 1) ^ 1);
        int i, j, k;
        tile_pos(b, T, threadIdx.x, &i, &j, &k);
        if (i >= b.n[0] || j >= b.n[1] || k >= b.n[2]) continue;
        deriv_cell<R, true, FXT>(b, i, j, k, stage);
    }
}

// ---- k_assemble: D + F, RK stage combine, fused ctoprim/flux/ghost write-back -------------
// FXT: FP64 boxes that keep a fixed-point copy of the P set: the kFxLap / kFxFlux stencils read
// the copy of the set read (where it is usable), and the write-back also writes the copy of the
// set written, with the block's maxima of its fields (as k_assemble_fx).
template <class R, int STAGE, bool FXT, bool MRG = false>
__global__ void __launch_bounds__(kTileThreads, 2) k_assemble(const BoxView* __restrict__ boxes,
                                                         const Tile* __restrict__ tiles, int ntiles) {
    __shared__ int s_emax[NPF];
    int fx_box = -1, fx_set = 0;
    bool fx_bad = false;
    if (FXT) {
        if (threadIdx.x < NPF) s_emax[threadIdx.x] = 0;
        __syncthreads();
    }
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile T = tiles[t];
        const BoxView& b = boxes[T.box];
        if (FXT && T.box != fx_box) {
            fx_flush(boxes, fx_box, fx_set, s_emax, fx_bad);
            fx_bad = false;
            fx_box = T.box;
            fx_set = (b.sc->pbase ^ ((STAGE - 1) & 1)) ^ 1;
        }
        int i, j, k;
        tile_pos(b, T, threadIdx.x, &i, &j, &k);
        double cour = 0.0;
        int health = 0;
        // plain form, stage 3: the Courant number through FP32 candidates (below)
        constexpr bool kDefer = sizeof(R) == 8 && STAGE == 3;
        constexpr bool kPlainFx = sizeof(R) == 8 && FXT;
        CourantInput64 cq;
        float est = -1.0f;
        bool inside = false;
        if (i < b.n[0] && j < b.n[1] && k < b.n[2]) {
            const int pr = b.sc->pbase ^ ((STAGE - 1) & 1);
            const R* Pr = (const R*)b.P[pr];
            R* Pw = (R*)b.P[pr ^ 1];
            const R* S = (const R*)b.S;
            const long long c = cell_off(b, i, j, k), fs = b.fs;
            const R u0 = ld(Pr + PU * fs + c), v0 = ld(Pr + PV * fs + c), w0 = ld(Pr + PW * fs + c),
                    t0 = ld(Pr + PT * fs + c);
            // diffterm + hypterm (cpu/diffterm.cpp:155-311, cpu/hypterm.cpp:29-208); the plain form
            // with no branch between its exact sums, again with their fallbacks where one needs it
            R f[5];
            if constexpr (kPlainFx) {
                const bool usable = !b.sc->fx_bad[pr];
                bool xf = !usable;
                if (usable)
                    assemble_terms<R, true, kFxLap, kFxFlux, MRG>(b, Pr, S, c, u0, v0, w0, t0, f, &xf, b.X[pr],
                                                                  b.sc->fx_e[pr]);
                if (xf) assemble_terms_fallback<R>(b, Pr, S, c, u0, v0, w0, t0, f);
            } else if constexpr (sizeof(R) == 8) {
                bool xf = false;
                assemble_terms<R, true>(b, Pr, S, c, u0, v0, w0, t0, f, &xf);
                if (xf) assemble_terms_fallback<R>(b, Pr, S, c, u0, v0, w0, t0, f);
            } else {
                assemble_terms<R, false>(b, Pr, S, c, u0, v0, w0, t0, f, nullptr);
            }
            if (sizeof(R) == 4) {
                // mixed form: the P set holds ((E + p) - H_ref) u_d, so add -H_ref div(u);
                // div(u) = (S_x + S_y + S_z) / 2 with the same first-difference operator
                const R divu = (R)0.5 * (ld(S + SX * fs + c) + ld(S + SY * fs + c) + ld(S + SZ * fs + c));
                f[4] = fma(-(R)b.sc->H_ref, divu, f[4]);
            }
            // RK3 stage combine in FP64 (cpu/advance.cpp:78-85, 110-119, 144-153)
            const double dt = b.sc->dt;
            double un[5];
#pragma unroll
            for (int l = 0; l < 5; l++) {
                const long long e = c + l * fs;
                const double r = (double)f[l];
                if (STAGE == 1) {
                    un[l] = fma(dt, r, b.U[e]);
                    b.Us[e] = quarter(un[l]);  // U1 / 4
                } else if (STAGE == 2) {
                    un[l] = fma(0.75, b.U[e], fma(0.25 * dt, r, b.Us[e]));
                    b.Us[e] = sizeof(R) == 4 ? (2.0 / 3.0) * un[l] : un[l];  // mixed: (2/3) U2
                } else {
                    un[l] = sizeof(R) == 4 ? fma(1.0 / 3.0, b.U[e], fma((2.0 / 3.0) * dt, r, b.Us[e]))
                                           : fma(1.0 / 3.0, b.U[e], (2.0 / 3.0) * fma(dt, r, b.Us[e]));
                    b.U[e] = un[l];
                }
            }
            if (STAGE == 3 && b.host_out) store_host(b, i, j, k, un);
            if (kPlainFx) {
                // the maxima of stage 3's writes only (the step's result; the next step's stages
                // differ from it by one step's change, well inside the exponents' 4x headroom):
                // tracking every stage measured 1 % of the step
                FxSink sink{b.X[pr ^ 1], b.sc->fx_e[pr ^ 1], s_emax, false, kFxFields, STAGE == 3};
                epilogue_plain(b, (double*)Pw, c, i, j, k, un, &health, &cq, &sink);
                fx_bad |= sink.bad;
                if (kDefer) {
                    est = courant_plain_est(b, cq);
                    inside = true;
                }
            } else if (kDefer) {
                epilogue_plain(b, (double*)Pw, c, i, j, k, un, &health, &cq);
                est = courant_plain_est(b, cq);
                inside = true;
            } else {
                cour = epilogue<R>(b, Pw, c, i, j, k, un, STAGE == 3, &health);
            }
        }
        if (health) atomicOr(&b.sc->status, health);
        if (kDefer) {
            // The FP64 Courant number only where it can be the tile's maximum: with
            // |est - exact| <= eps * exact (eps = kCourantPlainEps = 2^-18, over twice the
            // estimate's bound), a cell whose estimate is below (1 - 4 eps) of the tile's largest
            // (below (1 - eps) / (1 + eps) of it, with margin) is below the exact value of that
            // largest estimate's cell, so the maximum over the candidates is the maximum over
            // the tile, bit for bit.  NaN or tiny estimates are always candidates, and all cells
            // are when an estimate overflowed.  Warps without a candidate skip the FP64 code.
            __shared__ float s_max[kTileThreads / 32];
            float m = est;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
            __syncthreads();
            m = s_max[0];
#pragma unroll
            for (int q = 1; q < kTileThreads / 32; q++) m = fmaxf(m, s_max[q]);
            __syncthreads();  // s_max is rewritten for the next tile
            const float thr = m * (1.0f - 4.0f * kCourantPlainEps);
            const float gcut = courant_running_max(b);
            if (inside && !courant_below(est, gcut) && (!(m <= 3.0e38f) || !(est < thr) || !(est > 1e-30f)))
                cour = courant_plain(b, cq);
        }
        if (STAGE == 3) courant_fold(b, cour);
    }
    if (FXT) fx_flush(boxes, fx_box, fx_set, s_emax, fx_bad);
}

// ---- k_refs: the mixed form's reference values from interior cell (0,0,0) of U ----------
__global__ void k_refs(const BoxView* __restrict__ boxes, int nboxes) {
    const int bx = blockIdx.x * blockDim.x + threadIdx.x;
    if (bx >= nboxes) return;
    const BoxView& b = boxes[bx];
    const long long c = cell_off(b, 0, 0, 0);
    const double rho = b.U[c], E = b.U[c + 4 * b.fs];
    const double rinv = 1.0 / rho;
    const double u = b.U[c + b.fs] * rinv, v = b.U[c + 2 * b.fs] * rinv, w = b.U[c + 3 * b.fs] * rinv;
    const double eint = E * rinv - 0.5 * (u * u + v * v + w * w);
    const double p = kGm1 * eint * rho;
    b.sc->p_ref = p;
    b.sc->e_ref = eint;
    b.sc->E_ref = E;
    b.sc->H_ref = E + p;
}

// ---- k_stepend: dt for the next step from the Courant max (cpu/advance.cpp:52-58) ----------
__global__ void k_stepend(const BoxView* __restrict__ boxes, int nboxes, int flip) {
    const int bx = blockIdx.x * blockDim.x + threadIdx.x;
    if (bx >= nboxes) return;
    BoxScalars* s = boxes[bx].sc;
    double courno = __longlong_as_double((long long)s->courno_bits);
    courno = (courno > 1.0e-50) ? courno : 1.0e-50;
    if (flip) {
        boxes[bx].dtlog[s->nsteps_done & (DTLOG_CAP - 1)] = s->dt;
        s->dt_last = s->dt;
        s->pbase ^= 1;
        s->nsteps_done += 1;
        s->fx_fresh = 0;
    }
    s->dt = boxes[bx].cfl / courno;
    s->courno_bits = 0ull;
    // A box on the fixed-point assembly: the next step's writes take their exponents from the
    // maxima of this step's writes (after an upload, of the uploaded P set; after a restore, the
    // restored ones)
    if (boxes[bx].fx) {
        if (flip || !s->fx_restore) {
            for (int f = 0; f < NPF; f++) s->fx_prev[f] = s->fx_cur[f];
        }
        for (int f = 0; f < NPF; f++) s->fx_cur[f] = 0;
        fx_prepare_one(boxes[bx], s->pbase ^ 1);  // written by the next stage 1 (whose derivative
                                                  // pass may ride with an upload)
    }
    s->fx_restore = 0;
}

// ---- k_fx_pass: the fixed-point copy of a box's uploaded P set ------------------------------
// CONVERT = false: the maxima of the P set's fields into fx_cur (a fresh upload).  CONVERT = true:
// the copy at exponents from those maxima, or, after a restore, at the restored exponents.
template <bool CONVERT>
__global__ void __launch_bounds__(kTileThreads) k_fx_pass(const BoxView* __restrict__ boxes,
                                                        const Tile* __restrict__ tiles, int ntiles) {
    __shared__ int s_emax[NPF];
    if (threadIdx.x < NPF) s_emax[threadIdx.x] = 0;
    __syncthreads();
    int fx_box = -1, fx_set = 0;
    bool bad = false;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile T = tiles[t];
        const BoxView& b = boxes[T.box];
        BoxScalars* sc = b.sc;
        const int W = sc->pbase;
        if (T.box != fx_box) {
            fx_flush(boxes, fx_box, fx_set, s_emax, bad);
            bad = false;
            fx_box = T.box;
            fx_set = W;
            if (CONVERT && !sc->fx_restore && threadIdx.x < NPF)
                sc->fx_e[W][threadIdx.x] = fx_exponent(sc->fx_cur[threadIdx.x]);
            if (CONVERT && !sc->fx_restore && threadIdx.x == 0) sc->fx_fresh = 1;
        }
        int i, j, k;
        tile_pos(b, T, threadIdx.x, &i, &j, &k);
        if (i < b.n[0] && j < b.n[1] && k < b.n[2]) {
            const double* P = (const double*)b.P[W];
            const long long c = cell_off(b, i, j, k);
#pragma unroll
            for (int f = 0; f < NPF; f++) {
                if (f >= b.fx) break;  // fields without a copy
                const double v = P[f * b.fs + c];
                if (!CONVERT) {
                    fx_track(s_emax + f, fx_efield(v));
                } else {
                    const int E = sc->fx_restore ? sc->fx_e[W][f] : fx_exponent(sc->fx_cur[f]);
                    store_img(b.X[W] + f * b.fs, b, c, i, j, k, fx_word(v, E, &bad), pimg(f));
                }
            }
        }
    }
    fx_flush(boxes, fx_box, fx_set, s_emax, bad);
}

// ---- launch helpers ---------------------------------------------------------------------
static int grid_for(const void* fn, int ntiles) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kTileThreads, 0);
    if (per < 1) per = 1;
    int g = nsm * per;
    return ntiles < g ? ntiles : g;
}

template <class R>
static cudaError_t launch_prim_t(const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    auto fn = k_prim<R>;
    fn<<<grid_for((const void*)fn, ntiles), kTileThreads, 0, st>>>(boxes, tiles, ntiles);
    return cudaGetLastError();
}
template <class R, bool FXT>
static cudaError_t launch_deriv_t(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    auto fn = k_deriv<R, FXT>;
    return launch_step(fn, grid_for((const void*)fn, ntiles), kTileThreads, 0, st, boxes, tiles, ntiles, stage);
}
template <class R, bool FXT, bool MRG = false>
static cudaError_t launch_assemble_t(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (stage == 1) {
        auto fn = k_assemble<R, 1, FXT, MRG>;
        return launch_step(fn, grid_for((const void*)fn, ntiles), kTileThreads, 0, st, boxes, tiles, ntiles);
    } else if (stage == 2) {
        auto fn = k_assemble<R, 2, FXT, MRG>;
        return launch_step(fn, grid_for((const void*)fn, ntiles), kTileThreads, 0, st, boxes, tiles, ntiles);
    } else {
        auto fn = k_assemble<R, 3, FXT, MRG>;
        return launch_step(fn, grid_for((const void*)fn, ntiles), kTileThreads, 0, st, boxes, tiles, ntiles);
    }
}

cudaError_t launch_prim(int precision, const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    return precision ? launch_prim_t<float>(boxes, tiles, ntiles, st) : launch_prim_t<double>(boxes, tiles, ntiles, st);
}
cudaError_t launch_deriv(int form, const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (form == kFormMixed) return launch_deriv_t<float, false>(boxes, tiles, ntiles, stage, st);
    if (form == kFormPlainFx) return launch_deriv_t<double, true>(boxes, tiles, ntiles, stage, st);
    return launch_deriv_t<double, false>(boxes, tiles, ntiles, stage, st);
}
cudaError_t launch_assemble(int form, const BoxView* boxes, const Tile* tiles, int ntiles, int stage,
                            cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (form == kFormMixed) return launch_assemble_t<float, false>(boxes, tiles, ntiles, stage, st);
    if (form == kFormPlainFx) return launch_assemble_t<double, true>(boxes, tiles, ntiles, stage, st);
    if (form == kFormPlainFxMerge) return launch_assemble_t<double, true, true>(boxes, tiles, ntiles, stage, st);
    return launch_assemble_t<double, false>(boxes, tiles, ntiles, stage, st);
}
cudaError_t launch_refs(const BoxView* boxes, int nboxes, cudaStream_t st) {
    if (nboxes <= 0) return cudaSuccess;
    k_refs<<<(nboxes + 127) / 128, 128, 0, st>>>(boxes, nboxes);
    return cudaGetLastError();
}
// ---- k_fx_adopt: a box switched onto its fixed-point copies between steps takes the maxima of
// the conversion just made for its next writes (k_stepend's bookkeeping without a step)
__global__ void k_fx_adopt(const BoxView* __restrict__ boxes, int nboxes) {
    const int bx = blockIdx.x * blockDim.x + threadIdx.x;
    if (bx >= nboxes) return;
    BoxScalars* s = boxes[bx].sc;
    for (int f = 0; f < NPF; f++) {
        s->fx_prev[f] = s->fx_cur[f];
        s->fx_cur[f] = 0;
    }
    fx_prepare_one(boxes[bx], s->pbase ^ 1);
}
cudaError_t launch_fx_adopt(const BoxView* boxes, int nboxes, cudaStream_t st) {
    if (nboxes <= 0) return cudaSuccess;
    k_fx_adopt<<<(nboxes + 127) / 128, 128, 0, st>>>(boxes, nboxes);
    return cudaGetLastError();
}
cudaError_t launch_fx_pass(bool convert, const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    if (convert)
        k_fx_pass<true><<<grid_for((const void*)k_fx_pass<true>, ntiles), kTileThreads, 0, st>>>(boxes, tiles, ntiles);
    else
        k_fx_pass<false><<<grid_for((const void*)k_fx_pass<false>, ntiles), kTileThreads, 0, st>>>(boxes, tiles, ntiles);
    return cudaGetLastError();
}
cudaError_t launch_stepend(const BoxView* boxes, int nboxes, int flip, cudaStream_t st) {
    if (nboxes <= 0) return cudaSuccess;
    return launch_step(k_stepend, (nboxes + 127) / 128, 128, 0, st, boxes, nboxes, flip);
}

}  // namespace cns
