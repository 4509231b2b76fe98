// cns_host.cu -- the reference-layout host array <-> a box, moved by the SMs themselves over
// the CPU-GPU link when the caller's array is page-locked (and so mapped into the device's
// address space).
//
// The reference's new_advance works in place on a host array U[i][j][k][l] with 4 ghost
// layers, component fastest (cpu/helper_functions.cpp:100-122).  Only the interior of the
// input matters (stage 1 refills the ghosts, cpu/advance.cpp:45), and on return the ghosts hold
// the periodic images of the last step's start state (stage 3 writes the interior only,
// cpu/advance.cpp:144-153).  Reading and writing the caller's array in place saves the staging
// copy in HBM and its conversion pass, moves only the interior on the way in (84 of 101 MB at
// 128^3), and for FP64 boxes runs the first ctoprim + Courant pass in the same kernel as the
// read, under the link time.
//
// One warp per run of up to 32 consecutive k cells of an (i, j) row: the run's 5 x 32 doubles
// are contiguous in the host array and move with lane-strided (coalesced) accesses through a
// per-warp shared-memory buffer; the device side is the box's structure-of-arrays layout.
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <vector>

#include "cns_fused.cuh"

#include "cns_internal.h"

namespace cns {

constexpr int kRun = 32, kWarps = 8;

struct RunIdx {
    int i, j, k0, cnt;
    long long a0;  // element offset of the run's first value in the host array
};

// Run w of the interior: rows (i, j) of the interior, runs of 32 along k.
__device__ __forceinline__ RunIdx interior_run(const BoxView& b, long long w) {
    const int runs = (b.n[2] + kRun - 1) / kRun;
    const int g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    RunIdx r;
    const int kr = (int)(w % runs);
    const long long row = w / runs;
    r.j = (int)(row % b.n[1]);
    r.i = (int)(row / b.n[1]);
    r.k0 = kr * kRun;
    r.cnt = min(kRun, b.n[2] - r.k0);
    r.a0 = (((long long)(r.i + CNS_NG) * g1 + (r.j + CNS_NG)) * g2 + (r.k0 + CNS_NG)) * CNS_NC;
    return r;
}

// Write the run's periodic images into the host array's ghost cells: the whole run shifted by
// +-n along i and/or j (rows of ghost cells), and its first / last 4 cells shifted along k.
// Every ghost cell has exactly one interior source, so no cell is written twice.
__device__ __forceinline__ void run_images(const BoxView& b, const RunIdx& r, const double* sw, double* h, int lane) {
    const int g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    // shift number a along i: 0, then +n if the row is in the low layer, then -n if in the high
    const bool ilo = r.i < CNS_NG, ihi = r.i >= b.n[0] - CNS_NG, jlo = r.j < CNS_NG, jhi = r.j >= b.n[1] - CNS_NG;
    const int ni = 1 + ilo + ihi, nj = 1 + jlo + jhi;
    const int klo = r.k0 < CNS_NG ? min(CNS_NG - r.k0, r.cnt) : 0;        // cells k < 4
    const int khi = max(b.n[2] - CNS_NG, r.k0) - r.k0;                    // first cell k >= n-4
    const long long kshift = (long long)b.n[2] * CNS_NC;
    for (int a = 0; a < ni; a++) {
        for (int c = 0; c < nj; c++) {
            const int di = a == 0 ? 0 : (a == 1 && ilo ? b.n[0] : -b.n[0]);
            const int dj = c == 0 ? 0 : (c == 1 && jlo ? b.n[1] : -b.n[1]);
            const long long base = r.a0 + ((long long)di * g1 + dj) * g2 * CNS_NC;
            if (a || c)
                for (int q = lane; q < r.cnt * CNS_NC; q += 32) h[base + q] = sw[q];
            for (int q = lane; q < klo * CNS_NC; q += 32) h[base + kshift + q] = sw[q];
            for (int q = khi * CNS_NC + lane; q < r.cnt * CNS_NC; q += 32) h[base - kshift + q] = sw[q];
        }
    }
}

// Host interior -> box U; with PRIM also the P set (with its ghost images), the health bits and
// the Courant number of the state, as k_prim does; with GHOSTS also the host array's ghost
// cells as the periodic images of its interior (what the reference's fill_boundary leaves
// there), written back over the link while the interior is read.
template <bool PRIM, bool GHOSTS>
__global__ void __launch_bounds__(kWarps * 32) k_host_upload(BoxView b, double* __restrict__ h) {
    __shared__ double s[kWarps][kRun * CNS_NC];
    const int lane = threadIdx.x & 31;
    double* sw = s[threadIdx.x >> 5];
    const long long nw = (long long)b.n[0] * b.n[1] * ((b.n[2] + kRun - 1) / kRun);
    for (long long w = blockIdx.x * (long long)kWarps + (threadIdx.x >> 5); w < nw; w += (long long)gridDim.x * kWarps) {
        const RunIdx r = interior_run(b, w);
        for (int q = lane; q < r.cnt * CNS_NC; q += 32) sw[q] = h[r.a0 + q];
        __syncwarp();
        if (GHOSTS) run_images(b, r, sw, h, lane);
        double cour = 0.0;
        int health = 0;
        if (lane < r.cnt) {
            const int k = r.k0 + lane;
            const long long c = cell_off(b, r.i, r.j, k);
            double un[CNS_NC];
#pragma unroll
            for (int l = 0; l < CNS_NC; l++) {
                un[l] = sw[lane * CNS_NC + l];
                b.U[c + l * b.fs] = un[l];
            }
            if (PRIM) cour = epilogue<double>(b, (double*)b.P[b.sc->pbase], c, r.i, r.j, k, un, true, &health);
        }
        if (PRIM) {
            if (health) atomicOr(&b.sc->status, health);
            courant_fold(b, cour);  // the whole warp takes part (w is warp-uniform)
        }
        __syncwarp();
    }
}

// Box U interior -> host interior.
__global__ void __launch_bounds__(kWarps * 32) k_host_download(BoxView b, double* __restrict__ h) {
    __shared__ double s[kWarps][kRun * CNS_NC];
    const int lane = threadIdx.x & 31;
    double* sw = s[threadIdx.x >> 5];
    const long long nw = (long long)b.n[0] * b.n[1] * ((b.n[2] + kRun - 1) / kRun);
    for (long long w = blockIdx.x * (long long)kWarps + (threadIdx.x >> 5); w < nw; w += (long long)gridDim.x * kWarps) {
        const RunIdx r = interior_run(b, w);
        if (lane < r.cnt) {
            const long long c = cell_off(b, r.i, r.j, r.k0 + lane);
#pragma unroll
            for (int l = 0; l < CNS_NC; l++) sw[lane * CNS_NC + l] = b.U[c + l * b.fs];
        }
        __syncwarp();
        for (int q = lane; q < r.cnt * CNS_NC; q += 32) h[r.a0 + q] = sw[q];
        __syncwarp();
    }
}

// Every ghost cell of the host array <- the periodic image of the box's current U (what the
// reference's fill_boundary leaves there, cpu/helper_functions.cpp:226-262).  Runs of 32 along
// k over all ghost-inclusive rows; a run with no ghost cell is skipped.
__global__ void __launch_bounds__(kWarps * 32) k_host_ghosts(BoxView b, double* __restrict__ h) {
    __shared__ double s[kWarps][kRun * CNS_NC];
    const int lane = threadIdx.x & 31;
    double* sw = s[threadIdx.x >> 5];
    const int g0 = b.n[0] + 2 * CNS_NG, g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    const int runs = (g2 + kRun - 1) / kRun;
    const long long nw = (long long)g0 * g1 * runs;
    for (long long w = blockIdx.x * (long long)kWarps + (threadIdx.x >> 5); w < nw; w += (long long)gridDim.x * kWarps) {
        const int kr = (int)(w % runs);
        const long long row = w / runs;
        const int J = (int)(row % g1), I = (int)(row / g1);
        const bool ghost_row = I < CNS_NG || I >= b.n[0] + CNS_NG || J < CNS_NG || J >= b.n[1] + CNS_NG;
        const int K0 = kr * kRun, cnt = min(kRun, g2 - K0);
        if (!ghost_row && K0 >= CNS_NG && K0 + cnt <= b.n[2] + CNS_NG) continue;  // warp-uniform
        const long long a0 = (((long long)I * g1 + J) * g2 + K0) * CNS_NC;
        if (lane < cnt) {
            const int K = K0 + lane;
            const int ii = (I - CNS_NG + b.n[0]) % b.n[0], jj = (J - CNS_NG + b.n[1]) % b.n[1],
                      kk = (K - CNS_NG + b.n[2]) % b.n[2];
            const long long c = cell_off(b, ii, jj, kk);
#pragma unroll
            for (int l = 0; l < CNS_NC; l++) sw[lane * CNS_NC + l] = b.U[c + l * b.fs];
        }
        __syncwarp();
        for (int q = lane; q < cnt * CNS_NC; q += 32) {
            const int K = K0 + q / CNS_NC;
            if (ghost_row || K < CNS_NG || K >= b.n[2] + CNS_NG) h[a0 + q] = sw[q];
        }
        __syncwarp();
    }
}

// ---- the upload fused with stage 1's derivative pass (FP64 boxes) -------------------------
// One persistent launch works through a queue built on the host (upload_deriv_queue): upload
// items (8 runs of one i-plane, planes in the order n-4 .. n-1, 0 .. n-5) interleaved with the
// derivative tiles of stage 1.  Each tile stands after the upload items of every plane it reads
// (its own planes and 4 on each side, periodically) and kDerivLag more planes, so that by the
// time a block takes it those planes are usually in.  Blocks take items in queue order from an
// atomic counter.  A tile waits for its planes' completion counts; every upload item it waits
// for stands earlier in the queue, so it was already taken by a running block that waits on
// nothing: the waits always end.  They are bounded all the same (about one second of global
// time; then HEALTH_TIMEOUT and the tile is skipped).  A warp publishes a finished run with a
// fence before counting it; a tile fences after seeing its counts and reads the P set from L2
// (deriv_cell<double, false>: it is written during this launch).
constexpr int kPlaneStart = CNS_NG;  // plane order: q = (i + 4) mod n
constexpr int kDerivLag = 8;         // planes (at 128^3 lags of 4 to 16 planes time the same)

__device__ __forceinline__ bool planes_ready(const volatile int* done, int n0, int lo, int hi, int target) {
    for (int p = lo; p <= hi; p++)
        if (done[(p % n0 + n0) % n0] < target) return false;
    return true;
}

template <bool GHOSTS>
__global__ void __launch_bounds__(kWarps * 32, 4) k_upload_deriv(BoxView b, double* __restrict__ h,
                                                               const Tile* __restrict__ tiles,
                                                               const int* __restrict__ queue, int nq, int* counter,
                                                               int* done) {
    __shared__ double s[kWarps][kRun * CNS_NC];
    __shared__ int s_item, s_ok;
    __shared__ float s_max[kWarps];
    __shared__ int s_emax[NPF];  // boxes with fixed-point copies: the block's P-field maxima
    if (threadIdx.x < NPF) s_emax[threadIdx.x] = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* sw = s[warp];
    const int runs = (b.n[2] + kRun - 1) / kRun, per_plane = b.n[1] * runs;
    const int items_per_plane = (per_plane + kWarps - 1) / kWarps;
    const int g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    for (;;) {
        if (threadIdx.x == 0) {
            const int pos = atomicAdd(counter, 1);
            s_item = pos < nq ? queue[pos] : INT_MIN;
        }
        __syncthreads();
        const int item = s_item;
        __syncthreads();  // s_item is rewritten next round
        if (item == INT_MIN) {
            // the maxima of the fields with copies, for the copies' exponents (k_fx_pass<true>)
            if (threadIdx.x < b.fx && s_emax[threadIdx.x] > 0) atomicMax(&b.sc->fx_cur[threadIdx.x], s_emax[threadIdx.x]);
            return;
        }
        if (item >= 0) {  // upload: run (item % items_per_plane) * 8 + warp of plane order q
            const int q = item / items_per_plane, rr = (item % items_per_plane) * kWarps + warp;
            const bool has = rr < per_plane;  // warp-uniform; warps without a run still join the barriers
            RunIdx r;
            r.i = (q + b.n[0] - kPlaneStart) % b.n[0];
            r.j = rr / runs;
            r.k0 = (rr % runs) * kRun;
            r.cnt = has ? min(kRun, b.n[2] - r.k0) : 0;
            r.a0 = (((long long)(r.i + CNS_NG) * g1 + (r.j + CNS_NG)) * g2 + (r.k0 + CNS_NG)) * CNS_NC;
            for (int x = lane; x < r.cnt * CNS_NC; x += 32) sw[x] = h[r.a0 + x];
            __syncwarp();
            if (GHOSTS && has) run_images(b, r, sw, h, lane);
            double cour = 0.0;
            int health = 0;
            float est = -1.0f;
            CourantInput64 cq;
            if (lane < r.cnt) {
                const int k = r.k0 + lane;
                const long long c = cell_off(b, r.i, r.j, k);
                double un[CNS_NC];
#pragma unroll
                for (int l = 0; l < CNS_NC; l++) {
                    un[l] = sw[lane * CNS_NC + l];
                    b.U[c + l * b.fs] = un[l];
                }
                double* P = (double*)b.P[b.sc->pbase];
                epilogue_plain(b, P, c, r.i, r.j, k, un, &health, &cq);
                est = courant_plain_est(b, cq);
                for (int f = 0; f < b.fx; f++) fx_track(s_emax + f, fx_efield(P[f * b.fs + c]));
            }
            // The Courant maximum through FP32 candidates over the item's 8 runs, as in stage 3
            // of k_assemble: the FP64 number only where it can be the largest, bit for bit.
            float m = est;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) s_max[warp] = m;
            __syncthreads();
            m = s_max[0];
#pragma unroll
            for (int w = 1; w < kWarps; w++) m = fmaxf(m, s_max[w]);
            const float thr = m * (1.0f - 4.0f * kCourantPlainEps);
            const float gcut = courant_running_max(b);
            if (lane < r.cnt && !courant_below(est, gcut) && (!(m <= 3.0e38f) || !(est < thr) || !(est > 1e-30f)))
                cour = courant_plain(b, cq);
            if (has) {
                if (health) atomicOr(&b.sc->status, health);
                courant_fold(b, cour);
                __threadfence();  // this lane's stores, before the run is counted
                __syncwarp();
                if (lane == 0) atomicAdd(&done[r.i], 1);
            }
        } else {  // stage 1's derivative pass on tile ~item, once the planes it reads are in
            const Tile T = tiles[~item];
            int lo, hi;
            if (b.tlog[0] == kLinearTile) {
                const long long plane = (long long)b.n[1] * b.n[2], last = (long long)b.n[0] * plane - 1;
                const long long p0 = (long long)T.k0 * kTileThreads;
                lo = (int)(p0 / plane);
                hi = (int)(min(p0 + kTileThreads - 1, last) / plane);
            } else {
                lo = T.i0;
                hi = min(T.i0 + (1 << b.tlog[0]), b.n[0]) - 1;
            }
            lo -= CNS_NG;
            hi += CNS_NG;
            if (hi - lo >= b.n[0]) lo = 0, hi = b.n[0] - 1;
            if (threadIdx.x == 0) {
                bool ok = planes_ready(done, b.n[0], lo, hi, per_plane);
                if (!ok) {
                    unsigned long long t0, t;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
                    do {
                        ok = planes_ready(done, b.n[0], lo, hi, per_plane);
                        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
                    } while (!ok && t - t0 < 1000000000ull);
                }
                if (!ok) atomicOr(&b.sc->status, HEALTH_TIMEOUT);
                __threadfence();  // the counted runs' stores, before this tile's loads
                s_ok = ok;
            }
            __syncthreads();
            const bool ok = s_ok;
            int i, j, k;
            tile_pos(b, T, threadIdx.x, &i, &j, &k);
            if (ok && i < b.n[0] && j < b.n[1] && k < b.n[2]) deriv_cell<double, false>(b, i, j, k, 1);
        }
    }
}

static int run_blocks(long long warps) {
    const long long b = (warps + kWarps - 1) / kWarps;
    return (int)(b > 1048576 ? 1048576 : (b < 1 ? 1 : b));
}

cudaError_t host_upload(const BoxView& v, double* h, bool prim, bool ghosts, cudaStream_t st) {
    const long long nw = (long long)v.n[0] * v.n[1] * ((v.n[2] + kRun - 1) / kRun);
    const int nb = run_blocks(nw), nt = kWarps * 32;
    if (prim && ghosts)
        k_host_upload<true, true><<<nb, nt, 0, st>>>(v, h);
    else if (prim)
        k_host_upload<true, false><<<nb, nt, 0, st>>>(v, h);
    else if (ghosts)
        k_host_upload<false, true><<<nb, nt, 0, st>>>(v, h);
    else
        k_host_upload<false, false><<<nb, nt, 0, st>>>(v, h);
    return cudaGetLastError();
}

cudaError_t host_download(const BoxView& v, double* h, cudaStream_t st) {
    const long long nw = (long long)v.n[0] * v.n[1] * ((v.n[2] + kRun - 1) / kRun);
    k_host_download<<<run_blocks(nw), kWarps * 32, 0, st>>>(v, h);
    return cudaGetLastError();
}

cudaError_t host_ghosts(const BoxView& v, double* h, cudaStream_t st) {
    const long long nw = (long long)(v.n[0] + 2 * CNS_NG) * (v.n[1] + 2 * CNS_NG) * ((v.n[2] + 2 * CNS_NG + kRun - 1) / kRun);
    k_host_ghosts<<<run_blocks(nw), kWarps * 32, 0, st>>>(v, h);
    return cudaGetLastError();
}

// The queue of k_upload_deriv for a box with tile list `tiles` (see there).
std::vector<int> upload_deriv_queue(const int n[3], const int tlog[3], const std::vector<Tile>& tiles) {
    const int runs = (n[2] + kRun - 1) / kRun, per_plane = n[1] * runs;
    const int items_per_plane = (per_plane + kWarps - 1) / kWarps;
    std::vector<std::vector<int>> after(n[0]);  // tiles to place after plane order q
    for (size_t t = 0; t < tiles.size(); t++) {
        int lo, hi;
        if (tlog[0] == kLinearTile) {
            const long long plane = (long long)n[1] * n[2], last = (long long)n[0] * plane - 1;
            const long long p0 = (long long)tiles[t].k0 * kTileThreads;
            lo = (int)(p0 / plane);
            hi = (int)(std::min(p0 + kTileThreads - 1, last) / plane);
        } else {
            lo = tiles[t].i0;
            hi = std::min(tiles[t].i0 + (1 << tlog[0]), n[0]) - 1;
        }
        lo -= CNS_NG;
        hi += CNS_NG;
        int qmax = 0;
        if (hi - lo >= n[0]) {
            qmax = n[0] - 1;
        } else {
            for (int p = lo; p <= hi; p++) qmax = std::max(qmax, (((p % n[0]) + n[0]) % n[0] + kPlaneStart) % n[0]);
        }
        after[std::min(qmax + kDerivLag, n[0] - 1)].push_back(~(int)t);
    }
    std::vector<int> q;
    q.reserve((size_t)n[0] * items_per_plane + tiles.size());
    for (int p = 0; p < n[0]; p++) {
        for (int it = 0; it < items_per_plane; it++) q.push_back(p * items_per_plane + it);
        q.insert(q.end(), after[p].begin(), after[p].end());
    }
    return q;
}

cudaError_t host_upload_deriv(const BoxView& v, double* h, bool ghosts, const Tile* tiles, const int* queue, int nq,
                              int* counters, cudaStream_t st) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const void* fn = ghosts ? (const void*)k_upload_deriv<true> : (const void*)k_upload_deriv<false>;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kWarps * 32, 0);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, nsm * per);
    e = cudaMemsetAsync(counters, 0, sizeof(int) * (v.n[0] + 1), st);
    if (e != cudaSuccess) return e;
    if (ghosts)
        k_upload_deriv<true><<<grid, kWarps * 32, 0, st>>>(v, h, tiles, queue, nq, counters + v.n[0], counters);
    else
        k_upload_deriv<false><<<grid, kWarps * 32, 0, st>>>(v, h, tiles, queue, nq, counters + v.n[0], counters);
    return cudaGetLastError();
}

// The device address of the host range [p, p + bytes), or null (the caller then stages through
// a copy).  Two kinds of host memory qualify:
//  * page-locked memory (cudaHostAlloc, cudaHostRegister): when all of the range lies inside one
//    such allocation that the device can address, checked against the allocation's extent as the
//    driver records it, so a kernel never touches host memory outside the caller's allocation;
//  * ordinary pageable memory (malloc, new, a numpy array), on a device that reads and writes it
//    through the host's own page tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables: a
//    GPU attached by NVLink-C2C, as on Grace-Blackwell), where the host address is the device
//    address.  The range is then the caller's array as its dimensions give it, exactly as the
//    reference's loops over the same array assume.  cns_set_pageable_in_place(0) turns this off.
static std::atomic<int> g_pageable_in_place{1};

static bool pageable_access(int dev) {
    static std::atomic<int> cache[64];  // per device: 0 unknown, 1 no, 2 yes
    if (dev < 0 || dev >= 64) return false;
    int c = cache[dev].load();
    if (c == 0) {
        int pma = 0, hpt = 0;
        if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            pma = hpt = 0;
        }
        c = (pma && hpt) ? 2 : 1;
        cache[dev].store(c);
    }
    return c == 2;
}

void set_pageable_in_place(int enable) { g_pageable_in_place.store(enable ? 1 : 0); }

typedef CUresult (*PointerGetAttributeFn)(void*, CUpointer_attribute, CUdeviceptr);

static PointerGetAttributeFn pointer_attr_fn() {
    static const PointerGetAttributeFn fn = [] {  // looked up once, thread-safely
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PointerGetAttributeFn)p;
        return (PointerGetAttributeFn) nullptr;
    }();
    return fn;
}

void* mapped_host_range(const void* p, size_t bytes) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // not a pointer the runtime knows; clear the (non-sticky) error
        return nullptr;
    }
    if (a.type == cudaMemoryTypeUnregistered) {
        int dev = -1;
        if (!g_pageable_in_place.load() || cudaGetDevice(&dev) != cudaSuccess || !pageable_access(dev)) return nullptr;
        return const_cast<void*>(p);
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    PointerGetAttributeFn get = pointer_attr_fn();
    if (!get) return nullptr;
    CUdeviceptr start = 0;
    size_t size = 0;
    const CUdeviceptr dp = (CUdeviceptr)a.devicePointer;
    if (get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, dp) != CUDA_SUCCESS) return nullptr;
    if (get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, dp) != CUDA_SUCCESS) return nullptr;
    if (dp < start || dp - start > size || bytes > size - (size_t)(dp - start)) return nullptr;
    return a.devicePointer;
}

}  // namespace cns
