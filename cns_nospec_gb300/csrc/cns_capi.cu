// cns_capi.cu -- the C ABI (include/cns_gb300.h): device-resident boxes and batches, the
// reference's host-array entry points, graphs and launch accounting.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cns_gb300.h"
#include "cns_common.cuh"
#include "cns_internal.h"

using namespace cns;

// ---- errors ------------------------------------------------------------------------------
static thread_local std::string g_err;

static int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
static int fail_cuda(cudaError_t e, const char* what, int line) {
    int code = (e == cudaErrorMemoryAllocation) ? CNS_ERR_NOMEM
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? CNS_ERR_NODEVICE
                                                                                : CNS_ERR_CUDA;
    return fail(code, "%s failed at cns_capi.cu:%d: %s", what, line, cudaGetErrorString(e));
}
#define CK(call)                                                             \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return fail_cuda(e_, #call, __LINE__);        \
    } while (0)

extern "C" const char* cns_last_error(void) { return g_err.c_str(); }
int cns::set_error(int code, const char* msg) {
    g_err = msg;
    return code;
}
extern "C" int cns_version(void) { return 100; }
extern "C" int cns_set_device(int device) {
    CK(cudaSetDevice(device));
    return CNS_OK;
}
extern "C" int cns_device_synchronize(void) {
    CK(cudaDeviceSynchronize());
    return CNS_OK;
}
extern "C" int cns_selftest_bounded_wait(int* status) {
    if (!status) return fail(CNS_ERR_INVALID, "null argument");
    CK(bounded_wait_selftest(status));
    return CNS_OK;
}
extern "C" int cns_selftest_exact_sums(const double* taps, int n, double* sums, int* ok) {
    if (!taps || !sums || !ok) return fail(CNS_ERR_INVALID, "null argument");
    if (n < 0 || n > (1 << 24)) return fail(CNS_ERR_INVALID, "n=%d outside 0..2^24", n);
    CK(exact_sums_selftest(taps, n, sums, ok));
    return CNS_OK;
}

extern "C" int cns_measure_fp64_peak(double* tflops) {
    if (!tflops) return fail(CNS_ERR_INVALID, "null argument");
    CK(probe_fp64(tflops));
    return CNS_OK;
}

// Keep freed box memory in the device's default pool instead of returning it to the driver
// at each synchronisation, so that admitting a box after another finished costs no driver
// allocation.
static cudaError_t keep_pool_warm(int dev) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), dev) != done.end()) return cudaSuccess;
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e != cudaSuccess) return e;
    unsigned long long thr = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (e == cudaSuccess) done.push_back(dev);
    return e;
}

// ---- geometry and coefficients ----------------------------------------------------------
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Geometry {
    int pk;
    long long sj, si, fs;
    size_t off_sc, off_dtlog, off_U, off_Us, off_P0, off_P1, off_S, off_view, off_tiles, off_aos, total;
    size_t off_xtiles, off_maps;  // mixed boxes: TMA-assembly tiles and tensor maps
    size_t off_X;                 // FP64 boxes: fixed-point copies of kFxFields fields of both P sets
    int ntiles;                   // capacity of the tile list (largest candidate shape)
    int nxtiles;                  // TMA-assembly tiles (8 x 8 x 32 cells)
};

static int validate_desc(const cns_box_desc* d) {
    if (!d) return fail(CNS_ERR_INVALID, "null box description");
    for (int a = 0; a < 3; a++) {
        if (d->n[a] < CNS_NG) return fail(CNS_ERR_INVALID, "n[%d]=%d: each axis needs >= %d interior cells", a, d->n[a], CNS_NG);
        if (d->n[a] > 4096) return fail(CNS_ERR_CAPACITY, "n[%d]=%d above 4096", a, d->n[a]);
        if (!(d->dx[a] > 0.0) || !std::isfinite(d->dx[a])) return fail(CNS_ERR_INVALID, "dx[%d] must be positive", a);
    }
    if (!(d->cfl > 0.0)) return fail(CNS_ERR_INVALID, "cfl must be positive");
    if (!(d->eta >= 0.0) || !(d->alam >= 0.0)) return fail(CNS_ERR_INVALID, "eta and alam must be >= 0");
    if (d->precision != CNS_FP64 && d->precision != CNS_MIXED) return fail(CNS_ERR_INVALID, "precision must be 0 or 1");
    return CNS_OK;
}

// ---- tile shapes ----------------------------------------------------------------------------
// Candidate tile shapes (log2 of the i, j, k extents; 256 cells each).  k is the unit-stride
// axis, so every candidate keeps at least 8 consecutive k cells in a warp.
// The last candidate is the linear tile (256 consecutive cells; cns_common.cuh).
static const int kShapes[][3] = {{1, 2, 5}, {0, 3, 5}, {2, 1, 5}, {0, 2, 6}, {1, 1, 6},
                                 {1, 3, 4}, {2, 2, 4}, {0, 4, 4}, {3, 1, 4}, {2, 3, 3}, {3, 2, 3}, {1, 4, 3},
                                 {kLinearTile, 0, 0}};
static const int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);
static const int kNumBlockShapes = kNumShapes - 1;  // the rectangular ones

static long long tile_count(const int n[3], const int tlog[3]) {
    if (tlog[0] == kLinearTile) return ((long long)n[0] * n[1] * n[2] + kTileThreads - 1) / kTileThreads;
    long long c = 1;
    for (int a = 0; a < 3; a++) c *= (n[a] + (1 << tlog[a]) - 1) >> tlog[a];
    return c;
}

// The candidate that pads the box least (ties: the earlier candidate in the list).
static void default_tlog(const int n[3], int out[3]) {
    long long best = -1;
    for (int s = 0; s < kNumBlockShapes; s++) {
        const long long cells = tile_count(n, kShapes[s]) * kTileThreads;
        if (best < 0 || cells < best) {
            best = cells;
            for (int a = 0; a < 3; a++) out[a] = kShapes[s][a];
        }
    }
}

// The order the persistent kernels take a box's tiles in: its i-planes one band of j rows at a
// time, the band as many rows as keep the stencils' window (the tile's planes and 4 on each side,
// the band's rows, the fields a cell carries: ~272 bytes in the plain form, ~160 in the mixed)
// within ~24 MB of L2.  At 256^3 the plain form's step is 3-4 % faster than in plain i-major
// order (16-32 rows, by tile shape; 8 rows is too few), where the window of whole planes
// (~180 MB) overflows L2, and the mixed form's 0.7 %.  Small boxes are one band.
static int cell_bytes(int precision) { return precision == CNS_MIXED ? 160 : 272; }
static int band_rows(const int n[3], int ti, int tj, int bytes) {
    const double window = 24e6 / ((double)n[2] * (ti + 2 * CNS_NG) * bytes);
    int rows = tj;
    while (rows * 2 <= window && rows < n[1]) rows *= 2;
    return rows;
}

static void append_tiles(const int n[3], const int tlog[3], int box_index, std::vector<Tile>& out,
                         int bytes = 272) {
    if (tlog[0] == kLinearTile) {
        const long long nt = tile_count(n, tlog);
        for (long long t = 0; t < nt; t++) out.push_back(Tile{box_index, 0, 0, (int)t});
        return;
    }
    const int ti = 1 << tlog[0], tj = 1 << tlog[1], tk = 1 << tlog[2];
    const int band = band_rows(n, ti, tj, bytes);
    for (int jb = 0; jb < n[1]; jb += band)
        for (int i0 = 0; i0 < n[0]; i0 += ti)
            for (int j0 = jb; j0 < n[1] && j0 < jb + band; j0 += tj)
                for (int k0 = 0; k0 < n[2]; k0 += tk) out.push_back(Tile{box_index, i0, j0, k0});
}

static Geometry geometry(const cns_box_desc* d) {
    Geometry g;
    const long long g0 = d->n[0] + 2 * CNS_NG, g1 = d->n[1] + 2 * CNS_NG, g2 = d->n[2] + 2 * CNS_NG;
    g.pk = (int)((g2 + 7) / 8 * 8);
    g.sj = g.pk;
    g.si = g1 * g.sj;
    g.fs = g0 * g.si;
    const size_t esz = d->precision == CNS_MIXED ? 4 : 8;
    g.ntiles = 0;  // capacity: the largest tile count over the candidate shapes
    for (int sh = 0; sh < kNumShapes; sh++) g.ntiles = std::max<long long>(g.ntiles, tile_count(d->n, kShapes[sh]));
    size_t o = 0;
    g.off_sc = o;      o = align256(o + sizeof(BoxScalars));
    g.off_dtlog = o;   o = align256(o + sizeof(double) * DTLOG_CAP);
    g.off_U = o;       o = align256(o + sizeof(double) * 5 * g.fs);
    g.off_Us = o;      o = align256(o + sizeof(double) * 5 * g.fs);
    g.off_P0 = o;      o = align256(o + esz * NPF * g.fs);
    g.off_P1 = o;      o = align256(o + esz * NPF * g.fs);
    g.off_S = o;       o = align256(o + esz * NSF * g.fs);
    g.off_view = o;    o = align256(o + sizeof(BoxView));
    g.off_tiles = o;   o = align256(o + sizeof(Tile) * g.ntiles);
    g.off_aos = o;     o = align256(o + sizeof(double) * CNS_NC * g0 * g1 * g2);
    g.off_X = o;
    if (d->precision != CNS_MIXED) o = align256(o + sizeof(long long) * 2 * kFxFields * g.fs);
    int xi, xj, xk;
    tma_tile_shape(&xi, &xj, &xk);
    g.nxtiles = 0;
    g.off_xtiles = g.off_maps = 0;
    {  // the TMA assemblies' tiles and tensor maps (both forms)
        g.nxtiles = ((d->n[0] + xi - 1) / xi) * ((d->n[1] + xj - 1) / xj) * ((d->n[2] + xk - 1) / xk);
        g.off_xtiles = o;  o = align256(o + sizeof(Tile) * g.nxtiles);
        g.off_maps = o;    o = align256(o + tma_maps_bytes());
    }
    g.total = o;
    return g;
}

static void append_xtiles(const int n[3], int box_index, std::vector<Tile>& out, int bytes = 272) {
    int xi, xj, xk;
    tma_tile_shape(&xi, &xj, &xk);
    const int band = band_rows(n, xi, xj, bytes);
    for (int jb = 0; jb < n[1]; jb += band)
        for (int i0 = 0; i0 < n[0]; i0 += xi)
            for (int j0 = jb; j0 < n[1] && j0 < jb + band; j0 += xj)
                for (int k0 = 0; k0 < n[2]; k0 += xk) out.push_back(Tile{box_index, i0, j0, k0});
}

template <class R>
static void cast_coefs(CoefT<R>& dst, const CoefT<double>& s) {
    const double* a = (const double*)&s;
    R* b = (R*)&dst;
    for (size_t i = 0; i < sizeof(CoefT<double>) / sizeof(double); i++) b[i] = (R)a[i];
}

static void fill_coefs(BoxView& v, const cns_box_desc* d) {
    const double A[4] = {kAlp, kBet, kGam, kDel};
    const double B[4] = {kOff1, kOff2, kOff3, kOff4};
    const double dxi[3] = {1.0 / d->dx[0], 1.0 / d->dx[1], 1.0 / d->dx[2]};
    CoefT<double>& c = v.c64;
    memset(&c, 0, sizeof c);
    double tsum = 0.0;
    // heat conduction alam lap(T) = (alam / c_v) lap(e): the P set carries e, not T
    const double alam_cv = d->alam * (1.0 / kCv);
    for (int a = 0; a < 3; a++) {
        for (int m = 0; m < 4; m++) {
            c.da[a][m] = A[m] * dxi[a];
            c.ha[a][m] = -A[m] * dxi[a];
            c.mx[a][m] = (d->eta * (1.0 / 3.0)) * A[m] * dxi[a];
            c.tl[a][m] = alam_cv * B[m] * (dxi[a] * dxi[a]);
        }
        c.da[a][4] = dxi[a] / kD1Den;
        c.ha[a][4] = -dxi[a] / kD1Den;
        c.mx[a][4] = (d->eta * (1.0 / 3.0)) * dxi[a] / kD1Den;
        c.tl[a][4] = alam_cv * (dxi[a] * dxi[a]) / kD2Den;
        tsum += dxi[a] * dxi[a];
        c.cour[a] = dxi[a];
    }
    c.tc = alam_cv * kCenter * tsum;
    for (int comp = 0; comp < 3; comp++) {
        double sum = 0.0;
        for (int a = 0; a < 3; a++) {
            const double w = d->eta * (comp == a ? 4.0 / 3.0 : 1.0) * (dxi[a] * dxi[a]);
            for (int m = 0; m < 4; m++) c.vl[comp][a][m] = w * B[m];
            c.vl[comp][a][4] = w / kD2Den;
            sum += w;
        }
        c.vc[comp] = kCenter * sum;
    }
    c.eta = d->eta;
    cast_coefs(v.c32, v.c64);
    // the merged Laplacian sums (u: j + k, v: i + k, w: i + j, e: all three) need equal factors
    v.lap_merge = c.vl[0][1][4] == c.vl[0][2][4] && c.vl[1][0][4] == c.vl[1][2][4] &&
                  c.vl[2][0][4] == c.vl[2][1][4] && c.tl[0][4] == c.tl[1][4] && c.tl[1][4] == c.tl[2][4];
}

// ---- boxes -------------------------------------------------------------------------------
struct cns_batch;

struct cns_box {
    int dev = 0;
    cns_box_desc desc{};
    Geometry geo{};
    BoxView view{};
    BoxView* d_view = nullptr;
    Tile* d_tiles = nullptr;
    double* d_aos = nullptr;
    BoxScalars* d_sc = nullptr;
    char* arena = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    bool primed = false;
    int ntiles = 0;  // tiles of the current shape (view.tlog)
    Tile* d_xtiles = nullptr;  // mixed boxes: tiles of the TMA assembly kernel
    int nxtiles = 0;
    int kernel = CNS_ASSEMBLE_DIRECT;  // which k_assemble a mixed box runs
    cudaGraphExec_t gexec = nullptr;
    cns_batch* batch = nullptr;
    double* host_out = nullptr;  // the source of the device view's host_out (see set_host_out)
    int* d_queue = nullptr;      // k_upload_deriv's work queue for the tile shape queue_tlog
    int nq = 0;
    int queue_tlog[3] = {0, 0, 0};
    int* d_counters = nullptr;   // its plane counts and queue position (n[0] + 1 ints)
    long long* a_X = nullptr;    // FP64 boxes: copies of kFxFields fields of both P sets (arena)
    long long* d_X = nullptr;    // copies of all NPF fields of both P sets: allocated when the box first
                                 // goes onto CNS_ASSEMBLE_TMA_FX (stream-ordered), kept until destroy
    int fx_kernel = -1;          // the fixed-point kernel the copies are kept for (-1: none)
};

extern "C" long long cns_box_bytes(const cns_box_desc* desc) {
    if (validate_desc(desc) != CNS_OK) return -1;
    return (long long)geometry(desc).total;
}

extern "C" int cns_box_create(const cns_box_desc* desc, cns_box** out) {
    if (!out) return fail(CNS_ERR_INVALID, "null output handle");
    *out = nullptr;
    int rc = validate_desc(desc);
    if (rc) return rc;
    cns_box* b = new (std::nothrow) cns_box();
    if (!b) return fail(CNS_ERR_NOMEM, "host allocation failed");
    b->desc = *desc;
    b->geo = geometry(desc);
    cudaError_t e = cudaGetDevice(&b->dev);
    if (e == cudaSuccess) e = keep_pool_warm(b->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    // stream-ordered allocation: freeing a finished box later needs no device-wide sync
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->arena, b->geo.total, b->own_stream);
    if (e != cudaSuccess) {
        if (b->own_stream) cudaStreamDestroy(b->own_stream);
        delete b;
        return fail_cuda(e, "cns_box_create", __LINE__);
    }
    b->stream = b->own_stream;
    const Geometry& g = b->geo;
    BoxView& v = b->view;
    memset(&v, 0, sizeof v);
    for (int a = 0; a < 3; a++) v.n[a] = desc->n[a];
    v.pk = g.pk;
    v.sj = g.sj;
    v.si = g.si;
    v.fs = g.fs;
    v.U = (double*)(b->arena + g.off_U);
    v.Us = (double*)(b->arena + g.off_Us);
    v.P[0] = b->arena + g.off_P0;
    v.P[1] = b->arena + g.off_P1;
    v.S = b->arena + g.off_S;
    v.sc = (BoxScalars*)(b->arena + g.off_sc);
    v.dtlog = (double*)(b->arena + g.off_dtlog);
    v.cfl = desc->cfl;
    v.precision = desc->precision;
    fill_coefs(v, desc);
    b->d_view = (BoxView*)(b->arena + g.off_view);
    b->d_tiles = (Tile*)(b->arena + g.off_tiles);
    b->d_aos = (double*)(b->arena + g.off_aos);
    b->d_sc = v.sc;
    if (desc->precision != CNS_MIXED) {
        // FP64 boxes start on the direct kernels on fixed-point copies of u, v, w, e
        b->a_X = (long long*)(b->arena + g.off_X);
        v.X[0] = b->a_X;
        v.X[1] = b->a_X + kFxFields * g.fs;
        v.fx = kFxFields;
        b->kernel = CNS_ASSEMBLE_FX;
        b->fx_kernel = CNS_ASSEMBLE_FX;
    }
    default_tlog(desc->n, v.tlog);
    std::vector<Tile> tiles;
    append_tiles(desc->n, v.tlog, 0, tiles, cell_bytes(desc->precision));
    b->ntiles = (int)tiles.size();
    std::vector<Tile> xtiles;
    std::vector<unsigned char> maps;
    {
        // the TMA assemblies need the box's tensor maps; without a driver entry point for them
        // the box stays on the direct kernel
        b->d_xtiles = (Tile*)(b->arena + g.off_xtiles);
        append_xtiles(desc->n, 0, xtiles, cell_bytes(desc->precision));
        b->nxtiles = (int)xtiles.size();
        maps.resize(tma_maps_bytes());
        if (tma_encode_maps(v, maps.data()) == cudaSuccess) {
            v.tma = b->arena + g.off_maps;
            if (desc->precision == CNS_MIXED) b->kernel = assemble_ws_fits() ? CNS_ASSEMBLE_TMA_WS : CNS_ASSEMBLE_TMA;
        }
    }
    e = cudaMemsetAsync(b->arena, 0, g.total, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_view, &v, sizeof v, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess && !xtiles.empty())
        e = cudaMemcpyAsync(b->d_xtiles, xtiles.data(), sizeof(Tile) * xtiles.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess && v.tma)
        e = cudaMemcpyAsync((void*)v.tma, maps.data(), maps.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(b->arena, b->own_stream);
        cudaStreamSynchronize(b->own_stream);
        cudaStreamDestroy(b->own_stream);
        delete b;
        return fail_cuda(e, "cns_box_create init", __LINE__);
    }
    *out = b;
    return CNS_OK;
}

extern "C" int cns_batch_remove(cns_batch* batch, cns_box* box);

static cudaStream_t batch_stream(cns_batch* bt);

extern "C" int cns_box_destroy(cns_box* b) {
    if (!b) return CNS_OK;
    cudaSetDevice(b->dev);
    if (b->batch) {
        // work already queued by the batch may still touch this box: order the free after it
        cudaEvent_t ev;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(ev, batch_stream(b->batch));
            cudaStreamWaitEvent(b->stream, ev, 0);
            cudaEventDestroy(ev);
        }
        cns_batch_remove(b->batch, b);
    }
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->d_queue || b->d_counters) {
        cudaStreamSynchronize(b->stream);
        cudaFree(b->d_queue);
        cudaFree(b->d_counters);
    }
    if (b->d_X) cudaFreeAsync(b->d_X, b->stream);
    cudaFreeAsync(b->arena, b->stream);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);  // released once its queued work is done
    delete b;
    return CNS_OK;
}

extern "C" int cns_box_set_stream(cns_box* b, void* stream) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    return CNS_OK;
}

// Prime a box whose U interior was just written: primitives/fluxes, Courant, first dt.
// `restore` (a snapshot's scalars) keeps its step count and reference values instead of
// deriving fresh ones, so a resumed run continues bit for bit.
// The plain form's fixed-point copy of the P set an upload just wrote (boxes on CNS_ASSEMBLE_FX
// or CNS_ASSEMBLE_TMA_FX): its fields' maxima (unless restored exponents are kept), then the copy.
static int fx_after_upload(cns_box* b, bool restored) {
    if (!b->view.fx) return CNS_OK;
    if (!restored) CK(launch_fx_pass(false, b->d_view, b->d_tiles, b->ntiles, b->stream));
    CK(launch_fx_pass(true, b->d_view, b->d_tiles, b->ntiles, b->stream));
    return CNS_OK;
}

static int prime(cns_box* b, const BoxScalars* restore = nullptr) {
    bool fx_restored = false;  // a restore whose saved fixed-point copy was usable keeps its exponents
    if (restore) {
        BoxScalars s;
        memset(&s, 0, sizeof s);
        s.nsteps_done = restore->nsteps_done;
        s.dt_last = restore->dt_last;
        s.p_ref = restore->p_ref;
        s.e_ref = restore->e_ref;
        s.E_ref = restore->E_ref;
        s.H_ref = restore->H_ref;
        // the saved P set becomes P[0]: its copy is made again at the saved exponents, and the next
        // writes take theirs from the saved maxima, so the run continues bit for bit
        fx_restored = b->view.fx && !restore->fx_bad[restore->pbase & 1];
        s.fx_restore = fx_restored ? 1 : 0;
        s.fx_fresh = fx_restored ? restore->fx_fresh : 0;
        for (int f = 0; f < NPF && fx_restored; f++) {
            s.fx_e[0][f] = restore->fx_e[restore->pbase & 1][f];
            s.fx_prev[f] = restore->fx_prev[f];
        }
        CK(cudaMemcpyAsync(b->d_sc, &s, sizeof s, cudaMemcpyHostToDevice, b->stream));
        CK(cudaStreamSynchronize(b->stream));  // s lives on this stack frame
    } else {
        CK(cudaMemsetAsync(b->d_sc, 0, sizeof(BoxScalars), b->stream));
        CK(launch_refs(b->d_view, 1, b->stream));
    }
    CK(launch_prim(b->desc.precision, b->d_view, b->d_tiles, b->ntiles, b->stream));
    int rc = fx_after_upload(b, fx_restored);
    if (rc) return rc;
    CK(launch_stepend(b->d_view, 1, 0, b->stream));
    b->primed = true;
    return CNS_OK;
}

extern "C" int cns_box_init_field(cns_box* b, const double amp[3], double perturb, unsigned long long seed) {
    if (!b || !amp) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    CK(op_init_field(b->view, amp[0], amp[1], amp[2], perturb, seed, b->stream));
    return prime(b);
}


static size_t aos_bytes(const cns_box* b) {
    return sizeof(double) * CNS_NC * (size_t)(b->desc.n[0] + 8) * (b->desc.n[1] + 8) * (b->desc.n[2] + 8);
}

extern "C" int cns_box_upload_device(cns_box* b, const double* U_dev) {
    if (!b || !U_dev) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    CK(op_aos_to_box(U_dev, b->view, b->stream));
    return prime(b);
}

// Host array -> box, primed, queued on the box's stream.  A page-locked array (h_map, its
// device address) is read in place, interior only; for FP64 boxes the first ctoprim + Courant
// pass is fused into that read, and with `ghosts` the array's ghost cells are written with the
// periodic images of its interior on the way.  Otherwise it is staged through the box's AoS
// buffer (and `ghosts` is left to the caller).
static int upload_host(cns_box* b, const double* U_host, double* h_map, bool ghosts) {
    if (!h_map) {
        CK(cudaMemcpyAsync(b->d_aos, U_host, aos_bytes(b), cudaMemcpyHostToDevice, b->stream));
        return cns_box_upload_device(b, b->d_aos);
    }
    const bool fp64 = b->desc.precision == CNS_FP64;
    CK(cudaMemsetAsync(b->d_sc, 0, sizeof(BoxScalars), b->stream));
    CK(host_upload(b->view, h_map, fp64, ghosts, b->stream));
    CK(launch_refs(b->d_view, 1, b->stream));
    if (!fp64) CK(launch_prim(b->desc.precision, b->d_view, b->d_tiles, b->ntiles, b->stream));
    int rc = fx_after_upload(b, false);
    if (rc) return rc;
    CK(launch_stepend(b->d_view, 1, 0, b->stream));
    b->primed = true;
    return CNS_OK;
}

// Box -> host array (interior, and with `ghosts` every ghost cell as its periodic image),
// queued on the box's stream; in place for a page-locked array, else staged.
static int download_host(cns_box* b, double* U_host, double* h_map, bool ghosts) {
    if (!h_map) {
        CK(op_box_to_aos(b->view, b->d_aos, ghosts ? 1 : 0, b->stream));
        CK(cudaMemcpyAsync(U_host, b->d_aos, aos_bytes(b), cudaMemcpyDeviceToHost, b->stream));
        return CNS_OK;
    }
    CK(host_download(b->view, h_map, b->stream));
    if (ghosts) CK(host_ghosts(b->view, h_map, b->stream));
    return CNS_OK;
}

extern "C" int cns_box_upload(cns_box* b, const double* U_host) {
    if (!b || !U_host) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    int rc = upload_host(b, U_host, (double*)mapped_host_range(U_host, aos_bytes(b)), false);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return CNS_OK;
}

extern "C" int cns_box_download_device(cns_box* b, double* U_dev) {
    if (!b || !U_dev) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    CK(op_box_to_aos(b->view, U_dev, 1, b->stream));
    return CNS_OK;
}

extern "C" int cns_box_download(cns_box* b, double* U_host) {
    if (!b || !U_host) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    int rc = download_host(b, U_host, (double*)mapped_host_range(U_host, aos_bytes(b)), true);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return CNS_OK;
}

// The tiles of one RK3 step, split by kernel: FP64 boxes, mixed boxes (their derivative pass
// always, their assembly when on the direct kernel), and mixed boxes on the TMA assembly.
struct WorkLists {
    const Tile* d64 = nullptr;  // the derivative pass of FP64 boxes
    int nd64 = 0;
    const Tile* a64 = nullptr;  // FP64 boxes on the direct assembly
    int na64 = 0;
    const Tile* x64 = nullptr;  // FP64 boxes on the TMA assembly
    int nx64 = 0;
    const Tile* d32 = nullptr;
    int nd32 = 0;
    const Tile* a32 = nullptr;
    int na32 = 0;
    const Tile* x32 = nullptr;
    int nx32 = 0;
    const Tile* w32 = nullptr;  // mixed boxes on the warp-specialised TMA assembly
    int nw32 = 0;
    const Tile* dx32 = nullptr;  // the derivative pass of mixed boxes on either TMA assembly
    int ndx32 = 0;
    const Tile* f64 = nullptr;  // FP64 boxes on the fixed-point TMA assembly
    int nf64 = 0;
    const Tile* dfx64 = nullptr;  // the derivative pass of FP64 boxes that keep fixed-point copies
    int ndfx64 = 0;
    const Tile* afx64 = nullptr;  // FP64 boxes on the direct assembly on fixed-point taps
    int nafx64 = 0;
    const Tile* afxm64 = nullptr;  // the same, boxes whose Laplacians take the merged sums
    int nafxm64 = 0;
};

// One RK3 step of the boxes behind `views`.  When `ev` is given, an event is recorded after
// every launch and the launch's kind appended to `kinds`.
// With skip_first_deriv the step starts at stage 1's assembly (its derivative pass already ran,
// fused with an upload).
static int enqueue_step(const BoxView* views, int nviews, const WorkLists& w, cudaStream_t st,
                        std::vector<cudaEvent_t>* ev, std::vector<int>* kinds, bool skip_first_deriv = false) {
    auto mark = [&](int kind) -> int {
        if (!ev) return CNS_OK;
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        CK(cudaEventRecord(e, st));
        ev->push_back(e);
        kinds->push_back(kind);
        return CNS_OK;
    };
    int rc;
    for (int stage = 1; stage <= 3; stage++) {
        if (w.nd64 && !(stage == 1 && skip_first_deriv)) {
            CK(launch_deriv(kFormPlain, views, w.d64, w.nd64, stage, st));
            if ((rc = mark(CNS_KERN_DERIV))) return rc;
        }
        if (w.ndfx64 && !(stage == 1 && skip_first_deriv)) {
            CK(launch_deriv(kFormPlainFx, views, w.dfx64, w.ndfx64, stage, st));
            if ((rc = mark(CNS_KERN_DERIV))) return rc;
        }
        if (w.nd32 && !(stage == 1 && skip_first_deriv)) {
            CK(launch_deriv(kFormMixed, views, w.d32, w.nd32, stage, st));
            if ((rc = mark(CNS_KERN_DERIV))) return rc;
        }
        if (w.ndx32 && !(stage == 1 && skip_first_deriv)) {
            CK(launch_deriv_tma(views, w.dx32, w.ndx32, stage, st));
            if ((rc = mark(CNS_KERN_DERIV))) return rc;
        }
        if (w.na64) {
            CK(launch_assemble(kFormPlain, views, w.a64, w.na64, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nafx64) {
            CK(launch_assemble(kFormPlainFx, views, w.afx64, w.nafx64, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nafxm64) {
            CK(launch_assemble(kFormPlainFxMerge, views, w.afxm64, w.nafxm64, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nx64) {
            CK(launch_assemble_tma64(views, w.x64, w.nx64, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nf64) {
            CK(launch_assemble_fx(views, w.f64, w.nf64, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.na32) {
            CK(launch_assemble(kFormMixed, views, w.a32, w.na32, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nx32) {
            CK(launch_assemble_tma(views, w.x32, w.nx32, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
        if (w.nw32) {
            CK(launch_assemble_ws(views, w.w32, w.nw32, stage, st));
            if ((rc = mark(CNS_KERN_ASSEMBLE))) return rc;
        }
    }
    CK(launch_stepend(views, nviews, 1, st));
    return mark(CNS_KERN_STEPEND);
}

static WorkLists box_lists(const cns_box* b) {
    WorkLists w;
    if (b->desc.precision == CNS_MIXED) {
        if (b->kernel == CNS_ASSEMBLE_TMA)
            w.dx32 = w.x32 = b->d_xtiles, w.ndx32 = w.nx32 = b->nxtiles;
        else if (b->kernel == CNS_ASSEMBLE_TMA_WS)
            w.dx32 = w.w32 = b->d_xtiles, w.ndx32 = w.nw32 = b->nxtiles;
        else
            w.d32 = w.a32 = b->d_tiles, w.nd32 = w.na32 = b->ntiles;
    } else {
        if (b->view.fx)
            w.dfx64 = b->d_tiles, w.ndfx64 = b->ntiles;
        else
            w.d64 = b->d_tiles, w.nd64 = b->ntiles;
        if (b->kernel == CNS_ASSEMBLE_TMA)
            w.x64 = b->d_xtiles, w.nx64 = b->nxtiles;
        else if (b->kernel == CNS_ASSEMBLE_TMA_FX)
            w.f64 = b->d_xtiles, w.nf64 = b->nxtiles;
        else if (b->kernel == CNS_ASSEMBLE_FX && b->view.lap_merge)
            w.afxm64 = b->d_tiles, w.nafxm64 = b->ntiles;
        else if (b->kernel == CNS_ASSEMBLE_FX)
            w.afx64 = b->d_tiles, w.nafx64 = b->ntiles;
        else
            w.a64 = b->d_tiles, w.na64 = b->ntiles;
    }
    return w;
}

static int capture_step(cudaStream_t st, cudaGraphExec_t* out, const BoxView* views, int nviews, const WorkLists& w) {
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(views, nviews, w, st, nullptr, nullptr);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture", __LINE__);
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate", __LINE__);
    return CNS_OK;
}

extern "C" int cns_box_launches_per_step(const cns_box* b) { return b ? 7 : 0; }

extern "C" int cns_box_advance(cns_box* b, int nsteps) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    if (nsteps < 0) return fail(CNS_ERR_INVALID, "nsteps < 0");
    if (!b->primed) return fail(CNS_ERR_INVALID, "box has no state (upload first)");
    CK(cudaSetDevice(b->dev));
    if (!b->gexec) {
        int rc = capture_step(b->own_stream, &b->gexec, b->d_view, 1, box_lists(b));
        if (rc) return rc;
    }
    for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(b->gexec, b->stream));
    return CNS_OK;
}

// Device time of `launch` (graph replays on `st`) between two events on `st`; waits for it.
template <class F>
static int graph_ms(cudaStream_t st, F launch, double* ms) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail_cuda(e, "cudaEventCreate", __LINE__);
    }
    int rc = CNS_OK;
    e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) rc = launch();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float f = 0.f;
    if (e == cudaSuccess && rc == CNS_OK) e = cudaEventElapsedTime(&f, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (e != cudaSuccess) return fail_cuda(e, "graph timing", __LINE__);
    if (ms) *ms = f;
    return CNS_OK;
}

extern "C" int cns_box_advance_ms(cns_box* b, int nsteps, double* ms) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    CK(cudaSetDevice(b->dev));
    return graph_ms(b->stream, [&] { return cns_box_advance(b, nsteps); }, ms);
}

static int timed_run(cudaStream_t st, int nsteps, const BoxView* views, int nviews, const WorkLists& w,
                     double* kernel_ms, int* kernel_launches, double* total_ms) {
    std::vector<cudaEvent_t> ev;
    std::vector<int> kinds;
    ev.reserve(16 * nsteps + 1);
    kinds.reserve(16 * nsteps + 1);
    cudaEvent_t e0;
    CK(cudaEventCreate(&e0));
    CK(cudaEventRecord(e0, st));
    int rc = CNS_OK;
    for (int s = 0; s < nsteps && rc == CNS_OK; s++) rc = enqueue_step(views, nviews, w, st, &ev, &kinds);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == CNS_OK && e != cudaSuccess) rc = fail_cuda(e, "cudaStreamSynchronize", __LINE__);
    if (rc == CNS_OK) {
        for (int k = 0; k < CNS_KERN_COUNT; k++) {
            if (kernel_ms) kernel_ms[k] = 0.0;
            if (kernel_launches) kernel_launches[k] = 0;
        }
        cudaEvent_t prev = e0;
        for (size_t i = 0; i < ev.size(); i++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, prev, ev[i]);
            if (kernel_ms) kernel_ms[kinds[i]] += ms;
            if (kernel_launches) kernel_launches[kinds[i]] += 1;
            prev = ev[i];
        }
        if (total_ms) {
            float ms = 0.f;
            if (!ev.empty()) cudaEventElapsedTime(&ms, e0, ev.back());
            *total_ms = ms;
        }
    }
    for (auto x : ev) cudaEventDestroy(x);
    cudaEventDestroy(e0);
    return rc;
}

extern "C" int cns_box_advance_timed(cns_box* b, int nsteps, double* kernel_ms, int* kernel_launches,
                                     double* total_ms) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    if (nsteps < 0) return fail(CNS_ERR_INVALID, "nsteps < 0");
    if (!b->primed) return fail(CNS_ERR_INVALID, "box has no state (upload first)");
    CK(cudaSetDevice(b->dev));
    return timed_run(b->stream, nsteps, b->d_view, 1, box_lists(b), kernel_ms, kernel_launches, total_ms);
}

static int read_scalars(cns_box* b, BoxScalars* hs) {
    CK(cudaMemcpyAsync(hs, b->d_sc, sizeof *hs, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return CNS_OK;
}

extern "C" int cns_box_sync(cns_box* b, int* health_bits) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    CK(cudaSetDevice(b->dev));
    BoxScalars hs;
    int rc = read_scalars(b, &hs);
    if (rc) return rc;
    if (health_bits) *health_bits = hs.status;
    if (hs.status) return fail(CNS_ERR_NONFINITE, "box state went bad (health bits 0x%x)", hs.status);
    return CNS_OK;
}

extern "C" int cns_box_last_dt(cns_box* b, double* dt, int* nsteps_done) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    CK(cudaSetDevice(b->dev));
    BoxScalars hs;
    int rc = read_scalars(b, &hs);
    if (rc) return rc;
    if (dt) *dt = hs.dt_last;
    if (nsteps_done) *nsteps_done = hs.nsteps_done;
    return CNS_OK;
}

// ---- batches -----------------------------------------------------------------------------
struct cns_batch {
    int dev = 0;
    std::vector<cns_box*> members;
    BoxView* d_views = nullptr;
    Tile* d_tiles = nullptr;
    size_t cap_views = 0, cap_tiles = 0;
    int nviews = 0;
    WorkLists lists;  // into d_tiles
    cudaStream_t stream = nullptr, own_stream = nullptr;
    bool dirty = true;
    cudaGraphExec_t gexec = nullptr;
};

static cudaStream_t batch_stream(cns_batch* bt) { return bt->stream; }

// Make `later` wait for everything queued on `earlier` so far (no host blocking).
static int order_after(cudaStream_t later, cudaStream_t earlier) {
    if (later == earlier) return CNS_OK;
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, earlier);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(later, ev, 0);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return fail_cuda(e, "order_after", __LINE__);
    return CNS_OK;
}

extern "C" int cns_batch_create(cns_batch** out) {
    if (!out) return fail(CNS_ERR_INVALID, "null output handle");
    cns_batch* bt = new (std::nothrow) cns_batch();
    if (!bt) return fail(CNS_ERR_NOMEM, "host allocation failed");
    cudaError_t e = cudaGetDevice(&bt->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bt->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete bt;
        return fail_cuda(e, "cns_batch_create", __LINE__);
    }
    bt->stream = bt->own_stream;
    *out = bt;
    return CNS_OK;
}

extern "C" int cns_batch_destroy(cns_batch* bt) {
    if (!bt) return CNS_OK;
    cudaSetDevice(bt->dev);
    cudaStreamSynchronize(bt->stream);
    for (auto* b : bt->members) b->batch = nullptr;
    if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
    cudaFree(bt->d_views);
    cudaFree(bt->d_tiles);
    if (bt->own_stream) cudaStreamDestroy(bt->own_stream);
    delete bt;
    return CNS_OK;
}

extern "C" int cns_batch_set_stream(cns_batch* bt, void* stream) {
    if (!bt) return fail(CNS_ERR_INVALID, "null batch");
    bt->stream = stream ? (cudaStream_t)stream : bt->own_stream;
    return CNS_OK;
}

extern "C" int cns_batch_add(cns_batch* bt, cns_box* b) {
    if (!bt || !b) return fail(CNS_ERR_INVALID, "null argument");
    if (b->batch) return fail(CNS_ERR_INVALID, "box already belongs to a batch");
    if (b->dev != bt->dev) return fail(CNS_ERR_INVALID, "box and batch live on different devices");
    if (!b->primed) return fail(CNS_ERR_INVALID, "box has no state (upload first)");
    // work queued on the box's stream (an asynchronous init or upload) precedes the batch's
    int rc = order_after(bt->stream, b->stream);
    if (rc) return rc;
    bt->members.push_back(b);
    b->batch = bt;
    bt->dirty = true;
    return CNS_OK;
}

extern "C" int cns_batch_remove(cns_batch* bt, cns_box* b) {
    if (!bt || !b) return fail(CNS_ERR_INVALID, "null argument");
    auto it = std::find(bt->members.begin(), bt->members.end(), b);
    if (it == bt->members.end()) return fail(CNS_ERR_INVALID, "box is not in this batch");
    // later work on the box's own stream (download, free) follows the batch's queued steps
    int rc = order_after(b->stream, bt->stream);
    if (rc) return rc;
    bt->members.erase(it);
    b->batch = nullptr;
    bt->dirty = true;
    return CNS_OK;
}

extern "C" int cns_batch_size(const cns_batch* bt) { return bt ? (int)bt->members.size() : 0; }

static int batch_rebuild(cns_batch* bt, bool capture = true) {
    CK(cudaStreamSynchronize(bt->stream));
    std::vector<BoxView> views;
    std::vector<Tile> d64, a64, f64, d32, a32, x32, w32, dx32, dfx64, afx64, afxm64;  // the lists of WorkLists
    for (size_t m = 0; m < bt->members.size(); m++) {
        const cns_box* b = bt->members[m];
        views.push_back(b->view);
        if (b->desc.precision != CNS_MIXED) {
            // FP64 members: the direct assembly, on FP64 or fixed-point taps, or the fixed-point TMA one
            append_tiles(b->desc.n, b->view.tlog, (int)m, b->view.fx ? dfx64 : d64);
            if (b->kernel == CNS_ASSEMBLE_TMA_FX)
                append_xtiles(b->desc.n, (int)m, f64);
            else
                append_tiles(b->desc.n, b->view.tlog, (int)m,
                             b->kernel != CNS_ASSEMBLE_FX ? a64 : b->view.lap_merge ? afxm64 : afx64);
            continue;
        }
        if (b->kernel == CNS_ASSEMBLE_TMA || b->kernel == CNS_ASSEMBLE_TMA_WS) {
            append_xtiles(b->desc.n, (int)m, dx32, cell_bytes(CNS_MIXED));
            append_xtiles(b->desc.n, (int)m, b->kernel == CNS_ASSEMBLE_TMA ? x32 : w32, cell_bytes(CNS_MIXED));
        } else {
            append_tiles(b->desc.n, b->view.tlog, (int)m, d32, cell_bytes(CNS_MIXED));
            append_tiles(b->desc.n, b->view.tlog, (int)m, a32, cell_bytes(CNS_MIXED));
        }
    }
    std::vector<Tile> all;
    all.reserve(d64.size() + a64.size() + f64.size() + d32.size() + a32.size() + x32.size() + w32.size() + dx32.size() +
                dfx64.size() + afx64.size() + afxm64.size());
    for (auto* v : {&d64, &a64, &f64, &d32, &a32, &x32, &w32, &dx32, &dfx64, &afx64, &afxm64})
        all.insert(all.end(), v->begin(), v->end());
    const size_t nt = all.size();
    if (views.size() > bt->cap_views) {
        cudaFree(bt->d_views);
        bt->d_views = nullptr;
        bt->cap_views = std::max<size_t>(views.size(), 2 * bt->cap_views);
        CK(cudaMalloc((void**)&bt->d_views, sizeof(BoxView) * bt->cap_views));
    }
    if (nt > bt->cap_tiles) {
        cudaFree(bt->d_tiles);
        bt->d_tiles = nullptr;
        bt->cap_tiles = std::max<size_t>(nt, 2 * bt->cap_tiles);
        CK(cudaMalloc((void**)&bt->d_tiles, sizeof(Tile) * bt->cap_tiles));
    }
    if (!views.empty()) CK(cudaMemcpy(bt->d_views, views.data(), sizeof(BoxView) * views.size(), cudaMemcpyHostToDevice));
    if (!all.empty()) CK(cudaMemcpy(bt->d_tiles, all.data(), sizeof(Tile) * all.size(), cudaMemcpyHostToDevice));
    WorkLists& w = bt->lists;
    w = WorkLists();
    Tile* at = bt->d_tiles;
    w.d64 = at, w.nd64 = (int)d64.size(), at += d64.size();
    w.a64 = at, w.na64 = (int)a64.size(), at += a64.size();
    w.f64 = at, w.nf64 = (int)f64.size(), at += f64.size();
    w.d32 = at, w.nd32 = (int)d32.size(), at += d32.size();
    w.a32 = at, w.na32 = (int)a32.size(), at += a32.size();
    w.x32 = at, w.nx32 = (int)x32.size(), at += x32.size();
    w.w32 = at, w.nw32 = (int)w32.size(), at += w32.size();
    w.dx32 = at, w.ndx32 = (int)dx32.size(), at += dx32.size();
    w.dfx64 = at, w.ndfx64 = (int)dfx64.size(), at += dfx64.size();
    w.afx64 = at, w.nafx64 = (int)afx64.size(), at += afx64.size();
    w.afxm64 = at, w.nafxm64 = (int)afxm64.size();
    bt->nviews = (int)views.size();
    if (bt->gexec) {
        cudaGraphExecDestroy(bt->gexec);
        bt->gexec = nullptr;
    }
    if (!capture) {
        bt->dirty = true;  // tables are current, the graph is not
        return CNS_OK;
    }
    if (!views.empty()) {
        int rc = capture_step(bt->own_stream, &bt->gexec, bt->d_views, (int)views.size(), bt->lists);
        if (rc) return rc;
    }
    bt->dirty = false;
    return CNS_OK;
}

extern "C" int cns_batch_advance(cns_batch* bt, int nsteps) {
    if (!bt) return fail(CNS_ERR_INVALID, "null batch");
    if (nsteps < 0) return fail(CNS_ERR_INVALID, "nsteps < 0");
    CK(cudaSetDevice(bt->dev));
    if (bt->dirty) {
        int rc = batch_rebuild(bt);
        if (rc) return rc;
    }
    if (!bt->gexec) return CNS_OK;
    for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(bt->gexec, bt->stream));
    return CNS_OK;
}

extern "C" int cns_batch_advance_ms(cns_batch* bt, int nsteps, double* ms) {
    if (!bt) return fail(CNS_ERR_INVALID, "null batch");
    CK(cudaSetDevice(bt->dev));
    return graph_ms(bt->stream, [&] { return cns_batch_advance(bt, nsteps); }, ms);
}

extern "C" int cns_batch_sync(cns_batch* bt) {
    if (!bt) return fail(CNS_ERR_INVALID, "null batch");
    CK(cudaSetDevice(bt->dev));
    CK(cudaStreamSynchronize(bt->stream));
    return CNS_OK;
}

// ---- the reference's host-array entry points ---------------------------------------------
// A per-thread device workspace for the operator-level calls (grow-only).
struct Workspace {
    void* p = nullptr;
    size_t n = 0;
    int dev = -1;
    cudaStream_t st = nullptr;
    ~Workspace() {
        if (p) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
};
static thread_local Workspace g_ws;

static int workspace(size_t bytes, void** out, cudaStream_t* st) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (g_ws.dev != dev) {
        if (g_ws.p) cudaFree(g_ws.p);
        if (g_ws.st) cudaStreamDestroy(g_ws.st);
        g_ws.p = nullptr;
        g_ws.n = 0;
        g_ws.st = nullptr;
        g_ws.dev = dev;
        CK(cudaStreamCreateWithFlags(&g_ws.st, cudaStreamNonBlocking));
    }
    if (bytes > g_ws.n) {
        if (g_ws.p) cudaFree(g_ws.p);
        g_ws.p = nullptr;
        g_ws.n = 0;
        CK(cudaMalloc(&g_ws.p, bytes));
        g_ws.n = bytes;
    }
    *out = g_ws.p;
    *st = g_ws.st;
    return CNS_OK;
}

static int check_bounds(const int lo[3], const int hi[3], int ng) {
    if (!lo || !hi) return fail(CNS_ERR_INVALID, "null lo/hi");
    if (ng < CNS_NG) return fail(CNS_ERR_INVALID, "ng=%d: the 8th-order stencils need ng >= %d", ng, CNS_NG);
    for (int a = 0; a < 3; a++)
        if (hi[a] < lo[a]) return fail(CNS_ERR_INVALID, "hi[%d] < lo[%d]", a, a);
    return CNS_OK;
}

extern "C" int cns_ctoprim(const int lo[3], const int hi[3], const double* u, double* q, const double dx[3], int ng,
                           double* courno) {
    int rc = check_bounds(lo, hi, ng);
    if (rc) return rc;
    if (!u || !q || !dx) return fail(CNS_ERR_INVALID, "null array");
    long long np = 1;
    for (int a = 0; a < 3; a++) np *= (hi[a] - lo[a] + 1 + 2 * ng);
    const size_t need = sizeof(double) * (size_t)np * (5 + 5 + 6 + 6) + 256;
    void* ws;
    cudaStream_t st;
    if ((rc = workspace(need, &ws, &st))) return rc;
    double* d_aos_u = (double*)ws;
    double* d_u = d_aos_u + 5 * np;
    double* d_q = d_u + 5 * np;
    double* d_aos_q = d_q + 6 * np;
    unsigned long long* d_c = (unsigned long long*)(d_aos_q + 6 * np);
    CK(cudaMemcpyAsync(d_aos_u, u, sizeof(double) * 5 * np, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(d_c, 0, sizeof(unsigned long long), st));
    CK(op_aos_to_soa(d_aos_u, d_u, np, 5, st));
    CK(op_ctoprim(lo, hi, ng, d_u, d_q, dx, courno ? d_c : nullptr, st));
    CK(op_soa_to_aos(d_q, d_aos_q, np, 6, st));
    CK(cudaMemcpyAsync(q, d_aos_q, sizeof(double) * 6 * np, cudaMemcpyDeviceToHost, st));
    unsigned long long cb = 0;
    if (courno) CK(cudaMemcpyAsync(&cb, d_c, sizeof cb, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (courno) {
        double c;
        memcpy(&c, &cb, sizeof c);
        // cpu/ctoprim.cpp:69: courno = MAX(MAX(courmx, courmy), MAX(courmz, courno))
        if (c > *courno) *courno = c;
    }
    return CNS_OK;
}

extern "C" int cns_hypterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double* cons,
                           const double* q, double* flux) {
    int rc = check_bounds(lo, hi, ng);
    if (rc) return rc;
    if (!cons || !q || !flux || !dx) return fail(CNS_ERR_INVALID, "null array");
    long long np = 1, ni = 1;
    for (int a = 0; a < 3; a++) {
        np *= (hi[a] - lo[a] + 1 + 2 * ng);
        ni *= (hi[a] - lo[a] + 1);
    }
    const size_t need = sizeof(double) * (size_t)(np * 22 + ni * 10);
    void* ws;
    cudaStream_t st;
    if ((rc = workspace(need, &ws, &st))) return rc;
    double* a_c = (double*)ws;
    double* a_q = a_c + 5 * np;
    double* s_c = a_q + 6 * np;
    double* s_q = s_c + 5 * np;
    double* s_f = s_q + 6 * np;
    double* a_f = s_f + 5 * ni;
    CK(cudaMemcpyAsync(a_c, cons, sizeof(double) * 5 * np, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a_q, q, sizeof(double) * 6 * np, cudaMemcpyHostToDevice, st));
    CK(op_aos_to_soa(a_c, s_c, np, 5, st));
    CK(op_aos_to_soa(a_q, s_q, np, 6, st));
    CK(op_hypterm(lo, hi, ng, s_c, s_q, s_f, dx, st));
    CK(op_soa_to_aos(s_f, a_f, ni, 5, st));
    CK(cudaMemcpyAsync(flux, a_f, sizeof(double) * 5 * ni, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CNS_OK;
}

extern "C" int cns_diffterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double* q,
                            double* difflux, double eta, double alam) {
    int rc = check_bounds(lo, hi, ng);
    if (rc) return rc;
    if (!q || !difflux || !dx) return fail(CNS_ERR_INVALID, "null array");
    long long np = 1, ni = 1;
    for (int a = 0; a < 3; a++) {
        np *= (hi[a] - lo[a] + 1 + 2 * ng);
        ni *= (hi[a] - lo[a] + 1);
    }
    const size_t need = sizeof(double) * (size_t)(np * (6 + 6 + 9) + ni * 10);
    void* ws;
    cudaStream_t st;
    if ((rc = workspace(need, &ws, &st))) return rc;
    double* a_q = (double*)ws;
    double* s_q = a_q + 6 * np;
    double* tmp = s_q + 6 * np;
    double* s_d = tmp + 9 * np;
    double* a_d = s_d + 5 * ni;
    CK(cudaMemcpyAsync(a_q, q, sizeof(double) * 6 * np, cudaMemcpyHostToDevice, st));
    CK(op_aos_to_soa(a_q, s_q, np, 6, st));
    CK(op_diffterm(lo, hi, ng, s_q, tmp, s_d, dx, eta, alam, st));
    CK(op_soa_to_aos(s_d, a_d, ni, 5, st));
    CK(cudaMemcpyAsync(difflux, a_d, sizeof(double) * 5 * ni, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CNS_OK;
}

extern "C" int cns_fill_boundary(double* U, const int dim[3], const int dim_ng[3]) {
    if (!U || !dim || !dim_ng) return fail(CNS_ERR_INVALID, "null argument");
    for (int a = 0; a < 3; a++) {
        if (dim[a] < CNS_NG) return fail(CNS_ERR_INVALID, "dim[%d]=%d < %d", a, dim[a], CNS_NG);
        if (dim_ng[a] != dim[a] + 2 * CNS_NG) return fail(CNS_ERR_INVALID, "dim_ng[%d] != dim[%d]+8", a, a);
    }
    const long long np = (long long)dim_ng[0] * dim_ng[1] * dim_ng[2];
    void* ws;
    cudaStream_t st;
    int rc = workspace(sizeof(double) * 5 * np, &ws, &st);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ws, U, sizeof(double) * 5 * np, cudaMemcpyHostToDevice, st));
    CK(op_fill_ghosts_aos((double*)ws, dim, 5, st));
    CK(cudaMemcpyAsync(U, ws, sizeof(double) * 5 * np, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CNS_OK;
}

// A per-thread cache of one box for the host-array advance entry points, so that repeated
// new_advance calls on the same problem reuse the device state allocation.
struct BoxCache {
    cns_box* box = nullptr;
    ~BoxCache() {
        if (box) cns_box_destroy(box);
    }
};
static thread_local BoxCache g_cache;

static bool same_desc(const cns_box_desc& a, const cns_box_desc& b) {
    return memcmp(a.n, b.n, sizeof a.n) == 0 && memcmp(a.dx, b.dx, sizeof a.dx) == 0 && a.cfl == b.cfl &&
           a.eta == b.eta && a.alam == b.alam && a.precision == b.precision;
}

static int cached_box(const cns_box_desc& d, cns_box** out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (g_cache.box && (g_cache.box->dev != dev || !same_desc(g_cache.box->desc, d))) {
        cns_box_destroy(g_cache.box);
        g_cache.box = nullptr;
    }
    if (!g_cache.box) {
        int rc = cns_box_create(&d, &g_cache.box);
        if (rc) return rc;
    }
    *out = g_cache.box;
    return CNS_OK;
}

// Copy a host state in, fill its ghosts (the reference's fill_boundary at the start of the
// step), run nsteps, and copy back the interior of the result with the ghosts of the last
// step's start state -- what the reference leaves in U (cpu/advance.cpp:45,144-153).
// Point the box's device view at a page-locked host array (or at nothing): stage 3 then also
// stores every cell's new state there.  Stream-ordered; the pointer is copied from the box
// itself, which outlives the copy.
static int set_host_out(cns_box* b, double* h_map) {
    b->host_out = h_map;
    b->view.host_out = h_map;
    CK(cudaMemcpyAsync((char*)b->d_view + offsetof(BoxView, host_out), &b->host_out, sizeof(double*),
                       cudaMemcpyHostToDevice, b->stream));
    return CNS_OK;
}

// Clears the device view's host pointer when the call returns, on every path: no later launch
// may write to the caller's memory after this call.
struct HostOutGuard {
    cns_box* b = nullptr;
    ~HostOutGuard() {
        if (b && b->host_out) {
            set_host_out(b, nullptr);
            cudaStreamSynchronize(b->stream);
        }
    }
};

// FP64 box, page-locked host array: upload it and enqueue the first RK3 step, with stage 1's
// derivative pass fused into the upload (k_upload_deriv, cns_host.cu): the FP64-bound
// derivatives run while the link-bound upload is still reading.  Same arithmetic, same bits as
// upload + step.
static int upload_first_step(cns_box* b, double* h_map, bool ghosts) {
    if (!b->d_queue || memcmp(b->queue_tlog, b->view.tlog, sizeof b->queue_tlog) != 0) {
        std::vector<Tile> tiles;
        append_tiles(b->desc.n, b->view.tlog, 0, tiles, cell_bytes(b->desc.precision));
        const std::vector<int> q = upload_deriv_queue(b->desc.n, b->view.tlog, tiles);
        CK(cudaStreamSynchronize(b->stream));
        cudaFree(b->d_queue);
        b->d_queue = nullptr;
        CK(cudaMalloc((void**)&b->d_queue, sizeof(int) * q.size()));
        CK(cudaMemcpy(b->d_queue, q.data(), sizeof(int) * q.size(), cudaMemcpyHostToDevice));
        b->nq = (int)q.size();
        memcpy(b->queue_tlog, b->view.tlog, sizeof b->queue_tlog);
    }
    if (!b->d_counters) CK(cudaMalloc((void**)&b->d_counters, sizeof(int) * (b->desc.n[0] + 1)));
    CK(cudaMemsetAsync(b->d_sc, 0, sizeof(BoxScalars), b->stream));
    CK(host_upload_deriv(b->view, h_map, ghosts, b->d_tiles, b->d_queue, b->nq, b->d_counters, b->stream));
    // (no k_refs: the FP64 form does not use the mixed form's reference values; the upload
    // also formed the maxima of the fields with copies, so only the copy pass is left)
    if (b->view.fx) CK(launch_fx_pass(true, b->d_view, b->d_tiles, b->ntiles, b->stream));
    CK(launch_stepend(b->d_view, 1, 0, b->stream));
    b->primed = true;
    return enqueue_step(b->d_view, 1, box_lists(b), b->stream, nullptr, nullptr, true);
}

static int host_advance(const cns_box_desc& d, double* U, int nsteps, double* dt_hist) {
    cns_box* b;
    int rc = cached_box(d, &b);
    if (rc) return rc;
    double* h_map = (double*)mapped_host_range(U, aos_bytes(b));
    HostOutGuard guard;
    guard.b = b;
    // the last step's start state supplies the ghosts: with at most one step that is the input
    const bool ghosts_on_upload = h_map && nsteps <= 1;
    // FP64 boxes on page-locked memory: the first step's derivative pass rides with the upload
    const bool fused = h_map && b->desc.precision == CNS_FP64 && nsteps >= 1;
    if (fused) {
        if (nsteps == 1 && (rc = set_host_out(b, h_map))) return rc;  // the first step is the last
        if ((rc = upload_first_step(b, h_map, ghosts_on_upload))) return rc;
        if (nsteps == 1 && (rc = set_host_out(b, nullptr))) return rc;
    } else if ((rc = upload_host(b, U, h_map, ghosts_on_upload))) {
        return rc;
    }
    int done = 0;
    while (done < nsteps) {
        const int chunk = std::min(nsteps - done, DTLOG_CAP);
        const int first = (done == 0 && fused) ? 1 : 0;  // steps of this chunk already enqueued
        if (done + chunk == nsteps && chunk > first) {
            if (chunk - 1 > first && (rc = cns_box_advance(b, chunk - 1 - first))) return rc;
            if (!h_map)
                CK(op_box_to_aos(b->view, b->d_aos, 1, b->stream));
            else if (!ghosts_on_upload)
                CK(host_ghosts(b->view, h_map, b->stream));
            // in place: the last step's stage 3 writes the interior straight to the caller
            if (h_map && (rc = set_host_out(b, h_map))) return rc;
            if ((rc = cns_box_advance(b, 1))) return rc;
            if (h_map && (rc = set_host_out(b, nullptr))) return rc;
        } else if (chunk > first && (rc = cns_box_advance(b, chunk - first))) {
            return rc;
        }
        if (dt_hist) {
            std::vector<double> log(DTLOG_CAP);
            CK(cudaMemcpyAsync(log.data(), b->view.dtlog, sizeof(double) * DTLOG_CAP, cudaMemcpyDeviceToHost, b->stream));
            CK(cudaStreamSynchronize(b->stream));
            for (int s = 0; s < chunk; s++) dt_hist[done + s] = log[(done + s) & (DTLOG_CAP - 1)];
        }
        done += chunk;
    }
    // in place, the array is complete: ghosts written at upload or before the last step, the
    // interior by the last stage 3 (or, with no step, the input itself)
    if (!h_map) {
        if (nsteps == 0) CK(op_box_to_aos(b->view, b->d_aos, 1, b->stream));
        if ((rc = download_host(b, U, nullptr, false))) return rc;
    }
    int health = 0;
    rc = cns_box_sync(b, &health);
    return rc;
}

extern "C" int cns_advance_host(double* U, const int n[3], const double dx[3], double cfl, double eta, double alam,
                                int nsteps, int precision, double* dt_hist) {
    if (!U || !n || !dx) return fail(CNS_ERR_INVALID, "null argument");
    if (nsteps < 0) return fail(CNS_ERR_INVALID, "nsteps < 0");
    cns_box_desc d;
    memset(&d, 0, sizeof d);
    for (int a = 0; a < 3; a++) {
        d.n[a] = n[a];
        d.dx[a] = dx[a];
    }
    d.cfl = cfl;
    d.eta = eta;
    d.alam = alam;
    d.precision = precision;
    int rc = validate_desc(&d);
    if (rc) return rc;
    return host_advance(d, U, nsteps, dt_hist);
}

extern "C" int cns_advance_f64(double* U, const int n[3], const double dx[3], double cfl, double eta, double alam,
                               int nsteps, double* dt_hist) {
    return cns_advance_host(U, n, dx, cfl, eta, alam, nsteps, CNS_FP64, dt_hist);
}
extern "C" int cns_advance_mixed(double* U, const int n[3], const double dx[3], double cfl, double eta, double alam,
                                 int nsteps, double* dt_hist) {
    return cns_advance_host(U, n, dx, cfl, eta, alam, nsteps, CNS_MIXED, dt_hist);
}

extern "C" int cns_set_pageable_in_place(int enable) {
    set_pageable_in_place(enable);
    return CNS_OK;
}

extern "C" int cns_host_in_place(const void* U, long long bytes, int* in_place) {
    if (!U || !in_place || bytes < 0) return fail(CNS_ERR_INVALID, "null argument or negative size");
    *in_place = mapped_host_range(U, (size_t)bytes) ? 1 : 0;
    return CNS_OK;
}

extern "C" int cns_new_advance(const cns_global_const_t* h, double* U, double* Unew, double* Q, double* D, double* F,
                               double* dt) {
    (void)Unew, (void)Q, (void)D, (void)F;
    if (!h || !U) return fail(CNS_ERR_INVALID, "null argument");
    if (h->ng != CNS_NG || h->nc != CNS_NC)
        return fail(CNS_ERR_INVALID, "ng=%d nc=%d: this build supports ng=%d, nc=%d", h->ng, h->nc, CNS_NG, CNS_NC);
    double dt1 = 0.0;
    int rc = cns_advance_host(U, h->dim, h->dx, h->cfl, h->eta, h->alam, 1, CNS_FP64, &dt1);
    if (rc == CNS_OK && dt) *dt = dt1;
    return rc;
}

// ---- binary snapshot: header + ghost-inclusive AoS state --------------------------------
struct SnapHeader {
    char magic[8];  // "CNSSNAP1"
    int32_t version, precision, n[3], ng;
    int64_t nsteps_done;
    double dx[3], cfl, eta, alam;
    double p_ref, e_ref, E_ref, H_ref, dt_last;
    int64_t payload_doubles;
    // version 2: the fixed-point exponents of the saved P set and the maxima the next writes take
    // theirs from (fx_valid = 0: none, they are derived again at load; 2: as 1, and the copy was
    // made from an upload, fx_fresh)
    int32_t fx_valid, fx_e[NPF], fx_prev[NPF];
};

extern "C" int cns_box_save(cns_box* b, const char* path) {
    if (!b || !path) return fail(CNS_ERR_INVALID, "null argument");
    if (!b->primed) return fail(CNS_ERR_INVALID, "box has no state");
    CK(cudaSetDevice(b->dev));
    std::vector<double> U(aos_bytes(b) / sizeof(double));
    BoxScalars hs;
    int rc = cns_box_download(b, U.data());
    if (rc) return rc;
    if ((rc = read_scalars(b, &hs))) return rc;
    SnapHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, "CNSSNAP1", 8);
    h.version = 2;
    h.precision = b->desc.precision;
    for (int a = 0; a < 3; a++) {
        h.n[a] = b->desc.n[a];
        h.dx[a] = b->desc.dx[a];
    }
    h.ng = CNS_NG;
    h.nsteps_done = hs.nsteps_done;
    h.cfl = b->desc.cfl;
    h.eta = b->desc.eta;
    h.alam = b->desc.alam;
    h.p_ref = hs.p_ref;
    h.e_ref = hs.e_ref;
    h.E_ref = hs.E_ref;
    h.H_ref = hs.H_ref;
    h.dt_last = hs.dt_last;
    h.payload_doubles = (int64_t)U.size();
    h.fx_valid = (b->view.fx && !hs.fx_bad[hs.pbase & 1]) ? (hs.fx_fresh ? 2 : 1) : 0;
    for (int q = 0; q < NPF; q++) {
        h.fx_e[q] = hs.fx_e[hs.pbase & 1][q];
        h.fx_prev[q] = hs.fx_prev[q];
    }
    FILE* f = fopen(path, "wb");
    if (!f) return fail(CNS_ERR_INVALID, "cannot create %s", path);
    bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(U.data(), sizeof(double), U.size(), f) == U.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? CNS_OK : fail(CNS_ERR_INVALID, "short write to %s", path);
}

extern "C" int cns_box_load(cns_box* b, const char* path) {
    if (!b || !path) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    FILE* f = fopen(path, "rb");
    if (!f) return fail(CNS_ERR_INVALID, "cannot open %s", path);
    SnapHeader h;
    std::vector<double> U(aos_bytes(b) / sizeof(double));
    // version 1 headers end before the fixed-point fields
    const size_t v1_bytes = offsetof(SnapHeader, fx_valid);
    memset(&h, 0, sizeof h);
    bool ok = fread(&h, v1_bytes, 1, f) == 1 && memcmp(h.magic, "CNSSNAP1", 8) == 0 &&
              (h.version == 1 || h.version == 2);
    if (ok && h.version == 2) ok = fread((char*)&h + v1_bytes, sizeof h - v1_bytes, 1, f) == 1;
    if (ok) {
        ok = h.precision == b->desc.precision && h.ng == CNS_NG && h.payload_doubles == (int64_t)U.size();
        for (int a = 0; a < 3; a++) ok = ok && h.n[a] == b->desc.n[a] && h.dx[a] == b->desc.dx[a];
        ok = ok && h.cfl == b->desc.cfl && h.eta == b->desc.eta && h.alam == b->desc.alam;
        if (!ok) {
            fclose(f);
            return fail(CNS_ERR_INVALID, "snapshot %s does not match this box (dims, dx, params or precision)", path);
        }
        ok = fread(U.data(), sizeof(double), U.size(), f) == U.size();
    }
    fclose(f);
    if (!ok) return fail(CNS_ERR_INVALID, "%s is not a complete snapshot", path);
    CK(cudaMemcpyAsync(b->d_aos, U.data(), aos_bytes(b), cudaMemcpyHostToDevice, b->stream));
    CK(op_aos_to_box(b->d_aos, b->view, b->stream));
    BoxScalars s;
    memset(&s, 0, sizeof s);
    s.nsteps_done = (int)h.nsteps_done;
    s.dt_last = h.dt_last;
    s.p_ref = h.p_ref;
    s.e_ref = h.e_ref;
    s.E_ref = h.E_ref;
    s.H_ref = h.H_ref;
    s.pbase = 0;
    s.fx_bad[0] = h.fx_valid ? 0 : 1;
    s.fx_fresh = h.fx_valid == 2 ? 1 : 0;
    for (int q = 0; q < NPF; q++) {
        s.fx_e[0][q] = h.fx_e[q];
        s.fx_prev[q] = h.fx_prev[q];
    }
    int rc = prime(b, &s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return CNS_OK;
}


// ---- tile shapes and the autotuner ---------------------------------------------------------
static int valid_tlog(const int t[3]) {
    if (t[0] == kLinearTile) return t[1] == 0 && t[2] == 0;
    for (int a = 0; a < 3; a++)
        if (t[a] < 0 || t[a] > 8) return 0;
    return t[0] + t[1] + t[2] == 8 && t[2] >= 3;
}

extern "C" int cns_box_get_tile(const cns_box* b, int tlog[3]) {
    if (!b || !tlog) return fail(CNS_ERR_INVALID, "null argument");
    for (int a = 0; a < 3; a++) tlog[a] = b->view.tlog[a];
    return CNS_OK;
}

// Apply a tile shape to a box's own work list and device view (the batch, if any, is rebuilt
// lazily).  Results do not depend on the shape: every cell's arithmetic is the same.
static int apply_tile(cns_box* b, const int tlog[3]) {
    if (!valid_tlog(tlog))
        return fail(CNS_ERR_INVALID, "tile shape: log2 extents in [0,8] summing to 8, k >= 3, or {-1, 0, 0} (linear)");
    if (tile_count(b->desc.n, tlog) > b->geo.ntiles) return fail(CNS_ERR_CAPACITY, "tile shape has too many tiles");
    CK(cudaStreamSynchronize(b->stream));
    if (b->batch) CK(cudaStreamSynchronize(batch_stream(b->batch)));
    for (int a = 0; a < 3; a++) b->view.tlog[a] = tlog[a];
    std::vector<Tile> tiles;
    append_tiles(b->desc.n, tlog, 0, tiles, cell_bytes(b->desc.precision));
    b->ntiles = (int)tiles.size();
    CK(cudaMemcpy(b->d_tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_view, &b->view, sizeof(BoxView), cudaMemcpyHostToDevice));
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->batch) b->batch->dirty = true;
    return CNS_OK;
}

extern "C" int cns_box_set_tile(cns_box* b, const int tlog[3]) {
    if (!b || !tlog) return fail(CNS_ERR_INVALID, "null argument");
    CK(cudaSetDevice(b->dev));
    return apply_tile(b, tlog);
}

// Keep a copy of the state (device AoS staging) and the scalars, and put them back: trial
// steps of the autotuner leave no trace, and the run continues bit for bit.
static int save_state(cns_box* b, BoxScalars* hs) {
    CK(op_box_to_aos(b->view, b->d_aos, 1, b->stream));
    return read_scalars(b, hs);
}
static int restore_state(cns_box* b, const BoxScalars* hs) {
    CK(op_aos_to_box(b->d_aos, b->view, b->stream));
    return prime(b, hs);
}

// A box on CNS_ASSEMBLE_FX or CNS_ASSEMBLE_TMA_FX keeps the fixed-point copy of the P set it reads
// (view.fx fields: u, v, w, e in the box's arena for the direct kernels; every field in a separate
// allocation for the TMA kernel); on any other kernel the copies are neither written nor read.
// Switching onto one of them between steps (or from one to the other) makes the copy of the
// current P set at once (maxima, then the copy) and takes those maxima for the next writes.
static int push_fx(cns_box* b) {
    const bool fp64 = b->desc.precision == CNS_FP64;
    const int fx = !fp64 ? 0 : b->kernel == CNS_ASSEMBLE_TMA_FX ? NPF : b->kernel == CNS_ASSEMBLE_FX ? kFxFields : 0;
    if (fx == b->view.fx && (!fx || b->fx_kernel == b->kernel)) return CNS_OK;
    CK(cudaStreamSynchronize(b->stream));
    if (b->batch) CK(cudaStreamSynchronize(batch_stream(b->batch)));
    if (fx == NPF && !b->d_X) {
        // copies of every field (two sets of the P fields' geometry, 64-bit words)
        const size_t bytes = sizeof(long long) * 2 * NPF * (size_t)b->view.fs;
        cudaError_t e = cudaMallocAsync((void**)&b->d_X, bytes, b->stream);
        if (e != cudaSuccess) {
            b->d_X = nullptr;
            cudaGetLastError();
            return fail(CNS_ERR_NOMEM, "fixed-point copies: %zu bytes of device memory not available", bytes);
        }
    }
    long long* base = fx == NPF ? b->d_X : b->a_X;
    b->view.X[0] = fx ? base : nullptr;
    b->view.X[1] = fx ? base + (long long)fx * b->view.fs : nullptr;
    b->view.fx = fx;
    b->fx_kernel = fx ? b->kernel : -1;
    std::vector<unsigned char> maps(tma_maps_bytes());
    if (b->view.tma) {  // the TMA kernels' tensor maps, with the copies' when every field has one
        CK(tma_encode_maps(b->view, maps.data()));
        CK(cudaMemcpyAsync((void*)b->view.tma, maps.data(), maps.size(), cudaMemcpyHostToDevice, b->stream));
    }
    CK(cudaMemcpyAsync((char*)b->d_view + offsetof(BoxView, X), b->view.X, sizeof b->view.X, cudaMemcpyHostToDevice,
                       b->stream));
    static const int kNone[2] = {0, 0}, kBoth[2] = {1, 1};
    CK(cudaMemcpyAsync(&b->d_sc->fx_bad[0], fx ? kNone : kBoth, sizeof kBoth, cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync((char*)b->d_view + offsetof(BoxView, fx), &b->view.fx, sizeof(int), cudaMemcpyHostToDevice,
                       b->stream));
    if (fx && b->primed) {
        int rc = fx_after_upload(b, false);
        if (rc) return rc;
        CK(launch_fx_adopt(b->d_view, 1, b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));  // `maps` lives on this stack frame
    if (b->batch) b->batch->dirty = true;
    return CNS_OK;
}

static int apply_kernel(cns_box* b, int kernel) {
    if (kernel != CNS_ASSEMBLE_DIRECT && kernel != CNS_ASSEMBLE_TMA && kernel != CNS_ASSEMBLE_TMA_WS &&
        kernel != CNS_ASSEMBLE_TMA_FX && kernel != CNS_ASSEMBLE_FX)
        return fail(CNS_ERR_INVALID, "unknown kernel %d", kernel);
    if (kernel == CNS_ASSEMBLE_TMA_FX && b->desc.precision != CNS_FP64)
        return fail(CNS_ERR_INVALID, "the fixed-point TMA assembly serves plain FP64 boxes only");
    if (kernel == CNS_ASSEMBLE_FX && b->desc.precision != CNS_FP64)
        return fail(CNS_ERR_INVALID, "the fixed-point assembly serves plain FP64 boxes only");
    if (kernel != CNS_ASSEMBLE_DIRECT && kernel != CNS_ASSEMBLE_FX && !b->view.tma)
        return fail(CNS_ERR_INVALID, "the TMA assemblies need the box's tensor maps");
    if (kernel == CNS_ASSEMBLE_TMA_WS && b->desc.precision != CNS_MIXED)
        return fail(CNS_ERR_INVALID, "the warp-specialised TMA assembly serves mixed-precision boxes only");
    if (kernel == b->kernel) return CNS_OK;
    CK(cudaStreamSynchronize(b->stream));
    if (b->batch) CK(cudaStreamSynchronize(batch_stream(b->batch)));
    b->kernel = kernel;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->batch) b->batch->dirty = true;
    return push_fx(b);
}

extern "C" int cns_box_get_kernel(const cns_box* b, int* kernel) {
    if (!b || !kernel) return fail(CNS_ERR_INVALID, "null argument");
    *kernel = b->kernel;
    return CNS_OK;
}

extern "C" int cns_box_set_kernel(cns_box* b, int kernel) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    CK(cudaSetDevice(b->dev));
    return apply_kernel(b, kernel);
}

extern "C" int cns_box_autotune(cns_box* b, int trial_steps, int tlog_out[3], int* kernel_out, double* best_ms) {
    if (!b) return fail(CNS_ERR_INVALID, "null box");
    if (!b->primed) return fail(CNS_ERR_INVALID, "box has no state (upload first)");
    if (b->batch) return fail(CNS_ERR_INVALID, "autotune the batch this box belongs to");
    if (trial_steps < 1) trial_steps = 1;
    CK(cudaSetDevice(b->dev));
    BoxScalars hs;
    int rc = save_state(b, &hs);
    if (rc) return rc;
    // mixed boxes: the three assemblies; FP64 boxes: the direct one only (their TMA assembly,
    // one block per SM, measured 23 % slower on GB300, is an explicit option)
    const int nkern = (b->desc.precision == CNS_MIXED && b->view.tma) ? 3 : 1;
    int best[3] = {b->view.tlog[0], b->view.tlog[1], b->view.tlog[2]}, best_k = b->kernel;
    // FP64 boxes keep their arithmetic: on the fixed-point TMA assembly (8x8x32 tiles, nothing to
    // tune but the derivative pass's shape) only the derivative pass's shapes are tried
    const bool keep_fx = b->kernel == CNS_ASSEMBLE_TMA_FX || b->kernel == CNS_ASSEMBLE_FX;
    // Two rounds over the candidates, each scored by its faster round: the shapes of a large box
    // differ by 1-3 %, about what one trial run varies by.
    const int ncand = nkern * kNumShapes;
    std::vector<double> score(ncand, 1e300);
    for (int round = 0; round < 2; round++) {
        for (int c = round ? 0 : -1; c < ncand; c++) {  // c = -1: a warm-up trial, not scored
            const int* t = kShapes[c < 0 ? 0 : c % kNumShapes];
            const int k = (c < 0 || keep_fx) ? b->kernel : c / kNumShapes;
            if ((rc = apply_tile(b, t)) || (rc = apply_kernel(b, k))) return rc;
            double ms = 0.0;
            // graph-replayed, as the box runs (the event-per-kernel path ranks the shapes
            // differently): one step to capture the graph and warm up, then the timed steps
            if ((rc = cns_box_advance(b, 1))) return rc;
            if ((rc = graph_ms(b->stream, [&] { return cns_box_advance(b, trial_steps); }, &ms))) return rc;
            if ((rc = restore_state(b, &hs))) return rc;
            if (c >= 0) score[c] = std::min(score[c], ms);
        }
    }
    double best_t = 1e300;
    for (int c = 0; c < ncand; c++) {
        if (score[c] < best_t) {
            best_t = score[c];
            best_k = keep_fx ? b->kernel : c / kNumShapes;
            for (int q = 0; q < 3; q++) best[q] = kShapes[c % kNumShapes][q];
        }
    }
    if ((rc = apply_tile(b, best)) || (rc = apply_kernel(b, best_k))) return rc;
    if ((rc = restore_state(b, &hs))) return rc;
    CK(cudaStreamSynchronize(b->stream));
    if (tlog_out)
        for (int q = 0; q < 3; q++) tlog_out[q] = best[q];
    if (kernel_out) *kernel_out = best_k;
    if (best_ms) *best_ms = best_t / trial_steps;
    return CNS_OK;
}

// Policy p = shape + (kNumShapes + 1) * kernel: shape 0 = every member on its least-padding
// shape, 1 + s = every member on kShapes[s]; kernel = the assembly kernel of the mixed members
// (0 direct, 1 TMA).
static int apply_policy(cns_batch* bt, int policy) {
    const int shape = policy % (kNumShapes + 1), kernel = policy / (kNumShapes + 1);
    for (auto* b : bt->members) {
        int t[3];
        if (shape == 0)
            default_tlog(b->desc.n, t);
        else
            for (int a = 0; a < 3; a++) t[a] = kShapes[shape - 1][a];
        int rc = apply_tile(b, t);
        if (rc) return rc;
        if (b->desc.precision == CNS_MIXED && b->view.tma && (rc = apply_kernel(b, kernel))) return rc;
    }
    return batch_rebuild(bt, false);
}

extern "C" int cns_batch_autotune(cns_batch* bt, int trial_steps, int* chosen_policy, double* best_ms) {
    if (!bt) return fail(CNS_ERR_INVALID, "null batch");
    if (bt->members.empty()) return CNS_OK;
    if (trial_steps < 1) trial_steps = 1;
    CK(cudaSetDevice(bt->dev));
    CK(cudaStreamSynchronize(bt->stream));
    std::vector<BoxScalars> saved(bt->members.size());
    int rc;
    for (size_t m = 0; m < bt->members.size(); m++)
        if ((rc = save_state(bt->members[m], &saved[m]))) return rc;
    auto restore_all = [&]() -> int {
        for (size_t m = 0; m < bt->members.size(); m++) {
            int r = restore_state(bt->members[m], &saved[m]);
            if (r) return r;
            CK(cudaStreamSynchronize(bt->members[m]->stream));
        }
        return CNS_OK;
    };
    bool any_tma = false;
    for (auto* b : bt->members) any_tma = any_tma || (b->desc.precision == CNS_MIXED && b->view.tma);
    const int npolicies = (kNumShapes + 1) * (any_tma ? 3 : 1);
    int best = 0;
    double best_t = 1e300;
    for (int policy = -1; policy < npolicies; policy++) {  // -1: warm-up with policy 0
        if ((rc = apply_policy(bt, policy < 0 ? 0 : policy))) return rc;
        double ms = 0.0;
        rc = timed_run(bt->stream, trial_steps, bt->d_views, bt->nviews, bt->lists, nullptr, nullptr, &ms);
        if (rc) return rc;
        if ((rc = restore_all())) return rc;
        if (policy >= 0 && ms < best_t) {
            best_t = ms;
            best = policy;
        }
    }
    if ((rc = apply_policy(bt, best))) return rc;
    if ((rc = restore_all())) return rc;
    if ((rc = batch_rebuild(bt, true))) return rc;
    if (chosen_policy) *chosen_policy = best;
    if (best_ms) *best_ms = best_t / trial_steps;
    return CNS_OK;
}
