/*
 * cns_gb300.h -- C ABI of the GB300-native CNS_NoSpec RK3 advance (libcns_gb300.so).
 *
 * The library replaces the reference's cpu/ hot path: new_advance and the operators it calls
 * (cpu/advance.cpp:13-154, cpu/ctoprim.cpp:11-105, cpu/hypterm.cpp:11-209,
 * cpu/diffterm.cpp:22-320, cpu/helper_functions.cpp:226-262).  Every entry point is plain C:
 * pointers and sizes, no C++ or torch types.  All return an int status (cns_status); on
 * failure cns_last_error() describes the cause.  Nothing here calls exit().
 *
 * Array layout at this boundary is the reference's host layout (allocate_4D,
 * cpu/helper_functions.cpp:100-122): one contiguous block of doubles indexed
 * [i][j][k][l], component l fastest, then k, then j, then i; i pairs with dx[0].
 * Ghost-inclusive arrays (U, Q) have n+2*ng cells per axis; D/F are interior-only.
 * A caller holding the reference's double**** trees passes &X[0][0][0][0].
 *
 * Threading: calls on different cns_box / cns_batch handles may run concurrently from
 * different host threads; one handle must not be used by two threads at once.  The
 * operator-level calls (cns_ctoprim, ...) share a per-thread device workspace.
 */
#ifndef CNS_GB300_H
#define CNS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define CNS_NG 4 /* ghost cells per side, cpu/header.h:16 */
#define CNS_NC 5 /* conserved components, cpu/header.h:15 */

typedef enum cns_status {
    CNS_OK = 0,
    CNS_ERR_INVALID = 1,   /* bad argument (sizes, ng, null pointer, ...) */
    CNS_ERR_NOMEM = 2,     /* device or host allocation failed */
    CNS_ERR_NONFINITE = 3, /* the state developed rho <= 0, e <= 0 or a non-finite value */
    CNS_ERR_CUDA = 4,      /* a CUDA runtime call failed */
    CNS_ERR_CAPACITY = 5,  /* a size above a documented maximum */
    CNS_ERR_NODEVICE = 6   /* no CUDA device */
} cns_status;

/* Health bits of a box (sticky; cns_box_sync): what made it return CNS_ERR_NONFINITE. */
typedef enum cns_health {
    CNS_HEALTH_NONPOS_RHO = 1,  /* density <= 0 somewhere */
    CNS_HEALTH_NONFINITE = 2,   /* a non-finite density or internal energy */
    CNS_HEALTH_NONPOS_EINT = 4, /* internal energy <= 0 somewhere */
    CNS_HEALTH_TIMEOUT = 8      /* a bounded wait inside a kernel gave up; that launch returned early */
} cns_health;

typedef enum cns_precision {
    CNS_FP64 = 0, /* plain form: FP64 state and arithmetic; part of the stencil sums exact in integers, rounded once to FP64 */
    CNS_MIXED = 1 /* FP32 primitives/stencils/fluxes; FP64 e = E/rho - |u|^2/2 and RK3 state */
} cns_precision;

/* Layout-compatible with the reference's parameter struct global_const_t
 * (cpu/header.h:47-86), so a caller can pass &h_const directly.  Only ng, nc, dim, dx, cfl,
 * eta and alam are read; MAX_TEMP is 27 (cpu/header.h:36-45). */
typedef struct cns_global_const {
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
} cns_global_const_t;

/* ---- library --------------------------------------------------------------------------- */
const char *cns_last_error(void);          /* message of this thread's last failure */
int cns_version(void);                     /* 100 * major + minor */
int cns_set_device(int device);            /* select the CUDA device for this host thread */
int cns_device_synchronize(void);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (a ~0.1 s probe kernel):
 * the roofline denominator of the FP64-bound stencil kernels. */
int cns_measure_fp64_peak(double *tflops);
/* Self-test of the bounded waits inside the library's kernels: one block waits on an
 * mbarrier that nothing arrives on; the wait gives up after about one second and the block
 * reports *status = CNS_HEALTH_TIMEOUT (8) instead of hanging.  No counterpart in the
 * reference. */
int cns_selftest_bounded_wait(int *status);
/* Self-test of the exact 8-tap stencil sums of the plain form as the device computes them:
 * for n sets of taps (taps[8q..8q+7] = f[+1..+4], f[-1..-4]) writes the sums with the
 * first-derivative weights (672, -168, 32, -3) to sums[2q] and with the second-derivative
 * weights (8064, -1008, 128, -9) to sums[2q+1], and ok[2q], ok[2q+1] = 0 where a sum takes the
 * FP64 fallback.  Host arrays; n <= 2^24.  No counterpart in the reference. */
int cns_selftest_exact_sums(const double *taps, int n, double *sums, int *ok);

/* ---- operator level: the reference's per-operator surface, host arrays ---------------- */

/* cpu/ctoprim.cpp:11-70 and 72-105 (header.h:99-115).  q over the ghost-inclusive box from u;
 * when courno != NULL, *courno = max(*courno, max over interior of (c+|u_d|)/dx_d), exactly
 * as the reference's courno argument.  lo/hi are ghost-offset interior bounds (lo = ng). */
int cns_ctoprim(const int lo[3], const int hi[3], const double *u, double *q, const double dx[3], int ng,
                double *courno);

/* cpu/hypterm.cpp:11-209 (header.h:118-126).  flux is interior-indexed [n0][n1][n2][5]. */
int cns_hypterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double *cons,
                const double *q, double *flux);

/* cpu/diffterm.cpp:22-320 (header.h:129-138).  difflux is interior-indexed [n0][n1][n2][5]. */
int cns_diffterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double *q,
                 double *difflux, double eta, double alam);

/* No counterpart in the reference (its diffterm mallocs nine temporaries per call,
 * cpu/diffterm.cpp:59-61).  diffterm for callers that cannot allocate device memory while
 * they run (memory owned by another allocator or a fixed budget, or loops that cannot take
 * cudaMalloc's synchronisation): q_dev ([g0][g1][g2][6]) and difflux_dev ([n0][n1][n2][5]) are
 * caller-owned DEVICE buffers in the reference layout; the temporaries live in one fixed
 * device array of CNS_NOALLOC_MAX_POINTS * 20 doubles (10.24 MB), present on every GPU that
 * loads the library until the process exits.  No cudaMalloc/cudaFree or other allocating call
 * is made.  Boxes above CNS_NOALLOC_MAX_POINTS ghost-inclusive points return
 * CNS_ERR_CAPACITY.  Asynchronous on `stream` (NULL = default stream).  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress): make it before any
 * stream capture.  All calls share the array, which keeps the last call's contents (every
 * element a call reads it first writes); calls that overlap on the GPU race. */
#define CNS_NOALLOC_MAX_POINTS 64000
int cns_diffterm_noalloc(const int lo[3], const int hi[3], int ng, const double dx[3], const double *q_dev,
                         double *difflux_dev, double eta, double alam, void *stream);

/* cpu/helper_functions.cpp:226-262 (helper_functions.h:172-176): periodic ghost fill of a
 * ghost-inclusive [dim+8]^3 x 5 block, in place. */
int cns_fill_boundary(double *U, const int dim[3], const int dim_ng[3]);

/* cpu/advance.cpp:13-154 (header.h:149-156): one RK3 step of U in place, dt out.
 * Parameters come from *h (the reference's h_const).  Per-axis dims are honoured (the
 * reference handles cubic boxes only).  As in the reference, U's ghost cells come back
 * holding the periodic fill made at the start of the step.  Unew, Q, D and F are accepted
 * for signature compatibility and are not touched (the device keeps its own state); they
 * may be NULL.  Each call copies U in and out; cns_box_* keeps the state resident. */
int cns_new_advance(const cns_global_const_t *h, double *U, double *Unew, double *Q, double *D, double *F,
                    double *dt);

/* nsteps RK3 steps of a host U (ghost-inclusive [n+8]^3 x 5) with one copy in and one out.
 * dt_hist (nullable) receives each step's dt.  precision: cns_precision. */
int cns_advance_host(double *U, const int n[3], const double dx[3], double cfl, double eta, double alam,
                     int nsteps, int precision, double *dt_hist);
/* cns_advance_host with precision CNS_FP64 / CNS_MIXED. */
int cns_advance_f64(double *U, const int n[3], const double dx[3], double cfl, double eta, double alam, int nsteps,
                    double *dt_hist);
int cns_advance_mixed(double *U, const int n[3], const double dx[3], double cfl, double eta, double alam, int nsteps,
                      double *dt_hist);

/* Host arrays: cns_new_advance, cns_advance_host, cns_box_upload and cns_box_download read and
 * write the caller's array in place from the GPU over the CPU-GPU link (interior only on the
 * way in; no staging copy) when
 *  - all of [U, U + bytes) lies in one page-locked allocation the device can address
 *    (cudaHostAlloc, cudaHostRegister, a pinned torch tensor), or
 *  - U is ordinary pageable memory (malloc, as the reference's allocate_4D uses) and the device
 *    reads host memory through the host's page tables (NVLink-C2C, as on Grace-Blackwell); the
 *    array must then hold the [n0+8][n1+8][n2+8][5] doubles its dimensions give, as it must for
 *    the reference's own loops.
 * Any other host memory is staged through a device buffer.  Results are bit-identical either way.
 * *in_place = 1 when `U` takes the in-place path.  No counterpart in the reference. */
int cns_host_in_place(const void *U, long long bytes, int *in_place);
/* enable = 0: pageable host arrays take the staged path even where the device could use them in
 * place (page-locked arrays are unaffected); 1 (the default): in place where the device can.
 * Process-wide.  No counterpart in the reference. */
int cns_set_pageable_in_place(int enable);

/* ---- device-resident boxes ------------------------------------------------------------- */
typedef struct cns_box cns_box;

typedef struct cns_box_desc {
    int n[3];       /* interior cells per axis, each >= 4 */
    double dx[3];   /* cell sizes */
    double cfl, eta, alam;
    int precision;  /* cns_precision */
} cns_box_desc;

/* bytes of device memory one box of this description holds */
long long cns_box_bytes(const cns_box_desc *desc);
int cns_box_create(const cns_box_desc *desc, cns_box **out);
int cns_box_destroy(cns_box *box);
/* Run the box's work on `stream` (a cudaStream_t; NULL = the box's own stream). */
int cns_box_set_stream(cns_box *box, void *stream);
/* Copy a host ghost-inclusive AoS state in (ghost cells are ignored) / out (ghost cells get
 * the periodic images of the interior).  Both block until the copy is done. */
int cns_box_upload(cns_box *box, const double *U_host);
int cns_box_download(cns_box *box, double *U_host);
/* Same, from/to a device AoS buffer, asynchronously on the box's stream. */
int cns_box_upload_device(cns_box *box, const double *U_dev);
int cns_box_download_device(cns_box *box, double *U_dev);
/* nsteps RK3 steps, asynchronous on the box's stream (replays a captured one-step graph). */
int cns_box_advance(cns_box *box, int nsteps);
/* cns_box_advance bracketed by two CUDA events on the box's stream: waits for the steps and
 * returns their device time in *ms (no counterpart in the reference; for benchmarks). */
int cns_box_advance_ms(cns_box *box, int nsteps, double *ms);
/* Same, without graphs, with a CUDA event around every kernel launch; fills
 * kernel_ms[CNS_KERN_COUNT] (summed device ms per kernel kind), kernel_launches[...] and
 * *total_ms (first to last event).  Blocks until done. */
enum { CNS_KERN_DERIV = 0, CNS_KERN_ASSEMBLE = 1, CNS_KERN_STEPEND = 2, CNS_KERN_PRIM = 3, CNS_KERN_COUNT = 4 };
int cns_box_advance_timed(cns_box *box, int nsteps, double *kernel_ms, int *kernel_launches, double *total_ms);
/* Blocks until the box's queued work is done; returns CNS_ERR_NONFINITE if the state
 * went bad (then *health_bits, if given, says how). */
int cns_box_sync(cns_box *box, int *health_bits);
int cns_box_last_dt(cns_box *box, double *dt, int *nsteps_done);
/* Kernel launches one cns_box_advance step issues (for launch accounting). */
int cns_box_launches_per_step(const cns_box *box);

/* Write the CNS_NoSpec initial field straight into the box (no host array): velocity
 * amplitudes scaled by amp[3], rho/u/v/w times (1 + perturb * U(-1, 1)) from the seeded
 * SplitMix64 stream of cns_nospec_gb300/initdata.py; then primes the box like an upload. */
int cns_box_init_field(cns_box *box, const double amp[3], double perturb, unsigned long long seed);
/* Checkpoint / resume: a binary snapshot (header + ghost-inclusive AoS state + the box's
 * step count and mixed-form reference values).  Loading into a box of the same description
 * resumes the run bit for bit.  Both block. */
int cns_box_save(cns_box *box, const char *path);
int cns_box_load(cns_box *box, const char *path);

/* ---- the reference's text formats (host only) ------------------------------------------ */
/* general_input: "ng nc ncells lo[3] hi[3] dx[3] cfl eta alam nsteps dt", derived fields as in
 * read_configurations (cpu/helper_functions.cpp:38-83). */
int cns_read_general_input(const char *path, cns_global_const_t *h);
int cns_write_general_input(const char *path, const cns_global_const_t *h);
/* ncomp components as read_3D reads them (cpu/helper_functions.cpp:166-175), i fastest, into
 * / from an [d0][d1][d2][ncomp] block (the multistep_input format, cpu/main.cpp:22-25). */
int cns_read_3d(const char *path, double *a, const int dims[3], int ncomp);
int cns_write_3d(const char *path, const double *a, const int dims[3], int ncomp);
/* print_4D dumps (cpu/helper_functions.cpp:85-98), "%.17e\t" per value; with_header adds the
 * two header lines cpu/main.cpp:36-40 writes before it (ncomp; the three dims). */
int cns_print_4d(const char *path, const double *a, const int dims[3], int ncomp, int with_header);
int cns_read_4d(const char *path, double *a, const int dims[3], int ncomp, int with_header);

/* ---- batches: many boxes advanced together, one launch per kernel and stage ------------ */
typedef struct cns_batch cns_batch;
int cns_batch_create(cns_batch **out);
int cns_batch_destroy(cns_batch *batch);
int cns_batch_set_stream(cns_batch *batch, void *stream);
int cns_batch_add(cns_batch *batch, cns_box *box);
int cns_batch_remove(cns_batch *batch, cns_box *box);
int cns_batch_size(const cns_batch *batch);
/* nsteps RK3 steps of every member (each with its own dt), replaying a captured graph of
 * one step (rebuilt when membership changes).  Asynchronous. */
int cns_batch_advance(cns_batch *batch, int nsteps);
int cns_batch_sync(cns_batch *batch);
/* cns_batch_advance bracketed by two CUDA events on the batch's stream: waits for the steps
 * and returns their device time in *ms (no counterpart in the reference; for benchmarks). */
int cns_batch_advance_ms(cns_batch *batch, int nsteps, double *ms);

/* ---- tile shapes and the autotuner -------------------------------------------------------
 * Work is cut into tiles of 256 cells (one per thread, k fastest across a warp); a box's tile
 * shape is tlog[3] = log2 of the tile's (i, j, k) extents, summing to 8 with tlog[2] >= 3, or
 * {-1, 0, 0}: linear tiles of 256 consecutive cells in the box's own order (no padding for any
 * box shape).
 * The shape changes only speed, never results: every cell's arithmetic is the same.
 * A new box starts on the candidate shape that pads it least. */
int cns_box_get_tile(const cns_box *box, int tlog[3]);
int cns_box_set_tile(cns_box *box, const int tlog[3]);
/* Assembly kernel of a box: CNS_ASSEMBLE_DIRECT (one cell per thread, stencil taps loaded
 * through L1), CNS_ASSEMBLE_TMA (8x8x32-cell tiles whose 20 stencil fields are staged in shared
 * memory by TMA tensor copies; for FP64 boxes with FP64 tensor maps and one block per SM),
 * CNS_ASSEMBLE_TMA_WS (mixed boxes only: the TMA kernel with one 512-thread block per SM split
 * into a stencil warp group and an FP64 write-back warp group working on consecutive tiles) or
 * CNS_ASSEMBLE_TMA_FX (FP64 boxes only: the TMA tiles with the stencil fields staged as 62-bit
 * fixed-point copies that the box keeps beside its FP64 fields, one exponent per field set from
 * the fields' largest magnitudes; each Laplacian and flux-divergence stencil an exact integer sum
 * rounded once and one FP64 operation; within ~2e-15 of the direct kernel, not bit-identical) or
 * CNS_ASSEMBLE_FX (FP64 boxes only: the direct kernels, with the stencils that the FP64 form sums
 * exactly on the integer pipes reading the same fixed-point copies instead of placing each FP64
 * tap's significand; within ~2e-15 of the direct kernel, not bit-identical).
 * DIRECT, TMA and TMA_WS give identical bits.  A new mixed box starts on a TMA kernel when the
 * driver provides the tensor-map encoder; a new FP64 box on CNS_ASSEMBLE_FX, the fastest for FP64
 * on GB300 (the FP64 pipe, not the loads, sets the time of the FP64 kernels; the copies take
 * 64 bytes a cell in the box's memory).  The autotuner keeps an FP64 box's kernel. */
enum { CNS_ASSEMBLE_DIRECT = 0, CNS_ASSEMBLE_TMA = 1, CNS_ASSEMBLE_TMA_WS = 2, CNS_ASSEMBLE_TMA_FX = 3,
       CNS_ASSEMBLE_FX = 4 };
int cns_box_get_kernel(const cns_box *box, int *kernel);
int cns_box_set_kernel(cns_box *box, int kernel);
/* Time trial_steps RK3 steps of the box on every candidate shape (the 12 rectangular ones and
 * the linear one; for mixed boxes, with each of the three assembly kernels), twice, and keep the
 * candidate whose faster run is the fastest; the box's state is restored afterwards, so the run
 * continues bit for bit.  Blocks. */
int cns_box_autotune(cns_box *box, int trial_steps, int tlog_out[3], int *kernel_out, double *best_ms_per_step);
/* Same for a batch.  Policy p = shape + 14 * kernel: shape 0 = every member on its
 * least-padding rectangular shape, 1 + s = every member on candidate shape s (s = 12: linear);
 * kernel = the assembly kernel of its mixed members.  The fastest policy is kept and the graph re-captured. */
int cns_batch_autotune(cns_batch *batch, int trial_steps, int *chosen_policy, double *best_ms_per_step);

#ifdef __cplusplus
}
#endif
#endif /* CNS_GB300_H */
