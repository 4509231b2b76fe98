// cns_internal.h -- launchers shared between the kernel files and the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <vector>
#include "cns_common.cuh"

namespace cns {

// Launch a step kernel in plain stream order.  Programmatic dependent launch (each kernel
// waiting on the device for its predecessor, its successor launched early to take the SMs as
// they drain) was measured again with the current kernels: without it a graph-replayed 256^3
// step is 1-1.5 % faster in FP64, 3 % faster in the mixed form, and cns_new_advance 1 % faster.
template <class... Params, class... Args>
cudaError_t launch_step(void (*fn)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    return cudaLaunchKernelEx(&cfg, fn, args...);
}

// record the calling thread's last error (read back by cns_last_error); returns `code`
int set_error(int code, const char* msg);

// fused RK3 stage kernels (cns_fused.cu); precision / form 0 = FP64 stencils, 1 = FP32 stencils,
// 2 = FP64 boxes that keep a fixed-point copy of the P set (part of the stencils on the copy),
// 3 = the same with the Laplacians' merged sums (boxes with lap_merge; assembly only)
constexpr int kFormPlain = 0, kFormMixed = 1, kFormPlainFx = 2, kFormPlainFxMerge = 3;
cudaError_t launch_prim(int precision, const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st);
cudaError_t launch_deriv(int form, const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
cudaError_t launch_assemble(int form, const BoxView* boxes, const Tile* tiles, int ntiles, int stage,
                            cudaStream_t st);
cudaError_t launch_refs(const BoxView* boxes, int nboxes, cudaStream_t st);
// the plain form's fixed-point copy of an uploaded P set: its fields' maxima (convert = false),
// then the copy (convert = true); k_fx_pass
cudaError_t launch_fx_pass(bool convert, const BoxView* boxes, const Tile* tiles, int ntiles, cudaStream_t st);
// a box switched onto its fixed-point copies between steps: maxima of the conversion -> exponents
cudaError_t launch_fx_adopt(const BoxView* boxes, int nboxes, cudaStream_t st);
// the TMA-staged assembly of mixed boxes (cns_tma.cu)
void tma_tile_shape(int* ti, int* tj, int* tk);
size_t tma_maps_bytes();
cudaError_t tma_encode_maps(const BoxView& v, void* out);
cudaError_t bounded_wait_selftest(int* status);
cudaError_t exact_sums_selftest(const double* taps, int n, double* sums, int* ok);
cudaError_t launch_assemble_tma(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
cudaError_t launch_assemble_tma64(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
// FP64 boxes on their fixed-point copies, TMA-staged (k_assemble_fx)
cudaError_t launch_assemble_fx(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
// the mixed form's derivative pass on the same tiles, TMA-staged (same bits as launch_deriv)
cudaError_t launch_deriv_tma(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
// the warp-specialised TMA assembly (same tiles, same bits): stencils and FP64 write-back overlap
cudaError_t launch_assemble_ws(const BoxView* boxes, const Tile* tiles, int ntiles, int stage, cudaStream_t st);
bool assemble_ws_fits();  // its 512-thread, 160 KB block fits on the current device
cudaError_t launch_stepend(const BoxView* boxes, int nboxes, int flip, cudaStream_t st);

// operator-level kernels and layout conversions (cns_ops.cu)
cudaError_t op_aos_to_soa(const double* aos, double* soa, long long npts, int nc, cudaStream_t st);
cudaError_t op_soa_to_aos(const double* soa, double* aos, long long npts, int nc, cudaStream_t st);
cudaError_t op_ctoprim(const int lo[3], const int hi[3], int ng, const double* u, double* q, const double dx[3],
                       unsigned long long* courno_bits, cudaStream_t st);
cudaError_t op_hypterm(const int lo[3], const int hi[3], int ng, const double* cons, const double* q, double* flux,
                       const double dx[3], cudaStream_t st);
cudaError_t op_diffterm(const int lo[3], const int hi[3], int ng, const double* q, double* tmp9, double* difflux,
                        const double dx[3], double eta, double alam, cudaStream_t st);
cudaError_t op_fill_ghosts_aos(double* aos, const int n[3], int nc, cudaStream_t st);
cudaError_t op_aos_to_box(const double* aos, const BoxView& b, cudaStream_t st);
cudaError_t op_box_to_aos(const BoxView& b, double* aos, int ghosts, cudaStream_t st);
cudaError_t probe_fp64(double* tflops);

// the reference-layout host array <-> a box over the CPU-GPU link, in place (cns_host.cu).
// `h` is the device address of a host array the device can address (mapped_host_range).
void* mapped_host_range(const void* p, size_t bytes);
void set_pageable_in_place(int enable);
// ghosts: also write the host array's ghost cells (periodic images of its interior)
cudaError_t host_upload(const BoxView& v, double* h, bool prim, bool ghosts, cudaStream_t st);
cudaError_t host_download(const BoxView& v, double* h, cudaStream_t st);
cudaError_t host_ghosts(const BoxView& v, double* h, cudaStream_t st);
// the FP64 upload fused with stage 1's derivative pass (k_upload_deriv): its work queue for a
// tile list, and the launch; counters = n[0] + 1 ints of device memory
std::vector<int> upload_deriv_queue(const int n[3], const int tlog[3], const std::vector<Tile>& tiles);
cudaError_t host_upload_deriv(const BoxView& v, double* h, bool ghosts, const Tile* tiles, const int* queue, int nq,
                              int* counters, cudaStream_t st);
cudaError_t op_init_field(const BoxView& b, double ax, double ay, double az, double perturb, unsigned long long seed,
                          cudaStream_t st);

}  // namespace cns
