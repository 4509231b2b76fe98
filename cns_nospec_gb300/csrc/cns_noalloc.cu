// cns_noalloc.cu -- cns_diffterm_noalloc: diffterm on caller-owned device buffers, with its
// scratch in a fixed device array instead of memory allocated per call.
//
// Who needs it: callers that must not allocate device memory once they are running -- code
// whose device memory is owned by another allocator or a fixed budget set at start-up, and
// loops where the implicit synchronisation and latency of cudaMalloc/cudaFree are not
// acceptable.  They pass device pointers for q and difflux; the temporaries diffterm needs
// (cpu/diffterm.cpp:59-61 mallocs nine of them per call) come from the array below.
//
// The array is a file-scope __device__ variable: it exists on every GPU on which this
// library's device code is loaded and stays there until the process exits.  Host code may
// not use its name as a device address (it is a host-side stand-in), so the first call on a
// device looks up the real address with cudaGetSymbolAddress, with that device current, and
// keeps it.  Do that first call before any stream capture.
#include <mutex>

#include "../../include/cns_gb300.h"
#include "cns_common.cuh"
#include "cns_internal.h"

namespace {

// Largest box: 64,000 ghost-inclusive points (e.g. 32^3 interior cells with 4 ghosts a side).
constexpr long long kMaxPoints = CNS_NOALLOC_MAX_POINTS;
// SoA copy of q (6 fields), the nine first derivatives, the interior SoA difflux (5 fields).
constexpr long long kScratchDoubles = kMaxPoints * (6 + 9 + 5);

__device__ __align__(256) double g_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

int scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cns::set_error(CNS_ERR_NODEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return cns::set_error(CNS_ERR_CAPACITY, "device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return cns::set_error(CNS_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return CNS_OK;
}

}  // namespace

extern "C" int cns_diffterm_noalloc(const int lo[3], const int hi[3], int ng, const double dx[3], const double* q_dev,
                                    double* difflux_dev, double eta, double alam, void* stream) {
    if (!lo || !hi || !dx || !q_dev || !difflux_dev) return cns::set_error(CNS_ERR_INVALID, "null argument");
    if (ng < CNS_NG) return cns::set_error(CNS_ERR_INVALID, "the 8th-order stencils need ng >= 4");
    long long np = 1, ni = 1;
    for (int a = 0; a < 3; a++) {
        if (hi[a] < lo[a]) return cns::set_error(CNS_ERR_INVALID, "hi < lo");
        np *= (long long)(hi[a] - lo[a] + 1 + 2 * ng);
        ni *= (long long)(hi[a] - lo[a] + 1);
    }
    if (np > kMaxPoints)
        return cns::set_error(CNS_ERR_CAPACITY,
                              "cns_diffterm_noalloc: box has more than CNS_NOALLOC_MAX_POINTS (64000) "
                              "ghost-inclusive points; use cns_diffterm");
    double* s = nullptr;
    int rc = scratch_address(&s);
    if (rc) return rc;
    // every scratch element read below is first written by this call, so nothing needs clearing
    double* s_q = s;             // 6 * np
    double* tmp = s + 6 * np;    // 9 * np
    double* s_d = tmp + 9 * np;  // 5 * ni
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cns::op_aos_to_soa(q_dev, s_q, np, 6, st);
    if (e == cudaSuccess) e = cns::op_diffterm(lo, hi, ng, s_q, tmp, s_d, dx, eta, alam, st);
    if (e == cudaSuccess) e = cns::op_soa_to_aos(s_d, difflux_dev, ni, 5, st);
    if (e != cudaSuccess) return cns::set_error(CNS_ERR_CUDA, cudaGetErrorString(e));
    return CNS_OK;
}
