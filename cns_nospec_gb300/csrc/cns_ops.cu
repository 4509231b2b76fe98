// cns_ops.cu -- operator-level kernels behind the reference's per-operator call surface
// (ctoprim, hypterm, diffterm, fill_boundary; cpu/header.h:98-139,
// cpu/helper_functions.h:172-176), and the layout conversions between the reference's host
// layout (AoS [i][j][k][l], cpu/helper_functions.cpp:100-122) and the device layouts.
//
// These kernels take whatever the caller put in the ghost cells (no periodicity is assumed),
// exactly as the reference operators do, so they can be checked one operator at a time.
// They work on an unpadded structure-of-arrays copy: elem(f, i, j, k) = f*np + (i*g1+j)*g2+k.
#include "cns_common.cuh"
#include "cns_internal.h"

namespace cns {

struct OpDims {
    int g[3];     // ghost-inclusive dims
    int lo[3];    // first interior index (ghost-inclusive numbering)
    int n[3];     // interior dims
    long long np; // g0*g1*g2
};

__device__ __forceinline__ long long op_idx(const OpDims& d, int i, int j, int k) {
    return ((long long)i * d.g[1] + j) * d.g[2] + k;
}

// AoS (component fastest) <-> unpadded SoA
__global__ void k_aos_to_soa(const double* __restrict__ aos, double* __restrict__ soa, long long npts, int nc) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x)
        for (int l = 0; l < nc; l++) soa[l * npts + p] = aos[p * nc + l];
}
__global__ void k_soa_to_aos(const double* __restrict__ soa, double* __restrict__ aos, long long npts, int nc) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x)
        for (int l = 0; l < nc; l++) aos[p * nc + l] = soa[l * npts + p];
}

// cpu/ctoprim.cpp:11-70.  q over the whole ghost-inclusive box; Courant over the interior.
__global__ void k_op_ctoprim(const double* __restrict__ u, double* __restrict__ q, OpDims d, double dx0, double dx1,
                             double dx2, unsigned long long* courno_bits) {
    const long long np = d.np;
    unsigned long long best = 0ull;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
        const double rho = u[p];
        const double rhoinv = 1.0 / rho;
        const double q1 = u[np + p] * rhoinv, q2 = u[2 * np + p] * rhoinv, q3 = u[3 * np + p] * rhoinv;
        const double eint = u[4 * np + p] * rhoinv - 0.5 * (q1 * q1 + q2 * q2 + q3 * q3);
        const double pr = (kGm1 * eint) * rho;
        q[p] = rho;
        q[np + p] = q1;
        q[2 * np + p] = q2;
        q[3 * np + p] = q3;
        q[4 * np + p] = pr;
        q[5 * np + p] = eint / kCv;
        if (courno_bits) {
            const int k = (int)(p % d.g[2]);
            const int j = (int)((p / d.g[2]) % d.g[1]);
            const int i = (int)(p / ((long long)d.g[2] * d.g[1]));
            if (i >= d.lo[0] && i < d.lo[0] + d.n[0] && j >= d.lo[1] && j < d.lo[1] + d.n[1] && k >= d.lo[2] &&
                k < d.lo[2] + d.n[2]) {
                const double c = sqrt(kGamma * pr / rho);
                const double cx = (c + fabs(q1)) / dx0, cy = (c + fabs(q2)) / dx1, cz = (c + fabs(q3)) / dx2;
                const double m = fmax(fmax(cx, cy), cz);
                const unsigned long long mb = dbits(m);
                if (!(mb >> 63) && mb > best) best = mb;
            }
        }
    }
    if (courno_bits) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long w = __shfl_xor_sync(0xffffffffu, best, o);
            best = (w > best) ? w : best;
        }
        if ((threadIdx.x & 31) == 0 && best) atomicMax(courno_bits, best);
    }
}

// cpu/hypterm.cpp:11-209.  One interior cell per thread; the three passes of the reference
// become three sums subtracted from zero.  flux is interior-indexed SoA (n0*n1*n2 per field).
__global__ void k_op_hypterm(const double* __restrict__ cons, const double* __restrict__ q, double* __restrict__ flux,
                             OpDims d, double dxi0, double dxi1, double dxi2) {
    const long long nint = (long long)d.n[0] * d.n[1] * d.n[2], np = d.np;
    const double A[4] = {kAlp, kBet, kGam, kDel};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nint; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % d.n[2]);
        const int j = (int)((p / d.n[2]) % d.n[1]);
        const int i = (int)(p / ((long long)d.n[2] * d.n[1]));
        const long long c = op_idx(d, i + d.lo[0], j + d.lo[1], k + d.lo[2]);
        const long long st[3] = {(long long)d.g[1] * d.g[2], d.g[2], 1};
        const double dxi[3] = {dxi0, dxi1, dxi2};
        double out[5] = {0, 0, 0, 0, 0};
        for (int ax = 0; ax < 3; ax++) {
            const long long s = st[ax];
            const int mc = 1 + ax;  // momentum component along the pass; q index of its velocity
            double v[5] = {0, 0, 0, 0, 0};
            for (int m = 1; m <= 4; m++) {
                const long long cp = c + m * s, cm = c - m * s;
                const double unp = q[mc * np + cp], unm = q[mc * np + cm];
                const double pp = q[4 * np + cp], pm = q[4 * np + cm];
                v[0] += A[m - 1] * (cons[mc * np + cp] - cons[mc * np + cm]);
                for (int l = 1; l <= 3; l++) {
                    double t = cons[l * np + cp] * unp - cons[l * np + cm] * unm;
                    if (l == mc) t += pp - pm;
                    v[l] += A[m - 1] * t;
                }
                v[4] += A[m - 1] * (cons[4 * np + cp] * unp - cons[4 * np + cm] * unm + (pp * unp - pm * unm));
            }
            for (int l = 0; l < 5; l++) out[l] -= v[l] * dxi[ax];
        }
        for (int l = 0; l < 5; l++) flux[l * nint + p] = out[l];
    }
}

// cpu/diffterm.cpp:73-151.  The nine first derivatives of (u,v,w) on their extended ranges:
// the derivative along axis a covers the interior along a and every ghost-inclusive position
// along the other two axes.  tmp holds 9 fields of np: (ux,vx,wx, uy,vy,wy, uz,vz,wz).
__global__ void k_op_diffterm_d1(const double* __restrict__ q, double* __restrict__ tmp, OpDims d, double dxi0,
                                 double dxi1, double dxi2) {
    const long long np = d.np;
    const double A[4] = {kAlp, kBet, kGam, kDel};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % d.g[2]);
        const int j = (int)((p / d.g[2]) % d.g[1]);
        const int i = (int)(p / ((long long)d.g[2] * d.g[1]));
        const int pos[3] = {i, j, k};
        const long long st[3] = {(long long)d.g[1] * d.g[2], d.g[2], 1};
        const double dxi[3] = {dxi0, dxi1, dxi2};
        for (int ax = 0; ax < 3; ax++) {
            if (pos[ax] < d.lo[ax] || pos[ax] >= d.lo[ax] + d.n[ax]) continue;
            for (int comp = 1; comp <= 3; comp++) {
                double s = 0.0;
                for (int m = 1; m <= 4; m++) s += A[m - 1] * (q[comp * np + p + m * st[ax]] - q[comp * np + p - m * st[ax]]);
                tmp[(ax * 3 + comp - 1) * np + p] = s * dxi[ax];
            }
        }
    }
}

// cpu/diffterm.cpp:154-315.  One interior cell per thread; difflux interior-indexed SoA.
__global__ void k_op_diffterm(const double* __restrict__ q, const double* __restrict__ tmp,
                              double* __restrict__ difflux, OpDims d, double dxi0, double dxi1, double dxi2,
                              double eta, double alam) {
    const long long nint = (long long)d.n[0] * d.n[1] * d.n[2], np = d.np;
    const double A[4] = {kAlp, kBet, kGam, kDel};
    const double B[4] = {kOff1, kOff2, kOff3, kOff4};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nint; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % d.n[2]);
        const int j = (int)((p / d.n[2]) % d.n[1]);
        const int i = (int)(p / ((long long)d.n[2] * d.n[1]));
        const long long c = op_idx(d, i + d.lo[0], j + d.lo[1], k + d.lo[2]);
        const long long st[3] = {(long long)d.g[1] * d.g[2], d.g[2], 1};
        const double dxi[3] = {dxi0, dxi1, dxi2};
        // second differences of q component comp along axis ax
        auto d2 = [&](int comp, int ax) {
            double s = kCenter * q[comp * np + c];
            for (int m = 1; m <= 4; m++) s += B[m - 1] * (q[comp * np + c + m * st[ax]] + q[comp * np + c - m * st[ax]]);
            return s * (dxi[ax] * dxi[ax]);
        };
        // first difference along ax of derivative field t (index into tmp)
        auto dd = [&](int t, int ax) {
            double s = 0.0;
            for (int m = 1; m <= 4; m++) s += A[m - 1] * (tmp[t * np + c + m * st[ax]] - tmp[t * np + c - m * st[ax]]);
            return s * dxi[ax];
        };
        enum { UX = 0, VX, WX, UY, VY, WY, UZ, VZ, WZ };
        const double fx = eta * ((4.0 / 3.0) * d2(1, 0) + d2(1, 1) + d2(1, 2) + (1.0 / 3.0) * (dd(VY, 0) + dd(WZ, 0)));
        const double fy = eta * (d2(2, 0) + (4.0 / 3.0) * d2(2, 1) + d2(2, 2) + (1.0 / 3.0) * (dd(UX, 1) + dd(WZ, 1)));
        const double fz = eta * (d2(3, 0) + d2(3, 1) + (4.0 / 3.0) * d2(3, 2) + (1.0 / 3.0) * (dd(UX, 2) + dd(VY, 2)));
        const double ux = tmp[UX * np + c], vy = tmp[VY * np + c], wz = tmp[WZ * np + c];
        const double divu = (2.0 / 3.0) * (ux + vy + wz);
        const double tauxx = 2.0 * ux - divu, tauyy = 2.0 * vy - divu, tauzz = 2.0 * wz - divu;
        const double tauxy = tmp[UY * np + c] + tmp[VX * np + c];
        const double tauxz = tmp[UZ * np + c] + tmp[WX * np + c];
        const double tauyz = tmp[VZ * np + c] + tmp[WY * np + c];
        double mech = tauxx * ux + tauyy * vy + tauzz * wz + tauxy * tauxy + tauxz * tauxz + tauyz * tauyz;
        mech = eta * mech + fx * q[np + c] + fy * q[2 * np + c] + fz * q[3 * np + c];
        difflux[p] = 0.0;
        difflux[nint + p] = fx;
        difflux[2 * nint + p] = fy;
        difflux[3 * nint + p] = fz;
        difflux[4 * nint + p] = alam * (d2(5, 0) + d2(5, 1) + d2(5, 2)) + mech;
    }
}

// cpu/helper_functions.cpp:226-262 on a ghost-inclusive AoS block: every ghost cell receives
// its periodic interior image.  The reference's z, y, x pass order yields exactly this for
// every ghost cell, edges and corners included, when each interior dim is >= NG.
__global__ void k_fill_ghosts_aos(double* __restrict__ aos, int n0, int n1, int n2, int nc) {
    const int g1 = n1 + 2 * CNS_NG, g2 = n2 + 2 * CNS_NG;
    const long long np = (long long)(n0 + 2 * CNS_NG) * g1 * g2;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % g2);
        const int j = (int)((p / g2) % g1);
        const int i = (int)(p / ((long long)g2 * g1));
        const int ii = (i - CNS_NG + n0) % n0 + CNS_NG, jj = (j - CNS_NG + n1) % n1 + CNS_NG,
                  kk = (k - CNS_NG + n2) % n2 + CNS_NG;
        if (ii == i && jj == j && kk == k) continue;
        const long long s = ((long long)ii * g1 + jj) * g2 + kk;
        for (int l = 0; l < nc; l++) aos[p * nc + l] = aos[s * nc + l];
    }
}

// host AoS (ghost-inclusive, 5 comps) -> box U interior
__global__ void k_aos_to_box(const double* __restrict__ aos, BoxView b) {
    const int g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    const long long nint = (long long)b.n[0] * b.n[1] * b.n[2];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nint; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % b.n[2]);
        const int j = (int)((p / b.n[2]) % b.n[1]);
        const int i = (int)(p / ((long long)b.n[2] * b.n[1]));
        const long long a = (((long long)(i + CNS_NG) * g1 + (j + CNS_NG)) * g2 + (k + CNS_NG)) * CNS_NC;
        const long long c = cell_off(b, i, j, k);
        for (int l = 0; l < CNS_NC; l++) b.U[c + l * b.fs] = aos[a + l];
    }
}

// box U -> host AoS.  ghosts: 1 = also write every ghost cell with its periodic image.
__global__ void k_box_to_aos(BoxView b, double* __restrict__ aos, int ghosts) {
    const int g0 = b.n[0] + 2 * CNS_NG, g1 = b.n[1] + 2 * CNS_NG, g2 = b.n[2] + 2 * CNS_NG;
    const long long np = (long long)g0 * g1 * g2;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % g2);
        const int j = (int)((p / g2) % g1);
        const int i = (int)(p / ((long long)g2 * g1));
        const int ii = (i - CNS_NG + b.n[0]) % b.n[0], jj = (j - CNS_NG + b.n[1]) % b.n[1],
                  kk = (k - CNS_NG + b.n[2]) % b.n[2];
        const bool inner = (ii + CNS_NG == i) && (jj + CNS_NG == j) && (kk + CNS_NG == k);
        if (!inner && !ghosts) continue;
        const long long c = cell_off(b, ii, jj, kk);
        for (int l = 0; l < CNS_NC; l++) aos[p * CNS_NC + l] = b.U[c + l * b.fs];
    }
}

// ---- host launchers ----------------------------------------------------------------------
static int blocks_for(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

static OpDims make_dims(const int lo[3], const int hi[3], int ng) {
    OpDims d;
    for (int a = 0; a < 3; a++) {
        d.n[a] = hi[a] - lo[a] + 1;
        d.g[a] = d.n[a] + 2 * ng;
        d.lo[a] = ng;
    }
    d.np = (long long)d.g[0] * d.g[1] * d.g[2];
    return d;
}

cudaError_t op_aos_to_soa(const double* aos, double* soa, long long npts, int nc, cudaStream_t st) {
    k_aos_to_soa<<<blocks_for(npts), 256, 0, st>>>(aos, soa, npts, nc);
    return cudaGetLastError();
}
cudaError_t op_soa_to_aos(const double* soa, double* aos, long long npts, int nc, cudaStream_t st) {
    k_soa_to_aos<<<blocks_for(npts), 256, 0, st>>>(soa, aos, npts, nc);
    return cudaGetLastError();
}
cudaError_t op_ctoprim(const int lo[3], const int hi[3], int ng, const double* u, double* q, const double dx[3],
                       unsigned long long* courno_bits, cudaStream_t st) {
    OpDims d = make_dims(lo, hi, ng);
    k_op_ctoprim<<<blocks_for(d.np), 256, 0, st>>>(u, q, d, dx[0], dx[1], dx[2], courno_bits);
    return cudaGetLastError();
}
cudaError_t op_hypterm(const int lo[3], const int hi[3], int ng, const double* cons, const double* q, double* flux,
                       const double dx[3], cudaStream_t st) {
    OpDims d = make_dims(lo, hi, ng);
    long long nint = (long long)d.n[0] * d.n[1] * d.n[2];
    k_op_hypterm<<<blocks_for(nint), 256, 0, st>>>(cons, q, flux, d, 1.0 / dx[0], 1.0 / dx[1], 1.0 / dx[2]);
    return cudaGetLastError();
}
cudaError_t op_diffterm(const int lo[3], const int hi[3], int ng, const double* q, double* tmp9, double* difflux,
                        const double dx[3], double eta, double alam, cudaStream_t st) {
    OpDims d = make_dims(lo, hi, ng);
    long long nint = (long long)d.n[0] * d.n[1] * d.n[2];
    const double a = 1.0 / dx[0], b = 1.0 / dx[1], c = 1.0 / dx[2];
    k_op_diffterm_d1<<<blocks_for(d.np), 256, 0, st>>>(q, tmp9, d, a, b, c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_op_diffterm<<<blocks_for(nint), 256, 0, st>>>(q, tmp9, difflux, d, a, b, c, eta, alam);
    return cudaGetLastError();
}
cudaError_t op_fill_ghosts_aos(double* aos, const int n[3], int nc, cudaStream_t st) {
    long long np = (long long)(n[0] + 8) * (n[1] + 8) * (n[2] + 8);
    k_fill_ghosts_aos<<<blocks_for(np), 256, 0, st>>>(aos, n[0], n[1], n[2], nc);
    return cudaGetLastError();
}
cudaError_t op_aos_to_box(const double* aos, const BoxView& b, cudaStream_t st) {
    long long nint = (long long)b.n[0] * b.n[1] * b.n[2];
    k_aos_to_box<<<blocks_for(nint), 256, 0, st>>>(aos, b);
    return cudaGetLastError();
}
cudaError_t op_box_to_aos(const BoxView& b, double* aos, int ghosts, cudaStream_t st) {
    long long np = (long long)(b.n[0] + 8) * (b.n[1] + 8) * (b.n[2] + 8);
    k_box_to_aos<<<blocks_for(np), 256, 0, st>>>(b, aos, ghosts);
    return cudaGetLastError();
}

}  // namespace cns

// ---- FP64 peak probe: the roofline denominator of the FP64-bound kernels -----------------
// Eight independent FMA chains per thread keep the FP64 pipe busy; every thread writes one
// value so nothing is dead code.
namespace cns {
__global__ void k_dfma_probe(double* out, double a, double b, int iters) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t probe_fp64(double* tflops) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    double* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double) * blocks * threads)) != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        k_dfma_probe<<<blocks, threads>>>(out, 0.999, 0.001, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // rep 0 warms up
    }
    e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return e;
}
}  // namespace cns

// ---- the CNS_NoSpec initial field generated on the device (serving requests) -------------
// Same field and perturbation stream as cns_nospec_gb300/initdata.py: cell-centred
// X = 2 pi (i + 1/2) / n0 etc., velocity amplitudes scaled by (ax, ay, az), rho, u, v, w times
// (1 + perturb * (2 U - 1)) with U from SplitMix64 at counter ((i*n1 + j)*n2 + k)*4 + field.
namespace cns {
__device__ __forceinline__ double splitmix_uniform(unsigned long long counter, unsigned long long seed) {
    unsigned long long z = counter + seed * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_init_field(BoxView b, double ax, double ay, double az, double perturb, unsigned long long seed) {
    const long long nint = (long long)b.n[0] * b.n[1] * b.n[2];
    const double twopi = 6.283185307179586476925286766559;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nint; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % b.n[2]);
        const int j = (int)((p / b.n[2]) % b.n[1]);
        const int i = (int)(p / ((long long)b.n[2] * b.n[1]));
        const double X = twopi * (i + 0.5) / b.n[0], Y = twopi * (j + 0.5) / b.n[1], Z = twopi * (k + 0.5) / b.n[2];
        double u = (1.1e4 * ax) * (sin(X) * sin(2 * Y) * sin(3 * Z));
        double v = (1.0e4 * ay) * (sin(2 * X) * sin(4 * Y) * sin(Z));
        double w = (1.2e4 * az) * (sin(3 * X) * cos(2 * Y) * sin(2 * Z));
        double rho = 1.0e-3 + 1.0e-5 * (sin(X) * cos(2 * Y) * cos(3 * Z));
        const double e = 2.5e9 + 1.0e-3 * (sin(X) * cos(2 * Y) * sin(2 * Z));
        if (perturb != 0.0) {
            const unsigned long long cnt = (unsigned long long)p * 4ull;
            rho *= 1.0 + perturb * (2.0 * splitmix_uniform(cnt, seed) - 1.0);
            u *= 1.0 + perturb * (2.0 * splitmix_uniform(cnt + 1, seed) - 1.0);
            v *= 1.0 + perturb * (2.0 * splitmix_uniform(cnt + 2, seed) - 1.0);
            w *= 1.0 + perturb * (2.0 * splitmix_uniform(cnt + 3, seed) - 1.0);
        }
        const long long c = cell_off(b, i, j, k);
        b.U[c] = rho;
        b.U[c + b.fs] = rho * u;
        b.U[c + 2 * b.fs] = rho * v;
        b.U[c + 3 * b.fs] = rho * w;
        b.U[c + 4 * b.fs] = rho * (e + (u * u + v * v + w * w) / 2.0);
    }
}

cudaError_t op_init_field(const BoxView& b, double ax, double ay, double az, double perturb, unsigned long long seed,
                          cudaStream_t st) {
    const long long nint = (long long)b.n[0] * b.n[1] * b.n[2];
    long long blocks = (nint + 255) / 256;
    k_init_field<<<(int)(blocks > 4096 ? 4096 : blocks), 256, 0, st>>>(b, ax, ay, az, perturb, seed);
    return cudaGetLastError();
}
}  // namespace cns
