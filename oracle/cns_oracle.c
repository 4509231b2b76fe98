/*
 * cns_oracle.c -- CPU restatement of the CNS_NoSpec RK3 advance (the reference's cpu/ path).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the GPU library: only
 * tests, the smoke check and the benchmark's CPU-baseline leg load it, and only as the
 * checker or the timed CPU baseline.  Nothing in the product path calls it.
 *
 * Layout (same as the reference's allocate_4D, cpu/helper_functions.cpp:100-122): one flat
 * block of doubles indexed [i][j][k][l] with the component l fastest, then k, then j, then i.
 * Ghost-inclusive arrays (U, Q) have dims n+2*ng per axis; D and F are interior-only (n per
 * axis), indexed from the interior origin (cpu/hypterm.cpp:8, cpu/diffterm.cpp:187).
 *
 * Every expression keeps the reference's floating-point evaluation order so that, compiled
 * with -O2 -ffp-contract=off, results are bit-identical to the reference compiled the same
 * way.  The oracle's tests check that bit-for-bit against the reference objects built by
 * oracle/Makefile, and against the committed fixtures in tests/golden/.
 *
 * Differences from the reference that do not change results:
 *   - the Courant maxima start at 0.0 (the reference leaves them uninitialised,
 *     cpu/ctoprim.cpp:21; every Courant term is positive, so a zero start equals the
 *     Fortran -huge start, fortran90/advance.f90:426-489);
 *   - oracle_advance takes per-axis dims (the reference's new_advance uses ncells and dim[0]
 *     for every axis, cpu/advance.cpp:34,110-113,144-147); for cubic boxes the two agree;
 *   - the loops carry OpenMP pragmas (the Fortran original threads the same loops,
 *     fortran90/advance.f90:244); every cell is independent and the Courant max is
 *     order-free, so the thread count does not change any bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NG_ 4
#define NC_ 5

/* 8th-order first-derivative coefficients, cpu/header.h:88-91. */
static const double ALP = 0.8E0;
static const double BET = -0.2E0;
static const double GAM = 4.0E0 / 105.0E0;
static const double DEL = -1.0E0 / 280.0E0;

/* 8th-order second-derivative coefficients, cpu/diffterm.cpp:48-52. */
static const double CENTER = -205.0E0 / 72.0E0;
static const double OFF1 = 8.0E0 / 5.0E0;
static const double OFF2 = -0.2E0;
static const double OFF3 = 8.0E0 / 315.0E0;
static const double OFF4 = -1.0E0 / 560.0E0;

/* Gas constants, cpu/ctoprim.cpp:23-24. */
static const double GAMMA = 1.4E0;
static const double CV = 8.3333333333E6;

/* flat index into an [d0][d1][d2][dl] block */
#define IX4(i, j, k, l, d1, d2, dl) ((((size_t)(i) * (d1) + (j)) * (d2) + (k)) * (dl) + (l))
#define IX3(i, j, k, d1, d2) (((size_t)(i) * (d1) + (j)) * (d2) + (k))

int oracle_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/*
 * Periodic ghost fill, cpu/helper_functions.cpp:226-262: z (k) ghosts over the interior
 * i,j; then y (j) ghosts over interior i and all k; then x (i) ghosts over all j,k.  The
 * pass order is what fills edges and corners.  dim = interior dims, dim_ng = dim + 2*NG.
 */
void oracle_fill_boundary(double *U, const int dim[3], const int dim_ng[3])
{
    const int d1 = dim_ng[1], d2 = dim_ng[2];
    int i, j, k, l;
    for (i = NG_; i < dim[0] + NG_; i++)
        for (j = NG_; j < dim[1] + NG_; j++)
            for (k = 0; k < NG_; k++)
                for (l = 0; l < NC_; l++) {
                    U[IX4(i, j, k, l, d1, d2, NC_)] = U[IX4(i, j, k + dim[2], l, d1, d2, NC_)];
                    U[IX4(i, j, k + dim[2] + NG_, l, d1, d2, NC_)] = U[IX4(i, j, k + NG_, l, d1, d2, NC_)];
                }
    for (i = NG_; i < dim[0] + NG_; i++)
        for (j = 0; j < NG_; j++)
            for (k = 0; k < dim_ng[2]; k++)
                for (l = 0; l < NC_; l++) {
                    U[IX4(i, j, k, l, d1, d2, NC_)] = U[IX4(i, j + dim[1], k, l, d1, d2, NC_)];
                    U[IX4(i, j + dim[1] + NG_, k, l, d1, d2, NC_)] = U[IX4(i, j + NG_, k, l, d1, d2, NC_)];
                }
    for (i = 0; i < NG_; i++)
        for (j = 0; j < dim_ng[1]; j++)
            for (k = 0; k < dim_ng[2]; k++)
                for (l = 0; l < NC_; l++) {
                    U[IX4(i, j, k, l, d1, d2, NC_)] = U[IX4(i + dim[0], j, k, l, d1, d2, NC_)];
                    U[IX4(i + dim[0] + NG_, j, k, l, d1, d2, NC_)] = U[IX4(i + NG_, j, k, l, d1, d2, NC_)];
                }
}

/*
 * Conserved -> primitive over the ghost-inclusive box, cpu/ctoprim.cpp:11-70 (with Courant)
 * and 72-105 (without).  q = (rho, u, v, w, p, T).  When courno != NULL the Courant maximum
 * over the interior is folded into *courno exactly as cpu/ctoprim.cpp:69 does.
 */
void oracle_ctoprim(const int lo[3], const int hi[3], const double *u, double *q,
                    const double dx[3], int ng, double *courno)
{
    const int d1 = hi[1] - lo[1] + 1 + 2 * ng, d2 = hi[2] - lo[2] + 1 + 2 * ng;
    int i;
#pragma omp parallel for schedule(static)
    for (i = lo[0] - ng; i <= hi[0] + ng; i++) {
        int j, k;
        for (j = lo[1] - ng; j <= hi[1] + ng; j++)
            for (k = lo[2] - ng; k <= hi[2] + ng; k++) {
                const double *uc = &u[IX4(i, j, k, 0, d1, d2, 5)];
                double *qc = &q[IX4(i, j, k, 0, d1, d2, 6)];
                double rhoinv = 1.0E0 / uc[0];
                double eint;
                qc[0] = uc[0];
                qc[1] = uc[1] * rhoinv;
                qc[2] = uc[2] * rhoinv;
                qc[3] = uc[3] * rhoinv;
                eint = uc[4] * rhoinv - 0.5E0 * (qc[1] * qc[1] + qc[2] * qc[2] + qc[3] * qc[3]);
                qc[4] = (GAMMA - 1.0E0) * eint * uc[0];
                qc[5] = eint / CV;
            }
    }
    if (courno != NULL) {
        double cmx = 0.0, cmy = 0.0, cmz = 0.0;
#pragma omp parallel for schedule(static) reduction(max : cmx, cmy, cmz)
        for (i = lo[0]; i <= hi[0]; i++) {
            int j, k;
            for (j = lo[1]; j <= hi[1]; j++)
                for (k = lo[2]; k <= hi[2]; k++) {
                    const double *qc = &q[IX4(i, j, k, 0, d1, d2, 6)];
                    double c = sqrt(GAMMA * qc[4] / qc[0]);
                    double cx = (c + fabs(qc[1])) / dx[0];
                    double cy = (c + fabs(qc[2])) / dx[1];
                    double cz = (c + fabs(qc[3])) / dx[2];
                    cmx = (cmx > cx) ? cmx : cx;
                    cmy = (cmy > cy) ? cmy : cy;
                    cmz = (cmz > cz) ? cmz : cz;
                }
        }
        {
            double a = (cmx > cmy) ? cmx : cmy;
            double b = (cmz > *courno) ? cmz : *courno;
            *courno = (a > b) ? a : b;
        }
    }
}

/*
 * Hyperbolic (convective) flux divergence, cpu/hypterm.cpp:11-209.  The x pass assigns the
 * flux, the y and z passes subtract their contributions in place; flux is interior-indexed.
 * Each difference keeps the reference's grouping: the pressure term rides inside the ALP..DEL
 * bracket of the momentum component along the pass direction, and (p*u) rides inside the
 * energy bracket.
 */
#define CQ(a, b, c, l) cons[IX4((a), (b), (c), (l), d1, d2, 5)]
#define QQ(a, b, c, l) q[IX4((a), (b), (c), (l), d1, d2, 6)]
#define FL(a, b, c, l) flux[IX4((a) - ng, (b) - ng, (c) - ng, (l), f1, f2, 5)]

/* one direction's stencil; offsets (di,dj,dk) select the pass axis, mc the momentum
 * component along it, qc the velocity component along it, dxi = 1/dx along it */
static void hyp_pass(const int lo[3], const int hi[3], int ng, const double *cons, const double *q,
                     double *flux, int di, int dj, int dk, int mc, int qc, double dxi, int first)
{
    const int d1 = hi[1] - lo[1] + 1 + 2 * ng, d2 = hi[2] - lo[2] + 1 + 2 * ng;
    const int f1 = hi[1] - lo[1] + 1, f2 = hi[2] - lo[2] + 1;
    int i;
#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k, l;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
#define CM(m, l) cons[IX4(i + (m) * di, j + (m) * dj, k + (m) * dk, (l), d1, d2, 5)]
#define QM(m, l) q[IX4(i + (m) * di, j + (m) * dj, k + (m) * dk, (l), d1, d2, 6)]
                double unp1 = QM(1, qc), unp2 = QM(2, qc), unp3 = QM(3, qc), unp4 = QM(4, qc);
                double unm1 = QM(-1, qc), unm2 = QM(-2, qc), unm3 = QM(-3, qc), unm4 = QM(-4, qc);
                double v[5];
                /* density: -d(rho u_d)/dx_d */
                v[0] = (ALP * (CM(1, mc) - CM(-1, mc)) + BET * (CM(2, mc) - CM(-2, mc)) +
                        GAM * (CM(3, mc) - CM(-3, mc)) + DEL * (CM(4, mc) - CM(-4, mc)));
                /* momenta: the component along the pass carries the pressure difference */
                for (l = 1; l <= 3; l++) {
                    if (l == mc)
                        v[l] = (ALP * (CM(1, l) * unp1 - CM(-1, l) * unm1 + (QM(1, 4) - QM(-1, 4))) +
                                BET * (CM(2, l) * unp2 - CM(-2, l) * unm2 + (QM(2, 4) - QM(-2, 4))) +
                                GAM * (CM(3, l) * unp3 - CM(-3, l) * unm3 + (QM(3, 4) - QM(-3, 4))) +
                                DEL * (CM(4, l) * unp4 - CM(-4, l) * unm4 + (QM(4, 4) - QM(-4, 4))));
                    else
                        v[l] = (ALP * (CM(1, l) * unp1 - CM(-1, l) * unm1) +
                                BET * (CM(2, l) * unp2 - CM(-2, l) * unm2) +
                                GAM * (CM(3, l) * unp3 - CM(-3, l) * unm3) +
                                DEL * (CM(4, l) * unp4 - CM(-4, l) * unm4));
                }
                /* energy: (E + p) u_d, written as E*u_d - E*u_d + (p*u_d - p*u_d) per pair */
                v[4] = (ALP * (CM(1, 4) * unp1 - CM(-1, 4) * unm1 + (QM(1, 4) * unp1 - QM(-1, 4) * unm1)) +
                        BET * (CM(2, 4) * unp2 - CM(-2, 4) * unm2 + (QM(2, 4) * unp2 - QM(-2, 4) * unm2)) +
                        GAM * (CM(3, 4) * unp3 - CM(-3, 4) * unm3 + (QM(3, 4) * unp3 - QM(-3, 4) * unm3)) +
                        DEL * (CM(4, 4) * unp4 - CM(-4, 4) * unm4 + (QM(4, 4) * unp4 - QM(-4, 4) * unm4)));
#undef CM
#undef QM
                for (l = 0; l < 5; l++) {
                    if (first)
                        FL(i, j, k, l) = -v[l] * dxi;
                    else
                        FL(i, j, k, l) = FL(i, j, k, l) - v[l] * dxi;
                }
            }
    }
}

void oracle_hypterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double *cons,
                    const double *q, double *flux)
{
    double dxinv[3];
    int d;
    for (d = 0; d < 3; d++) dxinv[d] = 1.0E0 / dx[d];
    hyp_pass(lo, hi, ng, cons, q, flux, 1, 0, 0, 1, 1, dxinv[0], 1);
    hyp_pass(lo, hi, ng, cons, q, flux, 0, 1, 0, 2, 2, dxinv[1], 0);
    hyp_pass(lo, hi, ng, cons, q, flux, 0, 0, 1, 3, 3, dxinv[2], 0);
}
#undef CQ
#undef FL

/*
 * Viscous and heat-conduction terms, cpu/diffterm.cpp:22-320.  The nine first derivatives
 * of (u,v,w) are formed on the extended ranges the mixed derivatives need (73-151): the
 * derivative along axis d covers the interior along d and the full ghost-inclusive range
 * along the other two axes.  difflux is interior-indexed; its density component is zero.
 */
void oracle_diffterm(const int lo[3], const int hi[3], int ng, const double dx[3], const double *q,
                     double *difflux, double eta, double alam)
{
    const int g0 = hi[0] - lo[0] + 1 + 2 * ng, d1 = hi[1] - lo[1] + 1 + 2 * ng, d2 = hi[2] - lo[2] + 1 + 2 * ng;
    const int f1 = hi[1] - lo[1] + 1, f2 = hi[2] - lo[2] + 1;
    const double OneThird = 1.0E0 / 3.0E0, TwoThirds = 2.0E0 / 3.0E0, FourThirds = 4.0E0 / 3.0E0;
    const size_t n3 = (size_t)g0 * d1 * d2;
    double dxinv[3];
    double *tmp = (double *)malloc(9 * n3 * sizeof(double));
    double *ux = tmp, *vx = tmp + n3, *wx = tmp + 2 * n3, *uy = tmp + 3 * n3, *vy = tmp + 4 * n3,
           *wy = tmp + 5 * n3, *uz = tmp + 6 * n3, *vz = tmp + 7 * n3, *wz = tmp + 8 * n3;
    int i, d;
    for (d = 0; d < 3; d++) dxinv[d] = 1.0E0 / dx[d];

#define D1(arr, di, dj, dk, l, h)                                                                           \
    ((ALP * (QQ(i + (di), j + (dj), k + (dk), l) - QQ(i - (di), j - (dj), k - (dk), l)) +                   \
      BET * (QQ(i + 2 * (di), j + 2 * (dj), k + 2 * (dk), l) - QQ(i - 2 * (di), j - 2 * (dj), k - 2 * (dk), l)) + \
      GAM * (QQ(i + 3 * (di), j + 3 * (dj), k + 3 * (dk), l) - QQ(i - 3 * (di), j - 3 * (dj), k - 3 * (dk), l)) + \
      DEL * (QQ(i + 4 * (di), j + 4 * (dj), k + 4 * (dk), l) - QQ(i - 4 * (di), j - 4 * (dj), k - 4 * (dk), l))) * \
     (h))

    for (i = lo[0] - ng; i <= hi[0] - ng; i++) {
        int j, k;
        for (j = lo[1] - ng; j <= hi[1] - ng; j++)
            for (k = lo[2] - ng; k <= hi[2] - ng; k++) difflux[IX4(i, j, k, 0, f1, f2, 5)] = 0.0E0;
    }

#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k;
        for (j = lo[1] - ng; j <= hi[1] + ng; j++)
            for (k = lo[2] - ng; k <= hi[2] + ng; k++) {
                size_t c = IX3(i, j, k, d1, d2);
                ux[c] = D1(ux, 1, 0, 0, 1, dxinv[0]);
                vx[c] = D1(vx, 1, 0, 0, 2, dxinv[0]);
                wx[c] = D1(wx, 1, 0, 0, 3, dxinv[0]);
            }
    }
#pragma omp parallel for schedule(static)
    for (i = lo[0] - ng; i <= hi[0] + ng; i++) {
        int j, k;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2] - ng; k <= hi[2] + ng; k++) {
                size_t c = IX3(i, j, k, d1, d2);
                uy[c] = D1(uy, 0, 1, 0, 1, dxinv[1]);
                vy[c] = D1(vy, 0, 1, 0, 2, dxinv[1]);
                wy[c] = D1(wy, 0, 1, 0, 3, dxinv[1]);
            }
    }
#pragma omp parallel for schedule(static)
    for (i = lo[0] - ng; i <= hi[0] + ng; i++) {
        int j, k;
        for (j = lo[1] - ng; j <= hi[1] + ng; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
                size_t c = IX3(i, j, k, d1, d2);
                uz[c] = D1(uz, 0, 0, 1, 1, dxinv[2]);
                vz[c] = D1(vz, 0, 0, 1, 2, dxinv[2]);
                wz[c] = D1(wz, 0, 0, 1, 3, dxinv[2]);
            }
    }
#undef D1

/* symmetric second difference of q component l along (di,dj,dk), scaled by h*h */
#define D2(di, dj, dk, l, h)                                                                                  \
    ((CENTER * QQ(i, j, k, l) + OFF1 * (QQ(i + (di), j + (dj), k + (dk), l) + QQ(i - (di), j - (dj), k - (dk), l)) + \
      OFF2 * (QQ(i + 2 * (di), j + 2 * (dj), k + 2 * (dk), l) + QQ(i - 2 * (di), j - 2 * (dj), k - 2 * (dk), l)) +  \
      OFF3 * (QQ(i + 3 * (di), j + 3 * (dj), k + 3 * (dk), l) + QQ(i - 3 * (di), j - 3 * (dj), k - 3 * (dk), l)) +  \
      OFF4 * (QQ(i + 4 * (di), j + 4 * (dj), k + 4 * (dk), l) + QQ(i - 4 * (di), j - 4 * (dj), k - 4 * (dk), l))) * \
     ((h) * (h)))
/* first difference of a derivative array along (di,dj,dk) */
#define T3(a, i_, j_, k_) a[IX3((i_), (j_), (k_), d1, d2)]
#define DD(a, di, dj, dk, h)                                                                             \
    ((ALP * (T3(a, i + (di), j + (dj), k + (dk)) - T3(a, i - (di), j - (dj), k - (dk))) +                \
      BET * (T3(a, i + 2 * (di), j + 2 * (dj), k + 2 * (dk)) - T3(a, i - 2 * (di), j - 2 * (dj), k - 2 * (dk))) + \
      GAM * (T3(a, i + 3 * (di), j + 3 * (dj), k + 3 * (dk)) - T3(a, i - 3 * (di), j - 3 * (dj), k - 3 * (dk))) + \
      DEL * (T3(a, i + 4 * (di), j + 4 * (dj), k + 4 * (dk)) - T3(a, i - 4 * (di), j - 4 * (dj), k - 4 * (dk)))) * \
     (h))
#define DF(l) difflux[IX4(i - ng, j - ng, k - ng, (l), f1, f2, 5)]

#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
                double uxx = D2(1, 0, 0, 1, dxinv[0]);
                double uyy = D2(0, 1, 0, 1, dxinv[1]);
                double uzz = D2(0, 0, 1, 1, dxinv[2]);
                double vyx = DD(vy, 1, 0, 0, dxinv[0]);
                double wzx = DD(wz, 1, 0, 0, dxinv[0]);
                DF(1) = eta * (FourThirds * uxx + uyy + uzz + OneThird * (vyx + wzx));
            }
    }
#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
                double vxx = D2(1, 0, 0, 2, dxinv[0]);
                double vyy = D2(0, 1, 0, 2, dxinv[1]);
                double vzz = D2(0, 0, 1, 2, dxinv[2]);
                double uxy = DD(ux, 0, 1, 0, dxinv[1]);
                double wzy = DD(wz, 0, 1, 0, dxinv[1]);
                DF(2) = eta * (vxx + FourThirds * vyy + vzz + OneThird * (uxy + wzy));
            }
    }
#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
                double wxx = D2(1, 0, 0, 3, dxinv[0]);
                double wyy = D2(0, 1, 0, 3, dxinv[1]);
                double wzz = D2(0, 0, 1, 3, dxinv[2]);
                double uxz = DD(ux, 0, 0, 1, dxinv[2]);
                double vyz = DD(vy, 0, 0, 1, dxinv[2]);
                DF(3) = eta * (wxx + wyy + FourThirds * wzz + OneThird * (uxz + vyz));
            }
    }
#pragma omp parallel for schedule(static)
    for (i = lo[0]; i <= hi[0]; i++) {
        int j, k;
        for (j = lo[1]; j <= hi[1]; j++)
            for (k = lo[2]; k <= hi[2]; k++) {
                size_t c = IX3(i, j, k, d1, d2);
                double txx = D2(1, 0, 0, 5, dxinv[0]);
                double tyy = D2(0, 1, 0, 5, dxinv[1]);
                double tzz = D2(0, 0, 1, 5, dxinv[2]);
                double divu = TwoThirds * (ux[c] + vy[c] + wz[c]);
                double tauxx = 2.E0 * ux[c] - divu;
                double tauyy = 2.E0 * vy[c] - divu;
                double tauzz = 2.E0 * wz[c] - divu;
                double tauxy = uy[c] + vx[c];
                double tauxz = uz[c] + wx[c];
                double tauyz = vz[c] + wy[c];
                double mechwork = tauxx * ux[c] + tauyy * vy[c] + tauzz * wz[c] + tauxy * tauxy + tauxz * tauxz +
                                  tauyz * tauyz;
                mechwork = eta * mechwork + DF(1) * QQ(i, j, k, 1) + DF(2) * QQ(i, j, k, 2) + DF(3) * QQ(i, j, k, 3);
                DF(4) = alam * (txx + tyy + tzz) + mechwork;
            }
    }
#undef D2
#undef DD
#undef T3
#undef DF
    free(tmp);
}
#undef QQ

/*
 * One or more RK3 steps, cpu/advance.cpp:13-154 (new_advance), with per-axis bounds.
 * U is ghost-inclusive [g0][g1][g2][5] and is updated in place.  Per step:
 *   fill_boundary(U); ctoprim(U) with Courant; dt = cfl/courno; D,F at U;
 *   Unew = U + dt(D+F);  fill; ctoprim; D,F at Unew;
 *   Unew = 3/4 U + 1/4 (Unew + dt(D+F));  fill; ctoprim; D,F;
 *   U    = 1/3 U + 2/3 (Unew + dt(D+F)).
 * As in the reference, U's ghost cells are left holding the fill made at the step's start.
 * dt_hist (optional) receives each step's dt.
 */
void oracle_advance(double *U, const int dim[3], const double dx[3], double cfl, double eta, double alam,
                    int nsteps, double *dt_hist)
{
    const int ng = NG_;
    int dim_ng[3], lo[3], hi[3], d, step;
    size_t gsz, isz;
    double *Unew, *Q, *D, *F;
    const double OneThird = 1.0E0 / 3.0E0, TwoThirds = 2.0E0 / 3.0E0;
    const double OneQuarter = 1.E0 / 4.E0, ThreeQuarters = 3.E0 / 4.E0;
    for (d = 0; d < 3; d++) {
        dim_ng[d] = dim[d] + 2 * ng;
        lo[d] = ng;
        hi[d] = dim[d] - 1 + ng;
    }
    gsz = (size_t)dim_ng[0] * dim_ng[1] * dim_ng[2];
    isz = (size_t)dim[0] * dim[1] * dim[2];
    Unew = (double *)calloc(gsz * 5, sizeof(double));
    Q = (double *)calloc(gsz * 6, sizeof(double));
    D = (double *)calloc(isz * 5, sizeof(double));
    F = (double *)calloc(isz * 5, sizeof(double));

    for (step = 0; step < nsteps; step++) {
        double courno = 1.0E-50, dt;
        int stage;
        oracle_fill_boundary(U, dim, dim_ng);
        oracle_ctoprim(lo, hi, U, Q, dx, ng, &courno);
        dt = cfl / courno;
        if (dt_hist) dt_hist[step] = dt;
        for (stage = 0; stage < 3; stage++) {
            const double *src = (stage == 0) ? U : Unew;
            int i;
            if (stage > 0) {
                oracle_fill_boundary(Unew, dim, dim_ng);
                oracle_ctoprim(lo, hi, Unew, Q, dx, ng, NULL);
            }
            oracle_diffterm(lo, hi, ng, dx, Q, D, eta, alam);
            oracle_hypterm(lo, hi, ng, dx, src, Q, F);
#pragma omp parallel for schedule(static)
            for (i = 0; i < dim[0]; i++) {
                int j, k, l;
                for (j = 0; j < dim[1]; j++)
                    for (k = 0; k < dim[2]; k++)
                        for (l = 0; l < 5; l++) {
                            size_t g = IX4(i + ng, j + ng, k + ng, l, dim_ng[1], dim_ng[2], 5);
                            size_t c = IX4(i, j, k, l, dim[1], dim[2], 5);
                            if (stage == 0)
                                Unew[g] = U[g] + dt * (D[c] + F[c]);
                            else if (stage == 1)
                                Unew[g] = ThreeQuarters * U[g] + OneQuarter * (Unew[g] + dt * (D[c] + F[c]));
                            else
                                U[g] = OneThird * U[g] + TwoThirds * (Unew[g] + dt * (D[c] + F[c]));
                        }
            }
        }
    }
    free(Unew);
    free(Q);
    free(D);
    free(F);
}
