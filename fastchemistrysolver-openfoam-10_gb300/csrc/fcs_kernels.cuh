#pragma once
// fcs_kernels.cuh -- sm_103a kernels of the per-cell stiff chemistry path.
//
//   integrate_kernel : persistent kernel; each cell group pulls cells from a
//                      device work queue and runs OptRodas34 /
//                      OptRosenbrock34 / OptSeulex with the reference's step
//                      size control over one CFD step
//   rhs_kernel       : f(y) per cell (FastChemistryModel::derivatives)
//   jac_kernel       : J(y), f(y) per cell (FastChemistryModel::jacobian)
//   rates_kernel     : calculate()/Qdot source terms per cell
//   classify_kernel  : Treact skip + active-cell queue
//
// Precision: MT = double is the FP64 method; MT = float is the mixed method
// (Jacobian storage and LU in FP32, one FP64-residual refinement sweep per
// linear solve, everything else FP64).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fcs_device.cuh"
#include "fcs_launch.h"

namespace fcs {

// ------------------------------------------------------------------------
// linear algebra of one attempt

struct CellCounters {
    long long attempts = 0, accepted = 0, jac = 0, lu = 0, rhs = 0, solves = 0, fallbacks = 0;
};

// Accepted size of the refinement correction relative to the solution
// (max norm); above it the FP32 factorisation is not trusted for this matrix
// and the attempt is redone in FP64.
constexpr double kRefineTol = 1e-3;

// FP64: A = c I - J into the LU view (in place for the single-matrix layout)
template<int G>
__device__ __noinline__ void form_iteration_matrix(const Grp<G>& g, const Slot<double>& s, int n, double c) {
    const int ld = s.ld;
    for (int idx = g.rank; idx < n * ld; idx += G) {
        const int i = idx / ld, j = idx - i * ld;
        if (j >= n) continue;
        const double v = -s.J[idx];
        s.LU[idx] = (i == j) ? v + c : v;
    }
    g.sync();
}

__device__ __forceinline__ float pow2_inverse(float m) {
    // 2^-e with e the binary exponent of m (exact scaling); 1 for 0/inf/nan
    if (!(m > 0.f) || !(m < 3.0e38f)) return 1.f;
    return ldexpf(1.f, -ilogbf(m));
}

// Mixed: LU32 = Dr (c I - J64) Dc in FP32 with power-of-two row and column
// equilibration (Dr, Dc kept in s.dr / s.dc, as doubles, for the solves).
// One narrowing per element; the equilibration runs on the FP32 pipe.
template<int G>
__device__ __noinline__ void form_iteration_matrix_scaled(const Grp<G>& g, const Slot<float>& s, int n,
                                                          double c) {
    const int ld = s.ld;
    float* LU = s.LU;
    float* dcf = s.r32;  // FP32 copy of the column scales (the solve vector is free until the solves)
    // pass 1: narrow c I - J to FP32 (the diagonal formed in FP64), row maxima,
    // row scaling applied in FP32 (exact: powers of two)
    for (int i = g.rank; i < n; i += G) {
        const double* Ji = s.J64 + (size_t)i * ld;
        float* Li = LU + (size_t)i * ld;
        float mx = 0.f;
        for (int j = 0; j < n; j++) {
            const float a = (j == i) ? float(c - Ji[j]) : -float(Ji[j]);
            Li[j] = a;
            mx = fmaxf(mx, fabsf(a));
        }
        const float ri = pow2_inverse(mx);
        s.dr[i] = double(ri);
        for (int j = 0; j < n; j++) Li[j] *= ri;
    }
    g.sync();
    // pass 2: column maxima of the row-scaled matrix
    for (int j = g.rank; j < n; j += G) {
        float mx = 0.f;
        for (int i = 0; i < n; i++) mx = fmaxf(mx, fabsf(LU[(size_t)i * ld + j]));
        const float cj = pow2_inverse(mx);
        s.dc[j] = double(cj);
        dcf[j] = cj;
    }
    g.sync();
    // pass 3: column scaling
    for (int i = g.rank; i < n; i += G) {
        float* Li = LU + (size_t)i * ld;
        for (int j = 0; j < n; j++) Li[j] *= dcf[j];
    }
    g.sync();
}

// Mixed solve: x0 = Dc LU32^-1 Dr b (FP32 vectors), r = b - (c x0 - J64 x0)
// in FP64, x = x0 + Dc LU32^-1 Dr r.  Returns false when the correction is
// not small (or not finite): the caller then repeats the work in FP64.
template<int G>
__device__ __noinline__ bool linear_solve_mixed(const Grp<G>& g, const DevMech& M, const Slot<float>& s,
                                                double c, double* b, double* tmp) {
    const int n = M.n, ld = s.ld;
    for (int i = g.rank; i < n; i += G) s.x32[i] = float(b[i] * s.dr[i]);
    lu_solve<G, float, float>(g, s.LU, n, ld, s.piv, s.invD, s.x32);
    for (int i = g.rank; i < n; i += G) tmp[i] = double(s.x32[i]) * s.dc[i];
    g.sync();
    for (int i = g.rank; i < n; i += G) {
        const double* Ji = s.J64 + (size_t)i * ld;
        double r = b[i] - c * tmp[i];
        for (int j = 0; j < n; j++) r = fma(Ji[j], tmp[j], r);
        s.r32[i] = float(r * s.dr[i]);
    }
    lu_solve<G, float, float>(g, s.LU, n, ld, s.piv, s.invD, s.r32);
    double dmax = 0, xmax = 0;
    for (int i = g.rank; i < n; i += G) {
        const double d = double(s.r32[i]) * s.dc[i];
        const double x = tmp[i] + d;
        b[i] = x;
        // running maxima of |d| and |x| on the bit patterns (NaN wins)
        const unsigned long long ad = static_cast<unsigned long long>(__double_as_longlong(fabs(d)));
        const unsigned long long ax = static_cast<unsigned long long>(__double_as_longlong(fabs(x)));
        if (ad > static_cast<unsigned long long>(__double_as_longlong(dmax))) dmax = fabs(d);
        if (ax > static_cast<unsigned long long>(__double_as_longlong(xmax))) xmax = fabs(x);
    }
    gmax2_nonneg(g, dmax, xmax, s.red);
    g.sync();
    return dmax <= kRefineTol * xmax && xmax < 1e300;
}

// Jacobian of the attempt: assembled in FP64 (cancellation between fast
// forward and reverse terms needs it), kept in FP32 in mixed precision.
template<int G, class MT>
__device__ __forceinline__ void jacobian_into(const Grp<G>& g, const DevMech& M, const Slot<MT>& s,
                                              const Slot<double>& sd, double p, double* y, double* f, int fast) {
    jac_eval<G, double>(g, M, sd, p, y, f, sd.J, fast);
}

template<int G, class MT>
__device__ __forceinline__ void factor_iteration(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double c) {
    if constexpr (sizeof(MT) == 8) form_iteration_matrix<G>(g, s, M.n, c);
    else form_iteration_matrix_scaled<G>(g, s, M.n, c);
    // the reaction-chunk arrays are free between a Jacobian and the next RHS
    lu_factor<G, MT>(g, s.LU, M.n, s.ld, s.piv, s.invD, reinterpret_cast<int*>(s.Kf));
}

template<int G, class MT>
__device__ __forceinline__ bool stage_solve(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double c,
                                            double* b, double* tmp) {
    if constexpr (sizeof(MT) == 8) {
        lu_solve<G, double, double>(g, s.LU, M.n, s.ld, s.piv, s.invD, b);
        return true;
    } else {
        return linear_solve_mixed<G>(g, M, s, c, b, tmp);
    }
}

// ------------------------------------------------------------------------
// Rosenbrock attempts

// OptRodas34::Rodas34Solve (OptRodas34.C:291-882), constants OptRodas34.H:105-149.
// Vectors: 0 y0, 1 yTemp, 2..6 k1..k5, 7 dy, 8 err, 9 dydx, 10 dfdx, 11 tmp
template<int G, class MT>
__device__ __noinline__ double rodas34_attempt(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                  const Slot<MT>& s, const Slot<double>& sd, double p, double dx,
                                  double invdx, CellCounters& cc) {
    const int n = M.n;
    double *y0 = s.v(0), *yTemp = s.v(1), *k1 = s.v(2), *k2 = s.v(3), *k3 = s.v(4), *k4 = s.v(5);
    double *k5 = s.v(6), *dy = s.v(7), *err = s.v(8), *dydx = s.v(9), *dfdx = s.v(10), *tmp = s.v(11);
    const double d1 = 0.25, d2 = -0.1043, d3 = 0.1035, d4 = -0.3620000000000023e-01;
    const double a21 = 0.1544e1, a31 = 0.9466785280815826, a32 = 0.2557011698983284;
    const double a41 = 0.3314825187068521e1, a42 = 0.2896124015972201e1, a43 = 0.9986419139977817;
    const double a51 = 0.1221224509226641e1, a52 = 0.6019134481288629e1, a53 = 0.1253708332932087e2,
                 a54 = -0.6878860361058950;
    const double c21 = -0.56688e1, c31 = -0.2430093356833875e1, c32 = -0.2063599157091915;
    const double c41 = -0.1073529058151375, c42 = -0.9594562251023355e1, c43 = -0.2047028614809616e2;
    const double c51 = 0.7496443313967647e1, c52 = -0.1024680431464352e2, c53 = -0.3399990352819905e2,
                 c54 = 0.1170890893206160e2;
    const double c61 = 0.8083246795921522e1, c62 = -0.7981132988064893e1, c63 = -0.3152159432874371e2,
                 c64 = 0.1631930543123136e2, c65 = -0.6058818238834054e1;
    const double invgamma = 1.0 / 0.25;

    jacobian_into<G, MT>(g, M, s, sd, p, y0, dfdx, o.jacobian);
    const double cdiag = 1.0 * invdx * invgamma;
    factor_iteration<G, MT>(g, M, s, cdiag);
    cc.jac++; cc.lu++; cc.rhs += 5; cc.solves += 6;

    const double dxd1 = dx * d1 + 1;
    for (int i = g.rank; i < n; i += G) k1[i] = dxd1 * dfdx[i];
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k1, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a21, k1[i], y0[i]);
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, e1 = c21 * invdx;
        for (int i = g.rank; i < n; i += G) k2[i] = fma(e1, k1[i], fma(dxd2, dfdx[i], dydx[i]));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k2, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a32, k2[i], fma(a31, k1[i], y0[i]));
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, e1 = c31 * invdx, e2 = c32 * invdx;
        for (int i = g.rank; i < n; i += G) k3[i] = fma(e2, k2[i], fma(e1, k1[i], fma(dxd3, dfdx[i], dydx[i])));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k3, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a43, k3[i], fma(a42, k2[i], fma(a41, k1[i], y0[i])));
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double dxd4 = dx * d4, e1 = c41 * invdx, e2 = c42 * invdx, e3 = c43 * invdx;
        for (int i = g.rank; i < n; i += G)
            k4[i] = fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], fma(dxd4, dfdx[i], dydx[i]))));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k4, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) {
        const double d = fma(a54, k4[i], fma(a53, k3[i], fma(a52, k2[i], a51 * k1[i])));
        dy[i] = d;
        yTemp[i] = y0[i] + d;
    }
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double e1 = c51 * invdx, e2 = c52 * invdx, e3 = c53 * invdx, e4 = c54 * invdx;
        for (int i = g.rank; i < n; i += G)
            k5[i] = fma(e4, k4[i], fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], dydx[i]))));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k5, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) {
        const double d = dy[i] + k5[i];
        dy[i] = d;
        yTemp[i] = y0[i] + d;
    }
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 2);
    {
        const double e1 = c61 * invdx, e2 = c62 * invdx, e3 = c63 * invdx, e4 = c64 * invdx, e5 = c65 * invdx;
        for (int i = g.rank; i < n; i += G)
            err[i] = fma(e5, k5[i], fma(e4, k4[i], fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], dydx[i])))));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, err, tmp)) return -1.0;
    double me = 0;
    for (int i = g.rank; i < n; i += G) {
        const double yt = y0[i] + dy[i] + err[i];
        yTemp[i] = yt;
        const double tol = o.absTol + o.relTol * fmax(fabs(y0[i]), fabs(yt));
        const double e = fabs(err[i]) / tol;
        me = (e > me || e != e) ? e : me;
    }
    return gmax(g, me, s.red);
}

// OptRosenbrock34::Rosenbrock34Solve (OptRosenbrock34.C:281-678), .H:127-158
template<int G, class MT>
__device__ __noinline__ double ros34_attempt(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                const Slot<MT>& s, const Slot<double>& sd, double p, double dx,
                                double invdx, CellCounters& cc) {
    const int n = M.n;
    double *y0 = s.v(0), *yTemp = s.v(1), *k1 = s.v(2), *k2 = s.v(3), *k3 = s.v(4), *k4 = s.v(5);
    double *err = s.v(8), *dydx = s.v(9), *dfdx = s.v(10), *tmp = s.v(11);
    const double a21 = 2, a31 = 48.0 / 25.0, a32 = 6.0 / 25.0;
    const double c21 = -8, c31 = 372.0 / 25.0, c32 = 12.0 / 5.0;
    const double c41 = -112.0 / 125.0, c42 = -54.0 / 125.0, c43 = -2.0 / 5.0;
    const double b1 = 19.0 / 9.0, b2 = 1.0 / 2.0, b3 = 25.0 / 108.0, b4 = 125.0 / 108.0;
    const double e1 = 34.0 / 108.0, e2 = 7.0 / 36.0, e4 = 125.0 / 108.0;
    const double d1 = 1.0 / 2.0, d2 = -3.0 / 2.0, d3 = 605.0 / 250.0, d4 = 29.0 / 250.0;
    const double invgamma = 1.0 / (1.0 / 2.0);

    jacobian_into<G, MT>(g, M, s, sd, p, y0, dfdx, o.jacobian);
    const double cdiag = invdx * invgamma;
    factor_iteration<G, MT>(g, M, s, cdiag);
    cc.jac++; cc.lu++; cc.rhs += 2; cc.solves += 4;

    const double dxd1 = dx * d1 + 1;
    for (int i = g.rank; i < n; i += G) k1[i] = dxd1 * dfdx[i];
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k1, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a21, k1[i], y0[i]);
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, f1 = c21 * invdx;
        for (int i = g.rank; i < n; i += G) k2[i] = fma(f1, k1[i], fma(dxd2, dfdx[i], dydx[i]));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k2, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a32, k2[i], fma(a31, k1[i], y0[i]));
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, f1 = c31 * invdx, f2 = c32 * invdx;
        for (int i = g.rank; i < n; i += G) k3[i] = fma(f2, k2[i], fma(f1, k1[i], fma(dxd3, dfdx[i], dydx[i])));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k3, tmp)) return -1.0;
    {
        const double dxd4 = dx * d4, f1 = c41 * invdx, f2 = c42 * invdx, f3 = c43 * invdx;
        for (int i = g.rank; i < n; i += G)
            k4[i] = fma(f3, k3[i], fma(f2, k2[i], fma(f1, k1[i], fma(dxd4, dfdx[i], dydx[i]))));
    }
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k4, tmp)) return -1.0;
    double me = 0;
    for (int i = g.rank; i < n; i += G) {
        const double yt = fma(b4, k4[i], fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i]))));
        yTemp[i] = yt;
        const double e = fma(e4, k4[i], fma(e2, k2[i], e1 * k1[i]));
        err[i] = e;
        const double tol = o.absTol + o.relTol * fmax(fabs(y0[i]), fabs(yt));
        const double r = fabs(e) / tol;
        me = (r > me || r != r) ? r : me;
    }
    return gmax(g, me, s.red);
}

// OptRodas23::Rodas23Solve (OptRodas23.C:202-315), constants OptRodas23.H:113-126:
// k2 reuses f(y0), two derivative evaluations per attempt.
template<int G, class MT>
__device__ __noinline__ double rodas23_attempt(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                  const Slot<MT>& s, const Slot<double>& sd, double p, double dx,
                                  double invdx, CellCounters& cc) {
    const int n = M.n;
    double *y0 = s.v(0), *yTemp = s.v(1), *k1 = s.v(2), *k2 = s.v(3), *k3 = s.v(4);
    double *dy = s.v(7), *err = s.v(8), *dydx = s.v(9), *dfdx = s.v(10), *tmp = s.v(11);
    const double d1 = 1.0 / 2.0, d2 = 3.0 / 2.0, a31 = 2, c21 = 4, c31 = 1, c32 = -1;
    const double c41 = 1, c42 = -1, c43 = -8.0 / 3.0;
    const double invgamma = 1.0 / (1.0 / 2.0);

    jacobian_into<G, MT>(g, M, s, sd, p, y0, dfdx, o.jacobian);
    const double cdiag = invdx * invgamma;
    factor_iteration<G, MT>(g, M, s, cdiag);
    cc.jac++; cc.lu++; cc.rhs += 2; cc.solves += 4;

    const double dxd1 = dx * d1, dxd2 = dx * d2;
    for (int i = g.rank; i < n; i += G) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k1, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) k2[i] = fma(dxd2, dfdx[i], dfdx[i]) + c21 * k1[i] / dx;
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k2, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) {
        dy[i] = a31 * k1[i];
        yTemp[i] = y0[i] + dy[i];
    }
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    for (int i = g.rank; i < n; i += G) k3[i] = dydx[i] + fma(c32, k2[i], c31 * k1[i]) / dx;
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k3, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) {
        dy[i] += k3[i];
        yTemp[i] = y0[i] + dy[i];
    }
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    for (int i = g.rank; i < n; i += G) err[i] = dydx[i] + fma(c43, k3[i], fma(c42, k2[i], c41 * k1[i])) / dx;
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, err, tmp)) return -1.0;
    double me = 0;
    for (int i = g.rank; i < n; i += G) {
        const double yt = y0[i] + dy[i] + err[i];
        yTemp[i] = yt;
        const double tol = o.absTol + o.relTol * fmax(fabs(y0[i]), fabs(yt));
        const double e = fabs(err[i]) / tol;
        me = (e > me || e != e) ? e : me;
    }
    return gmax(g, me, s.red);
}

// OptRosenbrock23::Rosenbrock23Solve (OptRosenbrock23.C:208-298), constants
// OptRosenbrock23.H:116-140: one derivative evaluation per attempt.
template<int G, class MT>
__device__ __noinline__ double ros23_attempt(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                const Slot<MT>& s, const Slot<double>& sd, double p, double dx,
                                double invdx, CellCounters& cc) {
    const int n = M.n;
    double *y0 = s.v(0), *yTemp = s.v(1), *k1 = s.v(2), *k2 = s.v(3), *k3 = s.v(4);
    double *err = s.v(8), *dydx = s.v(9), *dfdx = s.v(10), *tmp = s.v(11);
    const double a21 = 1;
    const double c21 = -1.0156171083877702091975600115545, c31 = 4.0759956452537699824805835358067;
    const double c32 = 9.2076794298330791242156818474003;
    const double b1 = 1, b2 = 6.1697947043828245592553615689730, b3 = -0.4277225654321857332623837380651;
    const double e1 = 0.5, e2 = -2.9079558716805469821718236208017, e3 = 0.2235406989781156962736090927619;
    const double gamma = 0.43586652150845899941601945119356, invgamma = 1.0 / gamma;
    const double d1 = 0.43586652150845899941601945119356, d2 = 0.24291996454816804366592249683314;
    const double d3 = 2.1851380027664058511513169485832;

    jacobian_into<G, MT>(g, M, s, sd, p, y0, dfdx, o.jacobian);
    const double cdiag = invdx * invgamma;
    factor_iteration<G, MT>(g, M, s, cdiag);
    cc.jac++; cc.lu++; cc.rhs += 1; cc.solves += 3;

    const double dxd1 = dx * d1, dxd2 = dx * d2, dxd3 = dx * d3;
    for (int i = g.rank; i < n; i += G) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k1, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) yTemp[i] = fma(a21, k1[i], y0[i]);
    g.sync();
    rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
    for (int i = g.rank; i < n; i += G) k2[i] = fma(dxd2, dfdx[i], dydx[i]) + c21 * k1[i] / dx;
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k2, tmp)) return -1.0;
    for (int i = g.rank; i < n; i += G) k3[i] = fma(dxd3, dfdx[i], dydx[i]) + fma(c32, k2[i], c31 * k1[i]) / dx;
    g.sync();
    if (!stage_solve<G, MT>(g, M, s, cdiag, k3, tmp)) return -1.0;
    double me = 0;
    for (int i = g.rank; i < n; i += G) {
        const double yt = fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i])));
        yTemp[i] = yt;
        const double e = fma(e3, k3[i], fma(e2, k2[i], e1 * k1[i]));
        err[i] = e;
        const double tol = o.absTol + o.relTol * fmax(fabs(y0[i]), fabs(yt));
        const double r = fabs(e) / tol;
        me = (r > me || r != r) ? r : me;
    }
    return gmax(g, me, s.red);
}

template<int G, class MT>
__device__ __forceinline__ double attempt_of(const Grp<G>& g, const DevMech& M, const KOpts& o, const Slot<MT>& s,
                                             const Slot<double>& sd, double p, double dx, double invdx,
                                             CellCounters& cc) {
    switch (o.solver) {
        case FCS_SOLVER_ROSENBROCK34: return ros34_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
        case FCS_SOLVER_RODAS23: return rodas23_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
        case FCS_SOLVER_ROSENBROCK23: return ros23_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
        default: return rodas34_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
    }
}

// ODESolve + adaptiveSolve (OptRodas34.C:123-289, OptRosenbrock34.C:127-279,
// OptRodas23.C:105-200, OptRosenbrock23.C:105-206),
// with bounded reject loops.  Returns FCS_CELL_*; y0 (vector 0) holds the state.
// One attempt in the slot's precision; in mixed precision an attempt whose
// FP32 factorisation fails the refinement check is redone in FP64.
template<int G, class MT>
__device__ __forceinline__ double rosenbrock_attempt(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                                     const Slot<MT>& s, const Slot<double>& sd, double p,
                                                     double dx, double invdx, CellCounters& cc) {
    double Err = attempt_of<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
    if constexpr (sizeof(MT) == 4) {
        if (Err == -1.0) {
            cc.fallbacks++;
            Err = attempt_of<G, double>(g, M, o, sd, sd, p, dx, invdx, cc);
        }
    }
    return Err;
}

template<int G, class MT>
__device__ int rosenbrock_integrate(const Grp<G>& g, const DevMech& M, const KOpts& o,
                                    const Slot<MT>& s, const Slot<double>& sd, double p, double xEnd,
                                    double& dxTryIO, CellCounters& cc) {
    const double SAFE = 0.9, ALPHA_INC = 0.2, ALPHA_DEC = 0.25, MIN_SCALE = 0.2, MAX_SCALE = 10;
    const double ratio = 5.904900000000001e-06;  // (MAX_SCALE/SAFE)^(-1/ALPHA_INC)
    const double safeMaxScale = SAFE * MAX_SCALE;
    const int n = M.n;
    double* y0 = s.v(0);
    double* yTemp = s.v(1);
    double dxTry = dxTryIO;
    bool last = false;
    double x = 0;
    for (int nStep = 0; nStep < o.maxSteps; nStep++) {
        const double dxTry0 = dxTry;
        if ((x + dxTry - xEnd) * (x + dxTry - 0.0) > 0) { last = true; dxTry = xEnd - x; }
        double dx = dxTry, invdx = 1.0 / dx;
        double Err = rosenbrock_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
        cc.attempts++;
        int rejects = 0;
        while (Err > 1) {
            if (++rejects > o.maxRejects) return FCS_CELL_DT_UNDERFLOW;
            const double scale = fmax(SAFE * pow(Err, -ALPHA_DEC), MIN_SCALE);
            dx *= scale;
            invdx = 1.0 / dx;
            Err = rosenbrock_attempt<G, MT>(g, M, o, s, sd, p, dx, invdx, cc);
            cc.attempts++;
        }
        if (!(Err == Err)) return FCS_CELL_NONFINITE;
        cc.accepted++;
        x += dx;
        for (int i = g.rank; i < n; i += G) y0[i] = yTemp[i];
        g.sync();
        dxTry = (Err > ratio) ? fmin(fmax(SAFE * pow(Err, -ALPHA_INC), MIN_SCALE), MAX_SCALE) * dx
                              : safeMaxScale * dx;
        if ((x - xEnd) * (xEnd - 0.0) >= 0) {
            if (nStep > 0 && last) dxTry = dxTry0;
            dxTryIO = dxTry;
            return FCS_CELL_OK;
        }
    }
    return FCS_CELL_MAX_STEPS;
}

// ------------------------------------------------------------------------
// Seulex: OptSeulex.C:34-94 (constants), 171-260, 262-560, 562-709, 711-734.
// Vectors: 0 y (state), 1 y0_, 2 ySeq, 3 scale, 4 yTemp, 5 dy, 6 dydx, 7 k9 (f), 11 tmp.
// Matrices: J = Jy (kept), LU = a (factored per order).

constexpr int kKMax = 12;
constexpr int kIMax = kKMax + 1;

struct SeulexConst {
    int nSeq[kIMax];
    double cpu[kIMax];
};

__device__ __forceinline__ SeulexConst seulex_const() {
    SeulexConst c;
    const double cpuFunc = 1, cpuJac = 5, cpuLU = 1, cpuSolve = 1;
    c.nSeq[0] = 2; c.nSeq[1] = 3;
    for (int i = 2; i < kIMax; i++) c.nSeq[i] = 2 * c.nSeq[i - 2];
    c.cpu[0] = cpuJac + cpuLU + c.nSeq[0] * (cpuFunc + cpuSolve);
    for (int k = 0; k < kKMax; k++) c.cpu[k + 1] = c.cpu[k] + (c.nSeq[k + 1] - 1) * (cpuFunc + cpuSolve) + cpuLU;
    return c;
}

__device__ __forceinline__ double seulex_coeff(const SeulexConst& c, int k, int l) {
    const double r = (double)c.nSeq[k] / c.nSeq[l];
    return 1 / (r - 1);
}

struct SeulexState {
    double theta;
    int kTarg;
    double dxOpt[kIMax], temp[kIMax];
};

// returns 1 on success, 0 when the sequence diverged (step reject), 2 when the
// mixed-precision solve needs FP64
template<int G, class MT>
__device__ __noinline__ int seul(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p,
                     const SeulexConst& sc, SeulexState& st, double dxTot, int k, CellCounters& cc) {
    const int n = M.n;
    double *y0_ = s.v(1), *ySeq = s.v(2), *scale = s.v(3), *yTemp = s.v(4), *dy = s.v(5), *dydx = s.v(6);
    double* tmp = s.v(11);
    const int nSteps = sc.nSeq[k];
    const double invdx = nSteps / dxTot;
    factor_iteration<G, MT>(g, M, s, invdx);
    cc.lu++;
    rhs_eval<G, MT>(g, M, s, p, y0_, dy, 1);
    cc.rhs++;
    if (!stage_solve<G, MT>(g, M, s, invdx, dy, tmp)) return 2;
    cc.solves++;
    for (int i = g.rank; i < n; i += G) yTemp[i] = y0_[i];
    g.sync();
    for (int nn = 1; nn < nSteps; nn++) {
        for (int i = g.rank; i < n; i += G) yTemp[i] += dy[i];
        g.sync();
        if (nn == 1 && k <= 1) {
            double a = 0;
            for (int i = g.rank; i < n; i += G) { const double q = dy[i] / scale[i]; a += q * q; }
            a = gsum(g, a, s.red);
            const double dy1 = sqrt(a);
            rhs_eval<G, MT>(g, M, s, p, yTemp, dydx, 1);
            cc.rhs++;
            for (int i = g.rank; i < n; i += G) dy[i] = dydx[i] - dy[i] * invdx;
            g.sync();
            if (!stage_solve<G, MT>(g, M, s, invdx, dy, tmp)) return 2;
            cc.solves++;
            // dy2 = vGreat as soon as one |dy_i| > sqrt(vGreat)
            double b = 0, big = 0;
            for (int i = g.rank; i < n; i += G) {
                if (fabs(dy[i]) > 1e150) big = 1;
                const double q = dy[i] / scale[i];
                b += q * q;
            }
            gsum2(g, b, big, s.red);
            const double dy2 = big > 0 ? 1e300 : sqrt(b);
            st.theta = dy2 / fmax(1.0, dy1 + kSmall);
            if (st.theta > 1.0) return 0;
        }
        rhs_eval<G, MT>(g, M, s, p, yTemp, dy, 1);
        cc.rhs++;
        if (!stage_solve<G, MT>(g, M, s, invdx, dy, tmp)) return 2;
        cc.solves++;
    }
    for (int i = g.rank; i < n; i += G) ySeq[i] = yTemp[i] + dy[i];
    g.sync();
    return 1;
}

struct SeulexStep { double dxTry; bool first, last, reject, prevReject, failed, needFp64; };

template<int G, class MT>
__device__ __noinline__ void seulex_step(const Grp<G>& g, const DevMech& M, const KOpts& o, const Slot<MT>& s,
                            const Slot<double>& sd, double p, const SeulexConst& sc, SeulexState& st,
                            double& x, SeulexStep& step, CellCounters& cc) {
    const int n = M.n;
    double *y = s.v(0), *y0_ = s.v(1), *ySeq = s.v(2), *scale = s.v(3), *k9 = s.v(7);
    double* table = s.table;
    const double jacRedo = fmin(1e-4, o.relTol);
    st.temp[0] = 1e15;
    double dx = step.dxTry;
    for (int i = g.rank; i < n; i += G) {
        y0_[i] = y[i];
        scale[i] = o.absTol + o.relTol * fabs(y[i]);
    }
    g.sync();
    st.dxOpt[0] = fabs(0.1 * dx);
    if (step.first || step.prevReject) st.theta = 2 * jacRedo;
    if (step.first) {
        const double logTol = -log10(o.relTol + o.absTol) * 0.6 + 0.5;
        int kt = (int)logTol;
        kt = kt < kKMax - 1 ? kt : kKMax - 1;
        st.kTarg = kt > 1 ? kt : 1;
    }
    bool jacUpdated = false;
    if (st.theta > jacRedo) {
        jacobian_into<G, MT>(g, M, s, sd, p, y, k9, o.jacobian);
        cc.jac++;
        jacUpdated = true;
    }
    int k = 0;
    double dxNew = fabs(dx);
    bool firstk = true;
    int passes = 0;
    while (firstk || step.reject) {
        if (++passes > o.maxRejects) { step.failed = true; return; }
        dx = dxNew;
        firstk = false;
        step.reject = false;
        double errOld = 0;
        cc.attempts++;
        for (k = 0; k <= st.kTarg + 1; k++) {
            const int ok = seul<G, MT>(g, M, s, p, sc, st, dx, k, cc);
            if (ok == 2) { step.needFp64 = true; return; }
            if (ok == 0) { step.reject = true; dxNew = fabs(dx) * 0.5; break; }
            if (k == 0) {
                for (int i = g.rank; i < n; i += G) y[i] = ySeq[i];
            } else {
                for (int i = g.rank; i < n; i += G) table[(k - 1) * n + i] = ySeq[i];
            }
            g.sync();
            if (k != 0) {
                // extrapolate (OptSeulex.C:711-734); each thread owns its columns i
                for (int j = k - 1; j > 0; j--) {
                    const double cf = seulex_coeff(sc, k, j);
                    for (int i = g.rank; i < n; i += G)
                        table[(j - 1) * n + i] = table[j * n + i] + cf * (table[j * n + i] - table[(j - 1) * n + i]);
                }
                const double c0 = seulex_coeff(sc, k, 0);
                double e2 = 0;
                for (int i = g.rank; i < n; i += G) {
                    const double yi = table[i] + c0 * (table[i] - y[i]);
                    y[i] = yi;
                    const double sc_i = o.absTol + o.relTol * fabs(y0_[i]);
                    scale[i] = sc_i;
                    const double q = (yi - table[i]) / sc_i;
                    e2 += q * q;
                }
                e2 = gsum(g, e2, s.red);
                const double err = sqrt(e2 / n);
                if (err > 1 / kSmall || (k > 1 && err >= errOld) || err != err) {
                    step.reject = true;
                    dxNew = fabs(dx) * 0.5;
                    break;
                }
                errOld = fmin(4 * err, 1.0);
                const double expo = 1.0 / (k + 1);
                const double facmin = pow(0.1, expo);
                double fac;
                if (err == 0) fac = 1.0 / facmin;
                else {
                    fac = 0.93 / pow(err / 0.8, expo);
                    fac = fmax(facmin / 4, fmin(1 / facmin, fac));
                }
                st.dxOpt[k] = fabs(dx * fac);
                st.temp[k] = sc.cpu[k] / st.dxOpt[k];
                if ((step.first || step.last) && err <= 1.0) break;
                if (k == st.kTarg - 1 && !step.prevReject && !step.first && !step.last) {
                    if (err <= 1.0) break;
                    else if (err > sc.nSeq[st.kTarg] * sc.nSeq[st.kTarg + 1] * 4.0) {
                        step.reject = true;
                        st.kTarg = k;
                        if (st.kTarg > 1 && st.temp[k - 1] < 0.7 * st.temp[k]) st.kTarg--;
                        dxNew = st.dxOpt[st.kTarg];
                        break;
                    }
                }
                if (k == st.kTarg) {
                    if (err <= 1.0) break;
                    else if (err > sc.nSeq[k + 1] * 2.0) {
                        step.reject = true;
                        if (st.kTarg > 1 && st.temp[k - 1] < 0.7 * st.temp[k]) st.kTarg--;
                        dxNew = st.dxOpt[st.kTarg];
                        break;
                    }
                }
                if (k == st.kTarg + 1) {
                    if (err > 1.0) {
                        step.reject = true;
                        if (st.kTarg > 1 && st.temp[st.kTarg - 1] < 0.7 * st.temp[st.kTarg]) st.kTarg--;
                        dxNew = st.dxOpt[st.kTarg];
                    }
                    break;
                }
            }
        }
        if (step.reject) {
            step.prevReject = true;
            if (!jacUpdated) {
                st.theta = 2.0 * jacRedo;
                jacobian_into<G, MT>(g, M, s, sd, p, y, k9, o.jacobian);
                cc.jac++;
                jacUpdated = true;
            }
        }
    }
    x += dx;
    int kopt;
    if (k == 1) kopt = 2;
    else if (k <= st.kTarg) {
        kopt = k;
        if (st.temp[k - 1] < 0.7 * st.temp[k]) kopt = k - 1;
        else if (st.temp[k] < 0.9 * st.temp[k - 1]) kopt = (k + 1 < kKMax - 1) ? k + 1 : kKMax - 1;
    } else {
        kopt = k - 1;
        if (k > 2 && st.temp[k - 2] < 0.7 * st.temp[k - 1]) kopt = k - 2;
        if (st.temp[k] < 0.9 * st.temp[kopt]) kopt = (k < kKMax - 1) ? k : kKMax - 1;
    }
    if (step.prevReject) {
        st.kTarg = kopt < k ? kopt : k;
        dxNew = fmin(fabs(dx), st.dxOpt[st.kTarg]);
        step.prevReject = false;
    } else {
        if (kopt <= k) dxNew = st.dxOpt[kopt];
        else {
            if (k < st.kTarg && st.temp[k] < 0.9 * st.temp[k - 1]) dxNew = st.dxOpt[k] * sc.cpu[kopt + 1] / sc.cpu[k];
            else dxNew = st.dxOpt[k] * sc.cpu[kopt] / sc.cpu[k];
        }
        st.kTarg = kopt;
    }
    step.dxTry = dxNew;
}

// Internal status: the mixed-precision integration of this cell must be redone in FP64.
constexpr int kNeedFp64 = 100;

template<int G, class MT>
__device__ int seulex_integrate(const Grp<G>& g, const DevMech& M, const KOpts& o, const Slot<MT>& s,
                                const Slot<double>& sd, double p, double xEnd, double& dxTryIO,
                                CellCounters& cc) {
    const SeulexConst sc = seulex_const();
    SeulexState st;
    st.theta = 0; st.kTarg = 1;
    for (int i = 0; i < kIMax; i++) { st.dxOpt[i] = 0; st.temp[i] = 0; }
    SeulexStep step{dxTryIO, true, false, false, false, false, false};
    double x = 0;
    const int n = M.n;
    for (int nStep = 0; nStep < o.maxSteps; nStep++) {
        const double dxTry0 = step.dxTry;
        step.reject = false;
        if ((x + step.dxTry - xEnd) * (x + step.dxTry - 0.0) > 0) { step.last = true; step.dxTry = xEnd - x; }
        if constexpr (sizeof(MT) == 4) {
            // A step whose FP32 factorisation fails the refinement check is
            // redone in FP64 from the step's start: controller state restored,
            // state vector from the step's saved copy (vector 1), and a fresh
            // Jacobian (the failed attempt may have replaced the kept one).
            const SeulexState st0 = st;
            const SeulexStep step0 = step;
            seulex_step<G, MT>(g, M, o, s, sd, p, sc, st, x, step, cc);
            if (step.needFp64) {
                cc.fallbacks++;
                st = st0;
                step = step0;
                st.theta = 1e300;
                for (int i = g.rank; i < n; i += G) s.v(0)[i] = s.v(1)[i];
                g.sync();
                seulex_step<G, double>(g, M, o, sd, sd, p, sc, st, x, step, cc);
            }
        } else {
            seulex_step<G, MT>(g, M, o, s, sd, p, sc, st, x, step, cc);
        }
        if (step.needFp64) return kNeedFp64;
        if (step.failed) return FCS_CELL_DT_UNDERFLOW;
        cc.accepted++;
        double bad = 0;
        for (int i = g.rank; i < n; i += G) if (!(s.v(0)[i] == s.v(0)[i])) bad = 1;
        if (gsum(g, bad, s.red) > 0) return FCS_CELL_NONFINITE;
        if (!(step.dxTry == step.dxTry) || step.dxTry <= 0) return FCS_CELL_DT_UNDERFLOW;
        if ((x - xEnd) * (xEnd - 0.0) >= 0) {
            if (nStep > 0 && step.last) step.dxTry = dxTry0;
            dxTryIO = step.dxTry;
            return FCS_CELL_OK;
        }
        step.first = false;
        if (step.reject) step.prevReject = true;
    }
    return FCS_CELL_MAX_STEPS;
}

// ------------------------------------------------------------------------
// kernels

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Persistent integration kernel: cell groups pull work from queue->head.
template<int G, class MT>
__global__ void __launch_bounds__(G == 32 ? 256 : G)
integrate_kernel(const DevMech M, const KOpts o, const SlotLayout L, CellIO io, WorkQueue q,
                 char* __restrict__ gws) {
    extern __shared__ __align__(16) char smem[];
    Grp<G> g;
    g.rank = threadIdx.x % G;
    const int gidInBlock = threadIdx.x / G;
    const int groupsPerBlock = blockDim.x / G;
    char* base;
    if (gws) base = gws + (size_t)(blockIdx.x * groupsPerBlock + gidInBlock) * L.bytes;
    else base = smem + (size_t)gidInBlock * L.bytes;
    const Slot<MT> s = make_slot<MT>(base, L, M);
    const Slot<double> sd = make_slot<double>(base, L, M);
    const int ns = M.ns, n = M.n;
    CellCounters cc;
    long long nCells = 0, nFailed = 0;
    double dtMin = 1e300;
    int* bcast = reinterpret_cast<int*>(s.red + 40);
    const int qn = q.nDev ? *q.nDev : q.n;
    for (;;) {
        if (g.rank == 0) bcast[0] = atomicAdd(q.head, 1);
        g.sync();
        const int idx = bcast[0];
        g.sync();
        if (idx >= qn) break;
        const long long c = q.order ? q.order[idx] : idx;
        const long long nc = io.nCells;
        const double deltaT = io.dtPerCell ? io.dtPerCell[c] : io.deltaT;
        const double T0 = io.T[c];
        const double p = io.p[c];
        double* y = s.v(0);
        for (int i = g.rank; i < ns; i += G) {
            const double Yi = io.Y[(size_t)i * nc + c];
            y[i] = Yi > 0 ? Yi : 0.0;
        }
        if (g.rank == 0) y[ns] = T0;
        g.sync();
        const double subDt0 = io.subDt[c];
        double subDt = subDt0;
        const long long att0 = cc.attempts;
        int st = FCS_CELL_OK;
        double timeLeft = deltaT;
        while (timeLeft > kSmall) {
            const double dtc = timeLeft;
            if (o.solver == FCS_SOLVER_SEULEX) {
                st = seulex_integrate<G, MT>(g, M, o, s, sd, p, dtc, subDt, cc);
                if constexpr (sizeof(MT) == 4) {
                    if (st == kNeedFp64) {
                        // redo the whole cell in FP64 from its initial state
                        cc.fallbacks++;
                        for (int i = g.rank; i < ns; i += G) {
                            const double Yi = io.Y[(size_t)i * nc + c];
                            y[i] = Yi > 0 ? Yi : 0.0;
                        }
                        if (g.rank == 0) y[ns] = T0;
                        g.sync();
                        subDt = subDt0;
                        st = seulex_integrate<G, double>(g, M, o, sd, sd, p, dtc, subDt, cc);
                    }
                }
            } else {
                st = rosenbrock_integrate<G, MT>(g, M, o, s, sd, p, dtc, subDt, cc);
            }
            timeLeft -= dtc;
            if (st != FCS_CELL_OK) break;
        }
        nCells++;
        if (st != FCS_CELL_OK) nFailed++;
        const double rho0 = io.rho0[c];
        for (int i = g.rank; i < ns; i += G) {
            const double Yn = y[i] > 0 ? y[i] : 0.0;
            const size_t a = (size_t)i * nc + c;
            const double Y0 = io.Y[a];
            if (io.RR) io.RR[a] = (Yn * rho0 - Y0 * rho0) / deltaT;
            io.Y[a] = Yn;
        }
        if (g.rank == 0) {
            io.T[c] = y[ns];
            dtMin = fmin(dtMin, subDt);
            io.subDt[c] = subDt < o.dtChemMax ? subDt : o.dtChemMax;
            if (io.status) io.status[c] = st;
            if (io.attempts) io.attempts[c] = (int)(cc.attempts - att0);
        }
        g.sync();
    }
    if (g.rank == 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_CELLS]), (unsigned long long)nCells);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_FAILED]), (unsigned long long)nFailed);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_ATTEMPTS]), (unsigned long long)cc.attempts);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_ACCEPTED]), (unsigned long long)cc.accepted);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_JAC]), (unsigned long long)cc.jac);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_LU]), (unsigned long long)cc.lu);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_RHS]), (unsigned long long)cc.rhs);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_SOLVES]), (unsigned long long)cc.solves);
        atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[ST_FALLBACK]), (unsigned long long)cc.fallbacks);
        if (nCells) atomicMin(io.dtMinBits, dbits(dtMin));
    }
}

// f(y) per cell: one group per cell, Y read-only (copied into the slot)
template<int G, class MT>
__global__ void __launch_bounds__(G == 32 ? 256 : G)
eval_kernel(const DevMech M, const KOpts o, const SlotLayout L, long long nc, const double* __restrict__ p,
            const double* __restrict__ T, const double* __restrict__ rho, const double* __restrict__ Y,
            double* __restrict__ out,
            double* __restrict__ Jout, double* __restrict__ Qdot, int mode, char* __restrict__ gws) {
    extern __shared__ __align__(16) char smem[];
    Grp<G> g;
    g.rank = threadIdx.x % G;
    const int gidInBlock = threadIdx.x / G;
    const int groupsPerBlock = blockDim.x / G;
    const long long c = (long long)blockIdx.x * groupsPerBlock + gidInBlock;
    char* base = gws ? gws + (size_t)(blockIdx.x * groupsPerBlock + gidInBlock) * L.bytes
                     : smem + (size_t)gidInBlock * L.bytes;
    const Slot<MT> s = make_slot<MT>(base, L, M);
    if (c >= nc) return;  // whole group exits together
    const int ns = M.ns, n = M.n;
    double* y = s.v(0);
    double* f = s.v(1);
    for (int i = g.rank; i < ns; i += G) y[i] = Y[(size_t)i * nc + c];
    if (g.rank == 0) y[ns] = T[c];
    g.sync();
    if (mode == 0) {
        rhs_eval<G, MT>(g, M, s, p[c], y, f, 1);
    } else if (mode == 1) {
        const Slot<double> sd = make_slot<double>(base, L, M);
        jac_eval<G, double>(g, M, sd, p[c], y, f, sd.J, o.jacobian);
        for (int idx = g.rank; idx < n * n; idx += G) {
            const int i = idx / n, j = idx - i * n;
            Jout[(size_t)c * n * n + idx] = sd.J[(size_t)i * s.ld + j];
        }
    } else if (mode == 2) {
        const double qd = rates_eval<G, MT>(g, M, s, p[c], T[c], rho[c], y, f);
        if (Qdot && g.rank == 0) Qdot[c] = qd;
    } else {
        const double tc = tc_eval<G, MT>(g, M, s, p[c], T[c], rho[c], y);
        if (g.rank == 0) out[c] = tc;
        return;
    }
    g.sync();
    const int nout = mode == 2 ? ns : n;
    for (int i = g.rank; i < nout; i += G) out[(size_t)i * nc + c] = f[i];
}

// ------------------------------------------------------------------------
// host-side launchers (instantiations)

template<int G, class MT>
inline cudaError_t launch_integrate_t(const LaunchCfg& lc, const DevMech& M, const KOpts& o,
                                      const SlotLayout& L, const CellIO& io, const WorkQueue& q,
                                      char* gws, cudaStream_t st) {
    auto k = integrate_kernel<G, MT>;
    const size_t sm = gws ? 0 : (size_t)L.bytes * (lc.block / G);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    // Slots in shared memory: all of the unified L1/shared memory as shared
    // memory (the slots set how many groups reside per SM).  Slots in the
    // global workspace: all of it as L1, which then caches the slots.
    {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             gws ? (int)cudaSharedmemCarveoutMaxL1
                                                 : (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
    }
    k<<<lc.grid, lc.block, sm, st>>>(M, o, L, io, q, gws);
    return cudaGetLastError();
}

template<int G, class MT>
inline cudaError_t launch_eval_t(const LaunchCfg& lc, const DevMech& M, const KOpts& o, const SlotLayout& L,
                                 long long nc, const double* p, const double* T, const double* rho,
                                 const double* Y, double* out, double* J, double* Qdot, int mode, char* gws,
                                 cudaStream_t st) {
    auto k = eval_kernel<G, MT>;
    const size_t sm = gws ? 0 : (size_t)L.bytes * (lc.block / G);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    k<<<lc.grid, lc.block, sm, st>>>(M, o, L, nc, p, T, rho, Y, out, J, Qdot, mode, gws);
    return cudaGetLastError();
}

template<int G, class MT>
inline cudaError_t attrs_t(int* maxThreadsOut, int* regsOut) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, integrate_kernel<G, MT>);
    if (e != cudaSuccess) return e;
    *maxThreadsOut = a.maxThreadsPerBlock;
    *regsOut = a.numRegs;
    return cudaSuccess;
}

}  // namespace fcs
