#pragma once
// fcs_lane.cuh -- the lane-per-cell mapping of the Rosenbrock-family
// integrator (OptRodas34, OptRosenbrock34, OptRodas23, OptRosenbrock23).
//
// One thread integrates one cell from start to end of the CFD step.  The 32
// lanes of a warp therefore run the same instruction stream on 32 different
// cells: every FP64 instruction carries 32 useful lanes, no barrier or
// cross-lane reduction is needed, and the mechanism data each instruction
// reads (one reaction record, one species' coefficients) is the same address
// for the whole warp (a broadcast from L1).  The cells' working sets live in
// a global-memory workspace interleaved across the lanes (fcs_lane_layout.h),
// so each per-lane array access of a warp is one 256-byte transaction.
//
// The attempt (Jacobian, LU, stages, error norm) is identical code for every
// cell; only the step-size controller and the cell hand-over differ between
// lanes.  A lane whose cell is done takes the next cell from the device work
// queue on its own (warp-aggregated atomic), so the lanes of a warp stay busy
// until the queue runs dry.
//
// Arithmetic follows the cell-group kernels (fcs_kernels.cuh) operation by
// operation -- the same rate expressions, the same order of every species and
// Jacobian accumulation (reaction order), the same LU with the reference's
// panel-local pivoting (the delayed 4-column update below applies each
// element's multiply-adds in the same order as the column-by-column
// version), the same solves -- except that the sums over species of the
// mixture scalars (rho M, Cp M, ...) run serially here instead of as
// butterfly reductions.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fcs_device.cuh"
#include "fcs_kernels.cuh"
#include "fcs_lane_layout.h"
#include "fcs_launch.h"

namespace fcs {

constexpr int kLanes = 32;

// A per-lane array: element e of this lane's array at p[e * 32].
template<class T>
struct LA {
    T* p;
    __device__ __forceinline__ T& operator[](int e) const { return p[(size_t)e * kLanes]; }
    __device__ __forceinline__ LA operator+(int e) const { return LA{p + (size_t)e * kLanes}; }
};

struct LaneSlot {
    int n, ns;
    LA<double> A, vec, C, B, Binv, Cp, Ha, dBdT, Mtb, tbF, invD;
    LA<int> piv;
    LA<float> LU32, x32;   // mixed precision
    LA<double> dr, dc;     // mixed precision equilibration
    LA<double> q, dq;      // per-reaction net rate and d/dT
    __device__ __forceinline__ LA<double> v(int k) const { return vec + k * n; }
};

__device__ __forceinline__ LaneSlot make_lane_slot(double* ws, const LaneLayout& L) {
    // ws: this warp's workspace; lane offset applied here
    const int lane = threadIdx.x & 31;
    double* base = ws + lane;
    LaneSlot s;
    s.n = L.n;
    s.ns = L.ns;
    s.A = LA<double>{base + (size_t)L.offA * kLanes};
    s.vec = LA<double>{base + (size_t)L.offVec * kLanes};
    const LA<double> sp{base + (size_t)L.offSp * kLanes};
    s.C = sp; s.B = sp + L.ns; s.Binv = sp + 2 * L.ns; s.Cp = sp + 3 * L.ns; s.Ha = sp + 4 * L.ns;
    s.dBdT = sp + 5 * L.ns;
    const int nt = L.nTB > 0 ? L.nTB : 1;
    s.Mtb = LA<double>{base + (size_t)L.offTb * kLanes};
    s.tbF = s.Mtb + nt;
    s.invD = LA<double>{base + (size_t)L.offInvD * kLanes};
    s.piv = LA<int>{reinterpret_cast<int*>(ws + (size_t)L.offPiv * kLanes) + lane};
    s.LU32 = LA<float>{reinterpret_cast<float*>(ws + (size_t)L.offLU32 * kLanes) + lane};
    s.dr = LA<double>{base + (size_t)L.offScale * kLanes};
    s.dc = s.dr + L.n;
    s.x32 = LA<float>{reinterpret_cast<float*>(ws + (size_t)L.offX32 * kLanes) + lane};
    s.q = LA<double>{base + (size_t)L.offRx * kLanes};
    s.dq = s.q + (L.nr > 0 ? L.nr : 1);
    return s;
}

// A mechanism array indexed like a per-lane one (the same address in every
// lane): lane_map inputs.
struct LAC {
    const double* p;
    __device__ __forceinline__ double operator[](int e) const { return __ldg(p + e); }
};
// eff[e] * w
struct LAE {
    const double* p;
    double w;
    __device__ __forceinline__ double operator[](int e) const { return __ldg(p + e) * w; }
};

// Memory-level parallelism: a lane's array accesses go to L1/L2/HBM, so a
// loop whose iterations each wait for their own load runs at the memory
// latency.  The loops below issue the loads of several elements before they
// use or store any of them (the compiler cannot move a load above an earlier
// store to a per-lane array, which might alias).

// out[i] = f(in[i]...) for i < n, four elements per step
template<class F, class... In>
__device__ __forceinline__ void lane_map(int n, LA<double> out, F f, In... in) {
    int i = 0;
    for (; i + 4 <= n; i += 4) {
        double r0 = f(in[i]...), r1 = f(in[i + 1]...), r2 = f(in[i + 2]...), r3 = f(in[i + 3]...);
        out[i] = r0; out[i + 1] = r1; out[i + 2] = r2; out[i + 3] = r3;
    }
    #pragma unroll 1
    for (; i < n; i++) out[i] = f(in[i]...);
}

// ------------------------------------------------------------------------
// rates

// 1/Kc with the reference's clamp (inv_equilibrium_kc over per-lane arrays)
__device__ __forceinline__ double lane_inv_kc(const RxnInfo& x, const LA<double>& E, const LA<double>& Einv,
                                              const PFactor& pf) {
    double v = E[x.sl[0]];
    #pragma unroll 1
    for (int q = 1; q < x.nl; q++) v *= E[x.sl[q]];
    #pragma unroll 1
    for (int q = 0; q < x.nr; q++) v *= Einv[x.sr[q]];
    if (x.dnu != 0) v *= pressure_factor(pf, x.dnu);
    const double cl = inv_kc_clamp(x);
    return v > cl ? cl : v;
}

// The species values of a reaction with at most 3 reactants and 3 products,
// all loaded before any is used; products of 1..3 factors in the reference's
// order (first factor, then the next ones).
struct Tri { double a, b, c; };
__device__ __forceinline__ Tri lane_load3(const LA<double>& X, const uint8_t* s) {
    return Tri{X[s[0]], X[s[1]], X[s[2]]};  // unused slots hold species 0: a valid address
}
__device__ __forceinline__ double prod3(const Tri& t, int k) {
    double v = t.a;
    if (k > 1) v *= t.b;
    if (k > 2) v *= t.c;
    return v;
}
__device__ __forceinline__ double sum3(const Tri& t, int k) {
    double v = t.a;
    if (k > 1) v += t.b;
    if (k > 2) v += t.c;
    return v;
}
__device__ __forceinline__ bool short_reaction(const RxnInfo& x) { return x.nl <= 3 && x.nr <= 3; }

// 1/Kc of a short reaction from preloaded E (reactants) and 1/E (products)
__device__ __forceinline__ double inv_kc3(const RxnInfo& x, const Tri& e, const Tri& einv, const PFactor& pf) {
    double v = prod3(e, x.nl);
    v *= einv.a;
    if (x.nr > 1) v *= einv.b;
    if (x.nr > 2) v *= einv.c;
    if (x.dnu != 0) v *= pressure_factor(pf, x.dnu);
    const double cl = inv_kc_clamp(x);
    return v > cl ? cl : v;
}

// Third-body concentrations M_t = sum_j eff[t][j] C_j (ThirdBodyFactor1D)
__device__ __forceinline__ void lane_third_body(const DevMech& M, const LaneSlot& s) {
    const int ns = M.ns;
    #pragma unroll 1
    for (int t = 0; t < M.nTB; t++) {
        const double* e = M.eff + (size_t)t * ns;
        double m = 0;
        #pragma unroll 8
        for (int j = 0; j < ns; j++) m = fma(__ldg(&e[j]), s.C[j], m);
        s.Mtb[t] = m;
    }
}

// Forward rate constant of an ordinary (not special-block) reaction; PLOG
// also returns dk/dT.
__device__ __forceinline__ double lane_kf(const DevMech& M, const RxnInfo& x, double p, double logP, double logT,
                                          double invT, double* dkdT) {
    double Kf;
    if (x.kind == FCS_RXN_PLOG) {
        Kf = plog_rate(M, x.plog, p, logP, logT, invT, dkdT);
    } else if (x.tind) {
        Kf = x.A;
        *dkdT = 0;
    } else {
        Kf = x.A * fast_exp(fma(x.beta, logT, -(x.Ta * invT)));
        *dkdT = Kf * (fma(x.Ta, invT, x.beta) * invT);
    }
    return Kf;
}

// w_i = sum over the incidence list of species i (reaction order) of +-q[r],
// four entries' loads at a time: the same order as the cell-group gather.
__device__ __forceinline__ double lane_gather(const DevMech& M, const LA<double>& q, int i) {
    const int e1 = __ldg(&M.incOff[i + 1]);
    int e = __ldg(&M.incOff[i]);
    double w = 0.0;
    for (; e + 4 <= e1; e += 4) {
        const int v0 = __ldg(&M.inc[e]), v1 = __ldg(&M.inc[e + 1]), v2 = __ldg(&M.inc[e + 2]), v3 = __ldg(&M.inc[e + 3]);
        const double q0 = q[v0 >> 1], q1 = q[v1 >> 1], q2 = q[v2 >> 1], q3 = q[v3 >> 1];
        w = (v0 & 1) ? w + q0 : w - q0;
        w = (v1 & 1) ? w + q1 : w - q1;
        w = (v2 & 1) ? w + q2 : w - q2;
        w = (v3 & 1) ? w + q3 : w - q3;
    }
    #pragma unroll 1
    for (; e < e1; e++) {
        const int v = __ldg(&M.inc[e]);
        const double qq = q[v >> 1];
        w = (v & 1) ? w + qq : w - qq;
    }
    return w;
}

// RHS: FastChemistryModel::derivatives (FastChemistryModel.C:194-273 for mode
// 1, 340-417 for mode 2) over OptReaction::dNdtByV (ReactionRate.C:732-1503).
// YT is clamped (Y >= 0) in place; out[0..n) receives dY/dt and dT/dt.
__device__ __noinline__ void lane_rhs(const DevMech& M, const LaneSlot& s, double p, LA<double> YT,
                                      LA<double> out, int mode) {
    const int ns = M.ns;
    const double T = YT[ns];
    const double Tc = clampT(M, T);
    const double RuTByP = kRu * T / p;
    double part = 0;
    {
        int i = 0;
        for (; i + 4 <= ns; i += 4) {
            const double a0 = YT[i], a1 = YT[i + 1], a2 = YT[i + 2], a3 = YT[i + 3];
            const double y0 = a0 > 0 ? a0 : 0.0, y1 = a1 > 0 ? a1 : 0.0, y2 = a2 > 0 ? a2 : 0.0,
                         y3 = a3 > 0 ? a3 : 0.0;
            YT[i] = y0; YT[i + 1] = y1; YT[i + 2] = y2; YT[i + 3] = y3;
            part = fma(y0 * __ldg(&M.invW[i]), RuTByP, part);
            part = fma(y1 * __ldg(&M.invW[i + 1]), RuTByP, part);
            part = fma(y2 * __ldg(&M.invW[i + 2]), RuTByP, part);
            part = fma(y3 * __ldg(&M.invW[i + 3]), RuTByP, part);
        }
        #pragma unroll 1
        for (; i < ns; i++) {
            const double y0 = YT[i];
            const double y = y0 > 0 ? y0 : 0.0;
            YT[i] = y;
            part = fma(y * __ldg(&M.invW[i]), RuTByP, part);
        }
    }
    const double invrhoM = part;
    const double rhoM = 1.0 / invrhoM;
    const double logT = log(Tc), invT = 1.0 / Tc;
    const double Tp = mode == 2 ? T : Tc;
    #pragma unroll 1
    for (int i = 0; i < ns; i += 2) {
        // two species per step: both mass fractions loaded first
        const int i1 = i + 1 < ns ? i + 1 : i;
        const double ya = YT[i], yb = YT[i1];
        #pragma unroll
        for (int u = 0; u < 2; u++) {
            const int k = u ? i1 : i;
            if (u && i1 == i) break;
            const double invW = __ldg(&M.invW[k]);
            s.C[k] = rhoM * invW * (u ? yb : ya);
            const Nasa a = load_nasa(species_coeffs(M, k, Tc));
            const double Ei = fast_exp(gibbs_exponent(a, Tc, invT, logT));
            s.B[k] = Ei;
            s.Binv[k] = 1.0 / Ei;
            const double RuInvW = invW * kRu;
            s.Cp[k] = cp_of(a, Tp, RuInvW);
            s.Ha[k] = ha_of(a, Tp, RuInvW);
        }
    }
    lane_third_body(M, s);
    const PFactor pf = pressure_factors(Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    const int sp0 = M.spBegin, sp1 = M.spBegin + M.nSp;
    #pragma unroll 1
    for (int r = 0; r < M.nr; r++) {
        const RxnInfo x = load_rx(M.rx + r);
        const bool special = r >= sp0 && r < sp1;
        double Kf, Kr = 0, CF, CR;
        if (short_reaction(x)) {
            const Tri cl = lane_load3(s.C, x.sl), cr = lane_load3(s.C, x.sr);
            Tri el{0, 0, 0}, er{0, 0, 0};
            const bool viaKc = special ? x.rev == 1 : x.rev != 0;
            if (viaKc) { el = lane_load3(s.B, x.sl); er = lane_load3(s.Binv, x.sr); }
            const double Mt = x.tb >= 0 ? s.Mtb[x.tb] : 1.0;
            if (special) {
                const SpecialK k = special_rates_m(M, x, Mt, Tc, logT, invT, false);
                Kf = k.Kf;
                Kr = k.Kr;  // non-equilibrium: its own reverse rate
            } else {
                double dk;
                Kf = lane_kf(M, x, p, logP, logT, invT, &dk);
                if (x.tb >= 0) Kf *= Mt;
            }
            if (viaKc) Kr = Kf * inv_kc3(x, el, er, pf);
            CF = prod3(cl, x.nl);
            CR = prod3(cr, x.nr);
        } else {
            if (special) {
                const SpecialK k = special_rates_m(M, x, x.tb >= 0 ? s.Mtb[x.tb] : 1.0, Tc, logT, invT, false);
                Kf = k.Kf;
                Kr = k.Kr;
                if (x.rev == 1) Kr = Kf * lane_inv_kc(x, s.B, s.Binv, pf);
            } else {
                double dk;
                Kf = lane_kf(M, x, p, logP, logT, invT, &dk);
                if (x.tb >= 0) Kf *= s.Mtb[x.tb];
                if (x.rev) Kr = Kf * lane_inv_kc(x, s.B, s.Binv, pf);
            }
            CF = s.C[x.sl[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
            CR = s.C[x.sr[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        }
        s.q[r] = Kf * CF - Kr * CR;
    }
    double cpm = 0, dtd = 0;
    #pragma unroll 1
    for (int i = 0; i < ns; i++) {
        const double w = lane_gather(M, s.q, i);
        const double dY = (__ldg(&M.W[i]) * invrhoM) * w;
        out[i] = dY;
        cpm = fma(YT[i], s.Cp[i], cpm);
        dtd = fma(s.Ha[i], dY, dtd);
    }
    out[ns] = -dtd / cpm;
}

// J[rows of the reaction][j] -/+= d: reactant rows minus, product rows plus,
// in the reference's order (reactants then products).  dup: a species occurs
// more than once among the reaction's rows (then the updates of one element
// must follow each other); otherwise every row is loaded before any is stored.
__device__ __forceinline__ void lane_scatter_column(const RxnInfo& x, LA<double> J, int n, int j, double d,
                                                    bool dup) {
    if (!dup && x.nl <= 3 && x.nr <= 3) {
        double& a0 = J[x.sl[0] * n + j];
        double& a1 = J[x.sl[1] * n + j];
        double& a2 = J[x.sl[2] * n + j];
        double& b0 = J[x.sr[0] * n + j];
        double& b1 = J[x.sr[1] * n + j];
        double& b2 = J[x.sr[2] * n + j];
        const double va0 = a0, va1 = a1, va2 = a2, vb0 = b0, vb1 = b1, vb2 = b2;
        a0 = va0 - d;
        if (x.nl > 1) a1 = va1 - d;
        if (x.nl > 2) a2 = va2 - d;
        b0 = vb0 + d;
        if (x.nr > 1) b1 = vb1 + d;
        if (x.nr > 2) b2 = vb2 + d;
        return;
    }
    #pragma unroll 1
    for (int q = 0; q < x.nl; q++) { double& c = J[x.sl[q] * n + j]; c = c - d; }
    #pragma unroll 1
    for (int q = 0; q < x.nr; q++) { double& c = J[x.sr[q] * n + j]; c = c + d; }
}

__device__ __forceinline__ bool repeated_species(const RxnInfo& x) {
    // participants are warp-uniform: integer compares on the reaction record
    const int m = x.nl + x.nr;
    for (int a = 0; a < m; a++) {
        const int sa = a < x.nl ? x.sl[a] : x.sr[a - x.nl];
        for (int b = a + 1; b < m; b++) {
            const int sb = b < x.nl ? x.sl[b] : x.sr[b - x.nl];
            if (sa == sb) return true;
        }
    }
    return false;
}

// Analytic Jacobian (FastChemistryModel::jacobian, FastChemistryModel.C:489-572,
// over ddNdtByVdcTp, Jacobian.C:5-1004, and the dC/dY conversion,
// Jacobian.C:2814-2858 exact / 4541-4568 fast, 3709-3793 T column and row)
// into J (row-major n x n), f = dy/dt; YT clamped in place.
__device__ __noinline__ void lane_jac(const DevMech& M, const LaneSlot& s, double p, LA<double> YT, LA<double> f,
                                      LA<double> J, int fast) {
    const int ns = M.ns, n = M.n;
    lane_map(ns, YT, [](double y0) { return y0 > 0 ? y0 : 0.0; }, YT);
    const double T = YT[ns];
    const double Tc = clampT(M, T);
    const double RuTByP = (kRu * Tc) / p;
    double rs = 0, mws = 0;
    #pragma unroll 4
    for (int i = 0; i < ns; i++) {
        const double y = YT[i], invW = __ldg(&M.invW[i]);
        rs = fma(RuTByP, y * invW, rs);
        mws = fma(y, invW, mws);
    }
    const double logT = log(Tc), invT = 1.0 / Tc;
    const double rhoM = 1.0 / rs, invRhoM = rs, MW = 1.0 / mws;
    double cpm = 0, dcpm = 0;
    #pragma unroll 1
    for (int i = 0; i < ns; i++) {
        const double y = YT[i], invW = __ldg(&M.invW[i]);
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        s.C[i] = rhoM * y * invW;
        const double Ei = fast_exp(gibbs_exponent(a, Tc, invT, logT));
        s.B[i] = Ei;
        s.Binv[i] = 1.0 / Ei;
        s.dBdT[i] = fma(fma(a.a5, invT, a.a0), invT,
                        fma(fma(fma(a.a4 * 0.2, Tc, a.a3 * 0.25), Tc, a.a2 * (1.0 / 3.0)), Tc, a.a1 * 0.5));
        const double RuInvW = invW * kRu;
        const double cp = cp_of(a, Tc, RuInvW);
        const double dcp = RuInvW * fma(Tc, fma(Tc, fma(Tc, 4 * a.a4, 3 * a.a3), 2 * a.a2), a.a1);
        s.Cp[i] = cp;
        s.Ha[i] = ha_of(a, Tc, RuInvW);
        cpm = fma(y, cp, cpm);
        dcpm = fma(y, dcp, dcpm);
    }
    const double CpM = cpm, dCpMdT = dcpm;
    lane_third_body(M, s);
    {
        int idx = 0;
        const int m = ns * n;
        for (; idx + 4 <= m; idx += 4) { J[idx] = 0.0; J[idx + 1] = 0.0; J[idx + 2] = 0.0; J[idx + 3] = 0.0; }
        for (; idx < m; idx++) J[idx] = 0.0;
    }
    const PFactor pf = pressure_factors(Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    const int sp0 = M.spBegin, sp1 = M.spBegin + M.nSp;
    #pragma unroll 1
    for (int r = 0; r < M.nr; r++) {
        const RxnInfo x = load_rx(M.rx + r);
        const bool special = r >= sp0 && r < sp1;
        const bool shortr = short_reaction(x);
        double Kf, dKfdT, dKfdC = 0, Kr = 0, dKrdT = 0, dKrdC = 0;
        const bool viaKc = special ? x.rev == 1 : x.rev != 0;
        Tri cl{0, 0, 0}, cr{0, 0, 0};
        double Mt = 1.0;
        if (shortr) {
            cl = lane_load3(s.C, x.sl);
            cr = lane_load3(s.C, x.sr);
        }
        if (x.tb >= 0) Mt = s.Mtb[x.tb];
        if (special) {
            const SpecialK k = special_rates_m(M, x, Mt, Tc, logT, invT, true);
            Kf = k.Kf; dKfdT = k.dKfdT; dKfdC = k.dKfdC;
            Kr = k.Kr; dKrdT = k.dKrdT; dKrdC = k.dKrdC;
        } else {
            Kf = lane_kf(M, x, p, logP, logT, invT, &dKfdT);
            if (x.tb >= 0) {
                dKfdC = Kf;
                Kf *= Mt;
                dKfdT *= Mt;
            }
        }
        if (viaKc) {
            // Kr, dKr/dT and dKr/dM through Kc (JF* reversible branch); the Kc
            // term of dKr/dT is dropped when Kc sits on its clamp
            // (JacobianFunctionI.H:246-249)
            double invKc, sv, sl;
            if (shortr) {
                const Tri el = lane_load3(s.B, x.sl), er = lane_load3(s.Binv, x.sr);
                const Tri gl = lane_load3(s.dBdT, x.sl), gr = lane_load3(s.dBdT, x.sr);
                invKc = inv_kc3(x, el, er, pf);
                sv = sum3(gr, x.nr);
                sl = sum3(gl, x.nl);
            } else {
                invKc = lane_inv_kc(x, s.B, s.Binv, pf);
                sv = s.dBdT[x.sr[0]];
                #pragma unroll 1
                for (int q = 1; q < x.nr; q++) sv += s.dBdT[x.sr[q]];
                sl = s.dBdT[x.sl[0]];
                #pragma unroll 1
                for (int q = 1; q < x.nl; q++) sl += s.dBdT[x.sl[q]];
            }
            const double dKcdTByKc = (sv - sl) - x.dnu * invT;
            Kr = Kf * invKc;
            dKrdT = dKfdT * invKc - (invKc < inv_kc_clamp(x) ? Kr * dKcdTByKc : 0.0);
            dKrdC = dKfdC * invKc;
        }
        double CF, CR;
        if (shortr) {
            CF = prod3(cl, x.nl);
            CR = prod3(cr, x.nr);
        } else {
            CF = s.C[x.sl[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
            CR = s.C[x.sr[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        }
        s.q[r] = Kf * CF - Kr * CR;
        s.dq[r] = dKfdT * CF - dKrdT * CR;
        if (x.tb >= 0) s.tbF[x.tb] = dKfdC * CF - dKrdC * CR;
        // d q / d C_j for each reactant occurrence j: Kf times the other
        // reactant concentrations (the first occurrence of j skipped),
        // scattered down column j to the rows of the reaction
        const bool dup = repeated_species(x);
        #pragma unroll 1
        for (int qa = 0; qa < x.nl; qa++) {
            const int j = x.sl[qa];
            double d = Kf;
            if (shortr && !dup) {
                // distinct reactants: the occurrence skipped is qa itself
                if (qa != 0) d *= cl.a;
                if (qa != 1 && x.nl > 1) d *= cl.b;
                if (qa != 2 && x.nl > 2) d *= cl.c;
            } else {
                bool skipped = false;
                #pragma unroll 1
                for (int q = 0; q < x.nl; q++) {
                    if (!skipped && x.sl[q] == j) { skipped = true; continue; }
                    d *= s.C[x.sl[q]];
                }
            }
            lane_scatter_column(x, J, n, j, d, dup);
        }
        if (x.rev) {
            #pragma unroll 1
            for (int qb = 0; qb < x.nr; qb++) {
                const int j = x.sr[qb];
                double d = -Kr;
                if (shortr && !dup) {
                    if (qb != 0) d *= cr.a;
                    if (qb != 1 && x.nr > 1) d *= cr.b;
                    if (qb != 2 && x.nr > 2) d *= cr.c;
                } else {
                    bool skipped = false;
                    #pragma unroll 1
                    for (int q = 0; q < x.nr; q++) {
                        if (!skipped && x.sr[q] == j) { skipped = true; continue; }
                        d *= s.C[x.sr[q]];
                    }
                }
                lane_scatter_column(x, J, n, j, d, dup);
            }
        }
    }
    // third-body columns, J_ij += nu_i w_t E_tj (JF* third-body block)
    #pragma unroll 1
    for (int e = 0; e < M.nTbInc; e++) {
        const int v = __ldg(&M.tbInc[e]);
        const int i = v >> 16, t = (v >> 1) & 0x7fff;
        const double w = s.tbF[t];
        const double* eff = M.eff + (size_t)t * ns;
        LA<double> row = J + i * n;
        if (v & 1) lane_map(ns, row, [](double a, double b) { return a + b; }, row, LAE{eff, w});
        else lane_map(ns, row, [](double a, double b) { return a - b; }, row, LAE{eff, w});
    }
    // rows: production rate, temperature column and the dC/dY conversion
    // (diagonal scaling + rank-1 correction)
    double dtd = 0, dd = 0;
    #pragma unroll 1
    for (int i = 0; i < ns; i++) {
        LA<double> row = J + i * n;
        const double w = lane_gather(M, s.q, i);
        const double tc = lane_gather(M, s.dq, i);
        const double WiByrhoM = invRhoM * __ldg(&M.W[i]);
        const double dY = w * WiByrhoM;
        double S = 0;
        #pragma unroll 8
        for (int k = 0; k < ns; k++) S = fma(row[k], s.C[k], S);
        const double tcol = WiByrhoM * (tc - S * invT) + invT * dY;
        if (fast) {
            lane_map(ns, row, [=](double a, double invWj) { return WiByrhoM * (a * (rhoM * invWj)) + (MW * invWj) * dY; },
                     row, LAC{M.invW});
        } else {
            const double K = dY - WiByrhoM * S;
            const double Wi = __ldg(&M.W[i]);
            lane_map(ns, row, [=](double a, double invWj) { return fma(a, Wi * invWj, (MW * invWj) * K); },
                     row, LAC{M.invW});
        }
        row[ns] = tcol;
        f[i] = dY;
        dtd = fma(s.Ha[i], dY, dtd);
        dd += dY * s.Cp[i] + tcol * s.Ha[i];
    }
    const double dTdt = -dtd / CpM;
    // temperature row (ddTdtdYT)
    #pragma unroll 1
    for (int j = 0; j < ns; j++) {
        double v = 0;
        #pragma unroll 8
        for (int i = 0; i < ns; i++) v -= J[i * n + j] * s.Ha[i];
        v -= s.Cp[j] * dTdt;
        J[ns * n + j] = v / CpM;
    }
    J[ns * n + ns] = (-dd - dTdt * dCpMdT) / CpM;
    f[ns] = dTdt;
}

// ------------------------------------------------------------------------
// linear algebra of one attempt, per lane

// FP64: A = c I - J in place
__device__ __noinline__ void lane_form_iteration(LA<double> A, int n, double c) {
    lane_map(n * n, A, [](double a) { return -a; }, A);
    #pragma unroll 4
    for (int i = 0; i < n; i++) { double& d = A[i * n + i]; d = d + c; }
}

// choose_pivot (LUsolver.C:106-246 panel rules) over a per-lane matrix
template<class T>
__device__ __forceinline__ int lane_choose_pivot(const LA<T>& A, int n, int k, int pos, int size) {
    const int cand = size - pos;
    if (cand <= 1) return k;
    if (pos == 0 && size >= 3) {
        int best = 0;
        double t = 0;
        #pragma unroll 1
        for (int c = 0; c < size; c++) {
            const double v = fabs(double(A[(k + c) * n + k]));
            if (t < v) { best = c; t = v; }
        }
        return k + best;
    }
    if (size == 4 && pos == 1) {
        // LUsolver.C:169-185: the running maximum keeps the signed value of row 2
        double t = fabs(double(A[k * n + k]));
        int best = 0;
        const double v1 = double(A[(k + 1) * n + k]);
        if (t < fabs(v1)) { best = 1; t = v1; }
        if (t < fabs(double(A[(k + 2) * n + k]))) best = 2;
        return k + best;
    }
    return (fabs(double(A[k * n + k])) < fabs(double(A[(k + 1) * n + k]))) ? k + 1 : k;
}

// LU with the reference's panel-local pivoting (LUsolver.C:106-246,
// 503-660, 3058-3143), blocked by panels of four columns: the panel's
// columns are factored and updated eagerly, the panel's U rows and the
// trailing block receive the panel's rank-4 update afterwards, each element
// in the same multiply-add order as the column-by-column factorisation.
// T: double (FP64 method) or float (the mixed method's FP32 factors; the
// reciprocal pivots are kept in double, rounded to float as in the cell groups).
template<class T>
__device__ __noinline__ void lane_lu(LA<T> A, int n, LA<int> piv, LA<double> invD) {
    const int rem = n & 3;
    int k0 = 0;
    #pragma unroll 1
    while (k0 < n) {
        const bool tail = k0 >= n - rem;
        const int size = tail ? rem : 4;
        if (size == 1) {
            invD[k0] = 1.0 / double(A[k0 * n + k0]);
            piv[k0] = k0;
            break;
        }
        const int k1 = k0 + size;
        // (a) the panel's columns
        #pragma unroll 1
        for (int k = k0; k < k1; k++) {
            const int pos = k - k0;
            const int pr = lane_choose_pivot(A, n, k, pos, size);
            double akk = double(A[pr * n + k]);
            if (akk == 0) akk = kPivEps;
            const T rinv = T(1.0 / akk);
            invD[k] = double(rinv);
            piv[k] = pr;
            if (pr != k) {
                LA<T> rk = A + k * n, rp = A + pr * n;
                int j = 0;
                for (; j + 4 <= n; j += 4) {
                    const T a0 = rk[j], a1 = rk[j + 1], a2 = rk[j + 2], a3 = rk[j + 3];
                    const T b0 = rp[j], b1 = rp[j + 1], b2 = rp[j + 2], b3 = rp[j + 3];
                    rk[j] = b0; rk[j + 1] = b1; rk[j + 2] = b2; rk[j + 3] = b3;
                    rp[j] = a0; rp[j + 1] = a1; rp[j + 2] = a2; rp[j + 3] = a3;
                }
                #pragma unroll 1
                for (; j < n; j++) { const T t = rk[j]; rk[j] = rp[j]; rp[j] = t; }
            }
            // column k below the diagonal times 1/pivot, then the rest of the
            // panel's columns in those rows (u: the pivot row's panel entries)
            const T u1 = k + 1 < k1 ? A[k * n + k + 1] : T(0);
            const T u2 = k + 2 < k1 ? A[k * n + k + 2] : T(0);
            const T u3 = k + 3 < k1 ? A[k * n + k + 3] : T(0);
            const int w = k1 - k - 1;  // remaining panel columns: 0..3
            // two rows per step, both rows' loads issued before any store
            int i = k + 1;
            #pragma unroll 1
            for (; i + 2 <= n; i += 2) {
                LA<T> ri = A + i * n, rj = ri + n;
                const T a = ri[k], c = rj[k];
                const T b1 = w > 0 ? ri[k + 1] : T(0), b2 = w > 1 ? ri[k + 2] : T(0), b3 = w > 2 ? ri[k + 3] : T(0);
                const T d1 = w > 0 ? rj[k + 1] : T(0), d2 = w > 1 ? rj[k + 2] : T(0), d3 = w > 2 ? rj[k + 3] : T(0);
                const T l = a * rinv, m = c * rinv;
                ri[k] = l;
                rj[k] = m;
                if (w > 0) { ri[k + 1] = fma(-l, u1, b1); rj[k + 1] = fma(-m, u1, d1); }
                if (w > 1) { ri[k + 2] = fma(-l, u2, b2); rj[k + 2] = fma(-m, u2, d2); }
                if (w > 2) { ri[k + 3] = fma(-l, u3, b3); rj[k + 3] = fma(-m, u3, d3); }
            }
            if (i < n) {
                LA<T> ri = A + i * n;
                const T a = ri[k];
                const T b1 = w > 0 ? ri[k + 1] : T(0), b2 = w > 1 ? ri[k + 2] : T(0), b3 = w > 2 ? ri[k + 3] : T(0);
                const T l = a * rinv;
                ri[k] = l;
                if (w > 0) ri[k + 1] = fma(-l, u1, b1);
                if (w > 1) ri[k + 2] = fma(-l, u2, b2);
                if (w > 2) ri[k + 3] = fma(-l, u3, b3);
            }
        }
        if (k1 >= n) break;
        // (b) the panel's U rows in the trailing columns
        #pragma unroll 1
        for (int k = k0 + 1; k < k1; k++) {
            LA<T> rk = A + k * n;
            const int nm = k - k0;  // 1..3 earlier panel rows
            const T l0 = rk[k0], l1 = nm > 1 ? rk[k0 + 1] : T(0), l2 = nm > 2 ? rk[k0 + 2] : T(0);
            const LA<T> m0 = A + k0 * n, m1 = A + (k0 + 1) * n, m2 = A + (k0 + 2) * n;
            #pragma unroll 1
            for (int j = k1; j < n; j += 2) {
                const bool two = j + 1 < n;
                const T a0 = rk[j], a1 = two ? rk[j + 1] : T(0);
                const T p0 = m0[j], p1 = two ? m0[j + 1] : T(0);
                const T q0 = nm > 1 ? m1[j] : T(0), q1 = nm > 1 && two ? m1[j + 1] : T(0);
                const T s0 = nm > 2 ? m2[j] : T(0), s1 = nm > 2 && two ? m2[j + 1] : T(0);
                T r0 = fma(-l0, p0, a0), r1 = fma(-l0, p1, a1);
                if (nm > 1) { r0 = fma(-l1, q0, r0); r1 = fma(-l1, q1, r1); }
                if (nm > 2) { r0 = fma(-l2, s0, r0); r1 = fma(-l2, s1, r1); }
                rk[j] = r0;
                if (two) rk[j + 1] = r1;
            }
        }
        // (c) the trailing block: A[i][j] -= sum over the panel's m, in order
        // (here size == 4: the remainder panel is the last one).  Four columns
        // at a time: the panel's U entries of those columns stay in registers
        // while the rows stream past, 8 loads per 16 multiply-adds.
        #pragma unroll 1
        for (int j = k1; j < n; j += 4) {
            const int nj = n - j;  // >= 1; the last chunk holds n % 4 columns
            T u[4][4];
            #pragma unroll
            for (int m = 0; m < 4; m++) {
                const LA<T> um = A + (k0 + m) * n + j;
                #pragma unroll
                for (int c = 0; c < 4; c++) u[m][c] = c < nj ? um[c] : T(0);
            }
            // two rows per step: 16 loads in flight before the stores
            int i = k1;
            #pragma unroll 1
            for (; i + 2 <= n; i += 2) {
                const LA<T> r0 = A + i * n, r1 = r0 + n;
                T l[2][4], a[2][4];
                #pragma unroll
                for (int m = 0; m < 4; m++) { l[0][m] = r0[k0 + m]; l[1][m] = r1[k0 + m]; }
                #pragma unroll
                for (int c = 0; c < 4; c++) {
                    a[0][c] = c < nj ? r0[j + c] : T(0);
                    a[1][c] = c < nj ? r1[j + c] : T(0);
                }
                #pragma unroll
                for (int h = 0; h < 2; h++) {
                    #pragma unroll
                    for (int c = 0; c < 4; c++) {
                        T r = a[h][c];
                        #pragma unroll
                        for (int m = 0; m < 4; m++) r = fma(-l[h][m], u[m][c], r);
                        a[h][c] = r;
                    }
                }
                #pragma unroll
                for (int c = 0; c < 4; c++) {
                    if (c < nj) { r0[j + c] = a[0][c]; r1[j + c] = a[1][c]; }
                }
            }
            if (i < n) {
                const LA<T> ri = A + i * n;
                T l[4], a[4];
                #pragma unroll
                for (int m = 0; m < 4; m++) l[m] = ri[k0 + m];
                #pragma unroll
                for (int c = 0; c < 4; c++) a[c] = c < nj ? ri[j + c] : T(0);
                #pragma unroll
                for (int c = 0; c < 4; c++) {
                    T r = a[c];
                    #pragma unroll
                    for (int m = 0; m < 4; m++) r = fma(-l[m], u[m][c], r);
                    if (c < nj) ri[j + c] = r;
                }
            }
        }
        k0 = k1;
    }
}

// Forward / back substitution with the factors of lane_lu (LUsolver.C:3145-3171,
// 4113-4152): the recorded interchanges, unit-lower forward sweep, upper
// backward sweep times the reciprocal pivots; in place on b.
template<class MT, class VT>
__device__ __noinline__ void lane_lu_solve(const LA<MT> A, int n, const LA<int> piv, const LA<double> invD,
                                           LA<VT> b) {
    #pragma unroll 1
    for (int j = 0; j < n; j++) {
        const int p = piv[j];
        if (p != j) { const VT t = b[j]; b[j] = b[p]; b[p] = t; }
    }
    // Both sweeps take four rows at a time: b[j] is loaded once for the four
    // rows, each row still sums its terms in the order of the row-by-row sweep
    // (the terms of the four rows' own triangle last, in that order).
    int i = 1;
    #pragma unroll 1
    for (; i + 4 <= n; i += 4) {
        const LA<MT> r0 = A + i * n, r1 = r0 + n, r2 = r1 + n, r3 = r2 + n;
        VT a0 = b[i], a1 = b[i + 1], a2 = b[i + 2], a3 = b[i + 3];
        #pragma unroll 4
        for (int j = 0; j < i; j++) {
            const VT bj = b[j];
            a0 = fma(-VT(r0[j]), bj, a0);
            a1 = fma(-VT(r1[j]), bj, a1);
            a2 = fma(-VT(r2[j]), bj, a2);
            a3 = fma(-VT(r3[j]), bj, a3);
        }
        a1 = fma(-VT(r1[i]), a0, a1);
        a2 = fma(-VT(r2[i]), a0, a2);
        a3 = fma(-VT(r3[i]), a0, a3);
        a2 = fma(-VT(r2[i + 1]), a1, a2);
        a3 = fma(-VT(r3[i + 1]), a1, a3);
        a3 = fma(-VT(r3[i + 2]), a2, a3);
        b[i] = a0; b[i + 1] = a1; b[i + 2] = a2; b[i + 3] = a3;
    }
    #pragma unroll 1
    for (; i < n; i++) {
        const LA<MT> ri = A + i * n;
        VT acc = b[i];
        #pragma unroll 8
        for (int j = 0; j < i; j++) acc = fma(-VT(ri[j]), b[j], acc);
        b[i] = acc;
    }
    i = n - 1;
    #pragma unroll 1
    for (; i >= 3; i -= 4) {
        const LA<MT> r0 = A + i * n, r1 = A + (i - 1) * n, r2 = A + (i - 2) * n, r3 = A + (i - 3) * n;
        VT a0 = b[i], a1 = b[i - 1], a2 = b[i - 2], a3 = b[i - 3];
        #pragma unroll 4
        for (int j = n - 1; j > i; j--) {
            const VT bj = b[j];
            a0 = fma(-VT(r0[j]), bj, a0);
            a1 = fma(-VT(r1[j]), bj, a1);
            a2 = fma(-VT(r2[j]), bj, a2);
            a3 = fma(-VT(r3[j]), bj, a3);
        }
        a0 = a0 * VT(invD[i]);
        a1 = fma(-VT(r1[i]), a0, a1);
        a2 = fma(-VT(r2[i]), a0, a2);
        a3 = fma(-VT(r3[i]), a0, a3);
        a1 = a1 * VT(invD[i - 1]);
        a2 = fma(-VT(r2[i - 1]), a1, a2);
        a3 = fma(-VT(r3[i - 1]), a1, a3);
        a2 = a2 * VT(invD[i - 2]);
        a3 = fma(-VT(r3[i - 2]), a2, a3);
        a3 = a3 * VT(invD[i - 3]);
        b[i] = a0; b[i - 1] = a1; b[i - 2] = a2; b[i - 3] = a3;
    }
    #pragma unroll 1
    for (; i >= 0; i--) {
        const LA<MT> ri = A + i * n;
        VT acc = b[i];
        #pragma unroll 8
        for (int j = n - 1; j > i; j--) acc = fma(-VT(ri[j]), b[j], acc);
        b[i] = acc * VT(invD[i]);
    }
}

// ------------------------------------------------------------------------
// Rosenbrock attempts, per lane (same stage arithmetic as fcs_kernels.cuh).
// Vectors: 0 y0, 1 yTemp, 2..6 k1..k5, 7 dy, 8 err, 9 dydx, 10 dfdx, 11 tmp, 12 tcAcc

// Mixed precision: the FP32 factors of Dr (c I - J) Dc with power-of-two row
// and column equilibration (Dr, Dc in s.dr / s.dc); one narrowing per
// element, the scaling exact.
__device__ __noinline__ void lane_form32(const LaneSlot& s, int n) {
    const LA<double> A = s.A;
    const LA<float> L = s.LU32;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        float mx = 0.f;
        int j = 0;
        for (; j + 4 <= n; j += 4) {
            const double a0 = A[i * n + j], a1 = A[i * n + j + 1], a2 = A[i * n + j + 2], a3 = A[i * n + j + 3];
            const float b0 = float(a0), b1 = float(a1), b2 = float(a2), b3 = float(a3);
            L[i * n + j] = b0; L[i * n + j + 1] = b1; L[i * n + j + 2] = b2; L[i * n + j + 3] = b3;
            mx = fmaxf(mx, fmaxf(fmaxf(fabsf(b0), fabsf(b1)), fmaxf(fabsf(b2), fabsf(b3))));
        }
        #pragma unroll 1
        for (; j < n; j++) {
            const float b = float(A[i * n + j]);
            L[i * n + j] = b;
            mx = fmaxf(mx, fabsf(b));
        }
        s.dr[i] = double(pow2_inverse(mx));
    }
    #pragma unroll 1
    for (int j = 0; j < n; j++) {
        float mx = 0.f;
        #pragma unroll 4
        for (int i = 0; i < n; i++) mx = fmaxf(mx, fabsf(L[i * n + j] * float(s.dr[i])));
        s.dc[j] = double(pow2_inverse(mx));
    }
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        const float ri = float(s.dr[i]);
        int j = 0;
        for (; j + 4 <= n; j += 4) {
            const float a0 = L[i * n + j], a1 = L[i * n + j + 1], a2 = L[i * n + j + 2], a3 = L[i * n + j + 3];
            const float c0 = float(s.dc[j]), c1 = float(s.dc[j + 1]), c2 = float(s.dc[j + 2]), c3 = float(s.dc[j + 3]);
            L[i * n + j] = a0 * ri * c0; L[i * n + j + 1] = a1 * ri * c1;
            L[i * n + j + 2] = a2 * ri * c2; L[i * n + j + 3] = a3 * ri * c3;
        }
        #pragma unroll 1
        for (; j < n; j++) L[i * n + j] = L[i * n + j] * ri * float(s.dc[j]);
    }
}

// Mixed solve (as the cell groups' linear_solve_mixed): x0 = Dc LU32^-1 Dr b in
// FP32, r = b - A64 x0 in FP64, x = x0 + Dc LU32^-1 Dr r.  False when the
// correction is not below 1e-3 of the solution (or not finite): the attempt
// is then redone in FP64.
__device__ __noinline__ bool lane_solve_mixed(const LaneSlot& s, int n, LA<double> b, LA<double> tmp) {
    const LA<float> x32 = s.x32, r32 = s.x32 + n;
    #pragma unroll 4
    for (int i = 0; i < n; i++) x32[i] = float(b[i] * s.dr[i]);
    lane_lu_solve<float, float>(s.LU32, n, s.piv, s.invD, x32);
    #pragma unroll 4
    for (int i = 0; i < n; i++) tmp[i] = double(x32[i]) * s.dc[i];
    // the FP64 residual, four rows at a time (tmp[j] loaded once for them)
    int i = 0;
    #pragma unroll 1
    for (; i + 4 <= n; i += 4) {
        const LA<double> A0 = s.A + i * n, A1 = A0 + n, A2 = A1 + n, A3 = A2 + n;
        double r0 = b[i], r1 = b[i + 1], r2 = b[i + 2], r3 = b[i + 3];
        #pragma unroll 4
        for (int j = 0; j < n; j++) {
            const double t = tmp[j];
            r0 = fma(-A0[j], t, r0);
            r1 = fma(-A1[j], t, r1);
            r2 = fma(-A2[j], t, r2);
            r3 = fma(-A3[j], t, r3);
        }
        r32[i] = float(r0 * s.dr[i]);
        r32[i + 1] = float(r1 * s.dr[i + 1]);
        r32[i + 2] = float(r2 * s.dr[i + 2]);
        r32[i + 3] = float(r3 * s.dr[i + 3]);
    }
    #pragma unroll 1
    for (; i < n; i++) {
        const LA<double> Ai = s.A + i * n;
        double r = b[i];
        #pragma unroll 8
        for (int j = 0; j < n; j++) r = fma(-Ai[j], tmp[j], r);
        r32[i] = float(r * s.dr[i]);
    }
    lane_lu_solve<float, float>(s.LU32, n, s.piv, s.invD, r32);
    double dmax = 0, xmax = 0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        const double d = double(r32[i]) * s.dc[i];
        const double x = tmp[i] + d;
        b[i] = x;
        dmax = fmax(dmax, fabs(d));
        xmax = fmax(xmax, fabs(x));
        if (!(d == d) || !(x == x)) dmax = 1e300;
    }
    return dmax <= kRefineTol * xmax && xmax < 1e300;
}

// The iteration matrix of an attempt: the FP64 Jacobian, A = c I - J in
// FP64, factored in FP64 (the FP64 method, or a mixed attempt redone in
// FP64) or in FP32 from its equilibrated copy (MIXED).
template<bool MIXED>
__device__ __forceinline__ void lane_jacobian_and_lu(const DevMech& M, const KOpts& o, const LaneSlot& s, double p,
                                                     double cdiag, bool fp64) {
    lane_jac(M, s, p, s.v(0), s.v(10), s.A, o.jacobian);
    lane_form_iteration(s.A, M.n, cdiag);
    if (MIXED && !fp64) {
        lane_form32(s, M.n);
        lane_lu<float>(s.LU32, M.n, s.piv, s.invD);
    } else {
        lane_lu<double>(s.A, M.n, s.piv, s.invD);
    }
}

template<bool MIXED>
__device__ __forceinline__ bool lane_solve(const LaneSlot& s, int n, LA<double> b, bool fp64) {
    if (MIXED && !fp64) return lane_solve_mixed(s, n, b, s.v(11));
    lane_lu_solve<double, double>(s.A, n, s.piv, s.invD, b);
    return true;
}

__device__ __forceinline__ double lane_err_norm(const KOpts& o, int n, const LA<double>& y0, const LA<double>& yt,
                                                const LA<double>& err) {
    double me = 0;
    #pragma unroll 4
    for (int i = 0; i < n; i++) {
        const double tol = o.absTol + o.relTol * fmax(fabs(y0[i]), fabs(yt[i]));
        const double e = fabs(err[i]) / tol;
        me = (e > me || e != e) ? e : me;
    }
    return me;
}

// OptRodas34::Rodas34Solve (OptRodas34.C:291-882), constants OptRodas34.H:105-149
template<bool MIXED>
__device__ __noinline__ double lane_rodas34(const DevMech& M, const KOpts& o, const LaneSlot& s, double p, double dx,
                                            double invdx, CellCounters& cc, bool fp64) {
    const int n = M.n;
    const LA<double> y0 = s.v(0), yTemp = s.v(1), k1 = s.v(2), k2 = s.v(3), k3 = s.v(4), k4 = s.v(5);
    const LA<double> k5 = s.v(6), dy = s.v(7), err = s.v(8), dydx = s.v(9), dfdx = s.v(10);
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
    const double cdiag = 1.0 * invdx * invgamma;
    lane_jacobian_and_lu<MIXED>(M, o, s, p, cdiag, fp64);
    cc.jac++; cc.lu++; cc.rhs += 5; cc.solves += 6;

    const double dxd1 = dx * d1 + 1;
    lane_map(n, k1, [=](double f) { return dxd1 * f; }, dfdx);
    if (!lane_solve<MIXED>(s, n, k1, fp64)) return -1.0;
    lane_map(n, yTemp, [=](double a, double y) { return fma(a21, a, y); }, k1, y0);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, e1 = c21 * invdx;
        lane_map(n, k2, [=](double a, double f, double g) { return fma(e1, a, fma(dxd2, f, g)); }, k1, dfdx, dydx);
    }
    if (!lane_solve<MIXED>(s, n, k2, fp64)) return -1.0;
    lane_map(n, yTemp, [=](double a, double b, double y) { return fma(a32, b, fma(a31, a, y)); }, k1, k2, y0);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, e1 = c31 * invdx, e2 = c32 * invdx;
        lane_map(n, k3, [=](double a, double b, double f, double g) { return fma(e2, b, fma(e1, a, fma(dxd3, f, g))); },
                 k1, k2, dfdx, dydx);
    }
    if (!lane_solve<MIXED>(s, n, k3, fp64)) return -1.0;
    lane_map(n, yTemp, [=](double a, double b, double c, double y) { return fma(a43, c, fma(a42, b, fma(a41, a, y))); },
             k1, k2, k3, y0);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double dxd4 = dx * d4, e1 = c41 * invdx, e2 = c42 * invdx, e3 = c43 * invdx;
        lane_map(n, k4, [=](double a, double b, double c, double f, double g) {
            return fma(e3, c, fma(e2, b, fma(e1, a, fma(dxd4, f, g))));
        }, k1, k2, k3, dfdx, dydx);
    }
    if (!lane_solve<MIXED>(s, n, k4, fp64)) return -1.0;
    lane_map(n, dy, [=](double a, double b, double c, double d) { return fma(a54, d, fma(a53, c, fma(a52, b, a51 * a))); },
             k1, k2, k3, k4);
    lane_map(n, yTemp, [](double y, double d) { return y + d; }, y0, dy);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double e1 = c51 * invdx, e2 = c52 * invdx, e3 = c53 * invdx, e4 = c54 * invdx;
        lane_map(n, k5, [=](double a, double b, double c, double d, double g) {
            return fma(e4, d, fma(e3, c, fma(e2, b, fma(e1, a, g))));
        }, k1, k2, k3, k4, dydx);
    }
    if (!lane_solve<MIXED>(s, n, k5, fp64)) return -1.0;
    lane_map(n, dy, [](double d, double k) { return d + k; }, dy, k5);
    lane_map(n, yTemp, [](double y, double d) { return y + d; }, y0, dy);
    lane_rhs(M, s, p, yTemp, dydx, 2);
    {
        const double e1 = c61 * invdx, e2 = c62 * invdx, e3 = c63 * invdx, e4 = c64 * invdx, e5 = c65 * invdx;
        lane_map(n, err, [=](double a, double b, double c, double d, double e, double g) {
            return fma(e5, e, fma(e4, d, fma(e3, c, fma(e2, b, fma(e1, a, g)))));
        }, k1, k2, k3, k4, k5, dydx);
    }
    if (!lane_solve<MIXED>(s, n, err, fp64)) return -1.0;
    lane_map(n, yTemp, [](double y, double d, double e) { return y + d + e; }, y0, dy, err);
    return lane_err_norm(o, n, y0, yTemp, err);
}

// OptRosenbrock34::Rosenbrock34Solve (OptRosenbrock34.C:281-678), .H:127-158
template<bool MIXED>
__device__ __noinline__ double lane_ros34(const DevMech& M, const KOpts& o, const LaneSlot& s, double p, double dx,
                                          double invdx, CellCounters& cc, bool fp64) {
    const int n = M.n;
    const LA<double> y0 = s.v(0), yTemp = s.v(1), k1 = s.v(2), k2 = s.v(3), k3 = s.v(4), k4 = s.v(5);
    const LA<double> err = s.v(8), dydx = s.v(9), dfdx = s.v(10);
    const double a21 = 2, a31 = 48.0 / 25.0, a32 = 6.0 / 25.0;
    const double c21 = -8, c31 = 372.0 / 25.0, c32 = 12.0 / 5.0;
    const double c41 = -112.0 / 125.0, c42 = -54.0 / 125.0, c43 = -2.0 / 5.0;
    const double b1 = 19.0 / 9.0, b2 = 1.0 / 2.0, b3 = 25.0 / 108.0, b4 = 125.0 / 108.0;
    const double e1 = 34.0 / 108.0, e2 = 7.0 / 36.0, e4 = 125.0 / 108.0;
    const double d1 = 1.0 / 2.0, d2 = -3.0 / 2.0, d3 = 605.0 / 250.0, d4 = 29.0 / 250.0;
    const double invgamma = 1.0 / (1.0 / 2.0);
    const double cdiag = invdx * invgamma;
    lane_jacobian_and_lu<MIXED>(M, o, s, p, cdiag, fp64);
    cc.jac++; cc.lu++; cc.rhs += 2; cc.solves += 4;

    const double dxd1 = dx * d1 + 1;
    #pragma unroll 1
    for (int i = 0; i < n; i++) k1[i] = dxd1 * dfdx[i];
    if (!lane_solve<MIXED>(s, n, k1, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) yTemp[i] = fma(a21, k1[i], y0[i]);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, f1 = c21 * invdx;
        #pragma unroll 1
        for (int i = 0; i < n; i++) k2[i] = fma(f1, k1[i], fma(dxd2, dfdx[i], dydx[i]));
    }
    if (!lane_solve<MIXED>(s, n, k2, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) yTemp[i] = fma(a32, k2[i], fma(a31, k1[i], y0[i]));
    lane_rhs(M, s, p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, f1 = c31 * invdx, f2 = c32 * invdx;
        #pragma unroll 1
        for (int i = 0; i < n; i++) k3[i] = fma(f2, k2[i], fma(f1, k1[i], fma(dxd3, dfdx[i], dydx[i])));
    }
    if (!lane_solve<MIXED>(s, n, k3, fp64)) return -1.0;
    {
        const double dxd4 = dx * d4, f1 = c41 * invdx, f2 = c42 * invdx, f3 = c43 * invdx;
        #pragma unroll 1
        for (int i = 0; i < n; i++)
            k4[i] = fma(f3, k3[i], fma(f2, k2[i], fma(f1, k1[i], fma(dxd4, dfdx[i], dydx[i]))));
    }
    if (!lane_solve<MIXED>(s, n, k4, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        yTemp[i] = fma(b4, k4[i], fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i]))));
        err[i] = fma(e4, k4[i], fma(e2, k2[i], e1 * k1[i]));
    }
    return lane_err_norm(o, n, y0, yTemp, err);
}

// OptRodas23::Rodas23Solve (OptRodas23.C:202-315), constants OptRodas23.H:113-126
template<bool MIXED>
__device__ __noinline__ double lane_rodas23(const DevMech& M, const KOpts& o, const LaneSlot& s, double p, double dx,
                                            double invdx, CellCounters& cc, bool fp64) {
    const int n = M.n;
    const LA<double> y0 = s.v(0), yTemp = s.v(1), k1 = s.v(2), k2 = s.v(3), k3 = s.v(4);
    const LA<double> dy = s.v(7), err = s.v(8), dydx = s.v(9), dfdx = s.v(10);
    const double d1 = 1.0 / 2.0, d2 = 3.0 / 2.0, a31 = 2, c21 = 4, c31 = 1, c32 = -1;
    const double c41 = 1, c42 = -1, c43 = -8.0 / 3.0;
    const double invgamma = 1.0 / (1.0 / 2.0);
    const double cdiag = invdx * invgamma;
    lane_jacobian_and_lu<MIXED>(M, o, s, p, cdiag, fp64);
    cc.jac++; cc.lu++; cc.rhs += 2; cc.solves += 4;

    const double dxd1 = dx * d1, dxd2 = dx * d2;
    #pragma unroll 1
    for (int i = 0; i < n; i++) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    if (!lane_solve<MIXED>(s, n, k1, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) k2[i] = fma(dxd2, dfdx[i], dfdx[i]) + c21 * k1[i] / dx;
    if (!lane_solve<MIXED>(s, n, k2, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        dy[i] = a31 * k1[i];
        yTemp[i] = y0[i] + dy[i];
    }
    lane_rhs(M, s, p, yTemp, dydx, 1);
    #pragma unroll 1
    for (int i = 0; i < n; i++) k3[i] = dydx[i] + fma(c32, k2[i], c31 * k1[i]) / dx;
    if (!lane_solve<MIXED>(s, n, k3, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        dy[i] = dy[i] + k3[i];
        yTemp[i] = y0[i] + dy[i];
    }
    lane_rhs(M, s, p, yTemp, dydx, 1);
    #pragma unroll 1
    for (int i = 0; i < n; i++) err[i] = dydx[i] + fma(c43, k3[i], fma(c42, k2[i], c41 * k1[i])) / dx;
    if (!lane_solve<MIXED>(s, n, err, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) yTemp[i] = y0[i] + dy[i] + err[i];
    return lane_err_norm(o, n, y0, yTemp, err);
}

// OptRosenbrock23::Rosenbrock23Solve (OptRosenbrock23.C:208-298), constants .H:116-140
template<bool MIXED>
__device__ __noinline__ double lane_ros23(const DevMech& M, const KOpts& o, const LaneSlot& s, double p, double dx,
                                          double invdx, CellCounters& cc, bool fp64) {
    const int n = M.n;
    const LA<double> y0 = s.v(0), yTemp = s.v(1), k1 = s.v(2), k2 = s.v(3), k3 = s.v(4);
    const LA<double> err = s.v(8), dydx = s.v(9), dfdx = s.v(10);
    const double a21 = 1;
    const double c21 = -1.0156171083877702091975600115545, c31 = 4.0759956452537699824805835358067;
    const double c32 = 9.2076794298330791242156818474003;
    const double b1 = 1, b2 = 6.1697947043828245592553615689730, b3 = -0.4277225654321857332623837380651;
    const double e1 = 0.5, e2 = -2.9079558716805469821718236208017, e3 = 0.2235406989781156962736090927619;
    const double gamma = 0.43586652150845899941601945119356, invgamma = 1.0 / gamma;
    const double d1 = 0.43586652150845899941601945119356, d2 = 0.24291996454816804366592249683314;
    const double d3 = 2.1851380027664058511513169485832;
    const double cdiag = invdx * invgamma;
    lane_jacobian_and_lu<MIXED>(M, o, s, p, cdiag, fp64);
    cc.jac++; cc.lu++; cc.rhs += 1; cc.solves += 3;

    const double dxd1 = dx * d1, dxd2 = dx * d2, dxd3 = dx * d3;
    #pragma unroll 1
    for (int i = 0; i < n; i++) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    if (!lane_solve<MIXED>(s, n, k1, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) yTemp[i] = fma(a21, k1[i], y0[i]);
    lane_rhs(M, s, p, yTemp, dydx, 1);
    #pragma unroll 1
    for (int i = 0; i < n; i++) k2[i] = fma(dxd2, dfdx[i], dydx[i]) + c21 * k1[i] / dx;
    if (!lane_solve<MIXED>(s, n, k2, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) k3[i] = fma(dxd3, dfdx[i], dydx[i]) + fma(c32, k2[i], c31 * k1[i]) / dx;
    if (!lane_solve<MIXED>(s, n, k3, fp64)) return -1.0;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
        yTemp[i] = fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i])));
        err[i] = fma(e3, k3[i], fma(e2, k2[i], e1 * k1[i]));
    }
    return lane_err_norm(o, n, y0, yTemp, err);
}

template<bool MIXED>
__device__ __forceinline__ double lane_attempt(const DevMech& M, const KOpts& o, const LaneSlot& s, double p,
                                               double dx, CellCounters& cc, bool fp64) {
    const double invdx = 1.0 / dx;
    switch (o.solver) {
        case FCS_SOLVER_ROSENBROCK34: return lane_ros34<MIXED>(M, o, s, p, dx, invdx, cc, fp64);
        case FCS_SOLVER_RODAS23: return lane_rodas23<MIXED>(M, o, s, p, dx, invdx, cc, fp64);
        case FCS_SOLVER_ROSENBROCK23: return lane_ros23<MIXED>(M, o, s, p, dx, invdx, cc, fp64);
        default: return lane_rodas34<MIXED>(M, o, s, p, dx, invdx, cc, fp64);
    }
}

// ------------------------------------------------------------------------
// the kernel

// Per-lane state of the step-size controller (ODESolve + adaptiveSolve,
// OptRodas34.C:123-289), kept across loop iterations so that every lane runs
// one attempt per iteration whatever its cell's progress.
struct LaneCtl {
    long long c;      // cell, or -1
    double p, deltaT, x, dxTry, dxTry0, dx;
    double sub0;      // the cell's initial sub-step (kept on failure, as ODESolve leaves it)
    int att;          // attempts on this cell
    int nStep, rejects;
    bool last, retry;
    bool redo;        // repeat the last attempt with the same step (mixed precision, now in FP64)
    bool fp64;        // this attempt in FP64: the mixed attempt's refinement check failed
};

// Three resident blocks of 128 threads per SM (the launch shape's default):
// up to 168 registers per thread, so the RHS and Jacobian run without spills.
template<class MT>
__global__ void __launch_bounds__(128, 3)
lane_integrate_kernel(const DevMech M, const KOpts o, const LaneLayout L, CellIO io, WorkQueue q,
                      double* __restrict__ ws) {
    const unsigned FULL = 0xffffffffu;
    constexpr bool kMixed = sizeof(MT) == 4;
    const int lane = threadIdx.x & 31;
    const long long gwarp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const LaneSlot s = make_lane_slot(ws + (size_t)gwarp * L.words * kLanes, L);
    const int ns = M.ns, n = M.n;
    const long long nc = io.nCells;
    const double SAFE = 0.9, ALPHA_INC = 0.2, ALPHA_DEC = 0.25, MIN_SCALE = 0.2, MAX_SCALE = 10;
    const double ratio = 5.904900000000001e-06;  // (MAX_SCALE/SAFE)^(-1/ALPHA_INC)
    const double safeMaxScale = SAFE * MAX_SCALE;
    const int qn = q.nDev ? *q.nDev : q.n;
    const LA<double> y = s.v(0), yTemp = s.v(1);
    CellCounters cc;
    long long nCells = 0, nFailed = 0;
    double dtMin = 1e300;
    LaneCtl k;
    k.c = -1;
    bool exhausted = false;
    for (;;) {
        // 1. lanes without a cell take the next ones from the queue
        const bool want = k.c < 0 && !exhausted;
        const unsigned m = __ballot_sync(FULL, want);
        if (m) {
            const int leader = __ffs(m) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(q.head, __popc(m));
            base = __shfl_sync(FULL, base, leader);
            if (want) {
                const int idx = base + __popc(m & ((1u << lane) - 1));
                if (idx >= qn) {
                    exhausted = true;
                } else {
                    const long long c = q.order ? q.order[idx] : idx;
                    k.c = c;
                    k.p = io.p[c];
                    k.deltaT = io.dtPerCell ? io.dtPerCell[c] : io.deltaT;
                    #pragma unroll 1
                    for (int i = 0; i < ns; i++) {
                        const double Yi = io.Y[(size_t)i * nc + c];
                        y[i] = Yi > 0 ? Yi : 0.0;
                    }
                    y[ns] = io.T[c];
                    k.x = 0;
                    k.sub0 = io.subDt[c];
                    k.dxTry = k.sub0;
                    k.nStep = 0;
                    k.att = 0;
                    k.last = false;
                    k.redo = false;
                    k.fp64 = false;
                    k.retry = false;
                }
            }
        }
        if (!__any_sync(FULL, k.c >= 0)) break;
        int st = -1;  // >= 0: the lane's cell finishes with this status
        if (k.c >= 0) {
            if (!(k.deltaT > kSmall)) {
                st = FCS_CELL_OK;  // nothing to integrate (transientSolve.H's loop does not run)
            } else {
                // 2. the step size of this attempt
                if (!k.retry && !k.redo) {
                    k.dxTry0 = k.dxTry;
                    if ((k.x + k.dxTry - k.deltaT) * (k.x + k.dxTry - 0.0) > 0) {
                        k.last = true;
                        k.dxTry = k.deltaT - k.x;
                    }
                    k.dx = k.dxTry;
                    k.rejects = 0;
                }
                // 3. one attempt (the same code on every lane)
                k.redo = false;
                const double Err = lane_attempt<kMixed>(M, o, s, k.p, k.dx, cc, k.fp64);
                if (kMixed && Err == -1.0) {
                    // the FP32 factors failed the refinement check: the same
                    // attempt again in FP64 (counted once, as in the cell groups)
                    cc.fallbacks++;
                    k.fp64 = true;
                    k.redo = true;
                } else {
                    k.fp64 = false;
                    cc.attempts++;
                    k.att++;
                    // 4. the controller
                    if (Err > 1) {
                        if (++k.rejects > o.maxRejects) {
                            st = FCS_CELL_DT_UNDERFLOW;
                        } else {
                            k.dx *= fmax(SAFE * pow(Err, -ALPHA_DEC), MIN_SCALE);
                            k.retry = true;
                        }
                    } else if (!(Err == Err)) {
                        st = FCS_CELL_NONFINITE;
                    } else {
                        cc.accepted++;
                        k.retry = false;
                        k.x += k.dx;
                        lane_map(n, y, [](double v) { return v; }, yTemp);
                        k.dxTry = (Err > ratio) ? fmin(fmax(SAFE * pow(Err, -ALPHA_INC), MIN_SCALE), MAX_SCALE) * k.dx
                                                : safeMaxScale * k.dx;
                        if ((k.x - k.deltaT) * (k.deltaT - 0.0) >= 0) {
                            if (k.nStep > 0 && k.last) k.dxTry = k.dxTry0;
                            st = FCS_CELL_OK;
                        } else if (++k.nStep >= o.maxSteps) {
                            st = FCS_CELL_MAX_STEPS;
                        }
                    }
                }
            }
        }
        // 5. a finished cell writes its results and frees the lane
        if (st >= 0) {
            const long long c = k.c;
            nCells++;
            if (st != FCS_CELL_OK) nFailed++;
            const double rho0 = io.rho0[c];
            #pragma unroll 1
            for (int i = 0; i < ns; i++) {
                const double Yn = y[i] > 0 ? y[i] : 0.0;
                const size_t a = (size_t)i * nc + c;
                const double Y0 = io.Y[a];
                if (io.RR) io.RR[a] = (Yn * rho0 - Y0 * rho0) / k.deltaT;
                io.Y[a] = Yn;
            }
            io.T[c] = y[ns];
            const double subDt = st == FCS_CELL_OK ? k.dxTry : k.sub0;
            dtMin = fmin(dtMin, subDt);
            io.subDt[c] = subDt < o.dtChemMax ? subDt : o.dtChemMax;
            if (io.status) io.status[c] = st;
            if (io.attempts) io.attempts[c] = k.att;
            k.c = -1;
        }
    }
    // every lane leaves the loop in the same iteration: warp sums, one atomic per warp
    long long v[ST_COUNT] = {};
    v[ST_CELLS] = nCells; v[ST_FAILED] = nFailed; v[ST_ATTEMPTS] = cc.attempts; v[ST_ACCEPTED] = cc.accepted;
    v[ST_JAC] = cc.jac; v[ST_LU] = cc.lu; v[ST_RHS] = cc.rhs; v[ST_SOLVES] = cc.solves;
    v[ST_FALLBACK] = cc.fallbacks;
    unsigned long long dm = nCells ? dbits(dtMin) : ~0ull;
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        #pragma unroll
        for (int t = 0; t < ST_COUNT; t++) v[t] += __shfl_down_sync(FULL, v[t], off);
        const unsigned long long u = __shfl_down_sync(FULL, dm, off);
        dm = u < dm ? u : dm;
    }
    if (lane == 0) {
        #pragma unroll
        for (int t = 0; t < ST_COUNT; t++)
            if (t != ST_SKIPPED && v[t]) atomicAdd(reinterpret_cast<unsigned long long*>(&io.stats[t]),
                                                   (unsigned long long)v[t]);
        if (v[ST_CELLS]) atomicMin(io.dtMinBits, dm);
    }
}

}  // namespace fcs
