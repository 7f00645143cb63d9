// fcs_device.cuh -- device building blocks of the per-cell stiff integrator.
//
// Execution model: a *cell group* of G threads (G = 32: one warp; G = 64..256:
// one thread block) owns one cell at a time and keeps the whole per-cell
// working set in a private slot of shared memory (or of global memory when it
// does not fit): the Jacobian / LU matrices, the stage vectors, the species
// and reaction scratch.  Threads own species rows i = rank (mod G).  All
// scalars that steer control flow (error norms, step sizes) come out of
// butterfly reductions, so every thread of a group holds bit-identical values
// and takes the same branches.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fcs_internal.h"
#include "../../include/fcs.h"

namespace fcs {

// ------------------------------------------------------------------------
// cell group

template<int G>
struct Grp {
    int rank;  // 0..G-1
    __device__ __forceinline__ void sync() const {
        if constexpr (G == 32) __syncwarp();
        else __syncthreads();
    }
};

// Sum over the group; every thread returns the same bits.
template<int G>
__device__ __forceinline__ double gsum(const Grp<G>& g, double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if constexpr (G == 32) {
        return v;
    } else {
        g.sync();
        if ((g.rank & 31) == 0) red[g.rank >> 5] = v;
        g.sync();
        double s = red[0];
#pragma unroll
        for (int w = 1; w < G / 32; w++) s += red[w];
        return s;
    }
}

// Two sums at once (fewer barriers).
template<int G>
__device__ __forceinline__ void gsum2(const Grp<G>& g, double& a, double& b, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if constexpr (G > 32) {
        g.sync();
        if ((g.rank & 31) == 0) { red[g.rank >> 5] = a; red[16 + (g.rank >> 5)] = b; }
        g.sync();
        double s = red[0], t = red[16];
#pragma unroll
        for (int w = 1; w < G / 32; w++) { s += red[w]; t += red[16 + w]; }
        a = s; b = t;
    }
}

template<int G>
__device__ __forceinline__ double gmax(const Grp<G>& g, double v, double* red) {
    // NaN-propagating max: a NaN anywhere makes the result NaN
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = (u > v || u != u) ? u : v;
    }
    if constexpr (G == 32) {
        return v;
    } else {
        g.sync();
        if ((g.rank & 31) == 0) red[g.rank >> 5] = v;
        g.sync();
        double s = red[0];
#pragma unroll
        for (int w = 1; w < G / 32; w++) s = (red[w] > s || red[w] != red[w]) ? red[w] : s;
        return s;
    }
}

// ------------------------------------------------------------------------
// slot layout (byte offsets inside one cell's workspace)

struct SlotLayout {
    int ld;            // matrix leading dimension (odd: conflict-free column walks)
    int offJ;          // Jacobian (MT)
    int offLU;         // LU factors (MT); == offJ when factored in place
    int offVec;        // NV vectors of n doubles
    int offSp;         // 6 species arrays (C, B, Cp, Ha, dBdT, dCpdT) [ns]
    int offInvD;       // [n] double
    int offPiv;        // [n] int
    int offRx;         // Kf, Kr, q, dqdT [nr] each
    int offTb;         // M, dKfdC, dKrdC, CF, CR [nTB] each
    int offTable;      // Seulex extrapolation table [12][n] doubles
    int offRed;        // 48 doubles of reduction / broadcast scratch
    int bytes;         // total, multiple of 16
};

constexpr int kNV = 16;  // stage / work vectors per slot

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// mtBytes: 8 for an FP64 matrix, 4 for FP32; twoMatrices: J kept beside LU
__host__ __device__ inline SlotLayout make_layout(int ns, int nr, int nTB, int mtBytes,
                                                  bool twoMatrices, bool seulex) {
    SlotLayout L;
    const int n = ns + 1;
    L.ld = n | 1;
    int o = 0;
    L.offJ = o;
    o = align16(o + n * L.ld * mtBytes);
    if (twoMatrices) { L.offLU = o; o = align16(o + n * L.ld * mtBytes); }
    else L.offLU = L.offJ;
    L.offVec = o;  o = align16(o + kNV * n * 8);
    L.offSp = o;   o = align16(o + 6 * ns * 8);
    L.offInvD = o; o = align16(o + n * 8);
    L.offPiv = o;  o = align16(o + n * 4);
    L.offRx = o;   o = align16(o + 4 * nr * 8);
    L.offTb = o;   o = align16(o + 5 * (nTB > 0 ? nTB : 1) * 8);
    L.offTable = o;
    if (seulex) o = align16(o + 12 * n * 8);
    L.offRed = o;  o = align16(o + 48 * 8);
    L.bytes = o;
    return L;
}

template<class MT>
struct Slot {
    int ld, n, ns;
    MT* J;
    MT* LU;
    double* vec;      // vec + k*n is vector k
    double *C, *B, *Cp, *Ha, *dBdT, *dCpdT;
    double* invD;
    int* piv;
    double *Kf, *Kr, *q, *dqdT;
    double *Mtb, *tbF, *tbR, *tbCF, *tbCR;
    double* table;
    double* red;
    __device__ double* v(int k) const { return vec + k * n; }
};

template<class MT>
__device__ __forceinline__ Slot<MT> make_slot(char* base, const SlotLayout& L, const DevMech& M) {
    Slot<MT> s;
    s.ld = L.ld; s.n = M.n; s.ns = M.ns;
    s.J = reinterpret_cast<MT*>(base + L.offJ);
    s.LU = reinterpret_cast<MT*>(base + L.offLU);
    s.vec = reinterpret_cast<double*>(base + L.offVec);
    double* sp = reinterpret_cast<double*>(base + L.offSp);
    s.C = sp; s.B = sp + M.ns; s.Cp = sp + 2 * M.ns; s.Ha = sp + 3 * M.ns;
    s.dBdT = sp + 4 * M.ns; s.dCpdT = sp + 5 * M.ns;
    s.invD = reinterpret_cast<double*>(base + L.offInvD);
    s.piv = reinterpret_cast<int*>(base + L.offPiv);
    double* rx = reinterpret_cast<double*>(base + L.offRx);
    s.Kf = rx; s.Kr = rx + M.nr; s.q = rx + 2 * M.nr; s.dqdT = rx + 3 * M.nr;
    double* tb = reinterpret_cast<double*>(base + L.offTb);
    const int nt = M.nTB > 0 ? M.nTB : 1;
    s.Mtb = tb; s.tbF = tb + nt; s.tbR = tb + 2 * nt; s.tbCF = tb + 3 * nt; s.tbCR = tb + 4 * nt;
    s.table = reinterpret_cast<double*>(base + L.offTable);
    s.red = reinterpret_cast<double*>(base + L.offRed);
    return s;
}

// ------------------------------------------------------------------------
// thermo (ThermoFunctionI.H)

__device__ __forceinline__ const double* species_coeffs(const DevMech& M, int i, double Tb) {
    // setPtrCoeffs (ThermoFunctionI.H:1-31)
    const double* base = M.coef + 16 * i;
    if (Tb < M.TcommonMin) return base;
    if (Tb > M.TcommonMax) return base + 8;
    return (Tb < __ldg(&M.Tcommon[i])) ? base : base + 8;
}

struct Nasa { double a0, a1, a2, a3, a4, a5, a6; };

__device__ __forceinline__ Nasa load_nasa(const double* a) {
    Nasa c;
    c.a0 = __ldg(a + 0); c.a1 = __ldg(a + 1); c.a2 = __ldg(a + 2); c.a3 = __ldg(a + 3);
    c.a4 = __ldg(a + 4); c.a5 = __ldg(a + 5); c.a6 = __ldg(a + 6);
    return c;
}

// exponent of exp(-G/RT) (ThermoFunctionI.H:539-636)
__device__ __forceinline__ double gibbs_exponent(const Nasa& a, double T, double invT, double logT) {
    double v = fma(a.a4 * 0.05, T, a.a3 * (1.0 / 12.0));
    v = fma(v, T, a.a2 * (1.0 / 6.0));
    v = fma(v, T, a.a1 * 0.5);
    v = fma(v, T, -(a.a5 * invT));
    v = v + a.a6;
    return fma(a.a0, logT - 1.0, v);
}

__device__ __forceinline__ double cp_of(const Nasa& a, double T, double RuInvW) {
    double v = fma(a.a4, T, a.a3);
    v = fma(v, T, a.a2);
    v = fma(v, T, a.a1);
    v = fma(v, T, a.a0);
    return RuInvW * v;
}

__device__ __forceinline__ double ha_of(const Nasa& a, double T, double RuInvW) {
    double v = fma(a.a4, T * 0.2, a.a3 * 0.25);
    v = fma(v, T, a.a2 * (1.0 / 3.0));
    v = fma(v, T, a.a1 * 0.5);
    v = fma(v, T, a.a0);
    v = fma(v, T, a.a5);
    return RuInvW * v;
}

__device__ __forceinline__ double clampT(const DevMech& M, double T) {
    T = T < M.TlowMin ? M.TlowMin : T;
    T = T > M.ThighMax ? M.ThighMax : T;
    return T;
}

// ------------------------------------------------------------------------
// rate constants

// PLOG: ln k linear in ln p between the bracketing rows, clamped to the end
// rows (ReactionRate.C:577-727, Jacobian.C:798-1000); returns k, sets dk/dT.
__device__ __forceinline__ double plog_rate(const DevMech& M, int ip, double p, double logP,
                                            double logT, double invT, double* dkdT) {
    const int o = __ldg(&M.plogOff[ip]);
    const int len = __ldg(&M.plogOff[ip + 1]) - o;
    const double* R = M.plogRow;
    double lk, dk;
    if (p <= __ldg(&R[4 * o])) {
        const double la = __ldg(&R[4 * o + 2]), b = __ldg(&R[4 * o + 3]), ta = __ldg(&M.plogTa[o]);
        lk = la + b * logT - ta * invT;
        dk = (b + ta * invT) * invT;
    } else if (p >= __ldg(&R[4 * (o + len - 1)])) {
        const int e = o + len - 1;
        const double la = __ldg(&R[4 * e + 2]), b = __ldg(&R[4 * e + 3]), ta = __ldg(&M.plogTa[e]);
        lk = la + b * logT - ta * invT;
        dk = (b + ta * invT) * invT;
    } else {
        int idx = 0;
        for (int j = 0; j < len - 1; j++) {
            if (__ldg(&R[4 * (o + j)]) <= p && p <= __ldg(&R[4 * (o + j + 1)])) { idx = j; break; }
        }
        const int a = o + idx, b = a + 1;
        const double lpa = __ldg(&R[4 * a + 1]), lpb = __ldg(&R[4 * b + 1]);
        const double laa = __ldg(&R[4 * a + 2]), lab = __ldg(&R[4 * b + 2]);
        const double ba = __ldg(&R[4 * a + 3]), bb = __ldg(&R[4 * b + 3]);
        const double ta = __ldg(&M.plogTa[a]), tb = __ldg(&M.plogTa[b]);
        const double fr = (logP - lpa) / (lpb - lpa);
        lk = laa + ba * logT - ta * invT + ((lab - laa) + (bb - ba) * logT - (tb - ta) * invT) * fr;
        dk = invT * (ba + ta * invT + (bb - ba + (tb - ta) * invT) * fr);
    }
    const double k = exp(lk);
    *dkdT = k * dk;
    return k;
}

// Kc = Kp (Pstd/(Ru T))^dnu clamped from below (ReactionFunctionI.H RF11..RF33,
// ChemicalEquilibriumFunctionI.H:14-25)
__device__ __forceinline__ double equilibrium_kc(const RxnInfo& x, const double* B, double PByRT) {
    double num = B[x.sr[0]];
    for (int q = 1; q < x.nr; q++) num *= B[x.sr[q]];
    double den = B[x.sl[0]];
    for (int q = 1; q < x.nl; q++) den *= B[x.sl[q]];
    double Kc = num / den;
    switch (x.dnu) {
        case -2: Kc = Kc * (1 / (PByRT * PByRT)); break;
        case -1: Kc = Kc * (1 / PByRT); break;
        case 1: Kc = Kc * PByRT; break;
        case 2: Kc = Kc * (PByRT * PByRT); break;
        default: break;
    }
    return Kc > kKcClamp ? Kc : kKcClamp;
}

__device__ __forceinline__ RxnInfo load_rx(const RxnInfo* p) {
    // 64-byte record, four 16-byte loads through the read-only path
    RxnInfo x;
    const double2* s = reinterpret_cast<const double2*>(p);
    double2* d = reinterpret_cast<double2*>(&x);
    d[0] = __ldg(s);
    d[1] = __ldg(s + 1);
    d[2] = __ldg(s + 2);
    d[3] = __ldg(s + 3);
    return x;
}

// ------------------------------------------------------------------------
// right-hand side: FastChemistryModel::derivatives (FastChemistryModel.C:194-273
// for mode 1, 340-417 for mode 2) over OptReaction::dNdtByV
// (ReactionRate.C:732-1503).  YT is clamped (Y >= 0) in place.

template<int G, class MT>
__device__ __noinline__ void rhs_eval(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p,
                         double* YT, double* out, int mode) {
    const int ns = M.ns;
    const double T = YT[ns];
    const double Tc = clampT(M, T);
    const double logT = log(Tc), invT = 1.0 / Tc;
    const double RuTByP = kRu * T / p;
    double part = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double y0 = YT[i];
        const double y = y0 > 0 ? y0 : 0.0;
        YT[i] = y;
        part = fma(y * __ldg(&M.invW[i]), RuTByP, part);
    }
    const double invrhoM = gsum(g, part, s.red);
    const double rhoM = 1.0 / invrhoM;
    const double Tp = mode == 2 ? T : Tc;
    for (int i = g.rank; i < ns; i += G) {
        const double invW = __ldg(&M.invW[i]);
        s.C[i] = rhoM * invW * YT[i];
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        s.B[i] = exp(gibbs_exponent(a, Tc, invT, logT));
        const double RuInvW = invW * kRu;
        s.Cp[i] = cp_of(a, Tp, RuInvW);
        s.Ha[i] = ha_of(a, Tp, RuInvW);
    }
    g.sync();
    for (int t = g.rank; t < M.nTB; t += G) {
        const double* e = M.eff + (size_t)t * ns;
        double m = 0;
        for (int j = 0; j < ns; j++) m = fma(__ldg(&e[j]), s.C[j], m);
        s.Mtb[t] = m;
    }
    g.sync();
    const double PByRT = kPstd / (kRu * Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    for (int r = g.rank; r < M.nr; r += G) {
        const RxnInfo x = load_rx(M.rx + r);
        double Kf;
        if (x.kind == FCS_RXN_PLOG) {
            double dk;
            Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dk);
        } else if (x.tind) {
            Kf = x.A;
        } else {
            Kf = x.A * exp(fma(x.beta, logT, -(x.Ta * invT)));
        }
        if (x.tb >= 0) Kf *= s.Mtb[x.tb];
        double Kr = 0;
        if (x.rev) Kr = Kf / equilibrium_kc(x, s.B, PByRT);
        double CF = s.C[x.sl[0]];
        for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
        double CR = s.C[x.sr[0]];
        for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        s.q[r] = Kf * CF - Kr * CR;
    }
    g.sync();
    double cpm = 0, dtd = 0;
    for (int i = g.rank; i < ns; i += G) {
        double w = 0;
        const int e1 = __ldg(&M.incOff[i + 1]);
        for (int e = __ldg(&M.incOff[i]); e < e1; e++) {
            const int v = __ldg(&M.inc[e]);
            const double qq = s.q[v >> 1];
            w = (v & 1) ? w + qq : w - qq;
        }
        const double dY = (__ldg(&M.W[i]) * invrhoM) * w;
        out[i] = dY;
        cpm = fma(YT[i], s.Cp[i], cpm);
        dtd = fma(s.Ha[i], dY, dtd);
    }
    gsum2(g, cpm, dtd, s.red);
    if (g.rank == 0) out[ns] = -dtd / cpm;
    g.sync();
}

// ------------------------------------------------------------------------
// FastChemistryModel::calculate (FastChemistryModel.C:715-755): concentrations
// from the given density without clamping, RR_i = dNdtByV_i W_i.  Returns
// -sum Hf_i RR_i (Qdot, FastChemistryModel.C:656-685) to every thread.

template<int G, class MT>
__device__ __noinline__ double rates_eval(const Grp<G>& g, const DevMech& M, const Slot<MT>& s,
                                          double p, double T, double rho, const double* Y, double* RR) {
    const int ns = M.ns;
    const double Tc = clampT(M, T);
    const double logT = log(Tc), invT = 1.0 / Tc;
    for (int i = g.rank; i < ns; i += G) {
        s.C[i] = rho * Y[i] / __ldg(&M.W[i]);
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        s.B[i] = exp(gibbs_exponent(a, Tc, invT, logT));
    }
    g.sync();
    for (int t = g.rank; t < M.nTB; t += G) {
        const double* e = M.eff + (size_t)t * ns;
        double m = 0;
        for (int j = 0; j < ns; j++) m = fma(__ldg(&e[j]), s.C[j], m);
        s.Mtb[t] = m;
    }
    g.sync();
    const double PByRT = kPstd / (kRu * Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    for (int r = g.rank; r < M.nr; r += G) {
        const RxnInfo x = load_rx(M.rx + r);
        double Kf;
        if (x.kind == FCS_RXN_PLOG) {
            double dk;
            Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dk);
        } else if (x.tind) {
            Kf = x.A;
        } else {
            Kf = x.A * exp(fma(x.beta, logT, -(x.Ta * invT)));
        }
        if (x.tb >= 0) Kf *= s.Mtb[x.tb];
        double Kr = 0;
        if (x.rev) Kr = Kf / equilibrium_kc(x, s.B, PByRT);
        double CF = s.C[x.sl[0]];
        for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
        double CR = s.C[x.sr[0]];
        for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        s.q[r] = Kf * CF - Kr * CR;
    }
    g.sync();
    double qd = 0;
    for (int i = g.rank; i < ns; i += G) {
        double w = 0;
        const int e1 = __ldg(&M.incOff[i + 1]);
        for (int e = __ldg(&M.incOff[i]); e < e1; e++) {
            const int v = __ldg(&M.inc[e]);
            const double qq = s.q[v >> 1];
            w = (v & 1) ? w + qq : w - qq;
        }
        const double rr = w * __ldg(&M.W[i]);
        RR[i] = rr;
        qd -= __ldg(&M.hf[i]) * rr;
    }
    qd = gsum(g, qd, s.red);
    g.sync();
    return qd;
}

// ------------------------------------------------------------------------
// analytic Jacobian: FastChemistryModel::jacobian (FastChemistryModel.C:489-572)
// over OptReaction::ddNdtByVdcTp (Jacobian.C:5-1004, JF11..JF33) and the dC/dY
// conversion (Jacobian.C:2814-2858 exact written as diagonal scaling plus a
// rank-1 correction, 4541-4568 fast, 3709-3741 T column, 3743-3793 T row).
// Writes J (row-major, leading dimension s.ld) and f = dy/dt; YT clamped in
// place.  Accumulation happens in MT (double, or float in mixed precision);
// rate constants, equilibrium constants and f stay double.

template<int G, class MT>
__device__ __noinline__ void jac_eval(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p,
                         double* YT, double* f, MT* J, int fast) {
    const int ns = M.ns, n = M.n, ld = s.ld;
    for (int i = g.rank; i < ns; i += G) {
        const double y0 = YT[i];
        YT[i] = y0 > 0 ? y0 : 0.0;
    }
    const double T = YT[ns];
    const double Tc = clampT(M, T);
    const double logT = log(Tc), invT = 1.0 / Tc;
    // JacobianThermo (ThermoFunctionI.H:33-371) at the clamped temperature
    const double RuTByP = (kRu * Tc) / p;
    double rs = 0, mws = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double y = YT[i], invW = __ldg(&M.invW[i]);
        rs = fma(RuTByP, y * invW, rs);
        mws = fma(y, invW, mws);
    }
    gsum2(g, rs, mws, s.red);
    const double rhoM = 1.0 / rs, invRhoM = rs, MW = 1.0 / mws;
    double cpm = 0, dcpm = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double y = YT[i], invW = __ldg(&M.invW[i]);
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        s.C[i] = rhoM * y * invW;
        s.B[i] = exp(gibbs_exponent(a, Tc, invT, logT));
        s.dBdT[i] = fma(fma(a.a5, invT, a.a0), invT,
                        fma(fma(fma(a.a4 * 0.2, Tc, a.a3 * 0.25), Tc, a.a2 * (1.0 / 3.0)), Tc, a.a1 * 0.5));
        const double RuInvW = invW * kRu;
        const double cp = cp_of(a, Tc, RuInvW);
        const double dcp = RuInvW * fma(Tc, fma(Tc, fma(Tc, 4 * a.a4, 3 * a.a3), 2 * a.a2), a.a1);
        s.Cp[i] = cp;
        s.dCpdT[i] = dcp;
        s.Ha[i] = ha_of(a, Tc, RuInvW);
        cpm = fma(y, cp, cpm);
        dcpm = fma(y, dcp, dcpm);
    }
    gsum2(g, cpm, dcpm, s.red);
    const double CpM = cpm, dCpMdT = dcpm;
    g.sync();
    for (int t = g.rank; t < M.nTB; t += G) {
        const double* e = M.eff + (size_t)t * ns;
        double m = 0;
        for (int j = 0; j < ns; j++) m = fma(__ldg(&e[j]), s.C[j], m);
        s.Mtb[t] = m;
    }
    g.sync();
    // per-reaction rate constants, their temperature derivatives and q
    const double PByRT = kPstd / (kRu * Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    for (int r = g.rank; r < M.nr; r += G) {
        const RxnInfo x = load_rx(M.rx + r);
        double Kf, dKfdT;
        if (x.kind == FCS_RXN_PLOG) {
            Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dKfdT);
        } else if (x.tind) {
            Kf = x.A; dKfdT = 0;
        } else {
            Kf = x.A * exp(fma(x.beta, logT, -(x.Ta * invT)));
            dKfdT = Kf * (fma(x.Ta, invT, x.beta) * invT);
        }
        double dKfdC = 0;
        if (x.tb >= 0) {
            const double Mt = s.Mtb[x.tb];
            dKfdC = Kf;
            Kf *= Mt;
            dKfdT *= Mt;
        }
        double Kr = 0, dKrdT = 0, invKc = 0;
        if (x.rev) {
            const double Kc = equilibrium_kc(x, s.B, PByRT);
            double sv = s.dBdT[x.sr[0]];
            for (int q = 1; q < x.nr; q++) sv += s.dBdT[x.sr[q]];
            double sl = s.dBdT[x.sl[0]];
            for (int q = 1; q < x.nl; q++) sl += s.dBdT[x.sl[q]];
            const double dKcdTByKc = (sv - sl) - x.dnu * invT;
            invKc = 1.0 / Kc;
            Kr = Kf * invKc;
            dKrdT = dKfdT * invKc - (Kc > kKcClamp ? Kr * dKcdTByKc : 0.0);
        }
        double CF = s.C[x.sl[0]];
        for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
        double CR = s.C[x.sr[0]];
        for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        s.Kf[r] = Kf;
        s.Kr[r] = Kr;
        s.q[r] = Kf * CF - Kr * CR;
        s.dqdT[r] = dKfdT * CF - dKrdT * CR;
        if (x.tb >= 0) {
            s.tbF[x.tb] = dKfdC;
            s.tbR[x.tb] = dKfdC * invKc;
            s.tbCF[x.tb] = CF;
            s.tbCR[x.tb] = CR;
        }
    }
    g.sync();
    // Row owners gather the concentration Jacobian of their species row in
    // reaction order, then convert the row to the mass-fraction Jacobian.
    double dtd = 0, dd = 0;
    for (int i = g.rank; i < ns; i += G) {
        MT* row = J + (size_t)i * ld;
        for (int j = 0; j < n; j++) row[j] = MT(0);
        double w = 0;
        const int e1 = __ldg(&M.incOff[i + 1]);
        for (int e = __ldg(&M.incOff[i]); e < e1; e++) {
            const int v = __ldg(&M.inc[e]);
            const int r = v >> 1;
            const bool prod = v & 1;
            const RxnInfo x = load_rx(M.rx + r);
            const double Kf = s.Kf[r], Kr = s.Kr[r];
            if (x.rev) {
                for (int pp = 0; pp < x.nr; pp++) {
                    double d = 1.0;
                    for (int qq = 0; qq < x.nr; qq++) if (qq != pp) d *= s.C[x.sr[qq]];
                    const double val = -Kr * d;
                    const int col = x.sr[pp];
                    row[col] = prod ? row[col] + MT(val) : row[col] - MT(val);
                }
            }
            const double qq = s.q[r];
            w = prod ? w + qq : w - qq;
            row[ns] = prod ? row[ns] + MT(s.dqdT[r]) : row[ns] - MT(s.dqdT[r]);
            for (int pp = 0; pp < x.nl; pp++) {
                double d = 1.0;
                for (int q2 = 0; q2 < x.nl; q2++) if (q2 != pp) d *= s.C[x.sl[q2]];
                const double val = Kf * d;
                const int col = x.sl[pp];
                row[col] = prod ? row[col] + MT(val) : row[col] - MT(val);
            }
            if (x.tb >= 0) {
                const double dF = s.tbF[x.tb], dR = s.tbR[x.tb];
                const double CF = s.tbCF[x.tb], CR = s.tbCR[x.tb];
                const double* eff = M.eff + (size_t)x.tb * ns;
                for (int j = 0; j < ns; j++) {
                    const double ej = __ldg(&eff[j]);
                    const double Wd = (dF * ej) * CF - (dR * ej) * CR;
                    row[j] = prod ? row[j] + MT(Wd) : row[j] - MT(Wd);
                }
            }
        }
        const double WiByrhoM = invRhoM * __ldg(&M.W[i]);
        const double dY = w * WiByrhoM;
        double S = 0;
        for (int k = 0; k < ns; k++) S = fma(double(row[k]), s.C[k], S);
        const double tcol = WiByrhoM * (double(row[ns]) - S * invT) + invT * dY;
        if (fast) {
            for (int j = 0; j < ns; j++) {
                const double mj = MW * __ldg(&M.invW[j]);
                row[j] = MT(WiByrhoM * (double(row[j]) * (rhoM * __ldg(&M.invW[j]))) + mj * dY);
            }
        } else {
            for (int j = 0; j < ns; j++) {
                const double invWj = __ldg(&M.invW[j]);
                const double mj = MW * invWj;
                row[j] = MT(WiByrhoM * fma(double(row[j]), rhoM * invWj, -(mj * S)) + mj * dY);
            }
        }
        row[ns] = MT(tcol);
        f[i] = dY;
        dtd = fma(s.Ha[i], dY, dtd);
        dd += dY * s.Cp[i] + tcol * s.Ha[i];
    }
    gsum2(g, dtd, dd, s.red);
    const double dTdt = -dtd / CpM;
    g.sync();
    // temperature row (ddTdtdYT): column owners
    for (int j = g.rank; j < ns; j += G) {
        double v = 0;
        for (int i = 0; i < ns; i++) v -= double(J[(size_t)i * ld + j]) * s.Ha[i];
        v -= s.Cp[j] * dTdt;
        J[(size_t)ns * ld + j] = MT(v / CpM);
    }
    if (g.rank == 0) {
        J[(size_t)ns * ld + ns] = MT((-dd - dTdt * dCpMdT) / CpM);
        f[ns] = dTdt;
    }
    g.sync();
}

// ------------------------------------------------------------------------
// LU with the reference's 4-row-panel pivoting (LUsolver.C:106-246 panel,
// 503-660 two- and three-row tails, 3058-3143 driver): partial pivoting
// restricted to the current panel, exact-zero pivots replaced by 2.22e-16,
// whole-row interchanges recorded LAPACK style.

template<class MT>
__device__ __forceinline__ int choose_pivot(const MT* A, int ld, int k, int pos, int size) {
    const int cand = size - pos;
    if (cand <= 1) return k;
    if (pos == 0 && size >= 3) {
        int best = 0;
        double t = 0;
        for (int c = 0; c < size; c++) {
            const double v = fabs(double(A[(size_t)(k + c) * ld + k]));
            if (t < v) { best = c; t = v; }
        }
        return k + best;
    }
    if (size == 4 && pos == 1) {
        // LUsolver.C:169-185: the running maximum keeps the signed value of row 2
        double t = fabs(double(A[(size_t)k * ld + k]));
        int best = 0;
        const double v1 = double(A[(size_t)(k + 1) * ld + k]);
        if (t < fabs(v1)) { best = 1; t = v1; }
        if (t < fabs(double(A[(size_t)(k + 2) * ld + k]))) best = 2;
        return k + best;
    }
    return (fabs(double(A[(size_t)k * ld + k])) < fabs(double(A[(size_t)(k + 1) * ld + k]))) ? k + 1 : k;
}

template<int G, class MT>
__device__ __noinline__ void lu_factor(const Grp<G>& g, MT* A, int n, int ld, int* piv, double* invD) {
    const int rem = n & 3;
    constexpr int TC = 8, TR = G / TC;
    const int tr = g.rank / TC, tc = g.rank % TC;
    for (int k = 0; k < n; k++) {
        const bool tail = k >= n - rem;
        const int size = tail ? rem : 4;
        const int pos = tail ? k - (n - rem) : (k & 3);
        if (size == 1) {
            if (g.rank == 0) { invD[k] = 1.0 / double(A[(size_t)k * ld + k]); piv[k] = k; }
            g.sync();
            break;
        }
        const int p = choose_pivot(A, ld, k, pos, size);
        if (p != k) {
            g.sync();  // every thread has read the pivot column before rows move
            MT* rk = A + (size_t)k * ld;
            MT* rp = A + (size_t)p * ld;
            for (int j = g.rank; j < n; j += G) { const MT t = rk[j]; rk[j] = rp[j]; rp[j] = t; }
            g.sync();
        }
        double akk = double(A[(size_t)k * ld + k]);
        if (akk == 0) akk = kPivEps;
        const MT rinv = MT(1.0 / akk);
        g.sync();  // all threads read a_kk before the multipliers overwrite column k
        if (g.rank == 0) { invD[k] = double(rinv); piv[k] = p; }
        for (int i = k + 1 + g.rank; i < n; i += G) A[(size_t)i * ld + k] *= rinv;
        g.sync();
        const MT* rk = A + (size_t)k * ld;
        for (int i = k + 1 + tr; i < n; i += TR) {
            MT* ri = A + (size_t)i * ld;
            const MT l = ri[k];
            for (int j = k + 1 + tc; j < n; j += TC) ri[j] = fma(-l, rk[j], ri[j]);
        }
        g.sync();
    }
}

// Forward/back substitution with the factors of lu_factor, applying the row
// interchanges first (LUsolver.C:3145-3171, 4113-4152).  b is a shared-slot
// vector of doubles; arithmetic in MT.
template<int G, class MT>
__device__ __noinline__ void lu_solve(const Grp<G>& g, const MT* A, int n, int ld, const int* piv,
                         const double* invD, double* b) {
    if constexpr (G == 32) {
        constexpr int NR = 8;  // up to 256 unknowns in registers
        const int lane = g.rank;
        __syncwarp();
        if (lane == 0) {
            for (int j = 0; j < n; j++) {
                const int pj = piv[j];
                if (pj != j) { const double t = b[pj]; b[pj] = b[j]; b[j] = t; }
            }
        }
        __syncwarp();
        MT x[NR];
#pragma unroll
        for (int u = 0; u < NR; u++) {
            const int i = lane + 32 * u;
            x[u] = i < n ? MT(b[i]) : MT(0);
        }
        for (int j = 0; j < n - 1; j++) {
            const MT bj = __shfl_sync(0xffffffffu, x[j >> 5], j & 31);
#pragma unroll
            for (int u = 0; u < NR; u++) {
                const int i = lane + 32 * u;
                if (i > j && i < n) x[u] = fma(-A[(size_t)i * ld + j], bj, x[u]);
            }
        }
        for (int j = n - 1; j >= 0; j--) {
            const MT xj = __shfl_sync(0xffffffffu, x[j >> 5], j & 31) * MT(invD[j]);
#pragma unroll
            for (int u = 0; u < NR; u++) {
                const int i = lane + 32 * u;
                if (i == j) x[u] = xj;
                else if (i < j) x[u] = fma(-A[(size_t)i * ld + j], xj, x[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < NR; u++) {
            const int i = lane + 32 * u;
            if (i < n) b[i] = double(x[u]);
        }
        __syncwarp();
    } else {
        g.sync();
        if (g.rank == 0) {
            for (int j = 0; j < n; j++) {
                const int pj = piv[j];
                if (pj != j) { const double t = b[pj]; b[pj] = b[j]; b[j] = t; }
            }
        }
        g.sync();
        for (int j = 0; j < n - 1; j++) {
            const double bj = b[j];
            for (int i = j + 1 + g.rank; i < n; i += G)
                b[i] = double(fma(-A[(size_t)i * ld + j], MT(bj), MT(b[i])));
            g.sync();
        }
        for (int j = n - 1; j >= 0; j--) {
            const double xj = double(MT(b[j]) * MT(invD[j]));
            for (int i = g.rank; i < j; i += G)
                b[i] = double(fma(-A[(size_t)i * ld + j], MT(xj), MT(b[i])));
            g.sync();
            if (g.rank == 0) b[j] = xj;
            g.sync();
        }
    }
}

}  // namespace fcs
