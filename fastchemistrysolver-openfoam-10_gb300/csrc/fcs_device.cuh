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

// log(Tc) and 1/Tc for the whole group.  With several warps, thread 0
// computes them and publishes them through red[44..45]; the caller's next
// group reduction (which synchronises) makes them visible -- call
// thermo_scalars_read after it.  A single warp computes them in every lane.
template<int G>
__device__ __forceinline__ void thermo_scalars_publish(const Grp<G>& g, double Tc, double* red) {
    if constexpr (G > 32) {
        if (g.rank == 0) { red[44] = log(Tc); red[45] = 1.0 / Tc; }
    }
}

template<int G>
__device__ __forceinline__ void thermo_scalars_read(const Grp<G>& g, double Tc, const double* red, double& logT,
                                                    double& invT) {
    if constexpr (G > 32) {
        logT = red[44];
        invT = red[45];
    } else {
        logT = log(Tc);
        invT = 1.0 / Tc;
    }
}

// Two maxima at once of non-negative values (or NaN, which wins), compared
// as integers on their bit patterns: the order of non-negative doubles is the
// order of their bits, and NaN patterns sit above +inf.  No FP64 compares.
template<int G>
__device__ __forceinline__ void gmax2_nonneg(const Grp<G>& g, double& a, double& b, double* red) {
    unsigned long long x = static_cast<unsigned long long>(__double_as_longlong(a));
    unsigned long long y = static_cast<unsigned long long>(__double_as_longlong(b));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, x, o);
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, y, o);
        x = u > x ? u : x;
        y = v > y ? v : y;
    }
    if constexpr (G > 32) {
        unsigned long long* r = reinterpret_cast<unsigned long long*>(red);
        g.sync();
        if ((g.rank & 31) == 0) { r[g.rank >> 5] = x; r[16 + (g.rank >> 5)] = y; }
        g.sync();
        x = r[0];
        y = r[16];
#pragma unroll
        for (int w = 1; w < G / 32; w++) {
            x = r[w] > x ? r[w] : x;
            y = r[16 + w] > y ? r[16 + w] : y;
        }
    }
    a = __longlong_as_double(static_cast<long long>(x));
    b = __longlong_as_double(static_cast<long long>(y));
}

// ------------------------------------------------------------------------
// slot layout (byte offsets inside one cell's workspace)

struct SlotLayout {
    int ld;            // matrix leading dimension (odd: conflict-free column walks)
    int offJ64, offLU64;  // FP64 views of the Jacobian / LU factors (LU64 == J64: in place)
    int offJ32, offLU32;  // FP32 views (mixed precision), inside the same matrix region
    int offVec;        // kNV vectors of n doubles
    int offVec32;      // 2 vectors of n floats (mixed-precision solves)
    int offSp;         // 7 species arrays (C, E, Einv, Cp, Ha, dBdT, dCpdT) [ns]
    int offInvD;       // [n] double
    int offScale;      // row / column equilibration factors [2n] double (mixed precision)
    int offPiv;        // [n] int
    int offRx;         // Kf, Kr, q, dqdT [rc] each: one chunk of reactions
    int rc;            // reactions per chunk (at most nr)
    int offCur;        // [ns] int: per-species incidence cursor across chunks
    int offTb;         // M (third-body concentration), third-body column weight [nTB] each
    int offTable;      // Seulex extrapolation table [12][n] doubles
    int offRed;        // 48 doubles of reduction / broadcast scratch
    int bytes;         // total, multiple of 16
};

constexpr int kNV = 12;  // stage / work vectors per slot

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// Matrix region:
//   FP64 Rosenbrock : one FP64 matrix, factored in place
//   FP64 Seulex     : FP64 Jacobian + FP64 LU (the Jacobian is reused across orders)
//   mixed Rosenbrock: FP32 Jacobian + FP32 LU; the FP64 view (Jacobian assembly in
//                     FP64, and the FP64 fallback attempt) overlays both
//   mixed Seulex    : as FP64 Seulex, with the two FP32 matrices inside the FP64 Jacobian
// rc: reactions per chunk (clamped to [1, nr]); the host picks it so that the
// chunks are no smaller than needed for the most cells per SM.
__host__ __device__ inline SlotLayout make_layout(int ns, int nr, int nTB, bool mixed, bool seulex, int rc) {
    SlotLayout L;
    const int n = ns + 1;
    L.ld = n | 1;
    const int m64 = align16(n * L.ld * 8), m32 = align16(n * L.ld * 4);
    int o = 0;
    L.offJ64 = 0;
    if (seulex) { L.offLU64 = m64; o = 2 * m64; }   // FP64 Jacobian (kept) + FP64 LU
    else if (mixed) { L.offLU64 = 0; o = m64 + m32; } // FP64 Jacobian (kept) + FP32 LU; FP64 fallback in place
    else { L.offLU64 = 0; o = m64; }                 // FP64 matrix factored in place
    L.offJ32 = 0;                                    // (unused: the Jacobian stays FP64)
    L.offLU32 = m64;                                 // after the FP64 Jacobian (inside LU64 for Seulex)
    L.offVec = o;   o = align16(o + kNV * n * 8);
    L.offVec32 = o; if (mixed) o = align16(o + 2 * n * 4);
    L.offSp = o;    o = align16(o + 7 * ns * 8);
    L.offInvD = o;  o = align16(o + n * 8);
    L.offScale = o; if (mixed) o = align16(o + 2 * n * 8);
    L.offPiv = o;   o = align16(o + n * 4);
    L.rc = rc < 1 ? 1 : (nr > 0 && rc > nr ? nr : rc);
    L.offRx = o;    o = align16(o + (4 * L.rc * 8 > n * 4 ? 4 * L.rc * 8 : n * 4));  // also the LU's permutation scratch
    L.offCur = o;   o = align16(o + ns * 4);
    L.offTb = o;    o = align16(o + 2 * (nTB > 0 ? nTB : 1) * 8);
    L.offTable = o;
    if (seulex) o = align16(o + 12 * n * 8);
    L.offRed = o;   o = align16(o + 48 * 8);
    L.bytes = o;
    return L;
}

template<class MT>
struct Slot {
    int ld, n, ns;
    MT* J;
    MT* LU;
    double* vec;      // vec + k*n is vector k
    float *x32, *r32; // FP32 solve vectors (mixed precision)
    double* J64;      // the FP64 Jacobian (== J for MT = double)
    double *C, *B, *Binv, *Cp, *Ha, *dBdT, *dCpdT;   // B = exp(-G/RT), Binv = 1/B
    double* invD;
    double *dr, *dc;
    int* piv;
    double *Kf, *Kr, *q, *dqdT;   // one chunk of reactions: index r - c0
    int rc;                        // reactions per chunk
    int* cur;                      // per-species incidence cursor
    double *Mtb, *tbF;
    double* table;
    double* red;
    __device__ double* v(int k) const { return vec + k * n; }
};

template<class MT>
__device__ __forceinline__ Slot<MT> make_slot(char* base, const SlotLayout& L, const DevMech& M) {
    Slot<MT> s;
    s.ld = L.ld; s.n = M.n; s.ns = M.ns;
    if constexpr (sizeof(MT) == 8) {
        s.J = reinterpret_cast<MT*>(base + L.offJ64);
        s.LU = reinterpret_cast<MT*>(base + L.offLU64);
    } else {
        s.J = reinterpret_cast<MT*>(base + L.offJ32);
        s.LU = reinterpret_cast<MT*>(base + L.offLU32);
    }
    s.vec = reinterpret_cast<double*>(base + L.offVec);
    s.x32 = reinterpret_cast<float*>(base + L.offVec32);
    s.r32 = s.x32 + M.n;
    s.J64 = reinterpret_cast<double*>(base + L.offJ64);
    double* sp = reinterpret_cast<double*>(base + L.offSp);
    s.C = sp; s.B = sp + M.ns; s.Binv = sp + 2 * M.ns; s.Cp = sp + 3 * M.ns; s.Ha = sp + 4 * M.ns;
    s.dBdT = sp + 5 * M.ns; s.dCpdT = sp + 6 * M.ns;
    s.invD = reinterpret_cast<double*>(base + L.offInvD);
    s.dr = reinterpret_cast<double*>(base + L.offScale);
    s.dc = s.dr + M.n;
    s.piv = reinterpret_cast<int*>(base + L.offPiv);
    double* rx = reinterpret_cast<double*>(base + L.offRx);
    s.rc = L.rc;
    s.Kf = rx; s.Kr = rx + L.rc; s.q = rx + 2 * L.rc; s.dqdT = rx + 3 * L.rc;
    s.cur = reinterpret_cast<int*>(base + L.offCur);
    double* tb = reinterpret_cast<double*>(base + L.offTb);
    const int nt = M.nTB > 0 ? M.nTB : 1;
    s.Mtb = tb; s.tbF = tb + nt;
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
// exp(x) in FP64 by Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2):144-157, 1989), with 64 table entries:
//   x = (64 m + j) ln2/64 + r,  |r| <= ln2/128,
//   exp(x) = 2^m * 2^(j/64) * (1 + p(r)),  p(r) = r + r^2/2! + ... + r^5/5!
// (truncation below 4e-17).  N = 64 m + j is rounded with the 1.5*2^52
// shift, ln2/64 is split in a 36-bit head and a tail so N*head is exact, and
// 2^m is applied by adding m to the exponent field on the integer pipe.
// |x| > 707 (outside the range where 2^m stays a normal number) goes to the
// CUDA exp.  About 12 FP64 instructions.
__device__ const double kExp2Table[64] = {
    1.0, 1.0108892860517005, 1.0218971486541166, 1.0330248790212284,
    1.0442737824274138, 1.0556451783605572, 1.0671404006768237, 1.0787607977571199,
    1.0905077326652577, 1.102382583307841, 1.1143867425958924, 1.1265216186082418,
    1.1387886347566916, 1.1511892299529827, 1.1637248587775775, 1.1763969916502812,
    1.189207115002721, 1.202156731452703, 1.215247359980469, 1.22848053610687,
    1.241857812073484, 1.255380757024691, 1.2690509571917332, 1.2828700160787783,
    1.2968395546510096, 1.3109612115247644, 1.3252366431597413, 1.339667524053303,
    1.3542555469368927, 1.3690024229745905, 1.383909881963832, 1.3989796725383112,
    1.4142135623730951, 1.42961333839197, 1.4451808069770467, 1.460917794180647,
    1.4768261459394993, 1.4929077282912648, 1.5091644275934228, 1.5255981507445384,
    1.5422108254079407, 1.559004400237837, 1.5759808451078865, 1.593142151342267,
    1.6104903319492543, 1.6280274218573478, 1.645755478153965, 1.6636765803267364,
    1.681792830507429, 1.7001063537185235, 1.718619298122478, 1.7373338352737062,
    1.7562521603732995, 1.7753764925265212, 1.7947090750031072, 1.8142521755003989,
    1.8340080864093424, 1.8539791250833855, 1.8741676341103, 1.8945759815869656,
    1.9152065613971474, 1.9360617934922943, 1.9571441241754002, 1.978456026387951};

__device__ __forceinline__ double fast_exp(double x) {
    if (!(fabs(x) <= 707.0)) return exp(x);
    const double kInvL = 92.33248261689366;          // 64/ln2
    const double kL1 = 0.010830424696223417;         // head of ln2/64 (36 bits)
    const double kL2 = 2.572804622327669e-14;        // tail
    const double kShift = 6755399441055744.0;        // 1.5 * 2^52
    const double kk = fma(x, kInvL, kShift);
    const long long N = __double_as_longlong(kk) - 0x4338000000000000LL;
    const double Nf = kk - kShift;
    double r = fma(-Nf, kL1, x);
    r = fma(-Nf, kL2, r);
    double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    q = fma(r, q, 1.0 / 6.0);
    q = fma(r, q, 0.5);
    q = fma(r, q, 1.0);
    const double p = r * q;
    const double S = __ldg(&kExp2Table[N & 63]);
    const double res = fma(S, p, S);
    return __longlong_as_double(__double_as_longlong(res) + ((N >> 6) << 52));
}

// OptReaction::fastPow (OptReaction.H:1405-1420)
__device__ __forceinline__ double fast_pow_int(double x, int order) {
    double xx = order < 0 ? 1 / x : x;
    double y = 1;
    for (int i = order; i != 0; i /= 2) {
        if (i % 2) y *= xx;
        xx *= xx;
    }
    return y;
}

// Pstd/(Ru T) and its inverse: the pressure factor of 1/Kc is (Pstd/(Ru T))^(-dnu)
struct PFactor { double P, invP; };

__device__ __forceinline__ PFactor pressure_factors(double Tc) {
    PFactor f;
    f.invP = kRu * Tc / kPstd;
    f.P = 1.0 / f.invP;
    return f;
}

constexpr double kInvKcClamp = 1.0 / kKcClamp;
constexpr double kInvKcClampG = 1.0 / kKcClampG;

// (Pstd/(Ru T))^(-dnu): the reference's table for |dnu| <= 2
// (ChemicalEquilibriumFunctionI.H:14-25), fastPow beyond it (RFG/JFG)
__device__ __forceinline__ double pressure_factor(const PFactor& pf, int dnu) {
    switch (dnu) {
        case -2: return pf.P * pf.P;
        case -1: return pf.P;
        case 1: return pf.invP;
        case 2: return pf.invP * pf.invP;
        default: return fast_pow_int(pf.invP, dnu);
    }
}

// The clamp of 1/Kc: RFG/JFG (more than 3 species on a side) use the other constant
__device__ __forceinline__ double inv_kc_clamp(const RxnInfo& x) {
    return (x.nl > 3 || x.nr > 3) ? kInvKcClampG : kInvKcClamp;
}

// 1/Kc from per-species exp(-G/RT) and its inverse, no division:
// 1/Kc = prod_reactants E * prod_products 1/E * (Pstd/(Ru T))^-dnu, with the
// reference's lower clamp of Kc (ReactionFunctionI.H:17; RFG's for more than
// 3 species on a side) as an upper clamp.
__device__ __forceinline__ double inv_equilibrium_kc(const RxnInfo& x, const double* E, const double* Einv,
                                                     const PFactor& pf) {
    double v = E[x.sl[0]];
    // Species loops over a reaction stay rolled: unrolled over the 4 + 8 byte
    // slots of RxnInfo they raised the integrator's register spills.
    #pragma unroll 1
    for (int q = 1; q < x.nl; q++) v *= E[x.sl[q]];
    #pragma unroll 1
    for (int q = 0; q < x.nr; q++) v *= Einv[x.sr[q]];
    if (x.dnu != 0) v *= pressure_factor(pf, x.dnu);
    const double cl = inv_kc_clamp(x);
    return v > cl ? cl : v;
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
    const double k = fast_exp(lk);
    *dkdT = k * dk;
    return k;
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
// fall-off reactions (ReactionRate.C:370-519, Jacobian.C:426-713,
// pressureReactionFunctionI.H): Kf = M K0 F / (1 + Pr), Pr = K0 M / kInf,
// F = 1 (Lindemann), Troe or SRI.  K0 is the reaction's own Arrhenius rate,
// kInf and the F parameters come from DevMech::fo; Tc is the clamped
// temperature.  With deriv, also dKf/dT and dKf/dM; the SRI branch uses dF/dT
// at fixed Pr, as the reference does (no dF/dPr dPr/dT term), the Troe branch
// the total derivative.

struct FalloffK { double Kf, dKfdT, dKfdC; };

static __device__ __noinline__ FalloffK falloff_rate(const DevMech& M, const RxnInfo& x, double K0, double dK0dT,
                                                     double Mt, double Tc, double logT, double invT, bool deriv) {
    const double* f = M.fo + (size_t)x.fo * 8;
    const double A2 = __ldg(f), b2 = __ldg(f + 1), Ta2 = __ldg(f + 2);
    const double Kinf = A2 * fast_exp(fma(b2, logT, -(Ta2 * invT)));
    const double dKinfdT = Kinf * (fma(Ta2, invT, b2) * invT);
    FalloffK o{0, 0, 0};
    if (x.kind == FCS_RXN_LINDEMANN_FALLOFF) {
        if (!deriv) {
            const double Pr = (K0 * Mt) / Kinf;
            o.Kf = Mt * (K0 / (Pr + 1.0));
            return o;
        }
        const double invKinf = 1.0 / Kinf;
        const double Pr = (K0 * Mt) * invKinf;
        const double dPrdT = fma(Mt, dK0dT, -(Pr * dKinfdT)) * invKinf;
        const double tmp = 1.0 / (1.0 + Pr);
        o.dKfdT = fma(tmp, Pr * dKinfdT, ((tmp * tmp) * dPrdT) * Kinf);
        o.dKfdC = (K0 * tmp) * tmp;
        o.Kf = Mt * (tmp * K0);
        return o;
    }
    const double small = 1e-15;
    const double Pr = K0 * Mt / Kinf;
    const double logPr = log10(fmax(Pr, small));
    const double logTen = 2.302585092994045684;
    double F, dFdT = 0, dFdPr = 0;
    if (x.kind == FCS_RXN_TROE_FALLOFF) {
        const double alpha = __ldg(f + 3), Ts = __ldg(f + 4), Tss = __ldg(f + 5), Tsss = __ldg(f + 6);
        const double invTsss = 1.0 / Tsss, invTs = 1.0 / Ts;
        const double eTsss = fast_exp(-Tc * invTsss), eTss = fast_exp(-Tss * invT), eTs = fast_exp(-Tc * invTs);
        const double Fcent = (1 - alpha) * eTsss + alpha * eTs + eTss;
        const double logFcent = log10(fmax(Fcent, small));
        const double c = -0.4 - 0.67 * logFcent;
        const double n = 0.75 - 1.27 * logFcent;
        const double x1 = n - 0.14 * (logPr + c);
        const double invx1 = 1.0 / x1;
        const double x2 = (logPr + c) * invx1;
        const double x3 = 1 + (x2 * x2);
        const double invx3 = 1.0 / x3;
        const double x4 = logFcent * invx3;
        F = pow(10.0, x4);
        if (deriv) {
            const double dFcentdT = -(1 - alpha) * invTsss * eTsss - alpha * invTs * eTs + Tss * invT * invT * eTss;
            const double dlogFcentdT = Fcent >= small ? dFcentdT / Fcent / logTen : 0;
            const double dcdT = -0.67 * dlogFcentdT;
            const double dndT = -1.27 * dlogFcentdT;
            const double dx1dT = dndT - 0.14 * dcdT;
            const double dx2dT = (dcdT - x2 * dx1dT) * invx1;
            const double dx3dT = 2 * x2 * dx2dT;
            const double dx4dT = (dlogFcentdT - x4 * dx3dT) * invx3;
            const double dlogPrdPr = Pr >= small ? 1 / (logTen * Pr) : 0;
            const double dx1dPr = -0.14 * dlogPrdPr;
            const double dx2dPr = (dlogPrdPr - x2 * dx1dPr) * invx1;
            const double dx3dPr = 2 * x2 * dx2dPr;
            const double dx4dPr = -x4 * dx3dPr * invx3;
            dFdPr = logTen * F * dx4dPr;
            const double dPrdT = (Mt * dK0dT - Pr * dKinfdT) * (1.0 / Kinf);
            dFdT = logTen * F * dx4dT + dFdPr * dPrdT;
        }
    } else {
        const double a = __ldg(f + 3), b = __ldg(f + 4), c = __ldg(f + 5), d = __ldg(f + 6), e = __ldg(f + 7);
        const double X = 1 / (1 + (logPr * logPr));
        const double eb = fast_exp(-b * invT), ec = fast_exp(-Tc * (1.0 / c));
        const double psi = a * eb + ec;
        F = d * pow(psi, X) * pow(Tc, e);
        if (deriv) {
            const double dpsidT = a * b / (Tc * Tc) * eb - 1 / c * ec;
            dFdT = F * (X / psi * dpsidT + e / Tc);
            const double dlogPrdPr = Pr >= small ? 1 / (logTen * Pr) : 0;
            const double dXdPr = -(X * X) * 2 * logPr * dlogPrdPr;
            dFdPr = F * log(psi) * dXdPr;
        }
    }
    const double invOnePlusPr = 1.0 / (1 + Pr);
    if (deriv) {
        const double dPrdT = (Mt * dK0dT - Pr * dKinfdT) * (1.0 / Kinf);
        o.dKfdT = F * invOnePlusPr * (Pr * dKinfdT) + F * invOnePlusPr * invOnePlusPr * dPrdT * Kinf +
                  K0 * invOnePlusPr * dFdT * Mt;
        o.dKfdC = K0 * invOnePlusPr * (F * invOnePlusPr + Pr * dFdPr);
    }
    o.Kf = Mt * (invOnePlusPr * F * K0);
    return o;
}

// Rates of one reaction of the special block: fall-off, non-equilibrium (the
// reverse rate its own Arrhenius, ReactionRate.C:362-367, 540-544) or
// third-body; Kf and Kr include M, and with deriv the temperature derivatives
// and dKf/dM, dKr/dM (Jacobian.C:401-422).
struct SpecialK { double Kf, dKfdT, dKfdC, Kr, dKrdT, dKrdC; };

// Mt: the reaction's third-body concentration (1 when it has none).
static __device__ __forceinline__ SpecialK special_rates_m(const DevMech& M, const RxnInfo& x, const double Mt,
                                                        double Tc, double logT, double invT, bool deriv) {
    SpecialK o{0, 0, 0, 0, 0, 0};
    double K0 = x.A, dK0dT = 0;
    if (!x.tind) {
        K0 = x.A * fast_exp(fma(x.beta, logT, -(x.Ta * invT)));
        dK0dT = K0 * (fma(x.Ta, invT, x.beta) * invT);
    }
    if (x.fo >= 0) {
        const FalloffK k = falloff_rate(M, x, K0, dK0dT, Mt, Tc, logT, invT, deriv);
        o.Kf = k.Kf;
        o.dKfdT = k.dKfdT;
        o.dKfdC = k.dKfdC;
    } else if (x.tb >= 0) {
        o.dKfdC = K0;
        o.Kf = K0 * Mt;
        o.dKfdT = dK0dT * Mt;
    } else {
        o.Kf = K0;
        o.dKfdT = dK0dT;
    }
    if (x.nq >= 0) {
        const double* f = M.fo + (size_t)x.nq * 8;
        const double Ar = __ldg(f), br = __ldg(f + 1), Tar = __ldg(f + 2);
        const double Kr = Ar * fast_exp(fma(br, logT, -(Tar * invT)));
        const double dKrdT = Kr * (fma(Tar, invT, br) * invT);
        if (x.tb >= 0) {
            o.dKrdC = Kr;
            o.Kr = Kr * Mt;
            o.dKrdT = dKrdT * Mt;
        } else {
            o.Kr = Kr;
            o.dKrdT = dKrdT;
        }
    }
    return o;
}

static __device__ __forceinline__ SpecialK special_rates(const DevMech& M, const RxnInfo& x, const double* Mtb,
                                                      double Tc, double logT, double invT, bool deriv) {
    return special_rates_m(M, x, x.tb >= 0 ? Mtb[x.tb] : 1.0, Tc, logT, invT, deriv);
}

// ------------------------------------------------------------------------
// Reactions are evaluated in chunks of s.rc so that the per-reaction arrays
// of a cell slot hold one chunk, not the whole mechanism, where that lets
// more cells reside per SM (otherwise one chunk holds every reaction).  Every sum keeps its order: a species' terms
// are added in reaction order across the chunks, its incidence cursor
// (s.cur) carrying over from one chunk to the next.

// Net rates q of the reactions [c0, c1) into s.q[r - c0] (ReactionRate.C:521-575
// and the RF* functions).  The special block [spBegin, spBegin + nSp) of the
// packed order (first non-equilibrium to last fall-off reaction) runs in a
// loop of its own, so that the main loop carries neither the fall-off call
// nor a second Arrhenius.
template<int G, class MT>
__device__ __forceinline__ void net_rates_chunk(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p,
                                                double logP, double Tc, double logT, double invT,
                                                const PFactor& pf, int c0, int c1) {
    const int sp0 = M.spBegin, sp1 = M.spBegin + M.nSp;
    auto finish = [&](const int r, const RxnInfo& x, const double Kf, const double Kr) {
        double CF = s.C[x.sl[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
        double CR = s.C[x.sr[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        s.q[r - c0] = Kf * CF - Kr * CR;
    };
    for (int r = c0 + g.rank; r < c1; r += G) {
        if (r >= sp0 && r < sp1) continue;
        const RxnInfo x = load_rx(M.rx + r);
        double Kf;
        if (x.kind == FCS_RXN_PLOG) {
            double dk;
            Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dk);
        } else if (x.tind) {
            Kf = x.A;
        } else {
            Kf = x.A * fast_exp(fma(x.beta, logT, -(x.Ta * invT)));
        }
        if (x.tb >= 0) Kf *= s.Mtb[x.tb];
        double Kr = 0;
        if (x.rev) Kr = Kf * inv_equilibrium_kc(x, s.B, s.Binv, pf);
        finish(r, x, Kf, Kr);
    }
    for (int r = max(c0, sp0) + g.rank; r < min(c1, sp1); r += G) {
        const RxnInfo x = load_rx(M.rx + r);
        const SpecialK k = special_rates(M, x, s.Mtb, Tc, logT, invT, false);
        double Kr = k.Kr;  // non-equilibrium: its own reverse rate
        if (x.rev == 1) Kr = k.Kf * inv_equilibrium_kc(x, s.B, s.Binv, pf);
        finish(r, x, k.Kf, Kr);
    }
}

// acc[i] += the net rates of the chunk [c0, c1) for species i (+q as a
// product, -q as a reactant), in reaction order.
template<int G, class MT>
__device__ __forceinline__ void gather_chunk(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, int c0, int c1,
                                             double* acc) {
    for (int i = g.rank; i < M.ns; i += G) {
        double w = acc[i];
        int e = s.cur[i];
        const int e1 = __ldg(&M.incOff[i + 1]);
        for (; e < e1; e++) {
            const int v = __ldg(&M.inc[e]);
            if ((v >> 1) >= c1) break;
            const double qq = s.q[(v >> 1) - c0];
            w = (v & 1) ? w + qq : w - qq;
        }
        s.cur[i] = e;
        acc[i] = w;
    }
}

// Sum over the chunks: acc[i] = w_i for every species.
template<int G, class MT>
__device__ __forceinline__ void net_production(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p,
                                               double logP, double Tc, double logT, double invT,
                                               const PFactor& pf, double* acc) {
    for (int i = g.rank; i < M.ns; i += G) {
        s.cur[i] = __ldg(&M.incOff[i]);
        acc[i] = 0.0;
    }
    for (int c0 = 0; c0 < M.nr; c0 += s.rc) {
        const int c1 = min(M.nr, c0 + s.rc);
        net_rates_chunk<G, MT>(g, M, s, p, logP, Tc, logT, invT, pf, c0, c1);
        g.sync();
        gather_chunk<G, MT>(g, M, s, c0, c1, acc);
        if (c1 < M.nr) g.sync();  // the next chunk overwrites q
    }
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
    thermo_scalars_publish(g, Tc, s.red);
    const double RuTByP = kRu * T / p;
    double part = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double y0 = YT[i];
        const double y = y0 > 0 ? y0 : 0.0;
        YT[i] = y;
        part = fma(y * __ldg(&M.invW[i]), RuTByP, part);
    }
    const double invrhoM = gsum(g, part, s.red);
    double logT, invT;
    thermo_scalars_read(g, Tc, s.red, logT, invT);
    const double rhoM = 1.0 / invrhoM;
    const double Tp = mode == 2 ? T : Tc;
    for (int i = g.rank; i < ns; i += G) {
        const double invW = __ldg(&M.invW[i]);
        s.C[i] = rhoM * invW * YT[i];
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        const double Ei = fast_exp(gibbs_exponent(a, Tc, invT, logT));
        s.B[i] = Ei;
        s.Binv[i] = 1.0 / Ei;
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
    const PFactor pf = pressure_factors(Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    net_production<G, MT>(g, M, s, p, logP, Tc, logT, invT, pf, out);
    double cpm = 0, dtd = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double dY = (__ldg(&M.W[i]) * invrhoM) * out[i];
        out[i] = dY;
        cpm = fma(YT[i], s.Cp[i], cpm);
        dtd = fma(s.Ha[i], dY, dtd);
    }
    gsum2(g, cpm, dtd, s.red);
    if (g.rank == 0) out[ns] = -dtd / cpm;
    g.sync();
}

// ------------------------------------------------------------------------
// FastChemistryModel::tc (FastChemistryModel.C:589-651) over OptReaction::Tc
// (Tc.C:3-834): c = rho Y / W (not clamped); per reaction the forward and
// reverse molar rates summed over the products / reactants,
// wf = n_products Kf CF and wr = n_reactants Kr CR, with Kc from the ratio of
// Gibbs exponentials times fastPow(Pstd/(Ru T), dnu) clamped at
// 1.49011611938476e-8; tc = sum(w) / sum(w^2) * sum(c).  Returns tc to every
// thread.

template<int G, class MT>
__device__ __noinline__ double tc_eval(const Grp<G>& g, const DevMech& M, const Slot<MT>& s, double p, double T,
                                       double rho, const double* Y) {
    const int ns = M.ns;
    const double Tc = clampT(M, T);
    const double logT = log(Tc), invT = 1.0 / Tc;
    double sumc = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double ci = rho * Y[i] / __ldg(&M.W[i]);
        s.C[i] = ci;
        sumc += ci;
        const Nasa a = load_nasa(species_coeffs(M, i, Tc));
        s.B[i] = fast_exp(gibbs_exponent(a, Tc, invT, logT));
    }
    sumc = gsum(g, sumc, s.red);
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
    double sw = 0, sw2 = 0;
    // The special block [spBegin, spBegin + nSp) of the packed order (first
    // non-equilibrium to last fall-off reaction) runs in a loop of its own, so
    // that the main loop carries neither the fall-off call nor a second
    // Arrhenius.
    // Tc.C:578-600: the reverse rate only through Kc; a non-equilibrium
    // reaction counts with its forward rate alone
    auto finish = [&](const int r, const RxnInfo& x, const double Kf) {
        double Kr = 0;
        if (x.rev == 1) {
            double Kp = 1.0;
            #pragma unroll 1
            for (int q = 0; q < x.nl; q++) Kp = Kp / s.B[x.sl[q]];
            #pragma unroll 1
            for (int q = 0; q < x.nr; q++) Kp = Kp * s.B[x.sr[q]];
            double Kc = Kp * fast_pow_int(PByRT, x.dnu);
            Kc = Kc > 1.49011611938476e-8 ? Kc : 1.49011611938476e-8;
            Kr = Kf / Kc;
        }
        double CF = s.C[x.sl[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
        double CR = s.C[x.sr[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
        const double wf = x.nr * (Kf * CF), wr = x.nl * (Kr * CR);
        sw += wf + wr;
        sw2 = fma(wf, wf, fma(wr, wr, sw2));
    };
    for (int j = g.rank; j < M.nr - M.nSp; j += G) {
        const int r = j < M.spBegin ? j : j + M.nSp;
        const RxnInfo x = load_rx(M.rx + r);
        double Kf;
        if (x.kind == FCS_RXN_PLOG) {
            double dk;
            Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dk);
        } else if (x.tind) {
            Kf = x.A;
        } else {
            Kf = x.A * fast_exp(fma(x.beta, logT, -(x.Ta * invT)));
        }
        if (x.tb >= 0) Kf *= s.Mtb[x.tb];
        finish(r, x, Kf);
    }
    for (int r = M.spBegin + g.rank; r < M.spBegin + M.nSp; r += G) {
        const RxnInfo x = load_rx(M.rx + r);
        finish(r, x, special_rates(M, x, s.Mtb, Tc, logT, invT, false).Kf);
    }
    gsum2(g, sw, sw2, s.red);
    return sw2 == 0 ? 1e300 : sw / sw2 * sumc;
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
        const double Ei = fast_exp(gibbs_exponent(a, Tc, invT, logT));
        s.B[i] = Ei;
        s.Binv[i] = 1.0 / Ei;
    }
    g.sync();
    for (int t = g.rank; t < M.nTB; t += G) {
        const double* e = M.eff + (size_t)t * ns;
        double m = 0;
        for (int j = 0; j < ns; j++) m = fma(__ldg(&e[j]), s.C[j], m);
        s.Mtb[t] = m;
    }
    g.sync();
    const PFactor pf = pressure_factors(Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    net_production<G, MT>(g, M, s, p, logP, Tc, logT, invT, pf, RR);
    double qd = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double rr = RR[i] * __ldg(&M.W[i]);
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
    thermo_scalars_publish(g, Tc, s.red);
    // JacobianThermo (ThermoFunctionI.H:33-371) at the clamped temperature
    const double RuTByP = (kRu * Tc) / p;
    double rs = 0, mws = 0;
    for (int i = g.rank; i < ns; i += G) {
        const double y = YT[i], invW = __ldg(&M.invW[i]);
        rs = fma(RuTByP, y * invW, rs);
        mws = fma(y, invW, mws);
    }
    gsum2(g, rs, mws, s.red);
    double logT, invT;
    thermo_scalars_read(g, Tc, s.red, logT, invT);
    const double rhoM = 1.0 / rs, invRhoM = rs, MW = 1.0 / mws;
    double cpm = 0, dcpm = 0;
    for (int i = g.rank; i < ns; i += G) {
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
    // per-reaction rate constants, their temperature derivatives and q, one
    // chunk of reactions at a time (see net_rates_chunk)
    const PFactor pf = pressure_factors(Tc);
    const double logP = M.nPlog ? log(p) : 0.0;
    // Kr, dKr/dT and dKr/dM through Kc (JF* reversible branch)
    auto through_kc = [&](const RxnInfo& x, const double Kf, const double dKfdT, const double dKfdC,
                          double& Kr, double& dKrdT, double& dKrdC) {
        const double invKc = inv_equilibrium_kc(x, s.B, s.Binv, pf);
        double sv = s.dBdT[x.sr[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nr; q++) sv += s.dBdT[x.sr[q]];
        double sl = s.dBdT[x.sl[0]];
        #pragma unroll 1
        for (int q = 1; q < x.nl; q++) sl += s.dBdT[x.sl[q]];
        const double dKcdTByKc = (sv - sl) - x.dnu * invT;
        Kr = Kf * invKc;
        // the Kc term of dKr/dT is dropped when Kc sits on its clamp (JacobianFunctionI.H:246-249)
        dKrdT = dKfdT * invKc - (invKc < inv_kc_clamp(x) ? Kr * dKcdTByKc : 0.0);
        dKrdC = dKfdC * invKc;
    };
    // The running sums of the rows: f[i] collects w_i (the net production),
    // s.dCpdT[i] (free once CpM and dCpM/dT are formed) collects the
    // temperature-column sum of dq/dT.
    double* tcAcc = s.dCpdT;
    for (int i = g.rank; i < ns; i += G) {
        s.cur[i] = __ldg(&M.incOff[i]);
        f[i] = 0.0;
        tcAcc[i] = 0.0;
    }
    for (int idx = g.rank; idx < ns * ld; idx += G) J[idx] = MT(0);
    const int sp0 = M.spBegin, sp1 = M.spBegin + M.nSp;
    for (int c0 = 0; c0 < M.nr; c0 += s.rc) {
        const int c1 = min(M.nr, c0 + s.rc);
        auto finish = [&](const int r, const RxnInfo& x, const double Kf, const double dKfdT, const double dKfdC,
                          const double Kr, const double dKrdT, const double dKrdC) {
            double CF = s.C[x.sl[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nl; q++) CF *= s.C[x.sl[q]];
            double CR = s.C[x.sr[0]];
            #pragma unroll 1
            for (int q = 1; q < x.nr; q++) CR *= s.C[x.sr[q]];
            s.Kf[r - c0] = Kf;
            s.Kr[r - c0] = Kr;
            s.q[r - c0] = Kf * CF - Kr * CR;
            s.dqdT[r - c0] = dKfdT * CF - dKrdT * CR;
            // third-body weight w = dKf/dM CF - dKr/dM CR
            if (x.tb >= 0) s.tbF[x.tb] = dKfdC * CF - dKrdC * CR;
        };
        for (int r = c0 + g.rank; r < c1; r += G) {
            if (r >= sp0 && r < sp1) continue;
            const RxnInfo x = load_rx(M.rx + r);
            double Kf, dKfdT;
            if (x.kind == FCS_RXN_PLOG) {
                Kf = plog_rate(M, x.plog, p, logP, logT, invT, &dKfdT);
            } else if (x.tind) {
                Kf = x.A; dKfdT = 0;
            } else {
                Kf = x.A * fast_exp(fma(x.beta, logT, -(x.Ta * invT)));
                dKfdT = Kf * (fma(x.Ta, invT, x.beta) * invT);
            }
            double dKfdC = 0;
            if (x.tb >= 0) {
                const double Mt = s.Mtb[x.tb];
                dKfdC = Kf;
                Kf *= Mt;
                dKfdT *= Mt;
            }
            double Kr = 0, dKrdT = 0, dKrdC = 0;
            if (x.rev) through_kc(x, Kf, dKfdT, dKfdC, Kr, dKrdT, dKrdC);
            finish(r, x, Kf, dKfdT, dKfdC, Kr, dKrdT, dKrdC);
        }
        for (int r = max(c0, sp0) + g.rank; r < min(c1, sp1); r += G) {
            const RxnInfo x = load_rx(M.rx + r);
            SpecialK k = special_rates(M, x, s.Mtb, Tc, logT, invT, true);
            // non-equilibrium: the reverse Arrhenius (JacobianFunctionI.H:129-130, Jacobian.C:412-422)
            if (x.rev == 1) through_kc(x, k.Kf, k.dKfdT, k.dKfdC, k.Kr, k.dKrdT, k.dKrdC);
            finish(r, x, k.Kf, k.dKfdT, k.dKfdC, k.Kr, k.dKrdT, k.dKrdC);
        }
        g.sync();
        // Per species j and reaction r of the chunk (reaction order): the row
        // sums of j (w_j, dq/dT), and as the owner of column j, d q_r / d C_j
        // scattered down column j to the rows of reaction r (JF11..JF33
        // reverse and forward concentration terms).
        for (int j = g.rank; j < ns; j += G) {
            double w = f[j], tc = tcAcc[j];
            int e = s.cur[j];
            const int e1 = __ldg(&M.incOff[j + 1]);
            for (; e < e1; e++) {
                const int v = __ldg(&M.inc[e]);
                const int r = v >> 1;
                if (r >= c1) break;
                const bool prod = v & 1;
                const double qq = s.q[r - c0], dq = s.dqdT[r - c0];
                if (prod) { w += qq; tc += dq; } else { w -= qq; tc -= dq; }
                const RxnInfo x = load_rx(M.rx + r);
                double d;
                if (!prod) {
                    // forward: Kf * product of the other reactant concentrations
                    bool skipped = false;
                    d = s.Kf[r - c0];
                    #pragma unroll 1
                    for (int q = 0; q < x.nl; q++) {
                        if (!skipped && x.sl[q] == j) { skipped = true; continue; }
                        d *= s.C[x.sl[q]];
                    }
                } else {
                    if (!x.rev) continue;
                    bool skipped = false;
                    d = -s.Kr[r - c0];
                    #pragma unroll 1
                    for (int q = 0; q < x.nr; q++) {
                        if (!skipped && x.sr[q] == j) { skipped = true; continue; }
                        d *= s.C[x.sr[q]];
                    }
                }
                const MT md = MT(d);
                #pragma unroll 1
                for (int q = 0; q < x.nl; q++) { MT& c = J[(size_t)x.sl[q] * ld + j]; c = c - md; }
                #pragma unroll 1
                for (int q = 0; q < x.nr; q++) { MT& c = J[(size_t)x.sr[q] * ld + j]; c = c + md; }
            }
            s.cur[j] = e;
            f[j] = w;
            tcAcc[j] = tc;
        }
        g.sync();  // the next chunk overwrites Kf, Kr, q, dq/dT; the passes below read J
    }
    // (2) third-body columns, J_ij += nu_i w_t E_tj (JF* third-body block)
    for (int j = g.rank; j < ns; j += G) {
        for (int e = 0; e < M.nTbInc; e++) {
            const int v = __ldg(&M.tbInc[e]);
            const int i = v >> 16, t = (v >> 1) & 0x7fff;
            const double wd = __ldg(&M.eff[(size_t)t * ns + j]) * s.tbF[t];
            MT& c = J[(size_t)i * ld + j];
            c = (v & 1) ? c + MT(wd) : c - MT(wd);
        }
    }
    g.sync();
    // (3) row owners: production rate, temperature column and the dC/dY
    // conversion of the row (diagonal scaling + rank-1 correction)
    double dtd = 0, dd = 0;
    for (int i = g.rank; i < ns; i += G) {
        MT* row = J + (size_t)i * ld;
        const double w = f[i], tc = tcAcc[i];
        const double WiByrhoM = invRhoM * __ldg(&M.W[i]);
        const double dY = w * WiByrhoM;
        double S = 0;
        for (int k = 0; k < ns; k++) S = fma(double(row[k]), s.C[k], S);
        const double tcol = WiByrhoM * (tc - S * invT) + invT * dY;
        if (fast) {
            for (int j = 0; j < ns; j++) {
                const double invWj = __ldg(&M.invW[j]);
                row[j] = MT(WiByrhoM * (double(row[j]) * (rhoM * invWj)) + (MW * invWj) * dY);
            }
        } else {
            // Wi/rho (Jc_ij rho/Wj - m_j S) + m_j dY = Jc_ij (Wi/Wj) + m_j (dY - Wi/rho S)
            const double K = dY - WiByrhoM * S;
            const double Wi = __ldg(&M.W[i]);
            for (int j = 0; j < ns; j++) {
                const double invWj = __ldg(&M.invW[j]);
                row[j] = MT(fma(double(row[j]), Wi * invWj, (MW * invWj) * K));
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

// work: n ints of slot scratch that is free during the factorisation (the
// permutation is built there and copied over piv).
template<int G, class MT>
__device__ __noinline__ void lu_factor(const Grp<G>& g, MT* A, int n, int ld, int* piv, double* invD, int* work) {
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
        // One thread picks the pivot row and the reciprocal of the pivot
        // (read from that row before the interchange) and publishes both
        // through piv[k] / invD[k]: the FP64 division and compares are issued
        // once per column, not by every warp of the group.
        if (g.rank == 0) {
            const int pr = choose_pivot(A, ld, k, pos, size);
            double akk = double(A[(size_t)pr * ld + k]);
            if (akk == 0) akk = kPivEps;
            invD[k] = double(MT(1.0 / akk));
            piv[k] = pr;
        }
        g.sync();
        const int p = piv[k];
        const MT rinv = MT(invD[k]);
        if (p != k) {
            MT* rk = A + (size_t)k * ld;
            MT* rp = A + (size_t)p * ld;
            for (int j = g.rank; j < n; j += G) { const MT t = rk[j]; rk[j] = rp[j]; rp[j] = t; }
            g.sync();
        }
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
    // The interchange sequence as one gather permutation (P b)[i] = b[perm[i]]
    // for the solves, built in the slot scratch and written over piv.
    for (int i = g.rank; i < n; i += G) work[i] = i;
    g.sync();
    if (g.rank == 0) {
        for (int j = 0; j < n; j++) {
            const int pj = piv[j];
            if (pj != j) { const int t = work[j]; work[j] = work[pj]; work[pj] = t; }
        }
    }
    g.sync();
    for (int i = g.rank; i < n; i += G) piv[i] = work[i];
    g.sync();
}

// Forward/back substitution with the factors of lu_factor after the row
// interchanges (LUsolver.C:3145-3171, 4113-4152).  One warp of the group
// does the column sweeps (shared-memory vector, one __syncwarp per column);
// the other warps wait at the closing group barrier.  b is a slot vector of
// doubles; arithmetic in MT.
template<int G, class MT, class VT>
__device__ __noinline__ void lu_solve(const Grp<G>& g, const MT* A, int n, int ld, const int* perm,
                                      const double* invD, VT* b) {
    g.sync();
    if (g.rank < 32) {
        const int lane = g.rank;
        VT t[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int i = lane + 32 * u;
            t[u] = i < n ? b[perm[i]] : VT(0);
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int i = lane + 32 * u;
            if (i < n) b[i] = t[u];
        }
        __syncwarp();
        for (int j = 0; j < n - 1; j++) {
            const VT bj = b[j];
            for (int i = j + 1 + lane; i < n; i += 32) b[i] = fma(-VT(A[(size_t)i * ld + j]), bj, b[i]);
            __syncwarp();
        }
        for (int j = n - 1; j >= 0; j--) {
            const VT xj = b[j] * VT(invD[j]);
            for (int i = lane; i < j; i += 32) b[i] = fma(-VT(A[(size_t)i * ld + j]), xj, b[i]);
            __syncwarp();
            if (lane == (j & 31)) b[j] = xj;
        }
        __syncwarp();
    }
    g.sync();
}

}  // namespace fcs
