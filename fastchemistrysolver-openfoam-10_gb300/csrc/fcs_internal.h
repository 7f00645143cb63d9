// fcs_internal.h -- layouts shared by the host packing code and the sm_103a
// kernels of libfcs_cuda.so.
//
// Mechanism image in HBM (built once by pack_mechanism, read through L1):
//   * species arrays W, invW, Tcommon and the NASA-7 sets, 16 doubles per
//     species (low[0..6], pad, high[0..6], pad): one 128-byte line each;
//   * one 64-byte RxnInfo per reaction, in the reference's type-block order
//     (OptReaction.C:448-1175): constant Arrhenius, other Arrhenius,
//     third-body, PLOG;
//   * the dense third-body efficiency matrix [nTB][Ns] (ThirdBodyFactor1D);
//   * PLOG tables as (log p, log A, beta, Ta) rows;
//   * a species -> (reaction, sign) incidence list in reaction order, which
//     lets one thread own a species row and accumulate its production rate and
//     Jacobian row in exactly the order the reference's scatter updates it.
#pragma once
#include <stdint.h>

namespace fcs {

constexpr double kRu = 8314.470066505449722171761095523834228515625;  // OptReaction.H:404
constexpr double kPstd = 100000.0;                                    // OptReaction.H:409
constexpr double kKcClamp = 1.4901171103413047e-8;                    // ReactionFunctionI.H:17
constexpr double kKcClampG = 1.49011611938476e-8;                     // RFG/JFG: more than 3 per side
constexpr double kPivEps = 2.2204460492503131e-16;                    // LUsolver.C:154
constexpr double kSmall = 1.0e-15;                                    // OpenFOAM small
// reactants / products per reaction handled on the GPU (species indices are
// bytes: at most 255 species); the tutorial mechanisms have at most 3 / 7
constexpr int kMaxL = 4, kMaxR = 8;

struct RxnInfo {            // 64 bytes
    double A, beta, Ta;     // Arrhenius (OpenFOAM form k = A T^beta exp(-Ta/T))
    uint8_t sl[kMaxL];      // reactant species (repeated by stoichiometry)
    uint8_t sr[kMaxR];      // product species
    int8_t nl, nr;          // counts
    int8_t rev;             // 1 reversible (Kr = Kf / Kc), 2 non-equilibrium (Kr its own Arrhenius)
    int8_t kind;            // FCS_RXN_*
    int32_t tb;             // third-body row or -1
    int32_t plog;           // PLOG index or -1
    int32_t dnu;            // nr - nl
    int32_t tind;           // temperature independent (beta == 0 and Ta == 0)
    int32_t fo;             // fall-off index (kInf and F parameters in DevMech::fo) or -1
    int32_t nq;             // non-equilibrium reverse-rate index (A, beta, Ta in DevMech::fo) or -1
};
static_assert(sizeof(RxnInfo) == 64, "RxnInfo must stay 64 bytes");

struct DevMech {
    int ns, n, nr;
    int nTB, nPlog;
    int spBegin, nSp;       // special block of the packed order: first to last non-equilibrium or
                            // fall-off reaction
    double TlowMin, ThighMax, TcommonMin, TcommonMax;
    const double* W;        // [ns]
    const double* invW;     // [ns]
    const double* Tcommon;  // [ns]
    const double* coef;     // [ns][16]
    const RxnInfo* rx;      // [nr]
    const double* eff;      // [nTB][ns]
    const int* plogOff;     // [nPlog+1]
    const double* plogRow;  // [rows][4]: p, logP, logA, beta   (Ta in plogTa)
    const double* plogTa;   // [rows]
    const int* incOff;      // [ns+1]
    const int* inc;         // (reaction << 1) | (1 if product else 0)
    int nTbInc;             // third-body incidences (species row, third-body row, side)
    const int* tbInc;       // (row << 16) | (tb << 1) | (1 if product else 0), reaction order
    const double* hf;       // [ns] formation enthalpy at 298.15 K, J/kg (for Qdot)
    const double* fo;       // [n fall-off + n non-equilibrium][8]: kInf A, beta, Ta; Troe alpha, T*, T**,
                            // T*** / SRI a, b, c, d, e -- or the reverse A, beta, Ta of a non-equilibrium reaction
};

// Per-cell options the kernels need (copied by value into kernel params).
struct KOpts {
    int solver;             // FCS_SOLVER_*
    int jacobian;           // FCS_JACOBIAN_*
    int maxSteps;
    int maxRejects;
    double absTol, relTol;
    double Treact;
    double dtChemMax;
};

// Per-cell status / counters layout in the stats buffer (int64 each).
enum { ST_CELLS = 0, ST_SKIPPED, ST_FAILED, ST_ATTEMPTS, ST_ACCEPTED, ST_JAC, ST_LU,
       ST_RHS, ST_SOLVES, ST_FALLBACK, ST_COUNT };

}  // namespace fcs
