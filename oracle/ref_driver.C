// ref_driver.C -- builds the REFERENCE numerical core (its own, unmodified
// Reaction/, LUsolver/ and ODE/ sources, compiled from the reference tree by
// oracle/Makefile) into the test-only library oracle/_ref/libfcs_ref.so.
//
// What this file adds, because OpenFOAM-10 is not available to compile the
// reference's model layer:
//   * fill_reaction(): fills OptReaction's public members from an
//     fcs_mechanism_desc, restating OptReaction::readInfo
//     (src/Reaction/OptReaction.C:348-1339) for the Arrhenius, third-body and
//     PLOG reaction types;
//   * RefModel: the members of FastChemistryModel that the ODE templates use,
//     with derivatives()/jacobian() restated from
//     src/ChemistryModel/FastChemistryModel.C:194-273, 340-417, 489-572;
//   * the cell loop of FastChemistryModel_transientSolve.H:30-104.
// TEST INFRASTRUCTURE ONLY (oracle validation and golden-vector generation).
#include "OptReaction.H"
#include "Jacobian.C"
#include "ReactionRate.C"
#include "Tc.C"

#include "chemistrySolver.H"
#include "LUsolver.H"

#include <atomic>
#include <memory>
#include <mutex>
#include <thread>

#include "../include/fcs.h"

// OptReaction's constructor and destructor live in OptReaction.C, which needs
// OpenFOAM dictionaries; their bodies are restated here (OptReaction.C:339-346,
// 1340-1346): the flag constructor does nothing, the destructor frees buffer.
OptReaction::OptReaction(bool) : buffer(nullptr) {}
OptReaction::~OptReaction() { free(this->buffer); }

namespace {

struct RefConfig {
    const fcs_mechanism_desc* desc;
    int jacobian;            // 0 exact, 1 fast
    double absTol, relTol;
    int maxSteps;
    const double* p;         // per-cell pressure (li indexes it)
};

// OptReaction::readInfo restated for a flat description (OptReaction.C:348-1339)
void fill_reaction(OptReaction& R, const fcs_mechanism_desc* d)
{
    const unsigned ns = d->n_species, nr = d->n_reactions;
    R.speciesTable_.resize(ns);
    for (unsigned i = 0; i < ns; i++) R.speciesTable_[i] = "S" + std::to_string(i);
    R.nReactions = nr;
    R.nSpecies = ns;
    for (unsigned r = 0; r < nr; r++) {
        if (d->type[r] == FCS_RXN_ARRHENIUS) R.n_Arrhenius++;
        else if (d->type[r] == FCS_RXN_THIRD_BODY) R.n_ThirdBodyReaction++;
        else if (d->type[r] == FCS_RXN_PLOG) R.n_PlogReaction++;
        else if (d->type[r] >= FCS_RXN_LINDEMANN_FALLOFF && d->type[r] <= FCS_RXN_SRI_FALLOFF) R.n_Fall_Off_Reaction++;
        else if (d->type[r] == FCS_RXN_NONEQ) R.n_NonEquilibriumReversibleArrhenius++;
        else if (d->type[r] == FCS_RXN_NONEQ_THIRD_BODY) R.n_NonEquilibriumThirdBodyReaction++;
        else throw std::runtime_error("unsupported reaction type in reference driver");
    }
    R.Itbr[0] = 0;
    R.Itbr[1] = R.n_NonEquilibriumThirdBodyReaction;
    R.Itbr[2] = R.Itbr[1] + R.n_ThirdBodyReaction;
    R.Itbr[3] = R.Itbr[2] + R.n_Fall_Off_Reaction;
    R.Itbr[4] = R.Itbr[3] + R.n_ChemicallyActivated_Reaction;
    R.Itbr[5] = R.Itbr[4] + R.n_NonEquilibriumThirdBodyReaction;
    R.Ikf[0] = 0;
    R.Ikf[1] = R.n_Arrhenius;
    R.Ikf[2] = R.Ikf[1] + R.n_NonEquilibriumReversibleArrhenius;
    R.Ikf[3] = R.Ikf[2] + R.n_NonEquilibriumThirdBodyReaction;
    R.Ikf[4] = R.Ikf[3] + R.n_ThirdBodyReaction;
    R.Ikf[5] = R.Ikf[4] + R.n_Fall_Off_Reaction;
    R.Ikf[6] = R.Ikf[5] + R.n_ChemicallyActivated_Reaction;
    R.Ikf[7] = R.Ikf[6] + R.n_Global_Reaction;
    R.Ikf[8] = R.Ikf[7] + R.n_Fall_Off_Reaction;
    R.Ikf[9] = R.Ikf[8] + R.n_ChemicallyActivated_Reaction;
    R.Ikf[10] = R.Ikf[9] + R.n_NonEquilibriumReversibleArrhenius;
    R.Ikf[11] = R.Ikf[10] + R.n_NonEquilibriumThirdBodyReaction;
    R.offset_kinf = -R.Ikf[4] + R.Ikf[7];
    R.A.resize(R.Ikf[11]);
    R.beta.resize(R.Ikf[11]);
    R.Ta.resize(R.Ikf[11]);
    R.lhsIndex.resize(nr); R.lhsstoichCoeff.resize(nr);
    R.rhsIndex.resize(nr); R.rhsstoichCoeff.resize(nr);
    R.ThirdBodyFactor.resize(R.Itbr[5]);
    R.HCoeffs.resize(ns); R.LCoeffs.resize(ns);
    R.Tlow.resize(ns); R.Thigh.resize(ns); R.Tcommon.resize(ns);
    R.PtrCoeffs.resize(ns);
    R.W.resize(ns); R.invW.resize(ns);
    R.isIrreversible.assign(nr, 0);
    R.sameSpecies.assign(nr, 1);
    double TcMax = 0, TcMin = 1e10;
    for (unsigned i = 0; i < ns; i++) {
        R.Tcommon[i] = d->T_common[i];
        R.Tlow[i] = d->T_low[i];
        R.Thigh[i] = d->T_high[i];
        R.W[i] = d->W[i];
        R.invW[i] = 1.0 / d->W[i];
        for (int j = 0; j < 7; j++) {
            R.HCoeffs[i][j] = d->high_coeffs[i * 7 + j];
            R.LCoeffs[i][j] = d->low_coeffs[i * 7 + j];
        }
        TcMax = R.Tcommon[i] > TcMax ? R.Tcommon[i] : TcMax;
        TcMin = R.Tcommon[i] < TcMin ? R.Tcommon[i] : TcMin;
    }
    R.TcommonMin = TcMin;
    R.TcommonMax = TcMax;
    auto species = [&](unsigned r, unsigned idx) {
        for (int j = d->lhs_offset[r]; j < d->lhs_offset[r + 1]; j++) {
            R.lhsIndex[idx].push_back(d->lhs_species[j]);
            R.lhsstoichCoeff[idx].push_back(1);
        }
        for (int j = d->rhs_offset[r]; j < d->rhs_offset[r + 1]; j++) {
            R.rhsIndex[idx].push_back(d->rhs_species[j]);
            R.rhsstoichCoeff[idx].push_back(1);
        }
    };
    unsigned iA = 0;
    for (int pass = 0; pass < 2; pass++) {
        for (unsigned r = 0; r < nr; r++) {
            if (d->type[r] != FCS_RXN_ARRHENIUS) continue;
            const double b = d->arrhenius[3 * r + 1], t = d->arrhenius[3 * r + 2];
            const bool ti = (b == 0 && t == 0);
            if ((pass == 0) != ti) continue;
            if (!d->reversible[r]) R.isIrreversible[iA] = 1;
            R.A[iA] = d->arrhenius[3 * r];
            R.beta[iA] = b;
            R.Ta[iA] = t;
            species(r, iA);
            iA++;
        }
    }
    // non-equilibrium, then non-equilibrium third-body (OptReaction.C:610-700):
    // forward rate at the reaction's slot, reverse at Ikf[9] onwards,
    // isIrreversible = 2; the third-body kind takes forward row k and reverse
    // row Itbr[4] + k, both from the forward coefficients as the reference reads them
    unsigned jr = R.Ikf[9];
    unsigned k = 0;
    for (int kind : {FCS_RXN_NONEQ, FCS_RXN_NONEQ_THIRD_BODY}) {
        for (unsigned r = 0; r < nr; r++) {
            if (d->type[r] != kind) continue;
            R.isIrreversible[iA] = 2;
            R.A[iA] = d->arrhenius[3 * r];
            R.beta[iA] = d->arrhenius[3 * r + 1];
            R.Ta[iA] = d->arrhenius[3 * r + 2];
            R.A[jr] = d->arrhenius2[3 * r];
            R.beta[jr] = d->arrhenius2[3 * r + 1];
            R.Ta[jr] = d->arrhenius2[3 * r + 2];
            if (kind == FCS_RXN_NONEQ_THIRD_BODY) {
                R.ThirdBodyFactor[k].resize(ns);
                R.ThirdBodyFactor[R.Itbr[4] + k].resize(ns);
                for (unsigned s = 0; s < ns; s++) {
                    R.ThirdBodyFactor[k][s] = d->efficiencies[(size_t)r * ns + s];
                    R.ThirdBodyFactor[R.Itbr[4] + k][s] = d->efficiencies[(size_t)r * ns + s];
                }
                k++;
            }
            species(r, iA);
            iA++; jr++;
        }
    }
    for (unsigned r = 0; r < nr; r++) {
        if (d->type[r] != FCS_RXN_THIRD_BODY) continue;
        if (!d->reversible[r]) R.isIrreversible[iA] = 1;
        R.A[iA] = d->arrhenius[3 * r];
        R.beta[iA] = d->arrhenius[3 * r + 1];
        R.Ta[iA] = d->arrhenius[3 * r + 2];
        R.ThirdBodyFactor[k].resize(ns);
        for (unsigned s = 0; s < ns; s++) R.ThirdBodyFactor[k][s] = d->efficiencies[(size_t)r * ns + s];
        species(r, iA);
        iA++; k++;
    }
    // fall-off reactions: Lindemann, then Troe, then SRI (OptReaction.C:746-917); k0 at
    // the reaction's slot, kInf at Ikf[7] + (slot - Ikf[4]), a third-body row each
    for (int kind : {FCS_RXN_LINDEMANN_FALLOFF, FCS_RXN_TROE_FALLOFF, FCS_RXN_SRI_FALLOFF}) {
        for (unsigned r = 0; r < nr; r++) {
            if (d->type[r] != kind) continue;
            if (!d->reversible[r]) R.isIrreversible[iA] = 1;
            R.A[iA] = d->arrhenius[3 * r];
            R.beta[iA] = d->arrhenius[3 * r + 1];
            R.Ta[iA] = d->arrhenius[3 * r + 2];
            const unsigned begin = iA - R.Ikf[4] + R.Ikf[7];
            R.A[begin] = d->arrhenius2[3 * r];
            R.beta[begin] = d->arrhenius2[3 * r + 1];
            R.Ta[begin] = d->arrhenius2[3 * r + 2];
            R.ThirdBodyFactor[k].resize(ns);
            for (unsigned s = 0; s < ns; s++) R.ThirdBodyFactor[k][s] = d->efficiencies[(size_t)r * ns + s];
            const double* f = &d->falloff_params[(size_t)r * 5];
            if (kind == FCS_RXN_LINDEMANN_FALLOFF) {
                R.Lindemann.push_back(iA);
            } else if (kind == FCS_RXN_TROE_FALLOFF) {
                R.Troe.push_back(iA);
                R.alpha_.push_back(f[0]);
                R.Ts_.push_back(f[1]);
                R.Tss_.push_back(f[2]);
                R.Tsss_.push_back(f[3]);
            } else {
                R.SRI.push_back(iA);
                R.a_.push_back(f[0]);
                R.b_.push_back(f[1]);
                R.c_.push_back(f[2]);
                R.d_.push_back(f[3]);
                R.e_.push_back(f[4]);
            }
            species(r, iA);
            iA++; k++;
        }
    }
    R.invTs_.resize(R.Ts_.size());
    R.invTsss_.resize(R.Tsss_.size());
    for (size_t i = 0; i < R.Ts_.size(); i++) R.invTs_[i] = 1.0 / R.Ts_[i];
    for (size_t i = 0; i < R.Tsss_.size(); i++) R.invTsss_[i] = 1.0 / R.Tsss_[i];
    R.invc_.resize(R.c_.size());
    for (size_t i = 0; i < R.c_.size(); i++) R.invc_[i] = 1.0 / R.c_[i];
    R.ThirdBodyFactor1D.resize(R.ThirdBodyFactor.size() * ns);
    {
        unsigned c = 0;
        for (auto& row : R.ThirdBodyFactor) for (double v : row) R.ThirdBodyFactor1D[c++] = v;
    }
    const unsigned np = R.n_PlogReaction;
    R.Kf_Plog.resize(np); R.dKfdT_Plog.resize(np);
    R.APlog.resize(np); R.logAPlog.resize(np); R.betaPlog.resize(np); R.TaPlog.resize(np);
    R.Prange.resize(np); R.rDeltaP_.resize(np); R.logPi.resize(np); R.Pindex.resize(np);
    unsigned a = 0;
    for (unsigned r = 0; r < nr; r++) {
        if (d->type[r] != FCS_RXN_PLOG) continue;
        if (!d->reversible[r]) R.isIrreversible[iA] = 1;
        const unsigned ps = d->plog_offset[r + 1] - d->plog_offset[r];
        R.APlog[a].resize(ps); R.logAPlog[a].resize(ps); R.betaPlog[a].resize(ps);
        R.TaPlog[a].resize(ps); R.Prange[a].resize(ps); R.rDeltaP_[a].resize(ps - 1);
        R.logPi[a].resize(ps);
        for (unsigned i = 0; i < ps; i++) {
            const double* row = &d->plog_table[4 * (d->plog_offset[r] + i)];
            R.Prange[a][i] = row[0];
            R.APlog[a][i] = row[1];
            R.logAPlog[a][i] = std::log(row[1]);
            R.betaPlog[a][i] = row[2];
            R.TaPlog[a][i] = row[3];
            R.logPi[a][i] = std::log(row[0]);
        }
        for (unsigned i = 0; i + 1 < ps; i++) R.rDeltaP_[a][i] = 1.0 / (R.logPi[a][i] - R.logPi[a][i + 1]);
        species(r, iA);
        iA++; a++;
    }
    std::vector<int> sumVki(nr);
    for (unsigned i = 0; i < nr; i++) sumVki[i] = int(R.rhsIndex[i].size()) - int(R.lhsIndex[i].size());
    if (nr) R.Pow_pByRT_SumVki_.insert({sumVki[0], 0.0});
    for (unsigned i = 1; i < nr; i++)
        if (R.Pow_pByRT_SumVki_.find(sumVki[i]) == R.Pow_pByRT_SumVki_.end())
            R.Pow_pByRT_SumVki_.insert({sumVki[i], 0.0});
    R.Kf_.resize(R.Ikf[11]);
    R.dKfdT_.resize(R.Ikf[11]);
    R.dKfdC_.resize(R.Itbr[5]);
    R.tmp_M.resize(R.Itbr[5]);
    R.tmp_Exp.resize(R.nSpecies + R.Troe.size() * 3 + R.SRI.size() * 2);
    R.n_Temperature_Independent_Reaction = 0;
    for (unsigned i = 0; i < R.n_Arrhenius; i++)
        if (R.beta[i] == 0 && R.Ta[i] == 0) R.n_Temperature_Independent_Reaction++;
    for (unsigned i = 0; i < R.n_Temperature_Independent_Reaction; i++) {
        R.Kf_[i] = R.A[i];
        R.dKfdT_[i] = 0;
    }
    R.n_ = R.nSpecies + 1;
    const unsigned arrSize = std::max(R.nSpecies, 5u);
    if (posix_memalign(reinterpret_cast<void**>(&R.buffer), 32, 4 * arrSize * sizeof(double)))
        throw std::bad_alloc();
    std::memset(R.buffer, 0, 4 * arrSize * sizeof(double));
    R.ArrPtr.resize(arrSize);
    for (unsigned i = 0; i < arrSize; i++) R.ArrPtr[i] = R.buffer + 4 * i;
    R.TlowMin = 1e10;
    R.ThighMax = 1;
    for (unsigned i = 0; i < ns; i++) {
        if (R.TlowMin > R.Tlow[i]) R.TlowMin = R.Tlow[i];
        if (R.ThighMax < R.Thigh[i]) R.ThighMax = R.Thigh[i];
    }
    R.RFTable[1][1] = &OptReaction::RF11; R.RFTable[1][2] = &OptReaction::RF12;
    R.RFTable[1][3] = &OptReaction::RF13; R.RFTable[2][1] = &OptReaction::RF21;
    R.RFTable[2][2] = &OptReaction::RF22; R.RFTable[2][3] = &OptReaction::RF23;
    R.RFTable[3][1] = &OptReaction::RF31; R.RFTable[3][2] = &OptReaction::RF32;
    R.RFTable[3][3] = &OptReaction::RF33;
    R.lhsOffset.assign(nr + 1, 0);
    R.rhsOffset.assign(nr + 1, 0);
    for (unsigned i = 0; i < nr; i++) {
        R.lhsOffset[i + 1] = R.lhsOffset[i] + R.lhsIndex[i].size();
        for (unsigned s : R.lhsIndex[i]) R.lhsSpeciesIndex.push_back(s);
        R.rhsOffset[i + 1] = R.rhsOffset[i] + R.rhsIndex[i].size();
        for (unsigned s : R.rhsIndex[i]) R.rhsSpeciesIndex.push_back(s);
    }
    for (unsigned i = 0; i < nr; i++) {
        std::vector<unsigned> seen;
        bool dup = false;
        for (unsigned s : R.lhsIndex[i]) { if (std::find(seen.begin(), seen.end(), s) != seen.end()) dup = true; seen.push_back(s); }
        for (unsigned s : R.rhsIndex[i]) { if (std::find(seen.begin(), seen.end(), s) != seen.end()) dup = true; seen.push_back(s); }
        R.sameSpecies[i] = dup ? 1 : 0;
    }
}

}  // namespace

// The FastChemistryModel members the ODE templates call.
class RefModel {
public:
    RefConfig cfg;
    mutable OptReaction reaction;
    int nSpecie_, n_;
    mutable std::vector<double> c_;
    std::vector<double> buf;
    mutable double* YTpWork[12];
    mutable double* YTpYTpWork[3];
    Foam::dictionary coeffs;
    mutable long long nJac = 0, nRhs = 0;

    RefModel(const Foam::fluidReactionThermo& t)
        : cfg(*static_cast<RefConfig*>(t.cfg)), reaction(true)
    {
        fill_reaction(reaction, cfg.desc);
        nSpecie_ = cfg.desc->n_species;
        n_ = nSpecie_ + 1;
        c_.assign(nSpecie_, 0.0);
        buf.assign(12 * n_ + 3 * n_ * n_ + 8, 0.0);
        size_t pos = 0;
        for (int i = 0; i < 12; i++) { YTpWork[i] = &buf[pos]; pos += n_; }
        for (int i = 0; i < 3; i++) { YTpYTpWork[i] = &buf[pos]; pos += n_ * n_; }
        coeffs.kv["absTol"] = cfg.absTol;
        coeffs.kv["relTol"] = cfg.relTol;
        coeffs.kv["maxSteps"] = cfg.maxSteps;
    }
    ~RefModel() { free(reaction.buffer); reaction.buffer = nullptr; }
    int nSpecie() const { return nSpecie_; }
    const Foam::dictionary& subDict(const std::string&) const { return coeffs; }

    // FastChemistryModel.C:194-273 (7 arguments) and 340-417 (6 arguments)
    void derivs(double p, double* YT, double* dYTdt, double* Cp, double* Ha, double* ExpGbyRT, bool seven) const
    {
        nRhs++;
        const double T = YT[nSpecie_];
        for (int i = 0; i < nSpecie_; i++) YT[i] = YT[i] > 0 ? YT[i] : 0;
        const double RuTByP = reaction.Ru * T / p;
        double s = 0;
        for (int i = 0; i < nSpecie_; i++) s = std::fma(YT[i] * reaction.invW[i], RuTByP, s);
        const double invrhoM = s;
        const double rhoM = 1 / s;
        for (int i = 0; i < nSpecie_; i++) c_[i] = rhoM * reaction.invW[i] * YT[i];
        std::memset(dYTdt, 0, n_ * sizeof(double));
        if (seven) reaction.dNdtByV(p, T, c_.data(), dYTdt, ExpGbyRT, Cp, Ha);
        else { reaction.dNdtByV(p, T, c_.data(), dYTdt, Cp); reaction.CpHa(T, Cp, Ha); }
        double CpM = 0, dTdt = 0;
        for (int i = 0; i < nSpecie_; i++) {
            dYTdt[i] = (reaction.W[i] * invrhoM) * dYTdt[i];
            CpM = std::fma(YT[i], Cp[i], CpM);
            dTdt = std::fma(Ha[i], dYTdt[i], dTdt);
        }
        dYTdt[nSpecie_] = -dTdt / CpM;
    }
    void derivatives(double, int li, double* YT, double* dYTdt, double* Cp, double* Ha, double* E) const
    { derivs(cfg.p[li], YT, dYTdt, Cp, Ha, E, true); }
    void derivatives(double, int li, double* YT, double* dYTdt, double* Cp, double* Ha) const
    { derivs(cfg.p[li], YT, dYTdt, Cp, Ha, nullptr, false); }

    // FastChemistryModel.C:489-572
    void jacobian(double, double* YT_, int li, double* dYTdt, double* Jy) const
    {
        nJac++;
        for (int i = 0; i < nSpecie_; i++) YT_[i] = YT_[i] > 0 ? YT_[i] : 0;
        const double T = YT_[nSpecie_];
        const double p = cfg.p[li];
        double* Jc = YTpYTpWork[0];
        std::memset(Jc, 0, n_ * n_ * sizeof(double));
        std::memset(dYTdt, 0, n_ * sizeof(double));
        double* ExpNegGbyRT = YTpWork[3];
        double* dBdT = YTpWork[4];
        double* dCpdT = YTpWork[5];
        double* Cp = YTpWork[6];
        double* Ha = YTpWork[7];
        double* WiByrhoM = YTpWork[8];
        double* rhoMvj = YTpWork[10];
        reaction.ddNdtByVdcTp(p, T, YT_, c_.data(), dYTdt, ExpNegGbyRT, dBdT, dCpdT, Cp, Ha,
                              rhoMvj, WiByrhoM, Jc, true);
        const unsigned remain = reaction.nSpecies % 4;
        if (cfg.jacobian == FCS_JACOBIAN_FAST) {
            reaction.FastddYdtdY_Vec(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, dYTdt, YT_, Jy);
            reaction.ddYdtdTP_Vec(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, c_.data(), dYTdt, YT_, Jy);
            reaction.ddTdtdYT_Vec(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, Cp, dCpdT, Ha, dYTdt, YT_, Jy);
        } else if (remain == 0) {
            reaction.ddYdtdY_Vec1_0(Jc, rhoMvj, WiByrhoM, dYTdt, YT_, Jy);
            reaction.ddYdtdTP_Vec_0(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, c_.data(), dYTdt, YT_, Jy);
            reaction.ddTdtdYT_Vec_0(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, Cp, dCpdT, Ha, dYTdt, YT_, Jy);
        } else if (remain == 1) {
            reaction.ddYdtdY_Vec1_1(Jc, rhoMvj, WiByrhoM, dYTdt, YT_, Jy);
            reaction.ddYdtdTP_Vec_1(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, c_.data(), dYTdt, YT_, Jy);
            reaction.ddTdtdYT_Vec_1(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, Cp, dCpdT, Ha, dYTdt, YT_, Jy);
        } else if (remain == 2) {
            reaction.ddYdtdY_Vec1_2(Jc, rhoMvj, WiByrhoM, dYTdt, YT_, Jy);
            reaction.ddYdtdTP_Vec_2(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, c_.data(), dYTdt, YT_, Jy);
            reaction.ddTdtdYT_Vec_2(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, Cp, dCpdT, Ha, dYTdt, YT_, Jy);
        } else {
            reaction.ddYdtdY_Vec1_3(Jc, rhoMvj, WiByrhoM, dYTdt, YT_, Jy);
            reaction.ddYdtdTP_Vec_3(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, c_.data(), dYTdt, YT_, Jy);
            reaction.ddTdtdYT_Vec_3(ExpNegGbyRT, Jc, rhoMvj, WiByrhoM, Cp, dCpdT, Ha, dYTdt, YT_, Jy);
        }
    }
};

#include "OptRodas34.H"
#include "OptRodas34.C"
#include "OptRosenbrock34.H"
#include "OptRosenbrock34.C"
#include "OptSeulex.H"
#include "OptSeulex.C"
#include "OptRodas23.H"
#include "OptRodas23.C"
#include "OptRosenbrock23.H"
#include "OptRosenbrock23.C"

template class Foam::OptRodas34<RefModel>;
template class Foam::OptRosenbrock34<RefModel>;
template class Foam::OptSeulex<RefModel>;
template class Foam::OptRodas23<RefModel>;
template class Foam::OptRosenbrock23<RefModel>;

namespace {

struct Solver {
    virtual ~Solver() {}
    virtual void solve(double& p, double& T, Foam::scalarField& Y, int li, double& dt, double& sub) = 0;
    virtual RefModel& model() = 0;
};
template<class S> struct SolverT : Solver {
    S s;
    explicit SolverT(const Foam::fluidReactionThermo& t) : s(t) {}
    void solve(double& p, double& T, Foam::scalarField& Y, int li, double& dt, double& sub) override
    { s.solve(p, T, Y, li, dt, sub); }
    RefModel& model() override { return s; }
};

struct RefHandle {
    fcs_mechanism_desc desc;
    // deep copies of the description arrays
    std::vector<double> W, Tl, Th, Tc, hc, lc, arr, arr2, fo, eff, pt;
    std::vector<int32_t> type, rev, lo, ls, ro, rs, po;
    int solver, jacobian, maxSteps;
    double absTol, relTol;
};

std::unique_ptr<Solver> make_solver(RefHandle* h, RefConfig* cfg)
{
    Foam::fluidReactionThermo t{cfg};
    if (h->solver == FCS_SOLVER_RODAS34) return std::unique_ptr<Solver>(new SolverT<Foam::OptRodas34<RefModel>>(t));
    if (h->solver == FCS_SOLVER_ROSENBROCK34) return std::unique_ptr<Solver>(new SolverT<Foam::OptRosenbrock34<RefModel>>(t));
    if (h->solver == FCS_SOLVER_RODAS23) return std::unique_ptr<Solver>(new SolverT<Foam::OptRodas23<RefModel>>(t));
    if (h->solver == FCS_SOLVER_ROSENBROCK23) return std::unique_ptr<Solver>(new SolverT<Foam::OptRosenbrock23<RefModel>>(t));
    return std::unique_ptr<Solver>(new SolverT<Foam::OptSeulex<RefModel>>(t));
}

}  // namespace

extern "C" {

void* ref_create(const fcs_mechanism_desc* d, int solver, int jacobian, double absTol,
                 double relTol, int maxSteps)
{
    RefHandle* h = new RefHandle();
    const int ns = d->n_species, nr = d->n_reactions;
    h->W.assign(d->W, d->W + ns);
    h->Tl.assign(d->T_low, d->T_low + ns);
    h->Th.assign(d->T_high, d->T_high + ns);
    h->Tc.assign(d->T_common, d->T_common + ns);
    h->hc.assign(d->high_coeffs, d->high_coeffs + 7 * ns);
    h->lc.assign(d->low_coeffs, d->low_coeffs + 7 * ns);
    h->type.assign(d->type, d->type + nr);
    h->rev.assign(d->reversible, d->reversible + nr);
    h->lo.assign(d->lhs_offset, d->lhs_offset + nr + 1);
    h->ro.assign(d->rhs_offset, d->rhs_offset + nr + 1);
    h->ls.assign(d->lhs_species, d->lhs_species + d->lhs_offset[nr]);
    h->rs.assign(d->rhs_species, d->rhs_species + d->rhs_offset[nr]);
    h->arr.assign(d->arrhenius, d->arrhenius + 3 * nr);
    if (d->efficiencies) h->eff.assign(d->efficiencies, d->efficiencies + (size_t)nr * ns);
    else h->eff.assign((size_t)nr * ns, 1.0);
    if (d->arrhenius2) h->arr2.assign(d->arrhenius2, d->arrhenius2 + 3 * nr);
    else h->arr2.assign(3 * (size_t)nr, 0.0);
    if (d->falloff_params) h->fo.assign(d->falloff_params, d->falloff_params + 5 * (size_t)nr);
    else h->fo.assign(5 * (size_t)nr, 0.0);
    h->po.assign(d->plog_offset, d->plog_offset + nr + 1);
    h->pt.assign(d->plog_table, d->plog_table + 4 * (size_t)d->plog_offset[nr]);
    fcs_mechanism_desc& c = h->desc;
    std::memset(&c, 0, sizeof(c));
    c.n_species = ns; c.n_reactions = nr;
    c.W = h->W.data(); c.T_low = h->Tl.data(); c.T_high = h->Th.data(); c.T_common = h->Tc.data();
    c.high_coeffs = h->hc.data(); c.low_coeffs = h->lc.data();
    c.type = h->type.data(); c.reversible = h->rev.data();
    c.lhs_offset = h->lo.data(); c.lhs_species = h->ls.data();
    c.rhs_offset = h->ro.data(); c.rhs_species = h->rs.data();
    c.arrhenius = h->arr.data(); c.efficiencies = h->eff.data();
    c.arrhenius2 = h->arr2.data(); c.falloff_params = h->fo.data();
    c.plog_offset = h->po.data(); c.plog_table = h->pt.data();
    for (int r = 0; r < nr; r++)
        if (d->type[r] < FCS_RXN_ARRHENIUS || d->type[r] > FCS_RXN_NONEQ_THIRD_BODY) {
            delete h;
            return nullptr;
        }
    h->solver = solver; h->jacobian = jacobian; h->absTol = absTol; h->relTol = relTol;
    h->maxSteps = maxSteps;
    return h;
}

void ref_destroy(void* handle) { delete static_cast<RefHandle*>(handle); }

// Cell loop of FastChemistryModel_transientSolve.H:30-104 (serial path),
// run by n_threads independent solver instances pulling from one queue.
int ref_integrate(void* handle, int64_t n, double deltaT, const double* p, const double* rho0,
                  double* T, double* Y, double* subDt, double* RR, int32_t* status,
                  double Treact, double dtChemMax, double* deltaTMin, int64_t* counters,
                  int n_threads)
{
    RefHandle* h = static_cast<RefHandle*>(handle);
    const int ns = h->desc.n_species;
    std::atomic<int64_t> next(0);
    std::mutex mu;
    double dmin = Foam::great;
    int64_t nJac = 0, nRhs = 0, nFail = 0, nCells = 0;
    auto work = [&]() {
        RefConfig cfg{&h->desc, h->jacobian, h->absTol, h->relTol, h->maxSteps, p};
        std::unique_ptr<Solver> s = make_solver(h, &cfg);
        Foam::scalarField Y_(ns), Y0(ns);
        double lmin = Foam::great;
        int64_t lfail = 0, lcells = 0;
        for (;;) {
            const int64_t c = next.fetch_add(1);
            if (c >= n) break;
            double Tc = T[c];
            if (!(Tc > Treact)) {
                if (RR) for (int i = 0; i < ns; i++) RR[(size_t)i * n + c] = 0;
                if (status) status[c] = FCS_CELL_SKIPPED;
                continue;
            }
            double pc = p[c];
            for (int i = 0; i < ns; i++) Y_[i] = Y0[i] = Y[(size_t)i * n + c];
            double timeLeft = deltaT;
            int st = FCS_CELL_OK;
            try {
                while (timeLeft > Foam::small) {
                    double dt = timeLeft;
                    s->solve(pc, Tc, Y_, int(c), dt, subDt[c]);
                    timeLeft -= dt;
                }
            } catch (const Foam::fatal_error&) {
                st = FCS_CELL_MAX_STEPS;
                lfail++;
            }
            lcells++;
            lmin = std::min(lmin, subDt[c]);
            subDt[c] = std::min(subDt[c], dtChemMax);
            for (int i = 0; i < ns; i++) {
                if (RR) RR[(size_t)i * n + c] = (Y_[i] * rho0[c] - Y0[i] * rho0[c]) / deltaT;
                Y[(size_t)i * n + c] = Y_[i];
            }
            T[c] = Tc;
            if (status) status[c] = st;
        }
        std::lock_guard<std::mutex> g(mu);
        dmin = std::min(dmin, lmin);
        nJac += s->model().nJac;
        nRhs += s->model().nRhs;
        nFail += lfail;
        nCells += lcells;
    };
    if (n_threads <= 1) work();
    else {
        std::vector<std::thread> th;
        for (int t = 0; t < n_threads; t++) th.emplace_back(work);
        for (auto& x : th) x.join();
    }
    if (deltaTMin) *deltaTMin = std::min(dmin, 2 * deltaT);
    if (counters) {
        counters[0] = nJac; counters[1] = nRhs; counters[2] = nCells; counters[3] = nFail;
    }
    return nFail ? FCS_ERR_CELLS : FCS_OK;
}

int ref_rhs(void* handle, int64_t n, const double* p, const double* T, const double* Y, double* dydt)
{
    RefHandle* h = static_cast<RefHandle*>(handle);
    RefConfig cfg{&h->desc, h->jacobian, h->absTol, h->relTol, h->maxSteps, p};
    Foam::fluidReactionThermo t{&cfg};
    RefModel m(t);
    const int ns = h->desc.n_species, nn = ns + 1;
    std::vector<double> y(nn), f(nn), Cp(nn), Ha(nn), E(nn + 8);
    for (int64_t c = 0; c < n; c++) {
        for (int i = 0; i < ns; i++) y[i] = Y[(size_t)i * n + c];
        y[ns] = T[c];
        m.derivatives(0, int(c), y.data(), f.data(), Cp.data(), Ha.data(), E.data());
        for (int i = 0; i < nn; i++) dydt[(size_t)i * n + c] = f[i];
    }
    return 0;
}

int ref_jacobian(void* handle, int64_t n, const double* p, const double* T, const double* Y,
                 double* J, double* dydt)
{
    RefHandle* h = static_cast<RefHandle*>(handle);
    RefConfig cfg{&h->desc, h->jacobian, h->absTol, h->relTol, h->maxSteps, p};
    Foam::fluidReactionThermo t{&cfg};
    RefModel m(t);
    const int ns = h->desc.n_species, nn = ns + 1;
    std::vector<double> y(nn), f(nn);
    for (int64_t c = 0; c < n; c++) {
        for (int i = 0; i < ns; i++) y[i] = Y[(size_t)i * n + c];
        y[ns] = T[c];
        m.jacobian(0, y.data(), int(c), f.data(), &J[(size_t)c * nn * nn]);
        for (int i = 0; i < nn; i++) dydt[(size_t)i * n + c] = f[i];
    }
    return 0;
}

// FastChemistryModel::tc (FastChemistryModel.C:589-651) over OptReaction::Tc
// (Tc.C:3-834): c = rho Y / W, tc = sumW / sumWRateByCTot * sum(c)
int ref_tc(void* handle, int64_t n, const double* p, const double* T, const double* rho, const double* Y,
           double* tc)
{
    RefHandle* h = static_cast<RefHandle*>(handle);
    RefConfig cfg{&h->desc, h->jacobian, h->absTol, h->relTol, h->maxSteps, p};
    Foam::fluidReactionThermo t{&cfg};
    RefModel m(t);
    const int ns = h->desc.n_species;
    std::vector<double> c(ns);
    for (int64_t k = 0; k < n; k++) {
        double sumc = 0;
        for (int i = 0; i < ns; i++) {
            c[i] = rho[k] * Y[(size_t)i * n + k] / h->desc.W[i];
            sumc += c[i];
        }
        double sumW = 0, sumWR = 0;
        m.reaction.Tc(int(k), p[k], T[k], c.data(), sumW, sumWR);
        tc[k] = sumWR == 0 ? Foam::vGreat : sumW / sumWR * sumc;
    }
    return 0;
}

// LU of one matrix with the reference LUsolver (LUsolver.C:3058-3171)
int ref_lu_solve(int n, double* a, int nrhs, double* b)
{
    LUsolver lu(a, n);
    lu.Block4LUDecompose();
    for (int r = 0; r < nrhs; r++) lu.xSolve(&b[(size_t)r * n]);
    return 0;
}

}  // extern "C"
