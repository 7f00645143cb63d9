/*
 * FastChemistryModel.C -- member functions of the GPU chemistry model (see
 * FastChemistryModel.H).  Included by the header (template definitions).
 */
#include <cstdlib>
#include <fstream>
#include <string>

namespace Foam {

namespace fcsPlugin {

struct SpeciesNames {
    std::vector<std::string> names;
};

inline fcs_status collectNames(const fcs_mechanism_desc* d, const char* const* names, void* user) {
    SpeciesNames* s = static_cast<SpeciesNames*>(user);
    s->names.assign(names, names + d->n_species);
    return FCS_OK;
}

inline bool exists(const fileName& f) { return std::ifstream(f).good(); }

}  // namespace fcsPlugin

template<class ThermoType>
void FastChemistryModel<ThermoType>::check(fcs_status s, const char* call) const {
    if (s == FCS_OK) return;
    if (s == FCS_ERR_CELLS) {
        label failed = 0;
        for (int32_t v : status_) failed += (v != FCS_CELL_OK && v != FCS_CELL_SKIPPED);
        FatalErrorInFunction << call << ": the integration of " << failed
                             << " cell(s) did not finish (status per cell: maxSteps, non-finite or step "
                                "underflow): " << fcs_last_error_string(ctx_) << exit(FatalError);
    }
    FatalErrorInFunction << call << " failed (fcs status " << s << "): "
                         << (ctx_ ? fcs_last_error_string(ctx_) : "no context") << exit(FatalError);
}

template<class ThermoType>
FastChemistryModel<ThermoType>::FastChemistryModel(const fluidReactionThermo& thermo, int32_t solver)
    : basicChemistryModel(thermo), ctx_(nullptr), nSpecie_(0), nReaction_(0) {
    const char* dev = std::getenv("FCS_DEVICE");
    check(fcs_create(&ctx_, dev ? std::atoi(dev) : 0), "fcs_create");
    // chemistryProperties: solver coefficients, jacobian, Treact, maxChemicalTimeStep, FastChemistryGPU{}
    double ini = -1;
    check(fcs_read_chemistry_properties(dictPath().c_str(), &opt_, &ini), "fcs_read_chemistry_properties");
    if (opt_.solver != solver)
        FatalErrorInFunction << "chemistryType solver does not match the selected solver class" << exit(FatalError);
    check(fcs_set_options(ctx_, &opt_), "fcs_set_options");
    // the mechanism: constant/reactions and the species thermo
    const fileName constant = mesh_.time().constant();
    const fileName reactions = constant + "/reactions";
    fileName thermoFile = constant + "/speciesThermo";
    if (!fcsPlugin::exists(thermoFile)) thermoFile = constant + "/physicalProperties";
    check(fcs_load_mechanism_foam(ctx_, reactions.c_str(), thermoFile.c_str()), "fcs_load_mechanism_foam");
    int32_t ns = 0, nr = 0;
    check(fcs_mechanism_size(ctx_, &ns, &nr), "fcs_mechanism_size");
    nSpecie_ = ns;
    nReaction_ = nr;
    // the library's species order against the thermo's
    fcsPlugin::SpeciesNames lib;
    check(fcs_parse_mechanism_foam(reactions.c_str(), thermoFile.c_str(), fcsPlugin::collectNames, &lib),
          "fcs_parse_mechanism_foam");
    const wordList& sp = thermo.species();
    if (label(sp.size()) != ns)
        FatalErrorInFunction << "the thermo has " << sp.size() << " species, the mechanism " << ns
                             << exit(FatalError);
    thermoIndex_.assign(ns, -1);
    for (label k = 0; k < ns; k++) {
        for (label i = 0; i < label(sp.size()); i++)
            if (sp[i] == lib.names[k]) thermoIndex_[k] = i;
        if (thermoIndex_[k] < 0)
            FatalErrorInFunction << "species " << lib.names[k] << " of the mechanism is not in the thermo"
                                 << exit(FatalError);
    }
    hf_.assign(ns, 0.0);
    check(fcs_formation_enthalpy(ctx_, hf_.data()), "fcs_formation_enthalpy");
    // RR(i) follows the thermo's species order, as OpenFOAM's solvers index it
    RR_.setSize(ns);
    for (label k = 0; k < ns; k++) RR_.set(thermoIndex_[k], new volScalarField("RR." + lib.names[k], mesh_, 0.0));
}

template<class ThermoType>
FastChemistryModel<ThermoType>::~FastChemistryModel() {
    if (ctx_) fcs_destroy(ctx_);
}

// p, T, rho and Y (species-major in the library's order) of every cell
template<class ThermoType>
void FastChemistryModel<ThermoType>::gather() const {
    const label n = mesh_.nCells(), ns = nSpecie_;
    const tmp<volScalarField> trho(thermo_.rho());
    p_.assign(thermo_.p().begin(), thermo_.p().end());
    T_.assign(thermo_.T().begin(), thermo_.T().end());
    rho_.assign(trho().begin(), trho().end());
    Y_.resize(size_t(ns) * n);
    for (label k = 0; k < ns; k++) {
        const volScalarField& Yk = thermo_.Y()[thermoIndex_[k]];
        std::copy(Yk.begin(), Yk.end(), Y_.begin() + size_t(k) * n);
    }
}

template<class ThermoType>
scalar FastChemistryModel<ThermoType>::integrate(const double* deltaTPerCell, scalar deltaT) {
    const label n = mesh_.nCells(), ns = nSpecie_;
    if (!chemistry_) return great;
    gather();
    sub_.assign(deltaTChem_.begin(), deltaTChem_.end());
    RRbuf_.assign(size_t(ns) * n, 0.0);
    status_.assign(n, FCS_CELL_OK);
    fcs_step_stats stats;
    double dtMin = great;
    // T and Y are copies: the chemistry step leaves the thermo's fields as
    // they are and reports the change through RR (transientSolve.H:35-83)
    const fcs_status s = deltaTPerCell
        ? fcs_integrate_lts(ctx_, n, deltaTPerCell, p_.data(), rho_.data(), T_.data(), Y_.data(), sub_.data(),
                            RRbuf_.data(), status_.data(), &stats, &dtMin, 0)
        : fcs_integrate(ctx_, n, deltaT, p_.data(), rho_.data(), T_.data(), Y_.data(), sub_.data(), RRbuf_.data(),
                        status_.data(), &stats, &dtMin, 0);
    check(s, deltaTPerCell ? "fcs_integrate_lts" : "fcs_integrate");
    for (label k = 0; k < ns; k++)
        std::copy(RRbuf_.begin() + size_t(k) * n, RRbuf_.begin() + size_t(k + 1) * n, RR_[thermoIndex_[k]].begin());
    std::copy(sub_.begin(), sub_.end(), deltaTChem_.begin());
    return dtMin;
}

template<class ThermoType>
scalar FastChemistryModel<ThermoType>::solve(const scalar deltaT) {
    return integrate(nullptr, deltaT);
}

template<class ThermoType>
scalar FastChemistryModel<ThermoType>::solve(const scalarField& deltaT) {
    dt_.assign(deltaT.begin(), deltaT.end());
    return integrate(dt_.data(), 0.0);
}

template<class ThermoType>
void FastChemistryModel<ThermoType>::calculate() {
    if (!chemistry_) return;
    const label n = mesh_.nCells(), ns = nSpecie_;
    gather();
    RRbuf_.assign(size_t(ns) * n, 0.0);
    check(fcs_rates(ctx_, n, p_.data(), T_.data(), rho_.data(), Y_.data(), RRbuf_.data(), nullptr, 0), "fcs_rates");
    for (label k = 0; k < ns; k++)
        std::copy(RRbuf_.begin() + size_t(k) * n, RRbuf_.begin() + size_t(k + 1) * n, RR_[thermoIndex_[k]].begin());
}

template<class ThermoType>
tmp<volScalarField> FastChemistryModel<ThermoType>::tc() const {
    tmp<volScalarField> ttc(volScalarField::New("tc", mesh_, small));
    if (!chemistry_) return ttc;
    gather();
    check(fcs_tc(ctx_, mesh_.nCells(), p_.data(), T_.data(), rho_.data(), Y_.data(), ttc.ref().data(), 0), "fcs_tc");
    return ttc;
}

// -sum_i Hf_i RR_i over the last solve's (or calculate's) RR (FastChemistryModel.C:653-686)
template<class ThermoType>
tmp<volScalarField> FastChemistryModel<ThermoType>::Qdot() const {
    tmp<volScalarField> tQdot(volScalarField::New("Qdot", mesh_, 0.0));
    if (!chemistry_) return tQdot;
    volScalarField& Qdot = tQdot.ref();
    for (label k = 0; k < nSpecie_; k++) {
        const volScalarField::Internal& R = RR_[thermoIndex_[k]];
        for (label c = 0; c < mesh_.nCells(); c++) Qdot[c] -= hf_[k] * R[c];
    }
    return tQdot;
}

}  // namespace Foam
