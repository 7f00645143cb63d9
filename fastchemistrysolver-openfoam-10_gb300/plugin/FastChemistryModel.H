/*
 * FastChemistryModel.H -- the chemistry model of libFastChemistryModel.so,
 * the OpenFOAM-10 plugin, on the GPU.
 *
 * Drop-in for the reference plugin's model (src/ChemistryModel/FastChemistryModel.H:57-330):
 * same name ("FastChemistryModel"), same solvers registered with it
 * (odeChemistrySolvers.C here, src/odeChemistrySolvers.C:63-74 there), same
 * chemistryProperties keys, same basicChemistryModel overrides --
 * solve(scalar) (FastChemistryModel_transientSolve.H:2-104),
 * solve(scalarField) (FastChemistryModel_localEulerSolve.H:3-101), RR(i),
 * calculate() (FastChemistryModel.C:715-755), tc() (:588-651), Qdot()
 * (:653-686), nSpecie(), nReaction().  Where the reference integrates one cell
 * at a time on the CPU, this model hands all of the mesh's cells to the GPU
 * library in one call of its C ABI (include/fcs.h) and writes the results
 * back into the OpenFOAM fields.
 *
 * The mechanism is read by the library itself from the case's
 * constant/reactions and constant/speciesThermo (or physicalProperties), the
 * files the reference's OptReaction::readInfo reads; the solver options from
 * constant/chemistryProperties.  The GPU is FCS_DEVICE (default 0).
 *
 * Errors: a failed library call, or cells the integrator could not finish
 * (maxSteps, which the reference treats as fatal, OptRodas34.C:193), end the
 * run with FatalError, as in the reference.
 */
#ifndef FastChemistryModelGPU_H
#define FastChemistryModelGPU_H

#include <cstdint>
#include <vector>

#include "basicChemistryModel.H"
#include "fluidReactionThermo.H"
#include "volFields.H"

#include "fcs.h"

namespace Foam {

template<class ThermoType>
class FastChemistryModel : public basicChemistryModel {
public:
    static word typeName() { return "FastChemistryModel"; }

    // solver: FCS_SOLVER_* of the registered solver class
    FastChemistryModel(const fluidReactionThermo& thermo, int32_t solver);
    virtual ~FastChemistryModel();

    virtual label nSpecie() const { return nSpecie_; }
    virtual label nReaction() const { return nReaction_; }
    virtual const volScalarField::Internal& RR(const label i) const { return RR_[i]; }
    virtual volScalarField::Internal& RR(const label i) { return RR_[i]; }

    // Instantaneous source terms of every cell (FastChemistryModel.C:715-755)
    virtual void calculate();
    // One CFD step of chemistry for every cell (transientSolve.H:2-104):
    // RR_i = (Y_i(t+dt) - Y_i(t)) rho / dt; returns min(deltaTMin, 2 dt)
    virtual scalar solve(const scalar deltaT);
    // The same with a per-cell time step (localEulerSolve.H:3-101)
    virtual scalar solve(const scalarField& deltaT);
    virtual tmp<volScalarField> tc() const;
    virtual tmp<volScalarField> Qdot() const;

private:
    fcs_ctx* ctx_;
    fcs_options opt_;
    label nSpecie_, nReaction_;
    std::vector<label> thermoIndex_;   // library species k -> index in thermo().species()
    std::vector<double> hf_;           // formation enthalpies, J/kg
    PtrList<volScalarField::Internal> RR_;
    // host staging of the mesh's fields, species-major as the library takes them
    mutable std::vector<double> p_, T_, rho_, Y_, RRbuf_, sub_, dt_;
    mutable std::vector<int32_t> status_;

    void check(fcs_status s, const char* call) const;
    void gather() const;
    scalar integrate(const double* deltaTPerCell, scalar deltaT);
};

// The registered solver classes: each selects its integrator in the library.
template<class ChemistryModel>
struct OptRodas34 : ChemistryModel {
    explicit OptRodas34(const fluidReactionThermo& t) : ChemistryModel(t, FCS_SOLVER_RODAS34) {}
};
template<class ChemistryModel>
struct OptRosenbrock34 : ChemistryModel {
    explicit OptRosenbrock34(const fluidReactionThermo& t) : ChemistryModel(t, FCS_SOLVER_ROSENBROCK34) {}
};
template<class ChemistryModel>
struct OptSeulex : ChemistryModel {
    explicit OptSeulex(const fluidReactionThermo& t) : ChemistryModel(t, FCS_SOLVER_SEULEX) {}
};
template<class ChemistryModel>
struct OptRodas23 : ChemistryModel {
    explicit OptRodas23(const fluidReactionThermo& t) : ChemistryModel(t, FCS_SOLVER_RODAS23) {}
};
template<class ChemistryModel>
struct OptRosenbrock23 : ChemistryModel {
    explicit OptRosenbrock23(const fluidReactionThermo& t) : ChemistryModel(t, FCS_SOLVER_ROSENBROCK23) {}
};

}  // namespace Foam

#include "FastChemistryModel.C"

#endif
