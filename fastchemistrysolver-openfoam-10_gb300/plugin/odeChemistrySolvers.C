/*
 * odeChemistrySolvers.C -- the runtime-selection entries of
 * libFastChemistryModel.so: the solvers OptRosenbrock34, OptRosenbrock23,
 * OptRodas34, OptRodas23 and OptSeulex with the method FastChemistryModel
 * and the gas thermo sutherland / sensibleEnthalpy / janaf / perfectGas /
 * specie -- the names the reference plugin registers
 * (src/odeChemistrySolvers.C:63-74), so a case selects them unchanged:
 *
 *     chemistryType { solver OptRodas34; method FastChemistryModel; }
 *
 * in constant/chemistryProperties and libs ("libFastChemistryModel.so") in
 * system/controlDict.
 */
#include "FastChemistryModel.H"
#include "makeChemistrySolver.H"

namespace Foam {

typedefThermo(sutherlandTransport, sensibleEnthalpy, janafThermo, perfectGas, specie);

defineChemistrySolver(FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);
makeChemistrySolver(OptRosenbrock34, FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);
makeChemistrySolver(OptRosenbrock23, FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);
makeChemistrySolver(OptRodas34, FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);
makeChemistrySolver(OptRodas23, FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);
makeChemistrySolver(OptSeulex, FastChemistryModel, sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie);

}  // namespace Foam
