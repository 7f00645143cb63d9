// makeChemistrySolver.H -- stand-in for the OpenFOAM-10 macros that register a
// chemistry solver in basicChemistryModel's runtime selection table (see
// foamStub.H): typedefThermo names a thermo type, makeChemistrySolver adds
// "<solver><<method><<thermo>>>" with a constructor from the thermo.
#pragma once
#include "foamStub.H"

#define typedefThermo(Transport, Energy, Thermo, Equation, Specie)                           \
    struct Transport##Energy##Thermo##Equation##Specie {                                     \
        static ::Foam::word typeName() { return #Transport #Energy #Thermo #Equation #Specie; } \
    }

#define defineChemistrySolver(Model, ThermoPhysics)

#define makeChemistrySolver(Solver, Model, ThermoPhysics)                                             \
    typedef Solver<Model<ThermoPhysics>> Solver##Model##ThermoPhysics;                                \
    static ::Foam::basicChemistryModel::addthermoConstructorToTable<Solver##Model##ThermoPhysics>      \
        add##Solver##Model##ThermoPhysics##ConstructorToTable_(                                       \
            ::Foam::word(#Solver "<" #Model "<") + ThermoPhysics::typeName() + ">>")
