// basicChemistryModel.H -- stand-in for the OpenFOAM-10 header of that name (see foamStub.H).
#pragma once
#include "foamStub.H"
