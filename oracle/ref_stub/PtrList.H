#include "fvCFD.H"
