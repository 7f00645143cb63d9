// Stand-in for OpenFOAM's chemistrySolver<ChemistryModel> base and the matrix
// and list types the ODE templates use.  Test infrastructure.
#pragma once
#include "fvCFD.H"
namespace Foam {
struct labelField : std::vector<int> { using std::vector<int>::vector; };
typedef labelField labelList;
struct scalarSquareMatrix {
    int nr, nc;
    std::vector<double> v;
    scalarSquareMatrix(int a, int b) : nr(a), nc(b), v(size_t(a) * b) {}
    double& operator()(int i, int j) { return v[size_t(i) * nc + j]; }
    double operator()(int i, int j) const { return v[size_t(i) * nc + j]; }
    double* operator[](int i) { return &v[size_t(i) * nc]; }
    const double* operator[](int i) const { return &v[size_t(i) * nc]; }
};
typedef scalarSquareMatrix scalarRectangularMatrix;
struct fluidReactionThermo { void* cfg; };
template<class CM> struct chemistrySolver : public CM {
    chemistrySolver(const fluidReactionThermo& t) : CM(t) {}
};
}  // namespace Foam
#define forAll(list, i) for (int i = 0; i < int((list).size()); ++i)
#define TypeName(x) static const char* typeName_() { return x; }
