// Minimal stand-ins for the OpenFOAM types the reference numerical core
// names, so that its Reaction/, LUsolver/ and ODE/ sources compile unmodified
// into the test-only reference library (oracle/_ref).  Test infrastructure.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foam {
typedef double scalar;
typedef int label;
typedef std::string word;
constexpr double small = 1.0e-15, vSmall = 1.0e-300, great = 1.0e15, vGreat = 1.0e300;
inline double max(double a, double b) { return a > b ? a : b; }
inline double min(double a, double b) { return a < b ? a : b; }
inline double max(double a, int b) { return a > b ? a : b; }
inline double max(int a, double b) { return a > b ? a : b; }
inline double min(double a, int b) { return a < b ? a : b; }
inline double min(int a, double b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline double mag(double a) { return std::fabs(a); }
inline double sqr(double a) { return a * a; }
using std::pow; using std::sqrt; using std::log; using std::log10; using std::exp;

struct scalarField : std::vector<double> { using std::vector<double>::vector; };

// A flat key -> number dictionary: enough for <Solver>Coeffs lookups.
class dictionary {
public:
    std::map<std::string, double> kv;
    template<class T> T lookup(const std::string& k) const { return T(kv.at(k)); }
    template<class T> T lookupOrDefault(const std::string& k, T d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : T(it->second);
    }
};
class hashedWordList;

struct FatalStream { template<class T> FatalStream& operator<<(const T&) { return *this; } };
struct FatalExit {};
static FatalStream FatalErrorInFunction;
static FatalStream FatalError;
static const char nl = '\n';
inline FatalExit exit(FatalStream&) { return FatalExit(); }
struct fatal_error : std::runtime_error { fatal_error() : std::runtime_error("FatalError") {} };
inline FatalStream& operator<<(FatalStream& s, FatalExit) { throw fatal_error(); return s; }
}  // namespace Foam
using namespace Foam;
