/*
 * foamStub.H -- the few classes of OpenFOAM-10 that libFastChemistryModel.so
 * uses, reduced to what its sources need, so that the plugin can be compiled
 * and driven on a machine without OpenFOAM.  COMPILE-CHECK AND TEST SUPPORT
 * ONLY: with a real OpenFOAM-10 installation the plugin is built by wmake
 * against OpenFOAM's own headers (plugin/Make) and none of this is used.
 *
 * What is kept of each class is its name, the members the plugin calls and
 * their meaning:
 *   fvMesh                      nCells(), the case directory
 *   volScalarField (+::Internal) a named cell field (boundary values omitted)
 *   tmp<T>, autoPtr<T>, PtrList<T>
 *   fluidReactionThermo         T(), p(), rho(), Y(), species(), the mesh
 *   basicChemistryModel         the chemistry-model interface OpenFOAM's
 *                               solvers call (solve, RR, tc, Qdot, ...), its
 *                               runtime selection table keyed by
 *                               "<solver><<method><<thermo>>>" as in
 *                               chemistrySolver::New, the `chemistry` switch
 *                               and the per-cell deltaTChem field
 *   FatalErrorInFunction        throws Foam::error (OpenFOAM aborts the run)
 */
#ifndef FOAM_STUB_H
#define FOAM_STUB_H

#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foam {

typedef double scalar;
typedef int label;
typedef std::string word;
typedef std::string fileName;
typedef std::vector<word> wordList;

const scalar small = 1e-15;
const scalar great = 1e15;
const scalar vGreat = 1e300;

class scalarField : public std::vector<double> {
public:
    scalarField() = default;
    explicit scalarField(size_t n, double v = 0) : std::vector<double>(n, v) {}
};

// OpenFOAM's FatalError: an exception here (OpenFOAM prints and aborts)
class error : public std::runtime_error {
public:
    explicit error(const std::string& m) : std::runtime_error(m) {}
};

class errorStream {
    std::ostringstream os_;
    std::string where_;
public:
    explicit errorStream(const char* where) : where_(where) {}
    template<class T> errorStream& operator<<(const T& v) { os_ << v; return *this; }
    [[noreturn]] void raise() { throw error(where_ + ": " + os_.str()); }
};
struct exitToken {};
inline void operator<<(errorStream& s, const exitToken&) { s.raise(); }
inline void operator<<(errorStream&& s, const exitToken&) { s.raise(); }
#define FatalErrorInFunction ::Foam::errorStream(__func__)
#define FatalError ::Foam::exitToken()
inline exitToken exit(const exitToken& t) { return t; }

template<class T>
class tmp {
    std::shared_ptr<T> p_;
public:
    explicit tmp(T* p) : p_(p) {}
    T& ref() { return *p_; }
    const T& operator()() const { return *p_; }
    const T* operator->() const { return p_.get(); }
};

template<class T>
class autoPtr {
    std::unique_ptr<T> p_;
public:
    explicit autoPtr(T* p = nullptr) : p_(p) {}
    T& operator()() { return *p_; }
    T* operator->() { return p_.get(); }
    bool valid() const { return bool(p_); }
};

template<class T>
class PtrList {
    std::vector<std::unique_ptr<T>> v_;
public:
    PtrList() = default;
    label size() const { return label(v_.size()); }
    void setSize(label n) { v_.resize(n); }
    void set(label i, T* p) { v_[i].reset(p); }
    T& operator[](label i) { return *v_[i]; }
    const T& operator[](label i) const { return *v_[i]; }
};

class Time {
    fileName case_;
public:
    explicit Time(const fileName& caseDir) : case_(caseDir) {}
    fileName path() const { return case_; }
    fileName constant() const { return case_ + "/constant"; }
};

class fvMesh {
    label nCells_;
    Time time_;
public:
    fvMesh(label nCells, const fileName& caseDir) : nCells_(nCells), time_(caseDir) {}
    label nCells() const { return nCells_; }
    const Time& time() const { return time_; }
};

class volScalarField : public scalarField {
    word name_;
public:
    typedef volScalarField Internal;  // the internal field (no boundaries here)
    volScalarField(const word& name, const fvMesh& mesh, scalar v = 0) : scalarField(mesh.nCells(), v), name_(name) {}
    const word& name() const { return name_; }
    static tmp<volScalarField> New(const word& name, const fvMesh& mesh, scalar v = 0) {
        return tmp<volScalarField>(new volScalarField(name, mesh, v));
    }
};

class fluidReactionThermo {
    const fvMesh& mesh_;
    wordList species_;
    volScalarField T_, p_, rho_;
    PtrList<volScalarField> Y_;
public:
    fluidReactionThermo(const fvMesh& mesh, const wordList& species)
        : mesh_(mesh), species_(species), T_("T", mesh), p_("p", mesh), rho_("rho", mesh) {
        Y_.setSize(label(species.size()));
        for (label i = 0; i < label(species.size()); i++) Y_.set(i, new volScalarField("Y." + species[i], mesh));
    }
    const fvMesh& mesh() const { return mesh_; }
    const wordList& species() const { return species_; }
    volScalarField& T() { return T_; }
    const volScalarField& T() const { return T_; }
    volScalarField& p() { return p_; }
    const volScalarField& p() const { return p_; }
    volScalarField& rhoRef() { return rho_; }
    tmp<volScalarField> rho() const { return tmp<volScalarField>(new volScalarField(rho_)); }
    PtrList<volScalarField>& Y() { return Y_; }
    const PtrList<volScalarField>& Y() const { return Y_; }
};

class basicChemistryModel {
public:
    typedef std::function<basicChemistryModel*(const fluidReactionThermo&)> thermoConstructorPtr;
    typedef std::map<word, thermoConstructorPtr> thermoConstructorTable;
    static thermoConstructorTable& thermoConstructorTablePtr_();

    template<class Type>
    struct addthermoConstructorToTable {
        explicit addthermoConstructorToTable(const word& name) {
            thermoConstructorTablePtr_()[name] = [](const fluidReactionThermo& t) -> basicChemistryModel* {
                return new Type(t);
            };
        }
    };

    // Selects "<solver><<method><<thermo>>>" from constant/chemistryProperties
    // chemistryType{solver; method;} (thermo: the one name this stub knows)
    static autoPtr<basicChemistryModel> New(const fluidReactionThermo& thermo);

    explicit basicChemistryModel(const fluidReactionThermo& thermo);
    virtual ~basicChemistryModel() = default;

    const fvMesh& mesh() const { return mesh_; }
    const fluidReactionThermo& thermo() const { return thermo_; }
    // <case>/constant/chemistryProperties
    fileName dictPath() const { return mesh_.time().constant() + "/chemistryProperties"; }

    virtual label nSpecie() const = 0;
    virtual label nReaction() const = 0;
    virtual const volScalarField::Internal& RR(const label i) const = 0;
    virtual volScalarField::Internal& RR(const label i) = 0;
    virtual void calculate() = 0;
    virtual scalar solve(const scalar deltaT) = 0;
    virtual scalar solve(const scalarField& deltaT) = 0;
    virtual tmp<volScalarField> tc() const = 0;
    virtual tmp<volScalarField> Qdot() const = 0;

protected:
    const fvMesh& mesh_;
    const fluidReactionThermo& thermo_;
    bool chemistry_;                 // `chemistry on|off;`
    scalarField deltaTChem_;         // per-cell chemistry sub-step, carried between steps
    scalar deltaTChemIni_;           // initialChemicalTimeStep
};

}  // namespace Foam

#endif
