// driver.C -- TEST SUPPORT: a stand-in for the OpenFOAM solver that loads
// libFastChemistryModel.so the way controlDict `libs ("libFastChemistryModel.so")`
// does, selects the chemistry model from the case's chemistryProperties
// through basicChemistryModel::New, and calls it on a few cells (built
// against the OpenFOAM stub of plugin/foam_stub).
//
//   driver --list <plugin.so>
//       prints the solver names the plugin registered
//   driver <plugin.so> <case dir> <cells.bin> <out.bin> [lts]
//       cells.bin: int32 n, int32 ns, double dt, then p[n], T[n], rho[n] and
//       Y[ns][n] in the order of <case>/constant/species (one name per line);
//       out.bin: double deltaTMin, RR[ns][n] of the solve, tc[n], Qdot[n], then
//       RR[ns][n] after calculate() (RR in the species order of the case)
//   With `lts`, solve(scalarField) with deltaT of every cell = dt * (1 + c/n).
#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "basicChemistryModel.H"

extern "C" int foamStub_chemistry_solvers(char* out, int cap);

using namespace Foam;

int main(int argc, char** argv) {
    if (argc == 3 && std::string(argv[1]) == "--list") {
        if (!dlopen(argv[2], RTLD_NOW | RTLD_GLOBAL)) {
            std::cerr << dlerror() << "\n";
            return 2;
        }
        std::vector<char> buf(1 << 16);
        if (foamStub_chemistry_solvers(buf.data(), (int)buf.size()) < 0) return 2;
        std::cout << buf.data();
        return 0;
    }
    if (argc < 5) {
        std::cerr << "usage: driver --list <plugin.so> | driver <plugin.so> <case> <cells.bin> <out.bin> [lts]\n";
        return 2;
    }
    if (!dlopen(argv[1], RTLD_NOW | RTLD_GLOBAL)) {
        std::cerr << dlerror() << "\n";
        return 2;
    }
    const std::string caseDir = argv[2];
    const bool lts = argc > 5 && std::string(argv[5]) == "lts";
    wordList species;
    {
        std::ifstream f(caseDir + "/constant/species");
        for (std::string s; f >> s;) species.push_back(s);
    }
    std::ifstream in(argv[3], std::ios::binary);
    int32_t n = 0, ns = 0;
    double dt = 0;
    in.read(reinterpret_cast<char*>(&n), 4);
    in.read(reinterpret_cast<char*>(&ns), 4);
    in.read(reinterpret_cast<char*>(&dt), 8);
    if (!in || ns != (int32_t)species.size()) {
        std::cerr << "bad cells file\n";
        return 2;
    }
    fvMesh mesh(n, caseDir);
    fluidReactionThermo thermo(mesh, species);
    auto readField = [&](scalarField& f) { in.read(reinterpret_cast<char*>(f.data()), sizeof(double) * n); };
    readField(thermo.p());
    readField(thermo.T());
    readField(thermo.rhoRef());
    for (int32_t i = 0; i < ns; i++) readField(thermo.Y()[i]);
    if (!in) {
        std::cerr << "short cells file\n";
        return 2;
    }
    try {
        autoPtr<basicChemistryModel> chem = basicChemistryModel::New(thermo);
        scalar dtMin;
        if (lts) {
            scalarField dts(n);
            for (int32_t c = 0; c < n; c++) dts[c] = dt * (1.0 + double(c) / n);
            dtMin = chem->solve(dts);
        } else {
            dtMin = chem->solve(dt);
        }
        std::ofstream out(argv[4], std::ios::binary);
        auto write = [&](const double* p, size_t k) { out.write(reinterpret_cast<const char*>(p), sizeof(double) * k); };
        write(&dtMin, 1);
        for (int32_t i = 0; i < chem->nSpecie(); i++) write(chem->RR(i).data(), n);
        tmp<volScalarField> tc = chem->tc();
        tmp<volScalarField> Qdot = chem->Qdot();
        write(tc().data(), n);
        write(Qdot().data(), n);
        chem->calculate();
        for (int32_t i = 0; i < chem->nSpecie(); i++) write(chem->RR(i).data(), n);
        std::cout << "solvers-ok nSpecie " << chem->nSpecie() << " nReaction " << chem->nReaction() << " deltaTMin "
                  << dtMin << "\n";
    } catch (const Foam::error& e) {
        std::cerr << "FatalError: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
