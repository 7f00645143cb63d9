// foamStub.C -- the out-of-line parts of foamStub.H (compile-check and test
// support for the plugin; see foamStub.H).  Built as libfoamStub.so, which
// stands in for OpenFOAM's libchemistryModel: it owns the runtime selection
// table that libFastChemistryModel.so adds its solvers to when it is loaded.
#include "foamStub.H"

#include <cctype>
#include <fstream>

namespace Foam {

namespace {

// Whitespace / punctuation tokens of an OpenFOAM dictionary file, comments
// removed (enough for the few top-level keys read here).
std::vector<std::string> tokens(const fileName& path) {
    std::ifstream f(path);
    if (!f) throw error("cannot open " + path);
    std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<std::string> out;
    std::string cur;
    auto flush = [&]() { if (!cur.empty()) { out.push_back(cur); cur.clear(); } };
    for (size_t i = 0; i < text.size(); i++) {
        const char c = text[i];
        if (c == '/' && i + 1 < text.size() && text[i + 1] == '/') {
            while (i < text.size() && text[i] != '\n') i++;
            flush();
        } else if (c == '/' && i + 1 < text.size() && text[i + 1] == '*') {
            i += 2;
            while (i + 1 < text.size() && !(text[i] == '*' && text[i + 1] == '/')) i++;
            i++;
            flush();
        } else if (std::isspace(static_cast<unsigned char>(c))) {
            flush();
        } else if (c == '{' || c == '}' || c == ';') {
            flush();
            out.push_back(std::string(1, c));
        } else {
            cur += c;
        }
    }
    flush();
    return out;
}

// The value token after a top-level `key` (depth 0), or "".
std::string topLevel(const std::vector<std::string>& t, const std::string& key) {
    int depth = 0;
    for (size_t i = 0; i + 1 < t.size(); i++) {
        if (t[i] == "{") depth++;
        else if (t[i] == "}") depth--;
        else if (depth == 0 && t[i] == key) return t[i + 1];
    }
    return "";
}

// The value token after `key` inside the top-level dictionary `dict`, or "".
std::string inDict(const std::vector<std::string>& t, const std::string& dict, const std::string& key) {
    int depth = 0;
    for (size_t i = 0; i + 1 < t.size(); i++) {
        if (t[i] == "{") depth++;
        else if (t[i] == "}") depth--;
        else if (depth == 0 && t[i] == dict && t[i + 1] == "{") {
            int d = 0;
            for (size_t j = i + 1; j + 1 < t.size(); j++) {
                if (t[j] == "{") d++;
                else if (t[j] == "}") { if (--d == 0) break; }
                else if (d == 1 && t[j] == key) return t[j + 1];
            }
        }
    }
    return "";
}

}  // namespace

basicChemistryModel::thermoConstructorTable& basicChemistryModel::thermoConstructorTablePtr_() {
    static thermoConstructorTable table;
    return table;
}

basicChemistryModel::basicChemistryModel(const fluidReactionThermo& thermo)
    : mesh_(thermo.mesh()), thermo_(thermo), chemistry_(true), deltaTChemIni_(1e-7) {
    const std::vector<std::string> t = tokens(dictPath());
    const std::string on = topLevel(t, "chemistry");
    chemistry_ = !(on == "off" || on == "false" || on == "no" || on == "n" || on == "none");
    const std::string ini = topLevel(t, "initialChemicalTimeStep");
    if (!ini.empty()) deltaTChemIni_ = std::stod(ini);
    deltaTChem_ = scalarField(mesh_.nCells(), deltaTChemIni_);
}

autoPtr<basicChemistryModel> basicChemistryModel::New(const fluidReactionThermo& thermo) {
    const std::vector<std::string> t = tokens(thermo.mesh().time().constant() + "/chemistryProperties");
    const std::string solver = inDict(t, "chemistryType", "solver");
    const std::string method = inDict(t, "chemistryType", "method");
    const std::string name = solver + "<" + method + "<sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie>>";
    thermoConstructorTable& table = thermoConstructorTablePtr_();
    const auto it = table.find(name);
    if (it == table.end()) {
        std::string valid;
        for (const auto& kv : table) valid += "\n    " + kv.first;
        FatalErrorInFunction << "Unknown chemistry solver " << name << "; valid solvers are:" << valid
                             << exit(FatalError);
    }
    return autoPtr<basicChemistryModel>(it->second(thermo));
}

}  // namespace Foam

// The selection table's names, for the loader that emulates controlDict
// `libs (...)` in the tests.
extern "C" int foamStub_chemistry_solvers(char* out, int cap) {
    std::string s;
    for (const auto& kv : Foam::basicChemistryModel::thermoConstructorTablePtr_()) s += kv.first + "\n";
    if ((int)s.size() + 1 > cap) return -1;
    s.copy(out, s.size());
    out[s.size()] = 0;
    return (int)s.size();
}
