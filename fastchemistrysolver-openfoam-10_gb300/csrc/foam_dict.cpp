// foam_dict.cpp -- reader for the OpenFOAM dictionaries the plugin consumes:
// the `reactions` dictionary (with `reversibleArrheniusPLOG` /
// `ArrheniusData`, fall-off k0 / kInf / F / thirdBodyEfficiencies and
// non-equilibrium forward / reverse entries), the species thermo entries (`specie{molWeight}`,
// `thermodynamics{Tlow,Thigh,Tcommon,highCpCoeffs,lowCpCoeffs}`) and the
// `chemistryProperties` keys.  It builds an fcs_mechanism_desc the way
// OptReaction::readInfo (src/Reaction/OptReaction.C:348-1339) and
// readReactionInfo (OptReaction.C:29-173) interpret the same files, and
// fills fcs_options the way the FastChemistryModel and Opt<Solver>
// constructors read them (FastChemistryModel.C:45-168, OptRodas34.C:34-50).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fcs.h"

namespace {

struct Node;
using NodeP = std::shared_ptr<Node>;

// A value is a token (word/number/string) or a list of values; a dictionary
// is an ordered list of (keyword, dict-or-value-sequence) entries.
struct Node {
    enum Kind { TOKEN, LIST, DICT } kind = TOKEN;
    std::string tok;                         // TOKEN
    bool quoted = false;
    std::vector<NodeP> items;                // LIST
    std::vector<std::pair<std::string, NodeP>> entries;  // DICT; value is a DICT or a LIST of tokens
    const Node* find(const std::string& k) const {
        for (auto& e : entries) if (e.first == k) return e.second.get();
        return nullptr;
    }
};

struct Lexer {
    std::string s;
    size_t i = 0;
    std::string dir;
    std::string bad;  // an unterminated comment or string (the file cannot be read as OpenFOAM reads it)
    explicit Lexer(std::string text, std::string d) : s(std::move(text)), dir(std::move(d)) {}
    void skip() {
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') i++;
            } else if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                i += 2;
                while (i + 1 < s.size() && !(s[i] == '*' && s[i + 1] == '/')) i++;
                if (i + 1 >= s.size()) bad = "unterminated /* comment";
                i += 2;
            } else {
                return;
            }
        }
    }
    bool eof() { skip(); return i >= s.size(); }
    char peek() { skip(); return i < s.size() ? s[i] : '\0'; }
    // returns punctuation as a one-char token
    std::string next(bool* quoted = nullptr) {
        skip();
        if (quoted) *quoted = false;
        if (i >= s.size()) return "";
        const char c = s[i];
        if (c == '(' || c == ')' || c == '{' || c == '}' || c == ';' || c == '[' || c == ']') {
            i++;
            return std::string(1, c);
        }
        if (c == '"') {
            size_t j = i + 1;
            std::string out;
            while (j < s.size() && s[j] != '"') out += s[j++];
            if (j >= s.size()) bad = "unterminated string";
            i = j + 1;
            if (quoted) *quoted = true;
            return out;
        }
        // A word keeps balanced parentheses, as OpenFOAM's word tokens do
        // (species such as CH2(S)); a ')' with no '(' open in the word ends it.
        const bool word = std::isalpha((unsigned char)c) || c == '_';
        int depth = 0;
        size_t j = i;
        while (j < s.size() && !std::isspace((unsigned char)s[j])) {
            if (word && s[j] == '(') { depth++; j++; continue; }
            if (word && s[j] == ')' && depth > 0) { depth--; j++; continue; }
            if (std::strchr("(){};[]\"", s[j]) != nullptr) break;
            if (s[j] == '/' && j + 1 < s.size() && (s[j + 1] == '/' || s[j + 1] == '*')) break;
            j++;
        }
        if (j == i) j = i + 1;  // a character no token rule takes: returned alone, never stuck on it
        std::string out = s.substr(i, j - i);
        i = j;
        return out;
    }
};

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

std::string dirname_of(const std::string& p) {
    const size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

// Text that is not a dictionary: a NUL or another control character
// (OpenFOAM files are plain text; tabs, line and page breaks are whitespace).
bool has_control_characters(const std::string& t) {
    for (unsigned char c : t)
        if ((c < 0x20 && !std::isspace(c)) || c == 0x7f) return true;
    return false;
}

// `N ( ... )` with an integer N: OpenFOAM's sized list, whose size must be N
bool sized_list_mismatch(const std::vector<NodeP>& items) {
    if (items.size() < 2) return false;
    const Node* c = items[items.size() - 2].get();
    const Node* l = items.back().get();
    if (c->kind != Node::TOKEN || c->quoted || l->kind != Node::LIST || c->tok.empty()) return false;
    for (char ch : c->tok) if (!std::isdigit((unsigned char)ch)) return false;
    return std::strtoul(c->tok.c_str(), nullptr, 10) != l->items.size();
}

struct Parser {
    std::string err;
    bool followIncludes = true;
    int depth = 0;                        // nesting of lists and dictionaries
    static constexpr int kMaxDepth = 256;

    NodeP parse_list(Lexer& L) {  // after '('
        auto n = std::make_shared<Node>();
        n->kind = Node::LIST;
        if (++depth > kMaxDepth) { err = "lists nested too deeply"; --depth; return n; }
        for (;;) {
            if (L.eof()) { err = "unterminated list"; break; }
            bool q = false;
            std::string t = L.next(&q);
            if (!q && t == ")") break;
            if (!q && t == "(") {
                n->items.push_back(parse_list(L));
                if (!err.empty()) break;
                if (sized_list_mismatch(n->items)) { err = "list size differs from its count"; break; }
                continue;
            }
            auto tk = std::make_shared<Node>();
            tk->tok = t;
            tk->quoted = q;
            n->items.push_back(tk);
        }
        --depth;
        return n;
    }

    // parse dictionary entries until '}' (or EOF when top)
    void parse_dict(Lexer& L, Node& d, bool top) {
        if (++depth > kMaxDepth) { err = "dictionaries nested too deeply"; --depth; return; }
        parse_entries(L, d, top);
        --depth;
    }

    void parse_entries(Lexer& L, Node& d, bool top) {
        for (;;) {
            if (L.eof()) {
                if (!top) err = "unterminated dictionary";
                return;
            }
            bool q = false;
            std::string key = L.next(&q);
            if (!q && key == "}") {
                if (top) err = "unexpected }";
                return;
            }
            if (!q && key == ";") continue;
            if (!q && key == "#include") {
                bool q2 = false;
                std::string f = L.next(&q2);
                if (!followIncludes) continue;
                std::string path = (f.size() && f[0] == '/') ? f : L.dir + "/" + f;
                std::string text;
                if (!read_file(path, text)) continue;  // missing include: the keys it held stay absent
                if (has_control_characters(text)) { err = "control character in " + path; return; }
                Lexer sub(text, dirname_of(path));
                parse_dict(sub, d, true);
                if (err.empty() && !sub.bad.empty()) err = sub.bad + " in " + path;
                if (!err.empty()) return;
                continue;
            }
            if (!q && (key == "#includeEtc" || key == "#inputMode" || key == "#remove")) {
                L.next();
                continue;
            }
            if (L.peek() == '{') {
                L.next();
                auto sub = std::make_shared<Node>();
                sub->kind = Node::DICT;
                parse_dict(L, *sub, false);
                if (!err.empty()) return;
                d.entries.emplace_back(key, sub);
                continue;
            }
            // value tokens until ';'
            auto val = std::make_shared<Node>();
            val->kind = Node::LIST;
            for (;;) {
                if (L.eof()) { err = "missing ; after " + key; return; }
                bool q3 = false;
                std::string t = L.next(&q3);
                if (!q3 && t == ";") break;
                if (!q3 && t == "(") {
                    val->items.push_back(parse_list(L));
                    if (!err.empty()) return;
                    if (sized_list_mismatch(val->items)) { err = "list size differs from its count in " + key; return; }
                    continue;
                }
                if (!q3 && t == "}") { err = "unexpected } in value of " + key; return; }
                if (!q3 && t == "{") {
                    // uniform list N{v}: N copies of one element (thermo databases
                    // write unused coefficient sets as `7 { 0 }`)
                    char* end = nullptr;
                    const long count = val->items.empty() ? -1 : std::strtol(val->items.back()->tok.c_str(), &end, 10);
                    if (count < 0 || count > 1000000 || !end || *end) { err = "bad uniform list in " + key; return; }
                    bool q4 = false;
                    std::string e = L.next(&q4);
                    NodeP elem;
                    if (!q4 && e == "(") {
                        elem = parse_list(L);
                        if (!err.empty()) return;
                    }
                    else { elem = std::make_shared<Node>(); elem->tok = e; elem->quoted = q4; }
                    if (L.next() != "}") { err = "bad uniform list in " + key; return; }
                    auto lst = std::make_shared<Node>();
                    lst->kind = Node::LIST;
                    lst->items.assign((size_t)count, elem);
                    val->items.back() = lst;
                    continue;
                }
                auto tk = std::make_shared<Node>();
                tk->tok = t;
                tk->quoted = q3;
                val->items.push_back(tk);
            }
            d.entries.emplace_back(key, val);
        }
    }

    bool parse_file(const std::string& path, Node& root) {
        std::string text;
        if (!read_file(path, text)) { err = "cannot read " + path; return false; }
        if (has_control_characters(text)) { err = "control character in " + path; return false; }
        root.kind = Node::DICT;
        Lexer L(text, dirname_of(path));
        parse_dict(L, root, true);
        if (err.empty() && !L.bad.empty()) err = L.bad;
        return err.empty();
    }
};

bool as_double(const Node* v, double& out) {
    if (!v) return false;
    const Node* t = v;
    if (t->kind == Node::LIST) {
        // value entry: last token is the number (OpenFOAM allows dimensions before it)
        if (t->items.empty()) return false;
        t = t->items.back().get();
    }
    if (t->kind != Node::TOKEN) return false;
    char* end = nullptr;
    out = std::strtod(t->tok.c_str(), &end);
    return end && *end == '\0' && !t->tok.empty();
}

bool as_word(const Node* v, std::string& out) {
    if (!v || v->kind != Node::LIST || v->items.empty() || v->items[0]->kind != Node::TOKEN) return false;
    out = v->items[0]->tok;
    return true;
}

// `N ( a b c )` or `( a b c )` -> the inner list node
const Node* inner_list(const Node* v) {
    if (!v || v->kind != Node::LIST) return nullptr;
    for (auto& it : v->items) if (it->kind == Node::LIST) return it.get();
    return nullptr;
}

bool list_doubles(const Node* l, std::vector<double>& out) {
    out.clear();
    if (!l) return false;
    for (auto& it : l->items) {
        double v;
        if (!as_double(it.get(), v)) return false;
        out.push_back(v);
    }
    return true;
}

}  // namespace

namespace {

// Largest stoichiometric coefficient the reader expands (each unit is one
// species entry of the reaction; the GPU takes at most 4 reactant and 8
// product entries, fcs_load_mechanism refuses more).
constexpr int kMaxCoefficient = 64;

// Parses the reactions and thermo files into a flat description and hands it
// (with the species names) to visit; the arrays live until visit returns.
fcs_status parse_foam_files(const char* reactions_path, const char* thermo_path, fcs_mechanism_visitor visit,
                            void* user) {
    Parser P;
    Node rfile, tfile;
    if (!P.parse_file(reactions_path, rfile)) return FCS_ERR_PARSE;
    if (!P.parse_file(thermo_path, tfile)) return FCS_ERR_PARSE;
    // species list: in the reactions file (chemkinToFoam output) or the thermo file
    const Node* spv = rfile.find("species");
    if (!spv) spv = tfile.find("species");
    const Node* spl = inner_list(spv);
    if (!spl) return FCS_ERR_PARSE;
    std::vector<std::string> species;
    for (auto& it : spl->items) if (it->kind == Node::TOKEN) species.push_back(it->tok);
    const int ns = (int)species.size();
    std::map<std::string, int> index;
    for (int i = 0; i < ns; i++) index[species[i]] = i;
    std::vector<double> W(ns), Tl(ns), Th(ns), Tc(ns), hc(7 * ns), lc(7 * ns);
    for (int i = 0; i < ns; i++) {
        const Node* sd = tfile.find(species[i]);
        if (!sd || sd->kind != Node::DICT) return FCS_ERR_PARSE;
        const Node* spd = sd->find("specie");
        const Node* td = sd->find("thermodynamics");
        if (!spd || !td) return FCS_ERR_PARSE;
        if (!as_double(spd->find("molWeight"), W[i])) return FCS_ERR_PARSE;
        if (!as_double(td->find("Tlow"), Tl[i]) || !as_double(td->find("Thigh"), Th[i]) ||
            !as_double(td->find("Tcommon"), Tc[i]))
            return FCS_ERR_PARSE;
        std::vector<double> h, l;
        if (!list_doubles(inner_list(td->find("highCpCoeffs")), h) || h.size() != 7) return FCS_ERR_PARSE;
        if (!list_doubles(inner_list(td->find("lowCpCoeffs")), l) || l.size() != 7) return FCS_ERR_PARSE;
        for (int j = 0; j < 7; j++) { hc[7 * i + j] = h[j]; lc[7 * i + j] = l[j]; }
    }
    const Node* rd = rfile.find("reactions");
    if (!rd || rd->kind != Node::DICT) return FCS_ERR_PARSE;
    std::vector<int32_t> type, rev, lo{0}, ls, ro{0}, rs, po{0};
    std::vector<double> arr, arr2, eff, fp, pt;
    for (auto& e : rd->entries) {
        const Node* r = e.second.get();
        if (r->kind != Node::DICT) return FCS_ERR_PARSE;
        std::string tname, eq;
        if (!as_word(r->find("type"), tname)) return FCS_ERR_PARSE;
        if (!as_word(r->find("reaction"), eq)) return FCS_ERR_PARSE;
        int reversible = 1;
        std::string base;
        int kind = -1;
        if (tname == "nonEquilibriumReversibleArrhenius") kind = FCS_RXN_NONEQ;
        else if (tname == "nonEquilibriumReversibleThirdBodyArrhenius") kind = FCS_RXN_NONEQ_THIRD_BODY;
        else if (tname.rfind("irreversible", 0) == 0) { reversible = 0; base = tname.substr(12); }
        else if (tname.rfind("reversible", 0) == 0) { reversible = 1; base = tname.substr(10); }
        else return FCS_ERR_UNSUPPORTED;  // chemically activated, Landau-Teller and other unknown types
        if (kind < 0) {
            if (base == "Arrhenius") kind = FCS_RXN_ARRHENIUS;
            else if (base == "ThirdBodyArrhenius") kind = FCS_RXN_THIRD_BODY;
            else if (base == "ArrheniusPLOG") kind = FCS_RXN_PLOG;
            else if (base == "ArrheniusLindemannFallOff") kind = FCS_RXN_LINDEMANN_FALLOFF;
            else if (base == "ArrheniusTroeFallOff") kind = FCS_RXN_TROE_FALLOFF;
            else if (base == "ArrheniusSRIFallOff") kind = FCS_RXN_SRI_FALLOFF;
            else return FCS_ERR_UNSUPPORTED;
        }
        const bool noneq = kind == FCS_RXN_NONEQ || kind == FCS_RXN_NONEQ_THIRD_BODY;
        // reaction string (readReactionInfo, OptReaction.C:29-173): terms
        // separated by '+', sides by '=', integer coefficients expanded
        std::istringstream iss(eq);
        std::vector<std::string> words;
        std::string w;
        while (iss >> w) words.push_back(w);
        int eqpos = -1;
        for (int k = 0; k < (int)words.size(); k++) if (words[k] == "=") eqpos = k;
        if (eqpos < 0) return FCS_ERR_PARSE;
        // Each side is one or more terms joined by '+' (the reference skips
        // every '+' and would take "A + = B" or "= B" too; a side without a
        // species, or a dangling '+', is refused here).
        auto side = [&](int k0, int k1, std::vector<int32_t>& out) -> bool {
            bool expectTerm = true;
            for (int k = k0; k < k1; k++) {
                if (words[k] == "+") {
                    if (expectTerm) return false;
                    expectTerm = true;
                    continue;
                }
                if (!expectTerm) return false;
                expectTerm = false;
                const std::string& t = words[k];
                size_t first = 0;
                while (first < t.size() && (std::isdigit((unsigned char)t[first]) || t[first] == '.')) first++;
                int coef = 1;
                if (first > 0) {
                    char* end = nullptr;
                    const std::string num = t.substr(0, first);
                    const double v = std::strtod(num.c_str(), &end);
                    if (!end || *end || v != std::floor(v) || v < 1 || v > kMaxCoefficient) return false;
                    coef = (int)v;
                }
                auto it = index.find(t.substr(first));
                if (it == index.end()) return false;
                for (int c = 0; c < coef; c++) out.push_back(it->second);
            }
            return !expectTerm;
        };
        if (!side(0, eqpos, ls) || !side(eqpos + 1, (int)words.size(), rs)) return FCS_ERR_PARSE;
        lo.push_back((int32_t)ls.size());
        ro.push_back((int32_t)rs.size());
        type.push_back(kind);
        rev.push_back(reversible);
        const bool falloff = kind >= FCS_RXN_LINDEMANN_FALLOFF && kind <= FCS_RXN_SRI_FALLOFF;
        double A = 0, beta = 0, Ta = 0;
        // forward rate: the reaction dict, k0 (fall-off) or forward (non-equilibrium,
        // OptReaction.C:620-631)
        const Node* k0 = falloff ? r->find("k0") : noneq ? r->find("forward") : r;
        if (!k0 || !as_double(k0->find("A"), A) || !as_double(k0->find("beta"), beta) ||
            !as_double(k0->find("Ta"), Ta))
            return FCS_ERR_PARSE;
        arr.push_back(A); arr.push_back(beta); arr.push_back(Ta);
        double kA = 0, kb = 0, kt = 0;
        if (falloff || noneq) {
            // second Arrhenius: kInf, or the reverse rate of a non-equilibrium reaction
            const Node* ki = r->find(falloff ? "kInf" : "reverse");
            if (!ki || !as_double(ki->find("A"), kA) || !as_double(ki->find("beta"), kb) ||
                !as_double(ki->find("Ta"), kt))
                return FCS_ERR_PARSE;
        }
        arr2.push_back(kA); arr2.push_back(kb); arr2.push_back(kt);
        // Third-body efficiencies: required where the reference looks them up
        // (OptReaction.C:669, 724, 776, 830, 889); species the list leaves out
        // keep efficiency 1 (the reference indexes its table by species and
        // needs every species listed).
        std::vector<double> row(ns, 1.0);
        const Node* cnode = nullptr;
        if (kind == FCS_RXN_THIRD_BODY) cnode = r->find("coeffs");
        // the reference takes both directions' coefficients from the forward
        // dictionary (OptReaction.C:668-686)
        else if (kind == FCS_RXN_NONEQ_THIRD_BODY) cnode = k0->find("coeffs");
        else if (falloff) {
            const Node* tb = r->find("thirdBodyEfficiencies");
            if (!tb || tb->kind != Node::DICT) return FCS_ERR_PARSE;
            cnode = tb->find("coeffs");
        }
        const bool needsEfficiencies = kind == FCS_RXN_THIRD_BODY || kind == FCS_RXN_NONEQ_THIRD_BODY || falloff;
        if (needsEfficiencies && !cnode) return FCS_ERR_PARSE;
        if (cnode) {
            const Node* l = inner_list(cnode);
            if (!l) return FCS_ERR_PARSE;
            for (auto& it : l->items) {
                if (it->kind != Node::LIST || it->items.size() != 2) return FCS_ERR_PARSE;
                auto sp = index.find(it->items[0]->tok);
                double v;
                if (sp == index.end() || !as_double(it->items[1].get(), v)) return FCS_ERR_PARSE;
                row[sp->second] = v;
            }
        }
        eff.insert(eff.end(), row.begin(), row.end());
        // Troe (alpha, Ts, Tss, Tsss) and SRI (a..e) parameters: all required,
        // as the reference's lookups (OptReaction.C:841-844, 900-904)
        double f5[5] = {0, 0, 0, 0, 0};
        const Node* F = r->find("F");
        if (kind == FCS_RXN_TROE_FALLOFF) {
            if (!F || !as_double(F->find("alpha"), f5[0]) || !as_double(F->find("Ts"), f5[1]) ||
                !as_double(F->find("Tss"), f5[2]) || !as_double(F->find("Tsss"), f5[3]))
                return FCS_ERR_PARSE;
        } else if (kind == FCS_RXN_SRI_FALLOFF) {
            if (!F || !as_double(F->find("a"), f5[0]) || !as_double(F->find("b"), f5[1]) ||
                !as_double(F->find("c"), f5[2]) || !as_double(F->find("d"), f5[3]) || !as_double(F->find("e"), f5[4]))
                return FCS_ERR_PARSE;
        }
        fp.insert(fp.end(), f5, f5 + 5);
        int rows = 0;
        if (kind == FCS_RXN_PLOG) {
            const Node* ad = inner_list(r->find("ArrheniusData"));
            if (!ad) return FCS_ERR_PARSE;
            for (auto& it : ad->items) {
                std::vector<double> v;
                if (it->kind != Node::LIST || !list_doubles(it.get(), v) || v.size() != 4) return FCS_ERR_PARSE;
                pt.insert(pt.end(), v.begin(), v.end());
                rows++;
            }
        }
        po.push_back(po.back() + rows);
    }
    if (pt.empty()) pt.assign(4, 0.0);
    fcs_mechanism_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_species = ns;
    d.n_reactions = (int32_t)type.size();
    d.W = W.data(); d.T_low = Tl.data(); d.T_high = Th.data(); d.T_common = Tc.data();
    d.high_coeffs = hc.data(); d.low_coeffs = lc.data();
    d.type = type.data(); d.reversible = rev.data();
    d.lhs_offset = lo.data(); d.lhs_species = ls.data(); d.rhs_offset = ro.data(); d.rhs_species = rs.data();
    d.arrhenius = arr.data(); d.arrhenius2 = arr2.data(); d.efficiencies = eff.data();
    d.falloff_params = fp.data(); d.plog_offset = po.data(); d.plog_table = pt.data();
    std::vector<const char*> names(ns);
    for (int i = 0; i < ns; i++) names[i] = species[i].c_str();
    return visit(&d, names.data(), user);
}

// No C++ exception crosses the C ABI: a file the reader cannot take is
// FCS_ERR_PARSE, running out of host memory FCS_ERR_NOMEM.
fcs_status parse_foam(const char* reactions_path, const char* thermo_path, fcs_mechanism_visitor visit,
                      void* user) {
    if (!reactions_path || !thermo_path || !visit) return FCS_ERR_INVALID;
    try {
        return parse_foam_files(reactions_path, thermo_path, visit, user);
    } catch (const std::bad_alloc&) {
        return FCS_ERR_NOMEM;
    } catch (...) {
        return FCS_ERR_PARSE;
    }
}

fcs_status load_visitor(const fcs_mechanism_desc* d, const char* const*, void* ctx) {
    return fcs_load_mechanism(static_cast<fcs_ctx*>(ctx), d);
}

}  // namespace

extern "C" fcs_status fcs_load_mechanism_foam(fcs_ctx* ctx, const char* reactions_path, const char* thermo_path) {
    if (!ctx) return FCS_ERR_INVALID;
    return parse_foam(reactions_path, thermo_path, load_visitor, ctx);
}

extern "C" fcs_status fcs_parse_mechanism_foam(const char* reactions_path, const char* thermo_path,
                                               fcs_mechanism_visitor visit, void* user) {
    return parse_foam(reactions_path, thermo_path, visit, user);
}

namespace {

// A positive whole number that fits an int32 (maxSteps, maxRejects)
bool as_count(const Node* v, int32_t& out) {
    double d;
    if (!as_double(v, d) || !(d >= 1) || d > 2147483647.0 || d != std::floor(d)) return false;
    out = (int32_t)d;
    return true;
}

fcs_status read_chemistry_properties(const char* path, fcs_options* o, double* initial_sub_dt) {
    Parser P;
    P.followIncludes = false;  // `#include "reactions"` carries no solver keys
    Node root;
    if (!P.parse_file(path, root)) return FCS_ERR_PARSE;
    fcs_default_options(o);
    std::string solver = "OptRodas34";
    const Node* ct = root.find("chemistryType");
    if (ct && ct->kind == Node::DICT) as_word(ct->find("solver"), solver);
    if (solver == "OptRodas34") o->solver = FCS_SOLVER_RODAS34;
    else if (solver == "OptRosenbrock34") o->solver = FCS_SOLVER_ROSENBROCK34;
    else if (solver == "OptSeulex") o->solver = FCS_SOLVER_SEULEX;
    else if (solver == "OptRodas23") o->solver = FCS_SOLVER_RODAS23;
    else if (solver == "OptRosenbrock23") o->solver = FCS_SOLVER_ROSENBROCK23;
    else return FCS_ERR_UNSUPPORTED;
    std::string jac = "exact";
    if (as_word(root.find("jacobian"), jac)) {
        if (jac == "exact") o->jacobian = FCS_JACOBIAN_EXACT;
        else if (jac == "fast") o->jacobian = FCS_JACOBIAN_FAST;
        else return FCS_ERR_PARSE;
    }
    double v;
    if (as_double(root.find("Treact"), v)) o->T_react = v;
    if (as_double(root.find("maxChemicalTimeStep"), v)) o->delta_t_chem_max = v;
    if (initial_sub_dt) *initial_sub_dt = as_double(root.find("initialChemicalTimeStep"), v) ? v : -1.0;
    const Node* cd = root.find(solver + "Coeffs");
    if (!cd || cd->kind != Node::DICT) return FCS_ERR_PARSE;  // absTol/relTol are required
    if (!as_double(cd->find("absTol"), o->abs_tol) || !as_double(cd->find("relTol"), o->rel_tol))
        return FCS_ERR_PARSE;
    if (cd->find("maxSteps") && !as_count(cd->find("maxSteps"), o->max_steps)) return FCS_ERR_PARSE;
    const Node* gd = root.find("FastChemistryGPU");
    if (gd && gd->kind == Node::DICT) {
        std::string w;
        if (as_word(gd->find("precision"), w)) {
            if (w == "fp64") o->precision = FCS_PRECISION_FP64;
            else if (w == "mixed") o->precision = FCS_PRECISION_MIXED;
            else return FCS_ERR_PARSE;
        }
        if (as_word(gd->find("mapping"), w)) {
            if (w == "auto") o->mapping = FCS_MAPPING_AUTO;
            else if (w == "lane") o->mapping = FCS_MAPPING_LANE;
            else if (w == "warp") o->mapping = FCS_MAPPING_WARP;
            else if (w == "block64") o->mapping = FCS_MAPPING_BLOCK64;
            else if (w == "block128") o->mapping = FCS_MAPPING_BLOCK128;
            else if (w == "block256") o->mapping = FCS_MAPPING_BLOCK256;
            else return FCS_ERR_PARSE;
        }
        if (gd->find("maxRejects") && !as_count(gd->find("maxRejects"), o->max_rejects)) return FCS_ERR_PARSE;
    }
    return FCS_OK;
}

}  // namespace

extern "C" fcs_status fcs_read_chemistry_properties(const char* path, fcs_options* o, double* initial_sub_dt) {
    if (!path || !o) return FCS_ERR_INVALID;
    try {
        return read_chemistry_properties(path, o, initial_sub_dt);
    } catch (const std::bad_alloc&) {
        return FCS_ERR_NOMEM;
    } catch (...) {
        return FCS_ERR_PARSE;
    }
}
