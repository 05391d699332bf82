// mechanism.cpp - Cantera YAML -> flat Mechanism.  See mechanism.h.
//
// The interpretation of each YAML item follows the reference loader:
//  * reaction equations: parseReactionEquation (src/kinetics/Reaction.cpp:889-956)
//  * implicit / explicit third bodies: Reaction::setEquation (Reaction.cpp:389-555)
//    and ThirdBody::setName / setParameters (Reaction.cpp:777-830)
//  * rate-coefficient units: Reaction::calculateRateCoeffUnits (Reaction.cpp:576-617),
//    FalloffRate::setParameters (src/kinetics/Falloff.cpp:130-161),
//    UnitSystem::convertTo (src/base/Units.cpp:562-571)
//  * activation energies: UnitSystem::convertActivationEnergyTo (Units.cpp:706-718)
//  * Troe parameters: TroeRate::setFalloffCoeffs (Falloff.cpp:235-270)
//  * stoichiometry buckets: StoichManagerN::add (include/cantera/kinetics/StoichManager.h:676-722)
//  * molecular weights: Species::molecularWeight (src/thermo/Species.cpp:31-48) with the
//    element table of src/thermo/Elements.cpp:64-82
#include "mechanism.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <stdexcept>

#include "yaml_lite.h"

namespace gbchem {

namespace {

[[noreturn]] void fail(const std::string& file, int line, const std::string& msg) {
    std::ostringstream os;
    os << file;
    if (line > 0) os << ":" << line;
    os << ": " << msg;
    throw std::runtime_error(os.str());
}

// Atomic weights (kg/kmol) of the elements these mechanisms use.
double elementWeight(const std::string& e) {
    static const std::map<std::string, double> w = {
        {"H", 1.008},   {"He", 4.002602}, {"C", 12.011},  {"N", 14.007},
        {"O", 15.999},  {"F", 18.998403163}, {"Ne", 20.1797}, {"S", 32.06},
        {"Cl", 35.45},  {"Ar", 39.95},   {"Si", 28.085},  {"E", 5.485799090649e-4},
    };
    auto it = w.find(e);
    if (it == w.end()) return -1.0;
    return it->second;
}

bool startsWith(const std::string& s, const std::string& p) { return s.compare(0, p.size(), p) == 0; }
bool endsWith(const std::string& s, const std::string& p) {
    return s.size() >= p.size() && s.compare(s.size() - p.size(), p.size(), p) == 0;
}

std::vector<std::string> splitWs(const std::string& s) {
    std::vector<std::string> t;
    std::istringstream is(s);
    std::string w;
    while (is >> w) t.push_back(w);
    return t;
}

// A unit expression "a^p*b/c^q" as a factor to SI-kmol units and its dimensions
// (mass, length, time, temperature, current, quantity), after Units::Units(string)
// (reference src/base/Units.cpp:138-195): groups split at '*' and '/', a group after
// '/' in the denominator, an optional '^exponent', known units with an optional
// one-letter SI prefix.
struct UnitDim {
    double f = 1.0;
    double d[6] = {0, 0, 0, 0, 0, 0};   // M, L, T, Theta, I, Q
    bool same(const double* o) const {
        for (int i = 0; i < 6; i++)
            if (std::fabs(d[i] - o[i]) > 1e-12) return false;
        return true;
    }
};
constexpr double kDimPressure[6] = {1, -1, -2, 0, 0, 0};
constexpr double kDimEnergy[6] = {1, 2, -2, 0, 0, 0};
constexpr double kDimMolarEnergy[6] = {1, 2, -2, 0, 0, -1};
constexpr double kDimTemperature[6] = {0, 0, 0, 1, 0, 0};
constexpr double kDimLength[6] = {0, 1, 0, 0, 0, 0};
constexpr double kDimMass[6] = {1, 0, 0, 0, 0, 0};
constexpr double kDimTime[6] = {0, 0, 1, 0, 0, 0};
constexpr double kDimQuantity[6] = {0, 0, 0, 0, 0, 1};

bool baseUnit(const std::string& u, UnitDim& out) {
    struct B { const char* n; double f; double d[6]; };
    static const B table[] = {
        {"kg", 1.0, {1, 0, 0, 0, 0, 0}}, {"g", 1e-3, {1, 0, 0, 0, 0, 0}},
        {"m", 1.0, {0, 1, 0, 0, 0, 0}}, {"micron", 1e-6, {0, 1, 0, 0, 0, 0}},
        {"angstrom", 1e-10, {0, 1, 0, 0, 0, 0}},
        {"s", 1.0, {0, 0, 1, 0, 0, 0}}, {"min", 60.0, {0, 0, 1, 0, 0, 0}}, {"hr", 3600.0, {0, 0, 1, 0, 0, 0}},
        {"K", 1.0, {0, 0, 0, 1, 0, 0}}, {"C", 1.0, {0, 0, 0, 1, 0, 0}},
        {"A", 1.0, {0, 0, 0, 0, 1, 0}},
        {"mol", 1e-3, {0, 0, 0, 0, 0, 1}}, {"gmol", 1e-3, {0, 0, 0, 0, 0, 1}}, {"mole", 1e-3, {0, 0, 0, 0, 0, 1}},
        {"kmol", 1.0, {0, 0, 0, 0, 0, 1}}, {"kgmol", 1.0, {0, 0, 0, 0, 0, 1}},
        {"molec", 1.0 / kAvogadro, {0, 0, 0, 0, 0, 1}},
        {"J", 1.0, {1, 2, -2, 0, 0, 0}}, {"cal", 4.184, {1, 2, -2, 0, 0, 0}}, {"erg", 1e-7, {1, 2, -2, 0, 0, 0}},
        {"eV", 1.602176634e-19, {1, 2, -2, 0, 0, 0}},
        {"N", 1.0, {1, 1, -2, 0, 0, 0}}, {"dyn", 1e-5, {1, 1, -2, 0, 0, 0}},
        {"Pa", 1.0, {1, -1, -2, 0, 0, 0}}, {"atm", kOneAtm, {1, -1, -2, 0, 0, 0}}, {"bar", 1e5, {1, -1, -2, 0, 0, 0}},
        {"liter", 1e-3, {0, 3, 0, 0, 0, 0}}, {"L", 1e-3, {0, 3, 0, 0, 0, 0}}, {"l", 1e-3, {0, 3, 0, 0, 0, 0}},
        {"cc", 1e-6, {0, 3, 0, 0, 0, 0}},
    };
    for (const B& b : table)
        if (u == b.n) {
            out.f = b.f;
            for (int i = 0; i < 6; i++) out.d[i] = b.d[i];
            return true;
        }
    return false;
}

UnitDim parseUnits(const std::string& expr, const std::string& file, int line) {
    static const std::map<char, double> prefix = {
        {'Y', 1e24}, {'Z', 1e21}, {'E', 1e18}, {'P', 1e15}, {'T', 1e12}, {'G', 1e9}, {'M', 1e6},
        {'k', 1e3}, {'h', 1e2}, {'d', 1e-1}, {'c', 1e-2}, {'m', 1e-3}, {'u', 1e-6}, {'n', 1e-9},
        {'p', 1e-12}, {'f', 1e-15}, {'a', 1e-18}, {'z', 1e-21}, {'y', 1e-24}};
    UnitDim r;
    size_t start = 0;
    while (true) {
        size_t stop = expr.find_first_of("*/", start);
        std::string grp = expr.substr(start, stop == std::string::npos ? std::string::npos : stop - start);
        double e = 1.0;
        size_t caret = grp.find('^');
        if (caret != std::string::npos) {
            e = std::stod(grp.substr(caret + 1));
            grp = grp.substr(0, caret);
        }
        std::string u;
        for (char ch : grp)
            if (ch != ' ' && ch != '\t') u += ch;
        if (start > 0 && expr[start - 1] == '/') e = -e;
        UnitDim b;
        if (!baseUnit(u, b)) {
            auto pf = u.empty() ? prefix.end() : prefix.find(u[0]);
            if (pf == prefix.end() || !baseUnit(u.substr(1), b))
                fail(file, line, "unknown unit '" + u + "' in '" + expr + "'");
            b.f *= pf->second;
        }
        r.f *= std::pow(b.f, e);
        for (int i = 0; i < 6; i++) r.d[i] += b.d[i] * e;
        if (stop == std::string::npos) break;
        start = stop + 1;
    }
    return r;
}

// Split "value units" (a quantity with explicit units); false if the text is a plain number.
bool splitQuantity(const YNode& n, double& value, std::string& units) {
    std::string t = n.asString();
    size_t b = t.find_first_not_of(" \t");
    if (b == std::string::npos) return false;
    size_t sp = t.find_first_of(" \t", b);
    if (sp == std::string::npos) return false;
    value = std::stod(t.substr(b, sp - b));
    units = t.substr(sp + 1);
    return true;
}

// The unit system in force for a YAML node: the file's `units:` block, overlaid by any
// `units:` of an enclosing node (UnitSystem::setDefaults, reference src/base/Units.cpp:475-538).
struct FileUnits {
    double mass = 1.0;       // kg per unit
    double length = 1.0;     // m per unit
    double quantity = 1.0;   // kmol per unit
    double time = 1.0;       // s per unit
    double energy = 1.0;     // J per unit
    double pressure = 1.0;   // Pa per unit
    double eaFactor = 1.0;   // J/kmol per activation-energy unit
    bool eaIsTemperature = false;
    bool eaExplicit = false;
};

double dimFactor(const YNode& n, const double* dim, const char* what, const std::string& file) {
    UnitDim u = parseUnits(n.asString(), file, n.line);
    if (!u.same(dim)) fail(file, n.line, std::string("'") + n.asString() + "' is not a unit of " + what);
    return u.f;
}

FileUnits applyUnits(const YNode* u, FileUnits fu, const std::string& file) {
    if (!u) return fu;
    if (const YNode* n = u->find("mass")) fu.mass = dimFactor(*n, kDimMass, "mass", file);
    if (const YNode* n = u->find("length")) fu.length = dimFactor(*n, kDimLength, "length", file);
    if (const YNode* n = u->find("quantity")) fu.quantity = dimFactor(*n, kDimQuantity, "quantity", file);
    if (const YNode* n = u->find("time")) fu.time = dimFactor(*n, kDimTime, "time", file);
    if (const YNode* n = u->find("energy")) fu.energy = dimFactor(*n, kDimEnergy, "energy", file);
    if (const YNode* n = u->find("pressure")) fu.pressure = dimFactor(*n, kDimPressure, "pressure", file);
    if (const YNode* n = u->find("temperature"))
        if (n->asString() != "K") fail(file, n->line, "temperature unit must be K");
    if (const YNode* n = u->find("activation-energy")) {
        UnitDim a = parseUnits(n->asString(), file, n->line);
        fu.eaIsTemperature = false;
        if (a.same(kDimMolarEnergy)) fu.eaFactor = a.f;
        else if (a.same(kDimTemperature)) { fu.eaFactor = gasConstant(); fu.eaIsTemperature = true; }
        else if (a.same(kDimEnergy)) fu.eaFactor = a.f * kAvogadro;
        else fail(file, n->line, "'" + n->asString() + "' is not a unit of activation energy");
        fu.eaExplicit = true;
    } else if (!fu.eaExplicit) {
        fu.eaFactor = fu.energy / fu.quantity;
    }
    return fu;
}

FileUnits readUnits(const YNode& root, const std::string& file) {
    return applyUnits(root.find("units"), FileUnits{}, file);
}

// Rate coefficient of total order n (concentration^(1-n) / time) in SI-kmol units,
// following UnitSystem::convertTo's factor order: value * L^(3(n-1)) * T^-1 * Q^(1-n).
double convertRateCoeff(double value, double n, const FileUnits& fu) {
    double v = value;
    v = v * std::pow(fu.length, 3.0 * (n - 1.0));
    v = v * std::pow(fu.time, -1.0);
    v = v * std::pow(fu.quantity, 1.0 - n);
    return v;
}

// A rate coefficient given as a number (file units) or as "value units".
double readRateCoeff(const YNode& node, double n, const FileUnits& fu, const std::string& file) {
    double v;
    std::string units;
    if (!splitQuantity(node, v, units)) return convertRateCoeff(node.asDouble(), n, fu);
    UnitDim u = parseUnits(units, file, node.line);
    const double dim[6] = {0, 3.0 * (n - 1.0), -1, 0, 0, 1.0 - n};
    if (!u.same(dim)) fail(file, node.line, "units '" + units + "' do not match the reaction order");
    return v * u.f;
}

// A pressure given as a number (file units) or as "value units", in Pa.
double readPressure(const YNode& node, const FileUnits& fu, const std::string& file) {
    double v;
    std::string units;
    if (!splitQuantity(node, v, units)) return node.asDouble() * fu.pressure;
    UnitDim u = parseUnits(units, file, node.line);
    if (!u.same(kDimPressure)) fail(file, node.line, "'" + units + "' is not a unit of pressure");
    return v * u.f;
}

// A temperature given as a number or as "value K".
double readTemperature(const YNode& node, const std::string& file) {
    double v;
    std::string units;
    if (!splitQuantity(node, v, units)) return node.asDouble();
    UnitDim u = parseUnits(units, file, node.line);
    if (!u.same(kDimTemperature)) fail(file, node.line, "'" + units + "' is not a unit of temperature");
    return v * u.f;
}

double convertEa(const YNode& node, const FileUnits& fu, const std::string& file) {
    // Ea given as a number (file units) or as "value unit" (UnitSystem::convertActivationEnergy)
    double v;
    std::string units;
    if (!splitQuantity(node, v, units)) {
        if (fu.eaIsTemperature) return node.asDouble();
        return node.asDouble() * fu.eaFactor / gasConstant();
    }
    UnitDim a = parseUnits(units, file, node.line);
    if (a.same(kDimTemperature)) return v * a.f;
    if (a.same(kDimMolarEnergy)) return v * a.f / gasConstant();
    if (a.same(kDimEnergy)) return v * a.f * kAvogadro / gasConstant();
    fail(file, node.line, "'" + units + "' is not a unit of activation energy");
}

struct Arr { double A, b, EaR; };

Arr readArrhenius(const YNode& node, double order, const FileUnits& fu, const std::string& file) {
    Arr a{};
    if (node.isMap()) {
        a.A = readRateCoeff(node["A"], order, fu, file);
        a.b = node["b"].asDouble();
        a.EaR = node.has("Ea") ? convertEa(node["Ea"], fu, file) : 0.0;
    } else if (node.isSeq() && node.elems.size() >= 2) {
        a.A = readRateCoeff(node.elems[0], order, fu, file);
        a.b = node.elems[1].asDouble();
        a.EaR = node.elems.size() > 2 ? convertEa(node.elems[2], fu, file) : 0.0;
    } else {
        fail(file, node.line, "malformed rate constant");
    }
    return a;
}

struct ParsedReaction {
    std::map<std::string, double> reactants, products;   // name-ordered, as Composition
    bool reversible = true;
    bool hasThirdBody = false;
    std::string tbName;          // "M" or a species name
    bool tbMassAction = true;
    double tbDefault = 1.0;
    std::map<std::string, double> tbEff;
};

// Restatement of parseReactionEquation: tokens separated by whitespace, "(+M)" or
// "(+ M)" mark a falloff collider, a number token before a species is its coefficient.
void parseEquation(const std::string& eq, ParsedReaction& r, const std::string& file, int line) {
    std::vector<std::string> tok = splitWs(eq);
    tok.push_back("+");
    long last = -1;
    bool reac = true;
    for (long i = 1; i < (long)tok.size(); i++) {
        const std::string& t = tok[i];
        if (t == "+" || startsWith(t, "(+") || t == "<=>" || t == "=" || t == "=>") {
            std::string sp = tok[i - 1];
            double nu = 1.0;
            if (last >= 0 && tok[last] == "(+" && endsWith(sp, ")")) {
                sp = "(+" + sp;
            } else if (last == i - 1 && startsWith(sp, "(+") && endsWith(sp, ")")) {
                // falloff third body written without a space
            } else if (last == i - 2) {
                // species without coefficient
            } else if (last == i - 3) {
                char* e = nullptr;
                nu = std::strtod(tok[i - 2].c_str(), &e);
                if (e == tok[i - 2].c_str() || *e) fail(file, line, "cannot parse equation '" + eq + "'");
            } else {
                fail(file, line, "cannot parse equation '" + eq + "'");
            }
            if (reac) r.reactants[sp] += nu;
            else r.products[sp] += nu;
            last = i;
        }
        if (t == "<=>" || t == "=") { r.reversible = true; reac = false; }
        else if (t == "=>") { r.reversible = false; reac = false; }
    }
    if (reac) fail(file, line, "equation '" + eq + "' has no '<=>', '=' or '=>'");
}

bool isGeneric(const std::string& n) { return n == "M" || n == "(+M)" || n == "(+ M)"; }

// Restatement of Reaction::setEquation's collider detection and ThirdBody setup.
void detectThirdBody(const YNode& rn, const std::string& rateType, ParsedReaction& r,
                     const std::string& file) {
    const int line = rn.line;
    const std::string eq = rn["equation"].asString();
    if (rateType == "elementary") return;
    std::string third;
    int count = 0, countM = 0, countF = 0;
    for (auto& kv : r.reactants) {
        const std::string& name = kv.first;
        double nu = kv.second;
        auto pit = r.products.find(name);
        if (pit == r.products.end()) continue;
        if (countF == 0) third = name;
        int generic = isGeneric(third) ? 1 : 0;
        count++;
        countM += generic;
        auto tp = r.products.find(third);
        double pthird = tp == r.products.end() ? 0.0 : tp->second;
        if (nu > 1 && pthird > 1) { count++; countM += generic; }
        if (startsWith(name, "(+") && endsWith(name, ")")) countF++;
    }
    bool explicitFromEff = false;
    if (count == 0) {
        if (startsWith(rateType, "three-body"))
            fail(file, line, "reactants of '" + eq + "' contain no valid third-body collider");
        return;
    } else if (countF == 1) {
        // falloff collider takes precedence
    } else if (countM > 1) {
        fail(file, line, "multiple generic third-body colliders in '" + eq + "'");
    } else if (count > 1) {
        if (countM) {
            third = "M";
        } else if (rn.has("efficiencies")) {
            auto effs = rn["efficiencies"].asDoubleMap();
            if (effs.size() != 1 || !r.reactants.count(effs.begin()->first))
                fail(file, line, "ambiguous third-body colliders in '" + eq + "'");
            third = effs.begin()->first;
            explicitFromEff = true;
        } else if (rn.has("default-efficiency")) {
            fail(file, line, "ambiguous third-body colliders in '" + eq + "'");
        } else if (startsWith(rateType, "three-body")) {
            fail(file, line, "ambiguous third-body colliders in '" + eq + "'");
        } else {
            return;
        }
    } else if (third != "M" && !startsWith(rateType, "three-body") && !startsWith(third, "(+")) {
        double nreac = 0, nprod = 0;
        for (auto& kv : r.reactants) {
            if (std::trunc(kv.second) != kv.second) return;
            nreac += kv.second;
        }
        for (auto& kv : r.products) {
            if (std::trunc(kv.second) != kv.second) return;
            nprod += kv.second;
        }
        if (nreac != 3 && nprod != 3) return;
    }
    (void)explicitFromEff;
    // ThirdBody(third): "(+X)" / "(+ X)" marks a non-mass-action (falloff) collider X
    r.hasThirdBody = true;
    std::string name = third;
    r.tbMassAction = true;
    if (startsWith(third, "(+ ")) { r.tbMassAction = false; name = third.substr(3, third.size() - 4); }
    else if (startsWith(third, "(+")) { r.tbMassAction = false; name = third.substr(2, third.size() - 3); }
    r.tbName = name;
    if (name != "M") { r.tbDefault = 0.0; r.tbEff[name] = 1.0; }
    // strip the collider from both sides
    auto strip = [&](std::map<std::string, double>& side) {
        auto it = side.find(third);
        if (it == side.end()) fail(file, line, "logic error interpreting third body of '" + eq + "'");
        if (std::trunc(it->second) != 1) it->second -= 1.0;
        else side.erase(it);
    };
    strip(r.reactants);
    strip(r.products);
}

}  // namespace

int Mechanism::speciesIndex(const std::string& name) const {
    for (int k = 0; k < K; k++)
        if (speciesNames[k] == name) return k;
    return -1;
}

namespace {

std::mutex g_dirMu;
std::vector<std::string> g_dataDirs;

bool fileExists(const std::string& p) {
    std::ifstream f(p);
    return f.good();
}

// AnyMap::fromYamlFile's search order (reference src/base/AnyMap.cpp:1841-1856): next to
// the including file, then the working directory, then the data directories (the most
// recently added first).
std::string findInputFile(const std::string& name, const std::string& parent) {
    size_t sl = parent.find_last_of('/');
    if (sl != std::string::npos) {
        std::string c = parent.substr(0, sl) + "/" + name;
        if (fileExists(c)) return c;
    }
    if (fileExists(name)) return name;
    std::lock_guard<std::mutex> lk(g_dirMu);
    for (auto it = g_dataDirs.rbegin(); it != g_dataDirs.rend(); ++it) {
        std::string c = *it + "/" + name;
        if (fileExists(c)) return c;
    }
    fail(parent, 0, "input file '" + name + "' not found");
}

// A section of the current file ("name") or of another file ("file.yaml/name"), with the
// unit system of the file it lives in.
struct Section {
    const YNode* node;
    std::string file;
    FileUnits fu;
};

struct Sources {
    std::map<std::string, std::unique_ptr<YNode>> roots;   // other files, kept alive while loading
    Section resolve(const std::string& spec, const YNode& root, const std::string& path,
                    const FileUnits& fu, int line) {
        size_t sl = spec.rfind('/');
        if (sl == std::string::npos) {
            const YNode* n = root.find(spec);
            if (!n) fail(path, line, "could not find a section named '" + spec + "'");
            return Section{n, path, fu};
        }
        std::string f = findInputFile(spec.substr(0, sl), path);
        auto it = roots.find(f);
        if (it == roots.end()) it = roots.emplace(f, std::make_unique<YNode>(yamlParseFile(f))).first;
        const YNode* n = it->second->find(spec.substr(sl + 1));
        if (!n) fail(f, 0, "could not find a section named '" + spec.substr(sl + 1) + "'");
        return Section{n, f, readUnits(*it->second, f)};
    }
};

}  // namespace

void addDataDirectory(const std::string& dir) {
    std::lock_guard<std::mutex> lk(g_dirMu);
    std::string d = dir;
    while (d.size() > 1 && d.back() == '/') d.pop_back();
    if (std::find(g_dataDirs.begin(), g_dataDirs.end(), d) == g_dataDirs.end()) g_dataDirs.push_back(d);
}

Mechanism loadMechanism(const std::string& path, const std::string& phaseName) {
    YNode root = yamlParseFile(path);
    Mechanism m;
    m.source = path;
    FileUnits fu = readUnits(root, path);
    Sources src;

    // ---- phase ----
    const YNode& phases = root["phases"];
    if (!phases.isSeq() || phases.elems.empty()) fail(path, phases.line, "no phases");
    const YNode* ph = nullptr;
    for (auto& p : phases.elems) {
        if (phaseName.empty() || p["name"].asString() == phaseName) { ph = &p; break; }
    }
    if (!ph) fail(path, phases.line, "phase '" + phaseName + "' not found");
    m.phase = (*ph)["name"].asString();
    std::string thermoModel = (*ph)["thermo"].asString();
    if (thermoModel != "ideal-gas")
        fail(path, ph->line, "phase '" + m.phase + "' uses thermo model '" + thermoModel +
                                 "'; only ideal-gas phases are supported");
    if (const YNode* kinNode = ph->find("kinetics")) {
        std::string kin = kinNode->asString();
        if (kin != "gas" && kin != "bulk")
            fail(path, ph->line, "unsupported kinetics model '" + kin + "'");
    }

    // ---- species declarations (setupPhase / addSpecies, reference src/thermo/
    // ThermoFactory.cpp:177-199,262-304): a list of names from this file's 'species'
    // section, the keyword 'all', or a list of {section: names | all} where a section may
    // live in another file ---
    struct SpDef { std::string name; const YNode* node; std::string file; FileUnits fu; };
    std::vector<SpDef> defs;
    auto addSpecies = [&](const YNode& names, const Section& sec, int line) {
        if (!sec.node->isSeq()) fail(sec.file, sec.node->line, "species section is not a list");
        auto push = [&](const YNode& sp) {
            std::string nm = sp["name"].asString();
            for (auto& d : defs)
                if (d.name == nm) fail(path, line, "species '" + nm + "' is declared twice");
            defs.push_back(SpDef{nm, &sp, sec.file, sec.fu});
        };
        if (names.isScalar() && names.asString() == "all") {
            for (auto& sp : sec.node->elems) push(sp);
        } else if (names.isSeq()) {
            std::map<std::string, const YNode*> byName;
            for (auto& sp : sec.node->elems) byName[sp["name"].asString()] = &sp;
            for (auto& e : names.elems) {
                auto it = byName.find(e.asString());
                if (it == byName.end()) fail(path, names.line, "could not find a species named '" + e.asString() + "'");
                push(*it->second);
            }
        } else {
            fail(path, names.line, "could not parse the species declaration");
        }
    };
    YNode allKw;
    allKw.kind = YNode::Scalar;
    allKw.text = "all";
    if (const YNode* sl = ph->find("species")) {
        bool names = sl->isScalar() || (sl->isSeq() && (sl->elems.empty() || sl->elems[0].isScalar()));
        if (names) {
            addSpecies(*sl, src.resolve("species", root, path, fu, sl->line), sl->line);
        } else if (sl->isSeq()) {
            for (auto& item : sl->elems) {
                if (!item.isMap() || item.items.size() != 1)
                    fail(path, item.line, "a species source must be a single {section: names} item");
                addSpecies(item.items[0].second, src.resolve(item.items[0].first, root, path, fu, item.line), item.line);
            }
        } else {
            fail(path, sl->line, "could not parse the species declaration");
        }
    } else if (root.has("species")) {
        addSpecies(allKw, Section{&root["species"], path, fu}, ph->line);
    }
    m.K = (int)defs.size();
    for (auto& d : defs) m.speciesNames.push_back(d.name);

    // ---- elements: the declared list, or (no 'elements' key) those the species use, in
    // order of first use (ThermoPhase::addUndefinedElements) ----
    if (const YNode* el = ph->find("elements")) {
        m.elementNames = el->asStringVec();
    } else {
        for (auto& d : defs)
            for (auto& kv : (*d.node)["composition"].asDoubleMap())
                if (std::find(m.elementNames.begin(), m.elementNames.end(), kv.first) == m.elementNames.end())
                    m.elementNames.push_back(kv.first);
    }
    for (auto& e : m.elementNames) {
        double w = elementWeight(e);
        if (w < 0) fail(path, ph->line, "unknown element '" + e + "'");
        m.elementWeights.push_back(w);
    }

    // ---- species data ----
    const int E = (int)m.elementNames.size();
    m.atoms.assign((size_t)m.K * E, 0.0);
    bool prefSet = false;
    for (int k = 0; k < m.K; k++) {
        const YNode& s = *defs[k].node;
        const std::string& sfile = defs[k].file;
        auto comp = s["composition"].asDoubleMap();
        double w = 0.0;
        for (auto& kv : comp) {  // element-name order, as the reference's Composition map
            double ew = elementWeight(kv.first);
            if (ew < 0) fail(sfile, s.line, "unknown element '" + kv.first + "'");
            w += ew * kv.second;
            auto e = std::find(m.elementNames.begin(), m.elementNames.end(), kv.first);
            if (e == m.elementNames.end())
                fail(sfile, s.line, "species '" + m.speciesNames[k] + "' uses undeclared element '" + kv.first + "'");
            m.atoms[(size_t)k * E + (e - m.elementNames.begin())] = kv.second;
        }
        m.mw.push_back(w);
        const YNode& th = s["thermo"];
        if (th["model"].asString() != "NASA7")
            fail(sfile, th.line, "species '" + m.speciesNames[k] + "': only NASA7 thermo is supported");
        std::vector<double> tr = th["temperature-ranges"].asDoubleVec();
        const YNode& data = th["data"];
        if (tr.size() < 2 || tr.size() > 3 || data.elems.size() != tr.size() - 1)
            fail(sfile, th.line, "bad NASA7 temperature ranges / data");
        std::vector<double> lo = data.elems[0].asDoubleVec();
        std::vector<double> hi = tr.size() == 3 ? data.elems[1].asDoubleVec() : lo;
        if (lo.size() != 7 || hi.size() != 7) fail(sfile, th.line, "NASA7 polynomials need 7 coefficients");
        double pref = kOneAtm;
        if (const YNode* p = th.find("reference-pressure")) pref = readPressure(*p, defs[k].fu, sfile);
        if (prefSet && pref != m.Pref) fail(sfile, th.line, "species reference pressures differ");
        m.Pref = pref;
        prefSet = true;
        m.Tmin.push_back(tr.front());
        m.Tmax.push_back(tr.back());
        m.nasaTmid.push_back(tr.size() == 3 ? tr[1] : tr.back());
        for (int j = 0; j < 7; j++) m.nasaLow.push_back(lo[j]);
        for (int j = 0; j < 7; j++) m.nasaHigh.push_back(hi[j]);
    }

    // ---- reaction sections (addReactions, reference src/kinetics/KineticsFactory.cpp:
    // 108-218): the rule 'all', 'declared-species' (skip reactions naming undeclared
    // species) or 'none' for this file's 'reactions' section, or a list of sections ----
    std::vector<std::pair<Section, std::string>> rsecs;
    if (const YNode* rk = ph->find("reactions")) {
        if (rk->isScalar()) {
            if (root.has("reactions")) rsecs.push_back({Section{&root["reactions"], path, fu}, rk->asString()});
            else if (rk->asString() != "none")
                fail(path, rk->line, "the phase implies a 'reactions' section that does not exist");
        } else if (rk->isSeq()) {
            for (auto& it : rk->elems) {
                if (it.isScalar()) {
                    rsecs.push_back({src.resolve(it.asString(), root, path, fu, it.line), "all"});
                } else if (it.isMap() && it.items.size() == 1) {
                    rsecs.push_back({src.resolve(it.items[0].first, root, path, fu, it.line), it.items[0].second.asString()});
                } else {
                    fail(path, it.line, "could not parse the reactions declaration");
                }
            }
        } else {
            fail(path, rk->line, "could not parse the reactions declaration");
        }
    } else if (ph->has("kinetics")) {
        if (!root.has("reactions"))
            fail(path, ph->line, "the phase implies a 'reactions' section that does not exist; "
                                 "add 'reactions: none' for a kinetics model without reactions");
        rsecs.push_back({Section{&root["reactions"], path, fu}, "all"});
    }
    const bool skipUndeclaredTB = ph->has("skip-undeclared-third-bodies") &&
                                  (*ph)["skip-undeclared-third-bodies"].asBool();
    m.plogPtr.push_back(0);
    m.chebPtr.push_back(0);

    for (auto& sr : rsecs) {
        const std::string& rule = sr.second;
        if (rule == "none") continue;
        if (rule != "all" && rule != "declared-species")
            fail(path, ph->line, "unknown rule '" + rule + "' for adding reactions");
        const bool skipUndeclared = rule == "declared-species";
        const std::string& rfile = sr.first.file;
        if (!sr.first.node->isSeq()) fail(rfile, sr.first.node->line, "reaction section is not a list");
        for (auto& rn : sr.first.node->elems) {
            const FileUnits rfu = applyUnits(rn.find("units"), sr.first.fu, rfile);
            const std::string eq = rn["equation"].asString();
            std::string type = rn.has("type") ? rn["type"].asString() : std::string();
            ParsedReaction pr;
            parseEquation(eq, pr, rfile, rn.line);
            detectThirdBody(rn, type, pr, rfile);
            // species of the equation (and orders) must be declared, or the reaction is skipped
            // under 'declared-species' (Reaction::checkSpecies)
            {
                bool undeclared = false;
                for (auto* side : {&pr.reactants, &pr.products})
                    for (auto& kv : *side)
                        if (m.speciesIndex(kv.first) < 0) undeclared = true;
                if (const YNode* o = rn.find("orders"))
                    for (auto& kv : o->asDoubleMap())
                        if (m.speciesIndex(kv.first) < 0) undeclared = true;
                if (undeclared && skipUndeclared) continue;
            }
            // ThirdBody::setParameters
            if (pr.hasThirdBody) {
                if (const YNode* d = rn.find("default-efficiency")) {
                    double v = d->asDouble();
                    if (pr.tbName != "M" && v != 0.0)
                        fail(rfile, rn.line, "invalid default efficiency for explicit collider in '" + eq + "'");
                    pr.tbDefault = v;
                }
                if (const YNode* e = rn.find("efficiencies")) pr.tbEff = e->asDoubleMap();
                if (pr.tbName != "M" && (pr.tbEff.size() != 1 || pr.tbEff.begin()->first != pr.tbName))
                    fail(rfile, rn.line, "incompatible third-body collider definitions in '" + eq + "'");
                // ThirdBody::checkSpecies
                std::vector<std::string> und;
                for (auto& kv : pr.tbEff)
                    if (m.speciesIndex(kv.first) < 0) und.push_back(kv.first);
                if (!und.empty()) {
                    if (!skipUndeclaredTB)
                        fail(rfile, rn.line, "reaction '" + eq + "' defines third-body efficiencies for undeclared species '" + und[0] + "'");
                    if (pr.tbName != "M") continue;
                    for (auto& n : und) pr.tbEff.erase(n);
                }
            } else if (rn.has("efficiencies") || rn.has("default-efficiency")) {
                fail(rfile, rn.line, "reaction '" + eq + "' gives efficiencies but has no third body");
            }
            std::map<std::string, double> orders;
            if (const YNode* o = rn.find("orders")) orders = o->asDoubleMap();
            if (pr.reversible && !orders.empty())
                fail(rfile, rn.line, "reaction orders may only be given for irreversible reactions");

            // rate kind (Reaction::setRate checks, reference src/kinetics/Reaction.cpp:164-203)
            int kindv;
            bool falloff = false, chemAct = false;
            if (type.empty() || type == "elementary" || type == "Arrhenius") {
                kindv = pr.hasThirdBody ? kThreeBody : kArrhenius;
            } else if (type == "three-body" || type == "three-body-Arrhenius") {
                kindv = kThreeBody;
            } else if (type == "falloff" || type == "chemically-activated") {
                falloff = true;
                chemAct = type == "chemically-activated";
                int forms = (int)rn.has("Troe") + (int)rn.has("SRI") + (int)rn.has("Tsang");
                if (forms > 1) fail(rfile, rn.line, "more than one falloff function given for '" + eq + "'");
                kindv = rn.has("Troe") ? kTroe : rn.has("SRI") ? kSri : rn.has("Tsang") ? kTsang : kLindemann;
            } else if (type == "pressure-dependent-Arrhenius") {
                kindv = kPlog;
                if (pr.hasThirdBody && pr.tbName == "M")
                    fail(rfile, rn.line, "found superfluous 'M' in pressure-dependent-Arrhenius reaction '" + eq + "'");
            } else if (type == "Chebyshev") {
                kindv = kChebyshev;
                if (pr.hasThirdBody && pr.tbName == "M") {
                    // deprecated "(+M)" notation: the collider is dropped (Reaction.cpp:181-186)
                    pr.hasThirdBody = false;
                    pr.tbEff.clear();
                }
            } else {
                fail(rfile, rn.line, "unsupported reaction type '" + type + "' for '" + eq + "'");
            }
            if (kindv == kThreeBody && !pr.hasThirdBody)
                fail(rfile, rn.line, "three-body reaction '" + eq + "' has no collider");
            if (falloff) {
                if (!pr.hasThirdBody) fail(rfile, rn.line, "falloff reaction '" + eq + "' lacks a (+M) collider");
                if (pr.tbMassAction) fail(rfile, rn.line, "falloff collider of '" + eq + "' must use '(+M)'");
            } else if (pr.hasThirdBody && !pr.tbMassAction) {
                fail(rfile, rn.line, "'(+M)' collider used in non-falloff reaction '" + eq + "'");
            }
            if ((kindv == kPlog || kindv == kChebyshev) && pr.hasThirdBody)
                fail(rfile, rn.line, "third-body collider in pressure-dependent reaction '" + eq + "'");

            // species indices
            std::vector<int32_t> rk, pk;
            std::vector<double> rnu, pnu, rord;
            for (auto& kv : pr.reactants) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(rfile, rn.line, "undeclared species '" + kv.first + "' in '" + eq + "'");
                rk.push_back(k);
                rnu.push_back(kv.second);
            }
            for (auto& kv : pr.products) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(rfile, rn.line, "undeclared species '" + kv.first + "' in '" + eq + "'");
                pk.push_back(k);
                pnu.push_back(kv.second);
            }
            rord = rnu;
            for (auto& kv : orders) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(rfile, rn.line, "order given for undeclared species '" + kv.first + "'");
                auto at = std::find(rk.begin(), rk.end(), k);
                if (at != rk.end()) {
                    rord[at - rk.begin()] = kv.second;
                } else {
                    if (!rn.has("nonreactant-orders") || !rn["nonreactant-orders"].asBool())
                        fail(rfile, rn.line, "order given for non-reactant '" + kv.first + "'");
                    rk.push_back(k);
                    rnu.push_back(0.0);
                    rord.push_back(kv.second);
                }
            }
            // total order of the forward rate coefficient (calculateRateCoeffUnits)
            double order = 0.0;
            for (size_t j = 0; j < rk.size(); j++) order += rord[j];
            double dnv = 0.0;
            for (double v : pnu) dnv += v;
            for (auto& kv : pr.reactants) dnv -= kv.second;

            int irxn = m.R++;
            m.equations.push_back(eq);
            m.kind.push_back(kindv);
            m.chemAct.push_back(chemAct ? 1 : 0);
            m.reversible.push_back(pr.reversible ? 1 : 0);
            m.duplicate.push_back(rn.has("duplicate") && rn["duplicate"].asBool() ? 1 : 0);
            m.dn.push_back(dnv);
            double troe[4] = {0.0, 0.0, 0.0, 0.0};
            double fx[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
            const bool negA = rn.has("negative-A") && rn["negative-A"].asBool();
            if (falloff) {
                // FalloffRate::setParameters (reference src/kinetics/Falloff.cpp:130-161): the
                // low-pressure limit of a falloff reaction, or the high-pressure limit of a
                // chemically activated one, carries one more concentration order
                Arr hi = readArrhenius(rn["high-P-rate-constant"], chemAct ? order - 1.0 : order, rfu, rfile);
                Arr lo = readArrhenius(rn["low-P-rate-constant"], chemAct ? order : order + 1.0, rfu, rfile);
                if (hi.A * lo.A < 0) fail(rfile, rn.line, "falloff A factors differ in sign");
                if ((hi.A < 0 || lo.A < 0) && !negA)
                    fail(rfile, rn.line, "negative pre-exponential factor in '" + eq + "'");
                m.A.push_back(hi.A); m.b.push_back(hi.b); m.EaR.push_back(hi.EaR);
                m.A0.push_back(lo.A); m.b0.push_back(lo.b); m.Ea0R.push_back(lo.EaR);
                if (kindv == kTroe) {
                    const YNode& t = rn["Troe"];
                    double a = t["A"].asDouble(), T3 = t["T3"].asDouble(), T1 = t["T1"].asDouble();
                    troe[0] = a;
                    troe[1] = std::fabs(T3) < kSmallNumber ? INFINITY : 1.0 / T3;
                    troe[2] = std::fabs(T1) < kSmallNumber ? INFINITY : 1.0 / T1;
                    troe[3] = t.has("T2") ? t["T2"].asDouble() : 0.0;
                } else if (kindv == kSri) {
                    // SriRate::setFalloffCoeffs (reference src/kinetics/Falloff.cpp:363-390)
                    const YNode& t = rn["SRI"];
                    fx[0] = t["A"].asDouble();
                    fx[1] = t["B"].asDouble();
                    fx[2] = t["C"].asDouble();
                    if (fx[2] < 0.0) fail(rfile, t.line, "SRI parameter C is less than zero");
                    if (t.has("D") != t.has("E")) fail(rfile, t.line, "SRI needs 3 or 5 coefficients");
                    fx[3] = t.has("D") ? t["D"].asDouble() : 1.0;
                    fx[4] = t.has("E") ? t["E"].asDouble() : 0.0;
                    if (fx[3] < 0.0) fail(rfile, t.line, "SRI parameter D is less than zero");
                } else if (kindv == kTsang) {
                    // TsangRate::setFalloffCoeffs (reference src/kinetics/Falloff.cpp:453-468)
                    const YNode& t = rn["Tsang"];
                    fx[0] = t["A"].asDouble();
                    fx[1] = t.has("B") ? t["B"].asDouble() : 0.0;
                }
            } else if (kindv == kPlog) {
                // PlogRate::setParameters / setRates (reference src/kinetics/PlogRate.cpp:62-120)
                const YNode& rl = rn["rate-constants"];
                if (!rl.isSeq() || rl.elems.empty()) fail(rfile, rn.line, "PLOG reaction '" + eq + "' has no rate constants");
                std::vector<std::pair<double, Arr>> rates;   // (ln P, rate), stable by pressure
                for (auto& r : rl.elems) rates.push_back({std::log(readPressure(r["P"], rfu, rfile)), readArrhenius(r, order, rfu, rfile)});
                std::stable_sort(rates.begin(), rates.end(), [](const std::pair<double, Arr>& x, const std::pair<double, Arr>& y) { return x.first < y.first; });
                const int r0 = (int)m.plogA.size();
                std::vector<std::pair<int, int>> groups;
                std::vector<double> logps;
                for (size_t j = 0; j < rates.size(); j++) {
                    m.plogA.push_back(rates[j].second.A);
                    m.plogB.push_back(rates[j].second.b);
                    m.plogEaR.push_back(rates[j].second.EaR);
                    int idx = r0 + (int)j;
                    if (logps.empty() || logps.back() != rates[j].first) {
                        logps.push_back(rates[j].first);
                        groups.push_back({idx, idx + 1});
                    } else {
                        groups.back().second = idx + 1;
                    }
                }
                auto level = [&](double lp, std::pair<int, int> g) {
                    m.plogLogP.push_back(lp);
                    m.plogFirst.push_back(g.first);
                    m.plogLast.push_back(g.second);
                };
                level(-1000.0, groups.front());
                for (size_t g = 0; g < groups.size(); g++) level(logps[g], groups[g]);
                level(1000.0, groups.back());
                // PlogRate::validate (PlogRate.cpp:122-157): the summed rate at every given
                // pressure must be positive at 300, 500, 1000, 2000, 5000 and 10000 K
                const double Tv[] = {300.0, 500.0, 1000.0, 2000.0, 5000.0, 10000.0};
                for (auto& g : groups)
                    for (double T : Tv) {
                        double k = 0.0;
                        for (int q = g.first; q < g.second; q++)
                            k += m.plogA[q] * std::exp(m.plogB[q] * std::log(T) - m.plogEaR[q] * (1.0 / T));
                        if (!(k > 0))
                            fail(rfile, rn.line, "invalid PLOG rate coefficient for reaction '" + eq + "' at T = " + std::to_string(T));
                    }
                m.A.push_back(0.0); m.b.push_back(0.0); m.EaR.push_back(0.0);
                m.A0.push_back(0.0); m.b0.push_back(0.0); m.Ea0R.push_back(0.0);
            } else if (kindv == kChebyshev) {
                // ChebyshevRate::setParameters / setLimits (reference src/kinetics/ChebyshevRate.cpp:64-111)
                std::vector<std::vector<double>> rows;
                for (auto& r : rn["data"].elems) rows.push_back(r.asDoubleVec());
                if (rows.empty() || rows[0].empty()) fail(rfile, rn.line, "Chebyshev reaction '" + eq + "' has no data");
                for (auto& r : rows)
                    if (r.size() != rows[0].size()) fail(rfile, rn.line, "inconsistent number of Chebyshev coefficients in '" + eq + "'");
                const YNode& trn = rn["temperature-range"];
                const YNode& prn = rn["pressure-range"];
                if (trn.elems.size() != 2 || prn.elems.size() != 2) fail(rfile, rn.line, "Chebyshev ranges need two values");
                const double Tmin = readTemperature(trn.elems[0], rfile), Tmax = readTemperature(trn.elems[1], rfile);
                const double Pmin = readPressure(prn.elems[0], rfu, rfile), Pmax = readPressure(prn.elems[1], rfu, rfile);
                const double offset = convertRateCoeff(1.0, order, rfu);
                rows[0][0] += std::log10(offset);
                const double logPmin = std::log10(Pmin), logPmax = std::log10(Pmax);
                const double TminInv = 1.0 / Tmin, TmaxInv = 1.0 / Tmax;
                m.chebLim.push_back(-TminInv - TmaxInv);
                m.chebLim.push_back(1.0 / (TmaxInv - TminInv));
                m.chebLim.push_back(-logPmin - logPmax);
                m.chebLim.push_back(1.0 / (logPmax - logPmin));
                m.chebNT.push_back((int)rows.size());
                m.chebNP.push_back((int)rows[0].size());
                for (auto& r : rows)
                    for (double v : r) m.chebCoef.push_back(v);
                m.A.push_back(0.0); m.b.push_back(0.0); m.EaR.push_back(0.0);
                m.A0.push_back(0.0); m.b0.push_back(0.0); m.Ea0R.push_back(0.0);
            } else {
                double ord = order + ((kindv == kThreeBody) ? 1.0 : 0.0);
                Arr a = readArrhenius(rn["rate-constant"], ord, rfu, rfile);
                if (a.A < 0 && !negA)
                    fail(rfile, rn.line, "negative pre-exponential factor in '" + eq + "'");
                m.A.push_back(a.A); m.b.push_back(a.b); m.EaR.push_back(a.EaR);
                m.A0.push_back(0.0); m.b0.push_back(0.0); m.Ea0R.push_back(0.0);
            }
            if (kindv != kChebyshev) {
                m.chebNT.push_back(0);
                m.chebNP.push_back(0);
                for (int j = 0; j < 4; j++) m.chebLim.push_back(0.0);
            }
            m.plogPtr.push_back((int)m.plogLogP.size());
            m.chebPtr.push_back((int)m.chebCoef.size());
            for (int j = 0; j < 4; j++) m.troe.push_back(troe[j]);
            for (int j = 0; j < 5; j++) m.falloffX.push_back(fx[j]);

            // third-body table
            if (pr.hasThirdBody) {
                m.tbOfRxn.push_back((int)m.tbRxn.size());
                m.tbRxn.push_back(irxn);
                m.tbDefault.push_back(pr.tbDefault);
                m.tbMassAction.push_back(pr.tbMassAction ? 1 : 0);
                std::map<int, double> effByIndex;   // ascending species index
                for (auto& kv : pr.tbEff) {
                    int k = m.speciesIndex(kv.first);
                    if (k < 0) fail(rfile, rn.line, "third-body efficiency for undeclared species '" + kv.first + "'");
                    effByIndex[k] = kv.second;
                }
                if (m.tbPtr.empty()) m.tbPtr.push_back(0);
                for (auto& kv : effByIndex) {
                    m.tbSpecies.push_back(kv.first);
                    m.tbEffMinusDefault.push_back(kv.second - pr.tbDefault);
                }
                m.tbPtr.push_back((int)m.tbSpecies.size());
            } else {
                m.tbOfRxn.push_back(-1);
            }

            // stoichiometry + bucket classification
            auto bucketOf = [](const std::vector<double>& nu, const std::vector<double>& ord) {
                bool frac = false;
                for (size_t j = 0; j < nu.size(); j++)
                    if (std::fmod(nu[j], 1.0) != 0.0 || nu[j] != ord[j]) frac = true;
                if (frac || nu.size() > 3) return (int)kCN;
                double nrep = 0;
                for (double v : nu) nrep += v;
                if (nrep == 1) return (int)kC1;
                if (nrep == 2) return (int)kC2;
                if (nrep == 3) return (int)kC3;
                return (int)kCN;
            };
            if (m.reacPtr.empty()) m.reacPtr.push_back(0);
            for (size_t j = 0; j < rk.size(); j++) {
                m.reacK.push_back(rk[j]);
                m.reacOrder.push_back(rord[j]);
                m.reacNu.push_back(rnu[j]);
            }
            m.reacPtr.push_back((int)m.reacK.size());
            m.reacBucket.push_back(bucketOf(rnu, rord));
            if (m.prodPtr.empty()) m.prodPtr.push_back(0);
            for (size_t j = 0; j < pk.size(); j++) {
                m.prodK.push_back(pk[j]);
                m.prodNu.push_back(pnu[j]);
            }
            m.prodPtr.push_back((int)m.prodK.size());
            m.prodBucket.push_back(bucketOf(pnu, pnu));
        }
    }
    if (m.reacPtr.empty()) m.reacPtr.push_back(0);
    if (m.prodPtr.empty()) m.prodPtr.push_back(0);
    if (m.tbPtr.empty()) m.tbPtr.push_back(0);
    return m;
}

void equivalenceRatioMassFractions(const Mechanism& m, double phi, const double* fuelX,
                                   const double* oxX, double* Y) {
    if (phi < 0.0) throw std::runtime_error("equivalence ratio phi must be >= 0");
    const int K = m.K, E = (int)m.elementNames.size();
    auto toMass = [&](const double* X, std::vector<double>& y) {
        double s = 0.0;
        for (int k = 0; k < K; k++) s += X[k] * m.mw[k];
        if (!(s > 0.0)) throw std::runtime_error("empty fuel or oxidizer composition");
        for (int k = 0; k < K; k++) y[k] = X[k] * m.mw[k] / s;
    };
    std::vector<double> fuel(K), ox(K);
    toMass(fuelX, fuel);
    toMass(oxX, ox);
    auto eidx = [&](const char* e) {
        for (int i = 0; i < E; i++)
            if (m.elementNames[i] == e) return i;
        return -1;
    };
    const int iC = eidx("C"), iS = eidx("S"), iH = eidx("H"), iO = eidx("O");
    if (iO < 0) throw std::runtime_error("equivalence ratio needs element O");
    // O2 needed (per unit mass) to oxidise C -> CO2, S -> SO2, H -> H2O, minus O2 present
    auto o2need = [&](const std::vector<double>& y) {
        double req = 0.0, pres = 0.0, sum = 0.0;
        for (int k = 0; k < K; k++) {
            sum += y[k];
            double x = y[k] / m.mw[k];
            const double* a = &m.atoms[(size_t)k * E];
            if (iC >= 0) req += x * a[iC];
            if (iS >= 0) req += x * a[iS];
            if (iH >= 0) req += x * 0.25 * a[iH];
            pres += x * a[iO];
        }
        return req / sum - 0.5 * pres / sum;
    };
    double of = o2need(fuel), oo = o2need(ox);
    if (of < 0.0 || oo > 0.0)
        throw std::runtime_error("fuel contains too much oxygen or oxidizer contains not enough");
    double afr = of / (-oo);
    double sf = 0.0, so = 0.0, tot = 0.0;
    for (int k = 0; k < K; k++) { sf += fuel[k]; so += ox[k]; }
    for (int k = 0; k < K; k++) { Y[k] = phi * fuel[k] / sf + afr * ox[k] / so; tot += Y[k]; }
    for (int k = 0; k < K; k++) Y[k] /= tot;
}

std::vector<int32_t> preconditionerOrdering(const Mechanism& m) {
    const int K = m.K, N = K + 1;
    std::vector<int32_t> cp, ri;
    jacobianPattern(m, cp, ri);
    // symmetric structure of Jp + Jp^T over z = [T, n_1..n_K]: the species block's pattern, the
    // dense T row and column
    std::vector<std::vector<char>> adj(N, std::vector<char>(N, 0));
    for (int i = 1; i < N; i++) adj[0][i] = adj[i][0] = 1;
    for (int c = 0; c < K; c++)
        for (int q = cp[c]; q < cp[c + 1]; q++) {
            const int r = ri[q];
            if (r != c) adj[1 + r][1 + c] = adj[1 + c][1 + r] = 1;
        }
    // greedy minimum degree: eliminate the remaining node of least degree (ties: the lowest
    // index), joining its remaining neighbours into a clique (the fill its elimination makes)
    std::vector<char> alive(N, 1);
    std::vector<int32_t> order;
    order.reserve(N);
    for (int step = 0; step < N; step++) {
        int best = -1, bestDeg = N + 1;
        for (int v = 0; v < N; v++) {
            if (!alive[v]) continue;
            int d = 0;
            for (int u = 0; u < N; u++) d += alive[u] && adj[v][u];
            if (d < bestDeg) { bestDeg = d; best = v; }
        }
        std::vector<int> nb;
        for (int u = 0; u < N; u++)
            if (alive[u] && adj[best][u]) nb.push_back(u);
        for (int a : nb)
            for (int b : nb)
                if (a != b) adj[a][b] = 1;
        alive[best] = 0;
        order.push_back(best);
    }
    return order;
}

void jacobianPattern(const Mechanism& m, std::vector<int32_t>& colPtr, std::vector<int32_t>& rowIdx) {
    std::vector<std::set<int>> cols(m.K);
    for (int i = 0; i < m.R; i++) {
        std::set<int> rows, deps;
        for (int j = m.reacPtr[i]; j < m.reacPtr[i + 1]; j++) {
            if (m.reacNu[j] != 0.0) rows.insert(m.reacK[j]);
            deps.insert(m.reacK[j]);
        }
        for (int j = m.prodPtr[i]; j < m.prodPtr[i + 1]; j++) {
            rows.insert(m.prodK[j]);
            if (m.reversible[i]) deps.insert(m.prodK[j]);
        }
        int t = m.tbOfRxn[i];
        if (t >= 0) {
            if (m.tbDefault[t] != 0.0) {
                for (int k = 0; k < m.K; k++) deps.insert(k);
            } else {
                for (int j = m.tbPtr[t]; j < m.tbPtr[t + 1]; j++) deps.insert(m.tbSpecies[j]);
            }
        }
        for (int c : deps)
            for (int r : rows) cols[c].insert(r);
    }
    colPtr.assign(1, 0);
    rowIdx.clear();
    for (int c = 0; c < m.K; c++) {
        for (int r : cols[c]) rowIdx.push_back(r);
        colPtr.push_back((int32_t)rowIdx.size());
    }
}

}  // namespace gbchem
