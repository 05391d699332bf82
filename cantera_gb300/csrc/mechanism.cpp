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
#include <map>
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

// Unit factors of the file's `units:` block (defaults: m, kmol, s, J/kmol).
struct FileUnits {
    double length = 1.0;     // m per file length unit
    double quantity = 1.0;   // kmol per file quantity unit
    double time = 1.0;       // s per file time unit
    double eaFactor = 1.0;   // J/kmol per file activation-energy unit
    bool eaIsTemperature = false;
};

double lengthFactor(const std::string& u, const std::string& file) {
    if (u == "m") return 1.0;
    if (u == "cm") return 0.01;
    if (u == "mm") return 0.001;
    fail(file, 0, "unsupported length unit '" + u + "'");
}
double quantityFactor(const std::string& u, const std::string& file) {
    if (u == "kmol" || u == "kgmol") return 1.0;
    if (u == "mol" || u == "gmol" || u == "mole") return 1e-3;
    if (u == "molec") return 1.0 / kAvogadro;
    fail(file, 0, "unsupported quantity unit '" + u + "'");
}
double timeFactor(const std::string& u, const std::string& file) {
    if (u == "s") return 1.0;
    if (u == "min") return 60.0;
    if (u == "hr") return 3600.0;
    if (u == "ms") return 0.001;
    fail(file, 0, "unsupported time unit '" + u + "'");
}
// Activation-energy unit "energy/quantity" or "K"; returns J/kmol per unit.
double activationFactor(const std::string& u, bool& isT, const std::string& file) {
    isT = false;
    if (u == "K") { isT = true; return gasConstant(); }
    size_t slash = u.find('/');
    if (slash == std::string::npos) fail(file, 0, "unsupported activation-energy unit '" + u + "'");
    std::string e = u.substr(0, slash), q = u.substr(slash + 1);
    double ef;
    if (e == "J") ef = 1.0;
    else if (e == "kJ") ef = 1000.0;
    else if (e == "cal") ef = 4.184;
    else if (e == "kcal") ef = 4184.0;
    else fail(file, 0, "unsupported energy unit '" + e + "'");
    // Units("cal/mol"): 1 * 4.184 * pow(1e-3, -1)
    return ef * std::pow(quantityFactor(q, file), -1.0);
}

FileUnits readUnits(const YNode& root, const std::string& file) {
    FileUnits fu;
    const YNode* u = root.find("units");
    if (!u) return fu;
    if (const YNode* n = u->find("length")) fu.length = lengthFactor(n->asString(), file);
    if (const YNode* n = u->find("quantity")) fu.quantity = quantityFactor(n->asString(), file);
    if (const YNode* n = u->find("time")) fu.time = timeFactor(n->asString(), file);
    if (const YNode* n = u->find("activation-energy")) {
        fu.eaFactor = activationFactor(n->asString(), fu.eaIsTemperature, file);
    } else {
        // default activation energy unit: energy/quantity of the unit system
        fu.eaFactor = 1.0 / fu.quantity;
    }
    return fu;
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

double convertEa(const YNode& node, const FileUnits& fu, const std::string& file) {
    // Ea given as a number (file units) or as "value unit"
    std::string t = node.asString();
    size_t sp = t.find(' ');
    if (sp == std::string::npos) {
        double v = node.asDouble();
        return v * fu.eaFactor / gasConstant();
    }
    double v = std::stod(t.substr(0, sp));
    bool isT;
    double f = activationFactor(t.substr(sp + 1), isT, file);
    if (isT) return v;
    return v * f / gasConstant();
}

struct Arr { double A, b, EaR; };

Arr readArrhenius(const YNode& node, double order, const FileUnits& fu, const std::string& file) {
    Arr a{};
    if (node.isMap()) {
        a.A = convertRateCoeff(node["A"].asDouble(), order, fu);
        a.b = node["b"].asDouble();
        a.EaR = node.has("Ea") ? convertEa(node["Ea"], fu, file) : 0.0;
    } else if (node.isSeq() && node.elems.size() >= 2) {
        a.A = convertRateCoeff(node.elems[0].asDouble(), order, fu);
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

Mechanism loadMechanism(const std::string& path, const std::string& phaseName) {
    YNode root = yamlParseFile(path);
    Mechanism m;
    m.source = path;
    FileUnits fu = readUnits(root, path);

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
    m.elementNames = (*ph)["elements"].asStringVec();
    for (auto& e : m.elementNames) {
        double w = elementWeight(e);
        if (w < 0) fail(path, ph->line, "unknown element '" + e + "'");
        m.elementWeights.push_back(w);
    }
    const YNode& spList = (*ph)["species"];
    if (!spList.isSeq()) fail(path, spList.line, "phase species must be a list of names");
    m.speciesNames = spList.asStringVec();
    m.K = (int)m.speciesNames.size();

    // ---- species data ----
    const YNode& species = root["species"];
    std::map<std::string, const YNode*> spNode;
    for (auto& s : species.elems) spNode[s["name"].asString()] = &s;
    const int E = (int)m.elementNames.size();
    m.atoms.assign((size_t)m.K * E, 0.0);
    bool prefSet = false;
    for (int k = 0; k < m.K; k++) {
        auto it = spNode.find(m.speciesNames[k]);
        if (it == spNode.end()) fail(path, spList.line, "species '" + m.speciesNames[k] + "' not defined");
        const YNode& s = *it->second;
        auto comp = s["composition"].asDoubleMap();
        double w = 0.0;
        for (auto& kv : comp) {  // element-name order, as the reference's Composition map
            double ew = elementWeight(kv.first);
            if (ew < 0) fail(path, s.line, "unknown element '" + kv.first + "'");
            w += ew * kv.second;
            auto e = std::find(m.elementNames.begin(), m.elementNames.end(), kv.first);
            if (e == m.elementNames.end())
                fail(path, s.line, "species '" + m.speciesNames[k] + "' uses undeclared element '" + kv.first + "'");
            m.atoms[(size_t)k * E + (e - m.elementNames.begin())] = kv.second;
        }
        m.mw.push_back(w);
        const YNode& th = s["thermo"];
        if (th["model"].asString() != "NASA7")
            fail(path, th.line, "species '" + m.speciesNames[k] + "': only NASA7 thermo is supported");
        std::vector<double> tr = th["temperature-ranges"].asDoubleVec();
        const YNode& data = th["data"];
        if (tr.size() < 2 || tr.size() > 3 || data.elems.size() != tr.size() - 1)
            fail(path, th.line, "bad NASA7 temperature ranges / data");
        std::vector<double> lo = data.elems[0].asDoubleVec();
        std::vector<double> hi = tr.size() == 3 ? data.elems[1].asDoubleVec() : lo;
        if (lo.size() != 7 || hi.size() != 7) fail(path, th.line, "NASA7 polynomials need 7 coefficients");
        double pref = kOneAtm;
        if (const YNode* p = th.find("reference-pressure")) pref = p->asDouble();
        if (prefSet && pref != m.Pref) fail(path, th.line, "species reference pressures differ");
        m.Pref = pref;
        prefSet = true;
        m.Tmin.push_back(tr.front());
        m.Tmax.push_back(tr.back());
        m.nasaTmid.push_back(tr.size() == 3 ? tr[1] : tr.back());
        for (int j = 0; j < 7; j++) m.nasaLow.push_back(lo[j]);
        for (int j = 0; j < 7; j++) m.nasaHigh.push_back(hi[j]);
    }

    // ---- reactions ----
    std::string rxnKey = "reactions";
    if (const YNode* rk = ph->find("reactions")) {
        if (rk->isScalar()) {
            std::string v = rk->asString();
            if (v == "none") rxnKey = "";
            else if (v != "all" && v != "declared-species") rxnKey = v;
        } else {
            fail(path, rk->line, "only a single reaction section is supported");
        }
    }
    if (!rxnKey.empty()) {
        const YNode& rxns = root[rxnKey];
        for (auto& rn : rxns.elems) {
            const std::string eq = rn["equation"].asString();
            std::string type = rn.has("type") ? rn["type"].asString() : std::string();
            ParsedReaction pr;
            parseEquation(eq, pr, path, rn.line);
            detectThirdBody(rn, type, pr, path);
            // ThirdBody::setParameters
            if (pr.hasThirdBody) {
                if (const YNode* d = rn.find("default-efficiency")) {
                    double v = d->asDouble();
                    if (pr.tbName != "M" && v != 0.0)
                        fail(path, rn.line, "invalid default efficiency for explicit collider in '" + eq + "'");
                    pr.tbDefault = v;
                }
                if (const YNode* e = rn.find("efficiencies")) pr.tbEff = e->asDoubleMap();
                if (pr.tbName != "M" && (pr.tbEff.size() != 1 || pr.tbEff.begin()->first != pr.tbName))
                    fail(path, rn.line, "incompatible third-body collider definitions in '" + eq + "'");
            } else if (rn.has("efficiencies") || rn.has("default-efficiency")) {
                fail(path, rn.line, "reaction '" + eq + "' gives efficiencies but has no third body");
            }
            std::map<std::string, double> orders;
            if (const YNode* o = rn.find("orders")) orders = o->asDoubleMap();
            if (pr.reversible && !orders.empty())
                fail(path, rn.line, "reaction orders may only be given for irreversible reactions");

            // rate kind
            int kindv;
            bool falloff = false;
            if (type.empty() || type == "elementary" || type == "Arrhenius") kindv = pr.hasThirdBody ? kThreeBody : kArrhenius;
            else if (type == "three-body" || type == "three-body-Arrhenius") kindv = kThreeBody;
            else if (type == "falloff") { falloff = true; kindv = rn.has("Troe") ? kTroe : kLindemann; }
            else fail(path, rn.line, "unsupported reaction type '" + type + "' for '" + eq + "'");
            if (falloff && rn.has("SRI")) fail(path, rn.line, "SRI falloff is not supported");
            if (falloff && rn.has("Tsang")) fail(path, rn.line, "Tsang falloff is not supported");
            if (kindv == kThreeBody && !pr.hasThirdBody)
                fail(path, rn.line, "three-body reaction '" + eq + "' has no collider");
            if (falloff) {
                if (!pr.hasThirdBody) fail(path, rn.line, "falloff reaction '" + eq + "' lacks a (+M) collider");
                if (pr.tbMassAction) fail(path, rn.line, "falloff collider of '" + eq + "' must use '(+M)'");
            } else if (pr.hasThirdBody && !pr.tbMassAction) {
                fail(path, rn.line, "'(+M)' collider used in non-falloff reaction '" + eq + "'");
            }

            // species indices
            std::vector<int32_t> rk, pk;
            std::vector<double> rnu, pnu, rord;
            for (auto& kv : pr.reactants) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(path, rn.line, "undeclared species '" + kv.first + "' in '" + eq + "'");
                rk.push_back(k);
                rnu.push_back(kv.second);
            }
            for (auto& kv : pr.products) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(path, rn.line, "undeclared species '" + kv.first + "' in '" + eq + "'");
                pk.push_back(k);
                pnu.push_back(kv.second);
            }
            rord = rnu;
            for (auto& kv : orders) {
                int k = m.speciesIndex(kv.first);
                if (k < 0) fail(path, rn.line, "order given for undeclared species '" + kv.first + "'");
                auto at = std::find(rk.begin(), rk.end(), k);
                if (at != rk.end()) {
                    rord[at - rk.begin()] = kv.second;
                } else {
                    if (!rn.has("nonreactant-orders") || !rn["nonreactant-orders"].asBool())
                        fail(path, rn.line, "order given for non-reactant '" + kv.first + "'");
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
            m.reversible.push_back(pr.reversible ? 1 : 0);
            m.duplicate.push_back(rn.has("duplicate") && rn["duplicate"].asBool() ? 1 : 0);
            m.dn.push_back(dnv);
            double troe[4] = {0.0, 0.0, 0.0, 0.0};
            if (falloff) {
                Arr hi = readArrhenius(rn["high-P-rate-constant"], order, fu, path);
                Arr lo = readArrhenius(rn["low-P-rate-constant"], order + 1.0, fu, path);
                if (hi.A * lo.A < 0) fail(path, rn.line, "falloff A factors differ in sign");
                m.A.push_back(hi.A); m.b.push_back(hi.b); m.EaR.push_back(hi.EaR);
                m.A0.push_back(lo.A); m.b0.push_back(lo.b); m.Ea0R.push_back(lo.EaR);
                if (kindv == kTroe) {
                    const YNode& t = rn["Troe"];
                    double a = t["A"].asDouble(), T3 = t["T3"].asDouble(), T1 = t["T1"].asDouble();
                    troe[0] = a;
                    troe[1] = std::fabs(T3) < kSmallNumber ? INFINITY : 1.0 / T3;
                    troe[2] = std::fabs(T1) < kSmallNumber ? INFINITY : 1.0 / T1;
                    troe[3] = t.has("T2") ? t["T2"].asDouble() : 0.0;
                }
            } else {
                double ord = order + ((kindv == kThreeBody) ? 1.0 : 0.0);
                Arr a = readArrhenius(rn["rate-constant"], ord, fu, path);
                if (a.A < 0 && !(rn.has("negative-A") && rn["negative-A"].asBool()))
                    fail(path, rn.line, "negative pre-exponential factor in '" + eq + "'");
                m.A.push_back(a.A); m.b.push_back(a.b); m.EaR.push_back(a.EaR);
                m.A0.push_back(0.0); m.b0.push_back(0.0); m.Ea0R.push_back(0.0);
            }
            for (int j = 0; j < 4; j++) m.troe.push_back(troe[j]);

            // third-body table
            if (pr.hasThirdBody) {
                m.tbOfRxn.push_back((int)m.tbRxn.size());
                m.tbRxn.push_back(irxn);
                m.tbDefault.push_back(pr.tbDefault);
                m.tbMassAction.push_back(pr.tbMassAction ? 1 : 0);
                std::map<int, double> effByIndex;   // ascending species index
                for (auto& kv : pr.tbEff) {
                    int k = m.speciesIndex(kv.first);
                    if (k < 0) fail(path, rn.line, "third-body efficiency for undeclared species '" + kv.first + "'");
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
