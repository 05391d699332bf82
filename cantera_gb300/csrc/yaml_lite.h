// yaml_lite.h - a small YAML-subset reader for Cantera mechanism files.
//
// Cantera reads mechanisms through yaml-cpp (reference: src/base/AnyMap.cpp:1824-1860,
// AnyMap::fromYamlFile -> YAML::Load).  This reader covers the subset that
// Cantera-generated mechanism files use: block mappings and sequences nested by
// indentation (including "- key: value" items and sequences at the same indent as
// their key), flow mappings / sequences that may span lines, comments, single /
// double quoted scalars and literal / folded block scalars ("|", "|-", ">").
// Scalars are kept as text; typed access converts on demand.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gbchem {

struct YamlError : std::runtime_error {
    explicit YamlError(const std::string& m) : std::runtime_error(m) {}
};

class YNode {
public:
    enum Kind { Null, Scalar, Map, Seq };
    Kind kind = Null;
    std::string text;                                   // Scalar
    std::vector<std::pair<std::string, YNode>> items;   // Map (insertion order kept)
    std::vector<YNode> elems;                           // Seq
    int line = 0;                                       // 1-based source line

    bool isMap() const { return kind == Map; }
    bool isSeq() const { return kind == Seq; }
    bool isScalar() const { return kind == Scalar; }
    bool has(const std::string& key) const;
    const YNode& operator[](const std::string& key) const;   // throws if missing
    const YNode* find(const std::string& key) const;          // nullptr if missing
    double asDouble() const;
    std::string asString() const;
    bool asBool() const;
    std::vector<double> asDoubleVec() const;
    std::vector<std::string> asStringVec() const;
    // {name: number, ...} -> ordered map (ordered by key, as std::map does)
    std::map<std::string, double> asDoubleMap() const;
};

YNode yamlParseFile(const std::string& path);
YNode yamlParseString(const std::string& src);

}  // namespace gbchem
