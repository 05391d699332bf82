// yaml_lite.cpp - see yaml_lite.h.  Line-oriented block parser plus a recursive
// flow-collection parser.  Errors carry the 1-based source line.
#include "yaml_lite.h"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace gbchem {

namespace {

struct LLine {
    int indent;        // column of first non-space character
    std::string text;  // comment-stripped, right-trimmed content (flow continuations joined)
    int lineno;
    bool isBlockScalar = false;  // text holds the literal payload of a block scalar value
    std::string blockKey;        // "key" (or "-" for a sequence item) owning the payload
};

std::string rtrim(const std::string& s) {
    size_t e = s.find_last_not_of(" \t\r");
    return e == std::string::npos ? std::string() : s.substr(0, e + 1);
}
std::string trim(const std::string& s) {
    size_t b = s.find_first_not_of(" \t\r");
    if (b == std::string::npos) return std::string();
    size_t e = s.find_last_not_of(" \t\r");
    return s.substr(b, e - b + 1);
}

// Remove a trailing comment: '#' at line start or preceded by whitespace, outside quotes.
std::string stripComment(const std::string& s) {
    char q = 0;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (q) {
            if (c == q) {
                if (q == '\'' && i + 1 < s.size() && s[i + 1] == '\'') { i++; continue; }
                q = 0;
            } else if (q == '"' && c == '\\') {
                i++;
            }
            continue;
        }
        if ((c == '\'' || c == '"')) {
            // a quote only opens a quoted scalar at a token start
            if (i == 0 || std::isspace((unsigned char)s[i - 1]) || s[i - 1] == '[' ||
                s[i - 1] == '{' || s[i - 1] == ',' || s[i - 1] == ':' || s[i - 1] == '-') {
                q = c;
            }
            continue;
        }
        if (c == '#' && (i == 0 || std::isspace((unsigned char)s[i - 1]))) return s.substr(0, i);
    }
    return s;
}

// Net bracket depth of a string, ignoring quoted text.
int bracketBalance(const std::string& s) {
    int depth = 0;
    char q = 0;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (q) {
            if (c == q) q = 0;
            continue;
        }
        if (c == '\'' || c == '"') {
            if (i == 0 || std::isspace((unsigned char)s[i - 1]) || s[i - 1] == '[' ||
                s[i - 1] == '{' || s[i - 1] == ',' || s[i - 1] == ':')
                q = c;
            continue;
        }
        if (c == '[' || c == '{') depth++;
        if (c == ']' || c == '}') depth--;
    }
    return depth;
}

int indentOf(const std::string& s) {
    int n = 0;
    while (n < (int)s.size() && s[n] == ' ') n++;
    return n;
}

// Find the "key: value" separator (a ':' followed by space or end of text) outside
// quotes and brackets.  Returns npos if the text is not a mapping entry.
size_t findKeySep(const std::string& s) {
    char q = 0;
    int depth = 0;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (q) {
            if (c == q) q = 0;
            continue;
        }
        if ((c == '\'' || c == '"') && (i == 0)) { q = c; continue; }
        if (c == '[' || c == '{') depth++;
        else if (c == ']' || c == '}') depth--;
        else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t'))
            return i;
    }
    return std::string::npos;
}

std::string unquote(const std::string& s, int line) {
    if (s.size() >= 2 && s.front() == '\'' && s.back() == '\'') {
        std::string out;
        for (size_t i = 1; i + 1 < s.size(); i++) {
            out += s[i];
            if (s[i] == '\'' && i + 2 < s.size() && s[i + 1] == '\'') i++;
        }
        return out;
    }
    if (s.size() >= 2 && s.front() == '"' && s.back() == '"') {
        std::string out;
        for (size_t i = 1; i + 1 < s.size(); i++) {
            if (s[i] == '\\' && i + 2 < s.size()) {
                char n = s[++i];
                out += (n == 'n') ? '\n' : (n == 't') ? '\t' : n;
            } else {
                out += s[i];
            }
        }
        return out;
    }
    (void)line;
    return s;
}

class FlowParser {
public:
    FlowParser(const std::string& s, int line) : s_(s), line_(line) {}
    YNode parseValue() {
        skipWs();
        if (p_ >= s_.size()) return scalar("");
        char c = s_[p_];
        if (c == '[') return parseSeq();
        if (c == '{') return parseMap();
        return scalar(parsePlainOrQuoted(false));
    }
    void expectEnd() {
        skipWs();
        if (p_ != s_.size()) fail("trailing characters in flow collection");
    }

private:
    const std::string& s_;
    size_t p_ = 0;
    int line_;
    [[noreturn]] void fail(const std::string& m) {
        throw YamlError("YAML line " + std::to_string(line_) + ": " + m + " in '" + s_ + "'");
    }
    void skipWs() {
        while (p_ < s_.size() && std::isspace((unsigned char)s_[p_])) p_++;
    }
    YNode scalar(const std::string& t) {
        YNode n;
        n.kind = YNode::Scalar;
        n.text = t;
        n.line = line_;
        return n;
    }
    std::string parsePlainOrQuoted(bool isKey) {
        skipWs();
        if (p_ < s_.size() && (s_[p_] == '\'' || s_[p_] == '"')) {
            char q = s_[p_];
            size_t b = p_++;
            while (p_ < s_.size()) {
                if (s_[p_] == q) {
                    if (q == '\'' && p_ + 1 < s_.size() && s_[p_ + 1] == '\'') { p_ += 2; continue; }
                    break;
                }
                if (q == '"' && s_[p_] == '\\') p_++;
                p_++;
            }
            if (p_ >= s_.size()) fail("unterminated quoted scalar");
            p_++;
            return unquote(s_.substr(b, p_ - b), line_);
        }
        size_t b = p_;
        while (p_ < s_.size()) {
            char c = s_[p_];
            if (c == ',' || c == ']' || c == '}') break;
            if (isKey && c == ':' && (p_ + 1 == s_.size() || s_[p_ + 1] == ' ')) break;
            p_++;
        }
        return trim(s_.substr(b, p_ - b));
    }
    YNode parseSeq() {
        YNode n;
        n.kind = YNode::Seq;
        n.line = line_;
        p_++;  // '['
        skipWs();
        if (p_ < s_.size() && s_[p_] == ']') { p_++; return n; }
        while (true) {
            n.elems.push_back(parseValue());
            skipWs();
            if (p_ >= s_.size()) fail("unterminated flow sequence");
            if (s_[p_] == ',') { p_++; skipWs(); if (p_ < s_.size() && s_[p_] == ']') { p_++; break; } continue; }
            if (s_[p_] == ']') { p_++; break; }
            fail("expected ',' or ']'");
        }
        return n;
    }
    YNode parseMap() {
        YNode n;
        n.kind = YNode::Map;
        n.line = line_;
        p_++;  // '{'
        skipWs();
        if (p_ < s_.size() && s_[p_] == '}') { p_++; return n; }
        while (true) {
            std::string key = parsePlainOrQuoted(true);
            skipWs();
            if (p_ >= s_.size() || s_[p_] != ':') fail("expected ':' in flow mapping");
            p_++;
            YNode v = parseValue();
            n.items.emplace_back(key, std::move(v));
            skipWs();
            if (p_ >= s_.size()) fail("unterminated flow mapping");
            if (s_[p_] == ',') { p_++; skipWs(); if (p_ < s_.size() && s_[p_] == '}') { p_++; break; } continue; }
            if (s_[p_] == '}') { p_++; break; }
            fail("expected ',' or '}'");
        }
        return n;
    }
};

YNode inlineValue(const std::string& raw, int line) {
    std::string s = trim(raw);
    if (!s.empty() && (s[0] == '[' || s[0] == '{')) {
        FlowParser fp(s, line);
        YNode n = fp.parseValue();
        fp.expectEnd();
        return n;
    }
    YNode n;
    n.kind = YNode::Scalar;
    n.text = unquote(s, line);
    n.line = line;
    return n;
}

bool isBlockIndicator(const std::string& v) {
    if (v.empty()) return false;
    if (v[0] != '|' && v[0] != '>') return false;
    for (size_t i = 1; i < v.size(); i++)
        if (!(v[i] == '-' || v[i] == '+' || std::isdigit((unsigned char)v[i]))) return false;
    return true;
}

class BlockParser {
public:
    explicit BlockParser(std::vector<LLine> L) : L_(std::move(L)) {}
    YNode parseDocument() {
        if (L_.empty()) return YNode();
        size_t pos = 0;
        YNode n = parseBlock(pos, L_[0].indent);
        if (pos != L_.size())
            throw YamlError("YAML line " + std::to_string(L_[pos].lineno) + ": unexpected indentation");
        return n;
    }

private:
    std::vector<LLine> L_;
    static bool isSeqLine(const LLine& l) {
        return !l.isBlockScalar && (l.text == "-" || (l.text.size() >= 2 && l.text[0] == '-' && l.text[1] == ' '));
    }
    YNode parseBlock(size_t& pos, int indent) {
        if (isSeqLine(L_[pos])) return parseSeq(pos, indent);
        return parseMap(pos, indent);
    }
    YNode valueAfterKey(size_t& pos, int keyIndent, const std::string& value, int line) {
        // value is empty: nested block follows (deeper, or a sequence at the same indent)
        if (!value.empty()) return inlineValue(value, line);
        if (pos < L_.size() && L_[pos].isBlockScalar) {
            YNode n;
            n.kind = YNode::Scalar;
            n.text = L_[pos].text;
            n.line = L_[pos].lineno;
            pos++;
            return n;
        }
        if (pos < L_.size() && L_[pos].indent > keyIndent) return parseBlock(pos, L_[pos].indent);
        if (pos < L_.size() && L_[pos].indent == keyIndent && isSeqLine(L_[pos])) return parseSeq(pos, keyIndent);
        YNode n;
        n.line = line;
        return n;
    }
    YNode parseSeq(size_t& pos, int indent) {
        YNode n;
        n.kind = YNode::Seq;
        n.line = L_[pos].lineno;
        while (pos < L_.size() && L_[pos].indent == indent && isSeqLine(L_[pos])) {
            LLine& l = L_[pos];
            std::string rest = l.text.size() > 1 ? l.text.substr(1) : std::string();
            int extra = 1 + indentOf(rest);
            rest = trim(rest);
            if (rest.empty()) {
                pos++;
                n.elems.push_back(valueAfterKey(pos, indent, "", l.lineno));
                continue;
            }
            bool startsFlowOrQuote = rest[0] == '[' || rest[0] == '{' || rest[0] == '\'' || rest[0] == '"';
            if (!startsFlowOrQuote && findKeySep(rest) != std::string::npos) {
                // "- key: value" opens a mapping whose keys sit at indent + extra
                l.indent = indent + extra;
                l.text = rest;
                n.elems.push_back(parseMap(pos, l.indent));
            } else if (isSeqLine(LLine{0, rest, 0, false, {}})) {
                l.indent = indent + extra;
                l.text = rest;
                n.elems.push_back(parseSeq(pos, l.indent));
            } else {
                pos++;
                n.elems.push_back(inlineValue(rest, l.lineno));
            }
        }
        return n;
    }
    YNode parseMap(size_t& pos, int indent) {
        YNode n;
        n.kind = YNode::Map;
        n.line = L_[pos].lineno;
        while (pos < L_.size() && L_[pos].indent == indent && !isSeqLine(L_[pos])) {
            const LLine l = L_[pos];
            if (l.isBlockScalar)
                throw YamlError("YAML line " + std::to_string(l.lineno) + ": stray block scalar");
            size_t sep = findKeySep(l.text);
            if (sep == std::string::npos)
                throw YamlError("YAML line " + std::to_string(l.lineno) + ": expected 'key: value', got '" + l.text + "'");
            std::string key = unquote(trim(l.text.substr(0, sep)), l.lineno);
            std::string value = trim(l.text.substr(sep + 1));
            pos++;
            n.items.emplace_back(key, valueAfterKey(pos, indent, value, l.lineno));
        }
        if (pos < L_.size() && L_[pos].indent > indent)
            throw YamlError("YAML line " + std::to_string(L_[pos].lineno) + ": unexpected indentation");
        return n;
    }
};

std::vector<LLine> logicalLines(const std::string& src) {
    std::vector<std::string> raw;
    {
        std::stringstream ss(src);
        std::string ln;
        while (std::getline(ss, ln)) raw.push_back(ln);
    }
    std::vector<LLine> out;
    for (size_t i = 0; i < raw.size(); i++) {
        std::string t = rtrim(stripComment(raw[i]));
        if (trim(t).empty()) continue;
        if (trim(t) == "---" || trim(t) == "...") continue;
        int ind = indentOf(t);
        std::string body = t.substr(ind);
        // join continuation lines of an unbalanced flow collection
        int bal = bracketBalance(body);
        size_t j = i;
        while (bal > 0 && j + 1 < raw.size()) {
            j++;
            std::string c = trim(stripComment(raw[j]));
            if (c.empty()) continue;
            body += " " + c;
            bal = bracketBalance(body);
        }
        if (bal != 0) throw YamlError("YAML line " + std::to_string(i + 1) + ": unbalanced brackets");
        // a plain scalar value continues on following lines indented deeper than its key
        // (or than its "-"), folded with single spaces
        {
            std::string b2 = body;
            int keyCol = ind;
            if (b2.size() >= 2 && b2[0] == '-' && b2[1] == ' ') {
                size_t off = b2.find_first_not_of(' ', 1);
                if (off != std::string::npos) {
                    keyCol = ind + (int)off;
                    b2 = b2.substr(off);
                }
            }
            size_t ks = findKeySep(b2);
            std::string v = trim(ks != std::string::npos ? b2.substr(ks + 1) : b2);
            const int limit = ks != std::string::npos ? keyCol : ind;
            bool plain = !v.empty() && std::string("[{\"'&*!|>").find(v[0]) == std::string::npos;
            if (plain && j == i) {
                while (j + 1 < raw.size()) {
                    std::string c = rtrim(stripComment(raw[j + 1]));
                    if (trim(c).empty() || indentOf(c) <= limit) break;
                    body += " " + trim(c);
                    j++;
                }
            }
        }
        LLine L{ind, body, (int)i + 1, false, {}};
        out.push_back(L);
        // block scalar indicator at the end of "key: |" or "- |"
        std::string value;
        size_t sep = findKeySep(body);
        if (sep != std::string::npos) value = trim(body.substr(sep + 1));
        else if (body.size() >= 2 && body[0] == '-' && body[1] == ' ') value = trim(body.substr(2));
        if (isBlockIndicator(value)) {
            out.back().text = (sep != std::string::npos) ? body.substr(0, sep + 1) : std::string("-");
            bool folded = value[0] == '>';
            bool keepTrail = value.find('+') != std::string::npos;
            bool strip = value.find('-') != std::string::npos;
            std::vector<std::string> content;
            int bodyIndent = -1;
            size_t k = j + 1;
            for (; k < raw.size(); k++) {
                std::string r = rtrim(raw[k]);
                if (trim(r).empty()) { content.push_back(""); continue; }
                int ri = indentOf(r);
                if (ri <= ind) break;
                if (bodyIndent < 0) bodyIndent = ri;
                content.push_back(r.size() > (size_t)bodyIndent ? r.substr(bodyIndent) : std::string());
            }
            while (!keepTrail && !content.empty() && content.back().empty()) content.pop_back();
            std::string payload;
            for (size_t c = 0; c < content.size(); c++) {
                if (c) payload += folded ? " " : "\n";
                payload += content[c];
            }
            if (!strip && !payload.empty()) payload += "\n";
            LLine B{ind + 1, payload, (int)j + 2, false, {}};
            B.isBlockScalar = true;
            out.push_back(B);
            j = k - 1;
        }
        i = j;
    }
    return out;
}

}  // namespace

bool YNode::has(const std::string& key) const { return find(key) != nullptr; }

const YNode* YNode::find(const std::string& key) const {
    if (kind != Map) return nullptr;
    for (auto& kv : items)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

const YNode& YNode::operator[](const std::string& key) const {
    const YNode* n = find(key);
    if (!n) throw YamlError("YAML line " + std::to_string(line) + ": missing key '" + key + "'");
    return *n;
}

double YNode::asDouble() const {
    if (kind != Scalar) throw YamlError("YAML line " + std::to_string(line) + ": expected a number");
    const char* b = text.c_str();
    char* e = nullptr;
    double v = std::strtod(b, &e);
    if (e == b || trim(std::string(e)) != "")
        throw YamlError("YAML line " + std::to_string(line) + ": cannot convert '" + text + "' to a number");
    return v;
}

std::string YNode::asString() const {
    if (kind != Scalar) throw YamlError("YAML line " + std::to_string(line) + ": expected a scalar");
    return text;
}

bool YNode::asBool() const {
    std::string t = asString();
    if (t == "true" || t == "True" || t == "TRUE" || t == "yes") return true;
    if (t == "false" || t == "False" || t == "FALSE" || t == "no") return false;
    throw YamlError("YAML line " + std::to_string(line) + ": expected a boolean, got '" + t + "'");
}

std::vector<double> YNode::asDoubleVec() const {
    if (kind != Seq) throw YamlError("YAML line " + std::to_string(line) + ": expected a sequence");
    std::vector<double> v;
    for (auto& e : elems) v.push_back(e.asDouble());
    return v;
}

std::vector<std::string> YNode::asStringVec() const {
    if (kind != Seq) throw YamlError("YAML line " + std::to_string(line) + ": expected a sequence");
    std::vector<std::string> v;
    for (auto& e : elems) v.push_back(e.asString());
    return v;
}

std::map<std::string, double> YNode::asDoubleMap() const {
    if (kind != Map) throw YamlError("YAML line " + std::to_string(line) + ": expected a mapping");
    std::map<std::string, double> m;
    for (auto& kv : items) m[kv.first] = kv.second.asDouble();
    return m;
}

YNode yamlParseString(const std::string& src) {
    BlockParser bp(logicalLines(src));
    return bp.parseDocument();
}

YNode yamlParseFile(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw YamlError("cannot open file '" + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    return yamlParseString(ss.str());
}

}  // namespace gbchem
