// mc_xml.cpp -- see mc_xml.h.
#include "mc_xml.h"

#include <cstdlib>
#include <cstring>

namespace mc {

const std::string *XmlNode::attr(const char *key) const
{
    for (const auto &a : attrs)
        if (a.first == key) return &a.second;
    return nullptr;
}

const XmlNode *XmlNode::child(const char *nm) const
{
    for (const auto &c : children)
        if (c.name == nm) return &c;
    return nullptr;
}

double XmlNode::as_double(const char *key, double def) const
{
    const std::string *v = attr(key);
    if (!v) return def;
    return std::strtod(v->c_str(), nullptr);
}

long XmlNode::as_int(const char *key, long def) const
{
    const std::string *v = attr(key);
    if (!v) return def;
    return std::strtol(v->c_str(), nullptr, 10);
}

std::string XmlNode::as_string(const char *key, const char *def) const
{
    const std::string *v = attr(key);
    return v ? *v : std::string(def);
}

namespace {

struct Parser {
    const std::string &s;
    size_t i = 0;
    std::string err;

    explicit Parser(const std::string &text) : s(text) {}

    bool eof() const { return i >= s.size(); }
    static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }
    static bool namech(char c)
    {
        return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') ||
               c == '_' || c == '-' || c == '.' || c == ':';
    }
    void skip_space() { while (!eof() && space(s[i])) ++i; }
    bool starts(const char *lit) const { return s.compare(i, std::strlen(lit), lit) == 0; }

    bool skip_until(const char *lit)
    {
        size_t p = s.find(lit, i);
        if (p == std::string::npos) { err = std::string("unterminated markup, expected ") + lit; return false; }
        i = p + std::strlen(lit);
        return true;
    }

    static std::string decode(const std::string &v)
    {
        std::string o;
        o.reserve(v.size());
        for (size_t k = 0; k < v.size(); ++k) {
            if (v[k] == '&') {
                static const char *ent[][2] = {{"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"},
                                               {"&quot;", "\""}, {"&apos;", "'"}};
                bool hit = false;
                for (auto &e : ent) {
                    if (v.compare(k, std::strlen(e[0]), e[0]) == 0) {
                        o += e[1];
                        k += std::strlen(e[0]) - 1;
                        hit = true;
                        break;
                    }
                }
                if (!hit) o += v[k];
            } else {
                o += v[k];
            }
        }
        return o;
    }

    // skips text, comments, declarations; stops at '<' of an element or '</'
    bool skip_misc()
    {
        for (;;) {
            while (!eof() && s[i] != '<') ++i;
            if (eof()) return true;
            if (starts("<!--")) { if (!skip_until("-->")) return false; continue; }
            if (starts("<?")) { if (!skip_until("?>")) return false; continue; }
            if (starts("<![CDATA[")) { if (!skip_until("]]>")) return false; continue; }
            if (starts("<!")) { if (!skip_until(">")) return false; continue; }
            return true;
        }
    }

    bool element(XmlNode &n)
    {
        ++i;  // '<'
        size_t b = i;
        while (!eof() && namech(s[i])) ++i;
        if (i == b) { err = "element without a name"; return false; }
        n.name = s.substr(b, i - b);
        for (;;) {
            skip_space();
            if (eof()) { err = "unterminated start tag <" + n.name; return false; }
            if (s[i] == '/') {
                if (i + 1 < s.size() && s[i + 1] == '>') { i += 2; return true; }
                err = "bad '/' in <" + n.name; return false;
            }
            if (s[i] == '>') { ++i; break; }
            size_t ab = i;
            while (!eof() && namech(s[i])) ++i;
            if (i == ab) { err = "bad attribute in <" + n.name; return false; }
            std::string key = s.substr(ab, i - ab);
            skip_space();
            if (eof() || s[i] != '=') { err = "attribute " + key + " without a value"; return false; }
            ++i;
            skip_space();
            if (eof() || (s[i] != '"' && s[i] != '\'')) { err = "unquoted attribute " + key; return false; }
            char q = s[i++];
            size_t ve = s.find(q, i);
            if (ve == std::string::npos) { err = "unterminated attribute " + key; return false; }
            n.attrs.emplace_back(key, decode(s.substr(i, ve - i)));
            i = ve + 1;
        }
        // content
        for (;;) {
            if (!skip_misc()) return false;
            if (eof()) { err = "missing </" + n.name + ">"; return false; }
            if (starts("</")) {
                i += 2;
                size_t b2 = i;
                while (!eof() && namech(s[i])) ++i;
                if (s.compare(b2, i - b2, n.name) != 0) { err = "mismatched </" + s.substr(b2, i - b2) + ">"; return false; }
                skip_space();
                if (eof() || s[i] != '>') { err = "bad end tag"; return false; }
                ++i;
                return true;
            }
            n.children.emplace_back();
            if (!element(n.children.back())) return false;
        }
    }
};

}  // namespace

bool xml_parse(const std::string &text, XmlNode &doc, std::string &err)
{
    Parser p(text);
    doc = XmlNode();
    for (;;) {
        if (!p.skip_misc()) { err = p.err; return false; }
        if (p.eof()) break;
        if (p.starts("</")) { err = "stray end tag"; return false; }
        doc.children.emplace_back();
        if (!p.element(doc.children.back())) { err = p.err; return false; }
    }
    return true;
}

}  // namespace mc
