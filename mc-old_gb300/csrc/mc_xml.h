// mc_xml.h -- a small XML reader for the fixed-source input schema.
//
// The reference reads input.xml with pugixml (src/simulator/setup.cpp:33-35):
// a document whose top level holds several sibling elements, attributes in
// single or double quotes with optional blanks around '=', comments and an
// XML declaration.  This reader builds a DOM of elements and attributes only
// (text, comments, processing instructions and CDATA are skipped), which is
// all the schema uses.
#pragma once

#include <string>
#include <utility>
#include <vector>

namespace mc {

struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlNode> children;

    // attribute value or nullptr
    const std::string *attr(const char *key) const;
    // first child element with this name or nullptr
    const XmlNode *child(const char *name) const;
    // pugixml xml_attribute::as_double / as_int semantics: missing -> def,
    // otherwise strtod / strtol of the leading number (0 if none)
    double as_double(const char *key, double def = 0.0) const;
    long as_int(const char *key, long def = 0) const;
    std::string as_string(const char *key, const char *def = "") const;
};

// Parses text into doc (whose children are the top-level elements).  Returns
// false with a message on malformed input.
bool xml_parse(const std::string &text, XmlNode &doc, std::string &err);

}  // namespace mc
