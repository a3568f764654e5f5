// Minimal XML DOM for the FVM_TVD task file.
//
// The reference parses task.xml with TinyXML (src/tinyxml/*); this reader covers
// what the task schema uses: elements, attributes, text, comments, the XML
// declaration and the five predefined entities. Attribute numbers are read the
// way TinyXML's TiXmlElement::Attribute(name, double*/int*) reads them (atof /
// atoi semantics).
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace cfd2d {

struct XmlNode {
    std::string name;
    std::string text;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<XmlNode>> children;

    const XmlNode* child(const char* n) const;                        // first child element named n
    std::vector<const XmlNode*> children_named(const char* n) const;  // all, in document order
    const char* attr(const char* n) const;                            // nullptr if absent
};

// Parses a whole document; throws std::runtime_error with a line number on malformed input.
std::unique_ptr<XmlNode> xml_parse(const std::string& doc);
std::unique_ptr<XmlNode> xml_load(const std::string& path);

}  // namespace cfd2d
