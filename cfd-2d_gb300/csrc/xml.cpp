#include "xml.hpp"

#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace cfd2d {

const XmlNode* XmlNode::child(const char* n) const {
    for (auto& c : children)
        if (c->name == n) return c.get();
    return nullptr;
}

std::vector<const XmlNode*> XmlNode::children_named(const char* n) const {
    std::vector<const XmlNode*> out;
    for (auto& c : children)
        if (c->name == n) out.push_back(c.get());
    return out;
}

const char* XmlNode::attr(const char* n) const {
    for (auto& a : attrs)
        if (a.first == n) return a.second.c_str();
    return nullptr;
}

namespace {

struct Parser {
    const std::string& s;
    size_t i = 0;
    explicit Parser(const std::string& d) : s(d) {}

    [[noreturn]] void fail(const char* what) const {
        int line = 1;
        for (size_t k = 0; k < i && k < s.size(); k++) line += s[k] == '\n';
        throw std::runtime_error(std::string("XML parse error at line ") + std::to_string(line) + ": " + what);
    }
    bool eof() const { return i >= s.size(); }
    bool starts(const char* p) const { return s.compare(i, std::strlen(p), p) == 0; }
    void ws() { while (!eof() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r' || s[i] == '\n')) i++; }
    void skip_past(const char* p) {
        size_t k = s.find(p, i);
        if (k == std::string::npos) fail("unterminated markup");
        i = k + std::strlen(p);
    }
    static bool name_char(char c) {
        return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_' || c == '-' ||
               c == '.' || c == ':';
    }
    std::string name() {
        size_t b = i;
        while (!eof() && name_char(s[i])) i++;
        if (b == i) fail("expected a name");
        return s.substr(b, i - b);
    }
    static std::string decode(const std::string& raw) {
        std::string o;
        for (size_t k = 0; k < raw.size(); k++) {
            if (raw[k] != '&') { o += raw[k]; continue; }
            static const char* ent[][2] = {{"&lt;", "<"}, {"&gt;", ">"}, {"&amp;", "&"}, {"&quot;", "\""}, {"&apos;", "'"}};
            bool hit = false;
            for (auto& e : ent)
                if (raw.compare(k, std::strlen(e[0]), e[0]) == 0) { o += e[1]; k += std::strlen(e[0]) - 1; hit = true; break; }
            if (!hit) o += '&';
        }
        return o;
    }
    void misc() {  // comments, declarations, processing instructions between elements
        for (;;) {
            ws();
            if (starts("<?")) skip_past("?>");
            else if (starts("<!--")) skip_past("-->");
            else if (starts("<!")) skip_past(">");
            else return;
        }
    }
    std::unique_ptr<XmlNode> element() {
        if (eof() || s[i] != '<') fail("expected '<'");
        i++;
        auto n = std::make_unique<XmlNode>();
        n->name = name();
        for (;;) {
            ws();
            if (eof()) fail("unterminated start tag");
            if (starts("/>")) { i += 2; return n; }
            if (s[i] == '>') { i++; break; }
            std::string an = name();
            ws();
            if (eof() || s[i] != '=') fail("expected '=' after attribute name");
            i++;
            ws();
            if (eof() || (s[i] != '"' && s[i] != '\'')) fail("expected quoted attribute value");
            char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) fail("unterminated attribute value");
            n->attrs.emplace_back(an, decode(s.substr(i, e - i)));
            i = e + 1;
        }
        std::string text;
        for (;;) {
            if (eof()) fail("unterminated element");
            if (starts("</")) {
                i += 2;
                std::string en = name();
                if (en != n->name) fail("mismatched end tag");
                ws();
                if (eof() || s[i] != '>') fail("expected '>'");
                i++;
                break;
            }
            if (starts("<!--")) { skip_past("-->"); continue; }
            if (starts("<![CDATA[")) {
                size_t e = s.find("]]>", i);
                if (e == std::string::npos) fail("unterminated CDATA");
                text += s.substr(i + 9, e - i - 9);
                i = e + 3;
                continue;
            }
            if (starts("<?")) { skip_past("?>"); continue; }
            if (s[i] == '<') { n->children.push_back(element()); continue; }
            size_t e = s.find('<', i);
            if (e == std::string::npos) e = s.size();
            text += decode(s.substr(i, e - i));
            i = e;
        }
        // GetText(): the element's text with surrounding whitespace dropped
        size_t b = text.find_first_not_of(" \t\r\n");
        size_t e = text.find_last_not_of(" \t\r\n");
        n->text = b == std::string::npos ? std::string() : text.substr(b, e - b + 1);
        return n;
    }
};

}  // namespace

std::unique_ptr<XmlNode> xml_parse(const std::string& doc) {
    Parser p(doc);
    if (doc.compare(0, 3, "\xEF\xBB\xBF") == 0) p.i = 3;  // UTF-8 byte order mark
    p.misc();
    if (p.eof()) p.fail("no root element");
    // a document node holding the top-level elements, like TiXmlDocument
    auto root = std::make_unique<XmlNode>();
    while (!p.eof()) {
        root->children.push_back(p.element());
        p.misc();
    }
    return root;
}

std::unique_ptr<XmlNode> xml_load(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open '" + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    return xml_parse(ss.str());
}

}  // namespace cfd2d
