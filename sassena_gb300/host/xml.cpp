#include "xml.hpp"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace sassgpu {

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}

namespace {

std::string decode_entities(const std::string& s) {
    std::string out;
    out.reserve(s.size());
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] != '&') {
            out.push_back(s[i]);
            continue;
        }
        size_t semi = s.find(';', i);
        if (semi == std::string::npos) throw XmlError("unterminated entity");
        std::string ent = s.substr(i + 1, semi - i - 1);
        if (ent == "lt") out.push_back('<');
        else if (ent == "gt") out.push_back('>');
        else if (ent == "amp") out.push_back('&');
        else if (ent == "quot") out.push_back('"');
        else if (ent == "apos") out.push_back('\'');
        else if (!ent.empty() && ent[0] == '#') {
            long v = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')
                         ? std::strtol(ent.c_str() + 2, nullptr, 16)
                         : std::strtol(ent.c_str() + 1, nullptr, 10);
            if (v < 0 || v > 127) throw XmlError("non-ASCII character reference &" + ent + ";");
            out.push_back((char)v);
        } else {
            throw XmlError("unknown entity &" + ent + ";");
        }
        i = semi;
    }
    return out;
}

struct Parser {
    const std::string& s;
    size_t i = 0;
    explicit Parser(const std::string& str) : s(str) {}

    [[noreturn]] void fail(const std::string& what) {
        size_t line = 1;
        for (size_t k = 0; k < i && k < s.size(); ++k)
            if (s[k] == '\n') ++line;
        throw XmlError("XML parse error at line " + std::to_string(line) + ": " + what);
    }
    bool starts(const char* p) const { return s.compare(i, std::char_traits<char>::length(p), p) == 0; }
    void skip_until(const char* end) {
        size_t k = s.find(end, i);
        if (k == std::string::npos) fail(std::string("missing ") + end);
        i = k + std::char_traits<char>::length(end);
    }
    std::string name() {
        size_t b = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' ||
                                s[i] == '.' || s[i] == ':'))
            ++i;
        if (i == b) fail("expected a name");
        return s.substr(b, i - b);
    }
    void skip_ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }

    // Parse the content of `node` until its end tag (or end of input for the document).
    void content(XmlNode* node, bool document) {
        while (i < s.size()) {
            if (s[i] != '<') {
                size_t k = s.find('<', i);
                if (k == std::string::npos) k = s.size();
                node->text += decode_entities(s.substr(i, k - i));
                i = k;
                continue;
            }
            if (starts("<!--")) {
                skip_until("-->");
            } else if (starts("<![CDATA[")) {
                i += 9;
                size_t k = s.find("]]>", i);
                if (k == std::string::npos) fail("unterminated CDATA");
                node->text += s.substr(i, k - i);
                i = k + 3;
            } else if (starts("<?")) {
                skip_until("?>");
            } else if (starts("<!")) {
                skip_until(">");
            } else if (starts("</")) {
                if (document) fail("unexpected end tag");
                i += 2;
                std::string n = name();
                if (n != node->name) fail("end tag </" + n + "> does not match <" + node->name + ">");
                skip_ws();
                if (i >= s.size() || s[i] != '>') fail("expected '>'");
                ++i;
                return;
            } else {
                ++i;
                auto child = std::make_unique<XmlNode>();
                child->name = name();
                child->parent = node;
                bool self_closing = false;
                for (;;) {  // attributes are accepted and ignored (the configs use elements)
                    skip_ws();
                    if (i >= s.size()) fail("unterminated start tag");
                    if (s[i] == '>') {
                        ++i;
                        break;
                    }
                    if (starts("/>")) {
                        i += 2;
                        self_closing = true;
                        break;
                    }
                    name();
                    skip_ws();
                    if (i >= s.size() || s[i] != '=') fail("expected '=' in attribute");
                    ++i;
                    skip_ws();
                    if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) fail("expected quote");
                    char q = s[i++];
                    size_t k = s.find(q, i);
                    if (k == std::string::npos) fail("unterminated attribute value");
                    i = k + 1;
                }
                XmlNode* raw = child.get();
                node->children.push_back(std::move(child));
                if (!self_closing) content(raw, false);
            }
        }
        if (!document) fail("missing end tag for <" + node->name + ">");
    }
};

void collect_descendants(const XmlNode* n, const std::string& name, std::vector<const XmlNode*>& out) {
    for (const auto& c : n->children) {
        if (c->name == name) out.push_back(c.get());
        collect_descendants(c.get(), name, out);
    }
}

std::vector<std::string> split_path(const std::string& p) {
    std::vector<std::string> parts;
    std::string cur;
    for (char c : p) {
        if (c == '/') {
            if (!cur.empty()) parts.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(c);
        }
    }
    if (!cur.empty()) parts.push_back(cur);
    return parts;
}

}  // namespace

XmlDoc XmlDoc::parse(const std::string& content) {
    XmlDoc d;
    d.root_ = std::make_unique<XmlNode>();
    d.root_->name = "#document";
    Parser p(content);
    p.content(d.root_.get(), true);
    return d;
}

XmlDoc XmlDoc::load(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw XmlError("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse(ss.str());
}

std::vector<const XmlNode*> XmlDoc::query(const std::string& path, const XmlNode* ctx) const {
    std::vector<const XmlNode*> cur;
    std::vector<std::string> parts;
    if (path.rfind("//", 0) == 0) {
        parts = split_path(path.substr(2));
        if (parts.empty()) return cur;
        collect_descendants(root_.get(), parts[0], cur);
        parts.erase(parts.begin());
    } else if (!path.empty() && path[0] == '.') {
        if (!ctx) throw XmlError("relative path without a current element: " + path);
        cur.push_back(ctx);
        parts = split_path(path.substr(1));
    } else {
        cur.push_back(root_.get());
        parts = split_path(path);
    }
    for (const std::string& part : parts) {
        std::vector<const XmlNode*> next;
        for (const XmlNode* n : cur)
            for (const auto& c : n->children)
                if (c->name == part) next.push_back(c.get());
        cur.swap(next);
    }
    return cur;
}

bool XmlDoc::exists(const std::string& path, const XmlNode* ctx) const {
    return !query(path, ctx).empty();
}

std::string XmlDoc::get_string(const std::string& path, const XmlNode* ctx) const {
    auto v = query(path, ctx);
    if (v.empty()) throw XmlError("no element matches " + path);
    if (v.size() > 1) throw XmlError("Xpathexp is ambigious, multiple fields matched: " + path);
    return trim(v[0]->text);
}

double XmlDoc::get_double(const std::string& path, const XmlNode* ctx) const {
    std::string t = get_string(path, ctx);
    char* end = nullptr;
    double v = std::strtod(t.c_str(), &end);
    if (t.empty() || *end != '\0') throw XmlError("not a number at " + path + ": '" + t + "'");
    return v;
}

long long XmlDoc::get_long(const std::string& path, const XmlNode* ctx) const {
    std::string t = get_string(path, ctx);
    char* end = nullptr;
    long long v = std::strtoll(t.c_str(), &end, 10);
    if (t.empty() || *end != '\0') throw XmlError("not an integer at " + path + ": '" + t + "'");
    return v;
}

size_t XmlDoc::get_size(const std::string& path, const XmlNode* ctx) const {
    long long v = get_long(path, ctx);
    if (v < 0) throw XmlError("negative value at " + path);
    return (size_t)v;
}

bool XmlDoc::get_bool(const std::string& path, const XmlNode* ctx) const {
    std::string t = get_string(path, ctx);
    std::string u;
    for (char c : t) u.push_back((char)std::toupper((unsigned char)c));
    if (u == "TRUE" || u == "1") return true;
    if (u == "FALSE" || u == "0") return false;
    throw XmlError("not a boolean at " + path + ": '" + t + "'");
}

}  // namespace sassgpu
