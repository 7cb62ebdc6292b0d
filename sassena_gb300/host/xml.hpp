// Minimal XML reader for Sassena's configuration and database files.
//
// Replaces the libxml2-backed XMLInterface (src/io/xml_interface.cpp) for the
// subset of XPath the reference uses: "//a/b/c" (elements named a anywhere, then
// child path), "./a/b" (relative to the current element) and "." (the current
// element). Values are the element's trimmed text; booleans accept TRUE/FALSE
// (any case) and 0/1 as xml_interface.cpp:15-62 does.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sassgpu {

struct XmlError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct XmlNode {
    std::string name;
    std::string text;  // concatenated character data directly inside this element
    std::vector<std::unique_ptr<XmlNode>> children;
    XmlNode* parent = nullptr;
};

class XmlDoc {
public:
    static XmlDoc parse(const std::string& content);
    static XmlDoc load(const std::string& path);

    const XmlNode* root() const { return root_.get(); }

    // All elements matching `path` ("//a/b", "./a", "."), relative to `ctx` for
    // paths starting with "." (ctx may be null for absolute paths).
    std::vector<const XmlNode*> query(const std::string& path, const XmlNode* ctx = nullptr) const;
    bool exists(const std::string& path, const XmlNode* ctx = nullptr) const;

    // Value of the single element matching `path`; throws if none or ambiguous.
    std::string get_string(const std::string& path, const XmlNode* ctx = nullptr) const;
    double get_double(const std::string& path, const XmlNode* ctx = nullptr) const;
    long long get_long(const std::string& path, const XmlNode* ctx = nullptr) const;
    size_t get_size(const std::string& path, const XmlNode* ctx = nullptr) const;
    bool get_bool(const std::string& path, const XmlNode* ctx = nullptr) const;

private:
    std::unique_ptr<XmlNode> root_;  // synthetic document node; its children are top-level elements
};

std::string trim(const std::string& s);

}  // namespace sassgpu
