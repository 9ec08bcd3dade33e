// Minimal XML reader for URDF text: elements, attributes, nesting. Text content,
// comments, processing instructions, DOCTYPE and CDATA are skipped. Entity references
// in attribute values (&lt; &gt; &amp; &quot; &apos;) are decoded.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sgdyn {

struct XmlNode {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XmlNode>> children;

  const std::string* attr(const std::string& k) const {
    for (auto& a : attrs)
      if (a.first == k) return &a.second;
    return nullptr;
  }
  const XmlNode* child(const std::string& n) const {
    for (auto& c : children)
      if (c->name == n) return c.get();
    return nullptr;
  }
};

// Parses a document and returns its root element; throws std::runtime_error on
// malformed input.
std::unique_ptr<XmlNode> parse_xml(const std::string& text);

}  // namespace sgdyn
