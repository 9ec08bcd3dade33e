#include "xml.h"

#include <cctype>

namespace sgdyn {
namespace {

struct Parser {
  const std::string& s;
  size_t i = 0;

  [[noreturn]] void fail(const char* what) const {
    throw std::runtime_error(std::string("URDF XML parse error: ") + what + " at offset " + std::to_string(i));
  }
  bool starts(const char* p) const { return s.compare(i, std::char_traits<char>::length(p), p) == 0; }
  void skip_ws() {
    while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) i++;
  }
  void skip_until(const char* end) {
    size_t k = s.find(end, i);
    if (k == std::string::npos) fail("unterminated construct");
    i = k + std::char_traits<char>::length(end);
  }
  // Skips text, comments, PIs, DOCTYPE and CDATA until the next element tag.
  void skip_misc() {
    for (;;) {
      while (i < s.size() && s[i] != '<') i++;
      if (i >= s.size()) return;
      if (starts("<!--")) skip_until("-->");
      else if (starts("<?")) skip_until("?>");
      else if (starts("<![CDATA[")) skip_until("]]>");
      else if (starts("<!")) skip_until(">");
      else return;
    }
  }
  std::string read_name() {
    size_t b = i;
    while (i < s.size()) {
      unsigned char c = static_cast<unsigned char>(s[i]);
      if (std::isalnum(c) || c == '_' || c == ':' || c == '-' || c == '.') i++;
      else break;
    }
    if (b == i) fail("expected a name");
    return s.substr(b, i - b);
  }
  static std::string decode(const std::string& v) {
    std::string o;
    for (size_t k = 0; k < v.size(); k++) {
      if (v[k] == '&') {
        size_t e = v.find(';', k);
        if (e != std::string::npos) {
          std::string ent = v.substr(k + 1, e - k - 1);
          const char* rep = nullptr;
          if (ent == "lt") rep = "<";
          else if (ent == "gt") rep = ">";
          else if (ent == "amp") rep = "&";
          else if (ent == "quot") rep = "\"";
          else if (ent == "apos") rep = "'";
          if (rep) {
            o += rep;
            k = e;
            continue;
          }
        }
      }
      o += v[k];
    }
    return o;
  }
  std::unique_ptr<XmlNode> element() {
    if (i >= s.size() || s[i] != '<') fail("expected '<'");
    i++;
    auto n = std::make_unique<XmlNode>();
    n->name = read_name();
    for (;;) {
      skip_ws();
      if (i >= s.size()) fail("unterminated tag");
      if (s[i] == '/') {
        if (i + 1 >= s.size() || s[i + 1] != '>') fail("expected '/>'");
        i += 2;
        return n;
      }
      if (s[i] == '>') {
        i++;
        break;
      }
      std::string k = read_name();
      skip_ws();
      if (i >= s.size() || s[i] != '=') fail("expected '='");
      i++;
      skip_ws();
      if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) fail("expected quoted attribute value");
      char q = s[i++];
      size_t e = s.find(q, i);
      if (e == std::string::npos) fail("unterminated attribute value");
      n->attrs.emplace_back(k, decode(s.substr(i, e - i)));
      i = e + 1;
    }
    for (;;) {
      skip_misc();
      if (i >= s.size()) fail("missing closing tag");
      if (starts("</")) {
        i += 2;
        std::string nm = read_name();
        if (nm != n->name) fail("mismatched closing tag");
        skip_ws();
        if (i >= s.size() || s[i] != '>') fail("expected '>'");
        i++;
        return n;
      }
      n->children.push_back(element());
    }
  }
};

}  // namespace

std::unique_ptr<XmlNode> parse_xml(const std::string& text) {
  Parser p{text};
  p.skip_misc();
  if (p.i >= text.size()) p.fail("no root element");
  return p.element();
}

}  // namespace sgdyn
