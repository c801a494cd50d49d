// xml.cpp -- recursive-descent XML reader (see xml.h).
#include "xml.h"

#include <fstream>
#include <sstream>
#include <stdexcept>

namespace doma_host {

const XmlNode * XmlNode::child(const std::string & n) const
{
  for (const auto & c : children)
    if (c->name == n) return c.get();
  return nullptr;
}

std::string XmlNode::attr(const std::string & n, bool * found) const
{
  for (const auto & a : attrs)
    if (a.first == n) {
      if (found) *found = true;
      return a.second;
    }
  if (found) *found = false;
  return std::string();
}

bool XmlNode::has_attr(const std::string & n) const
{
  bool f = false;
  attr(n, &f);
  return f;
}

namespace {

class Reader {
public:
  explicit Reader(const std::string & t) : s_(t) {}

  std::unique_ptr<XmlNode> document()
  {
    auto root = std::make_unique<XmlNode>();
    root->name = "#document";
    for (;;) {
      skip_misc();
      if (eof()) break;
      if (peek() != '<') fail("text outside the root element");
      root->children.push_back(element());
    }
    return root;
  }

private:
  const std::string & s_;
  size_t p_ = 0;

  bool eof() const { return p_ >= s_.size(); }
  char peek(size_t k = 0) const { return p_ + k < s_.size() ? s_[p_ + k] : '\0'; }
  bool starts(const char * lit) const { return s_.compare(p_, std::char_traits<char>::length(lit), lit) == 0; }

  [[noreturn]] void fail(const std::string & what) const
  {
    size_t line = 1;
    for (size_t i = 0; i < p_ && i < s_.size(); ++i) line += s_[i] == '\n';
    throw std::runtime_error("XML parse error at line " + std::to_string(line) + ": " + what);
  }

  void skip_ws()
  {
    while (!eof() && (peek() == ' ' || peek() == '\t' || peek() == '\n' || peek() == '\r')) ++p_;
  }

  void skip_until(const char * end)
  {
    const size_t e = s_.find(end, p_);
    if (e == std::string::npos) fail(std::string("unterminated construct, expected ") + end);
    p_ = e + std::char_traits<char>::length(end);
  }

  // whitespace, comments, processing instructions and doctype between elements
  void skip_misc()
  {
    for (;;) {
      skip_ws();
      if (starts("<!--")) skip_until("-->");
      else if (starts("<?")) skip_until("?>");
      else if (starts("<!DOCTYPE")) skip_until(">");
      else return;
    }
  }

  static bool name_char(char c)
  {
    return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') ||
           c == '_' || c == '-' || c == '.' || c == ':';
  }

  std::string name()
  {
    const size_t b = p_;
    while (!eof() && name_char(peek())) ++p_;
    if (p_ == b) fail("expected a name");
    return s_.substr(b, p_ - b);
  }

  static std::string decode(const std::string & v)
  {
    std::string out;
    out.reserve(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      if (v[i] != '&') {
        out += v[i];
        continue;
      }
      const size_t e = v.find(';', i);
      if (e == std::string::npos) {
        out += v[i];
        continue;
      }
      const std::string ent = v.substr(i + 1, e - i - 1);
      if (ent == "lt") out += '<';
      else if (ent == "gt") out += '>';
      else if (ent == "amp") out += '&';
      else if (ent == "quot") out += '"';
      else if (ent == "apos") out += '\'';
      else if (!ent.empty() && ent[0] == '#') {
        const long c = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')
                           ? std::strtol(ent.c_str() + 2, nullptr, 16)
                           : std::strtol(ent.c_str() + 1, nullptr, 10);
        out += static_cast<char>(c >= 0 && c < 128 ? c : '?');
      } else {
        out += v.substr(i, e - i + 1);
      }
      i = e;
    }
    return out;
  }

  std::unique_ptr<XmlNode> element()
  {
    if (peek() != '<') fail("expected '<'");
    ++p_;
    auto node = std::make_unique<XmlNode>();
    node->name = name();
    for (;;) {
      skip_ws();
      if (starts("/>")) {
        p_ += 2;
        return node;
      }
      if (peek() == '>') {
        ++p_;
        break;
      }
      std::string an = name();
      skip_ws();
      if (peek() != '=') fail("expected '=' after attribute " + an);
      ++p_;
      skip_ws();
      const char q = peek();
      if (q != '"' && q != '\'') fail("expected a quoted value for attribute " + an);
      ++p_;
      const size_t e = s_.find(q, p_);
      if (e == std::string::npos) fail("unterminated attribute value");
      node->attrs.emplace_back(an, decode(s_.substr(p_, e - p_)));
      p_ = e + 1;
    }
    // content
    for (;;) {
      if (eof()) fail("unterminated element <" + node->name + ">");
      if (starts("<!--")) skip_until("-->");
      else if (starts("<![CDATA[")) skip_until("]]>");
      else if (starts("<?")) skip_until("?>");
      else if (starts("</")) {
        p_ += 2;
        const std::string n = name();
        if (n != node->name) fail("mismatched closing tag </" + n + "> for <" + node->name + ">");
        skip_ws();
        if (peek() != '>') fail("expected '>'");
        ++p_;
        return node;
      } else if (peek() == '<') {
        node->children.push_back(element());
      } else {
        ++p_;  // text content is not used by the schema
      }
    }
  }
};

}  // namespace

std::unique_ptr<XmlNode> parse_xml(const std::string & text)
{
  Reader r(text);
  return r.document();
}

std::unique_ptr<XmlNode> parse_xml_file(const std::string & path)
{
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("Failed to parse " + path + "\nFile was not found");
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_xml(ss.str());
}

}  // namespace doma_host
