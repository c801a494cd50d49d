// xml.h -- a small XML reader for DOMA's input decks (elements, attributes,
// comments, processing instructions, CDATA and text are accepted; text and
// comments are dropped).  It gives the host layer the lookups DOMA's parser
// makes through pugixml (src/InputParameters.cpp:51-88): child by name,
// attribute by name with a default, iteration over element children.
#pragma once

#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace doma_host {

struct XmlNode {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XmlNode>> children;

  // First child element with this name, or nullptr.
  const XmlNode * child(const std::string & n) const;
  // Attribute value; `found` reports whether it exists.
  std::string attr(const std::string & n, bool * found = nullptr) const;
  bool has_attr(const std::string & n) const;
};

// Parse a whole document; throws std::runtime_error with a line number on
// malformed input.  Returns a synthetic root whose children are the
// top-level elements.
std::unique_ptr<XmlNode> parse_xml(const std::string & text);
std::unique_ptr<XmlNode> parse_xml_file(const std::string & path);

}  // namespace doma_host
