// Minimal XML DOM used to read minimc problem files.
//
// minimc reads its input through pugixml after Xerces-C++ schema validation
// (reference src/XMLDocument.cpp:73-90). Neither library is available here, so
// this is a small project-written, non-validating parser that keeps the parts
// of the DOM the input format uses: elements, attributes, character data,
// comments and the <?xml?> prolog are handled; DTDs are not.  Semantic checks
// that the schema would have made are done by the model loader (mc_model.cpp).
#pragma once

#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace mcxml {

struct Node {
  enum class Kind { document, element, pcdata };
  Kind kind = Kind::element;
  std::string name;   // element name; empty for document and pcdata
  std::string value;  // pcdata text
  std::vector<std::pair<std::string, std::string>> attributes;
  std::vector<std::unique_ptr<Node>> children;
  Node* parent = nullptr;

  // first child element with the given name, or nullptr
  const Node* child(const std::string& n) const;
  // attribute value or nullptr
  const std::string* attribute(const std::string& n) const;
  // value of the first pcdata child ("" if none)
  const std::string& child_value() const;
  // child elements in document order
  std::vector<const Node*> elements() const;
  // "/minimc/general/histories"-style path of this node
  std::string path() const;
};

// Parses a complete document. Throws std::runtime_error with a line number on
// malformed input.
std::unique_ptr<Node> parse(const std::string& text);
std::unique_ptr<Node> parse_file(const std::string& path);

}  // namespace mcxml
