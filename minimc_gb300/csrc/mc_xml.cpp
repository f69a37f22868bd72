// Minimal non-validating XML parser (see mc_xml.hpp).
#include "mc_xml.hpp"

#include <cctype>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mcxml {

namespace {

const std::string kEmpty;

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

bool is_name_char(char c) {
  return std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' ||
         c == '.' || c == ':';
}

class Parser {
public:
  explicit Parser(const std::string& t) : s(t) {}

  std::unique_ptr<Node> run() {
    auto doc = std::make_unique<Node>();
    doc->kind = Node::Kind::document;
    skip_misc();
    if (pos >= s.size() || s[pos] != '<') fail("expected root element");
    doc->children.push_back(element(doc.get()));
    skip_misc();
    if (pos != s.size()) fail("content after root element");
    return doc;
  }

private:
  const std::string& s;
  size_t pos = 0;

  [[noreturn]] void fail(const std::string& what) const {
    size_t line = 1;
    for (size_t i = 0; i < pos && i < s.size(); i++) line += s[i] == '\n';
    throw std::runtime_error("XML parse error at line " + std::to_string(line) + ": " + what);
  }

  bool starts(const char* lit) const { return s.compare(pos, std::char_traits<char>::length(lit), lit) == 0; }

  void skip_ws() {
    while (pos < s.size() && is_ws(s[pos])) pos++;
  }

  void skip_until(const char* lit) {
    const size_t at = s.find(lit, pos);
    if (at == std::string::npos) fail(std::string("unterminated construct, expected ") + lit);
    pos = at + std::char_traits<char>::length(lit);
  }

  // whitespace, comments, processing instructions, doctype
  void skip_misc() {
    for (;;) {
      skip_ws();
      if (starts("<?")) skip_until("?>");
      else if (starts("<!--")) skip_until("-->");
      else if (starts("<!DOCTYPE")) skip_until(">");
      else return;
    }
  }

  std::string name() {
    const size_t b = pos;
    while (pos < s.size() && is_name_char(s[pos])) pos++;
    if (b == pos) fail("expected a name");
    return s.substr(b, pos - b);
  }

  std::string unescape(const std::string& raw) {
    std::string out;
    out.reserve(raw.size());
    for (size_t i = 0; i < raw.size(); i++) {
      if (raw[i] != '&') {
        out += raw[i];
        continue;
      }
      const size_t semi = raw.find(';', i);
      if (semi == std::string::npos) fail("unterminated entity");
      const std::string ent = raw.substr(i + 1, semi - i - 1);
      if (ent == "lt") out += '<';
      else if (ent == "gt") out += '>';
      else if (ent == "amp") out += '&';
      else if (ent == "quot") out += '"';
      else if (ent == "apos") out += '\'';
      else if (!ent.empty() && ent[0] == '#') {
        const long code = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')
                              ? std::stol(ent.substr(2), nullptr, 16)
                              : std::stol(ent.substr(1));
        if (code < 0x80) out += static_cast<char>(code);
        else fail("non-ASCII character reference");
      }
      else fail("unknown entity &" + ent + ";");
      i = semi;
    }
    return out;
  }

  std::unique_ptr<Node> element(Node* parent) {
    pos++;  // '<'
    auto node = std::make_unique<Node>();
    node->kind = Node::Kind::element;
    node->parent = parent;
    node->name = name();
    for (;;) {
      skip_ws();
      if (pos >= s.size()) fail("unterminated start tag");
      if (starts("/>")) {
        pos += 2;
        return node;
      }
      if (s[pos] == '>') {
        pos++;
        break;
      }
      std::string an = name();
      skip_ws();
      if (pos >= s.size() || s[pos] != '=') fail("expected '=' after attribute " + an);
      pos++;
      skip_ws();
      if (pos >= s.size() || (s[pos] != '"' && s[pos] != '\'')) fail("expected quoted attribute value");
      const char q = s[pos++];
      const size_t e = s.find(q, pos);
      if (e == std::string::npos) fail("unterminated attribute value");
      node->attributes.emplace_back(an, unescape(s.substr(pos, e - pos)));
      pos = e + 1;
    }
    // content
    std::string text;
    auto flush_text = [&]() {
      bool all_ws = true;
      for (char c : text) all_ws = all_ws && is_ws(c);
      if (!text.empty() && !all_ws) {
        auto pc = std::make_unique<Node>();
        pc->kind = Node::Kind::pcdata;
        pc->parent = node.get();
        pc->value = unescape(text);
        node->children.push_back(std::move(pc));
      }
      text.clear();
    };
    for (;;) {
      if (pos >= s.size()) fail("unterminated element <" + node->name + ">");
      if (starts("</")) {
        flush_text();
        pos += 2;
        const std::string close = name();
        if (close != node->name) fail("mismatched closing tag </" + close + "> for <" + node->name + ">");
        skip_ws();
        if (pos >= s.size() || s[pos] != '>') fail("expected '>'");
        pos++;
        return node;
      }
      if (starts("<!--")) {
        skip_until("-->");
        continue;
      }
      if (starts("<![CDATA[")) {
        pos += 9;
        const size_t e = s.find("]]>", pos);
        if (e == std::string::npos) fail("unterminated CDATA");
        flush_text();
        auto pc = std::make_unique<Node>();
        pc->kind = Node::Kind::pcdata;
        pc->parent = node.get();
        pc->value = s.substr(pos, e - pos);
        node->children.push_back(std::move(pc));
        pos = e + 3;
        continue;
      }
      if (starts("<?")) {
        skip_until("?>");
        continue;
      }
      if (s[pos] == '<') {
        flush_text();
        node->children.push_back(element(node.get()));
        continue;
      }
      text += s[pos++];
    }
  }
};

}  // namespace

const Node* Node::child(const std::string& n) const {
  for (const auto& c : children)
    if (c->kind == Kind::element && c->name == n) return c.get();
  return nullptr;
}

const std::string* Node::attribute(const std::string& n) const {
  for (const auto& a : attributes)
    if (a.first == n) return &a.second;
  return nullptr;
}

const std::string& Node::child_value() const {
  for (const auto& c : children)
    if (c->kind == Kind::pcdata) return c->value;
  return kEmpty;
}

std::vector<const Node*> Node::elements() const {
  std::vector<const Node*> out;
  for (const auto& c : children)
    if (c->kind == Kind::element) out.push_back(c.get());
  return out;
}

std::string Node::path() const {
  if (kind == Kind::document) return "";
  std::string p;
  for (const Node* n = this; n && n->kind != Kind::document; n = n->parent) p = "/" + n->name + p;
  return p;
}

std::unique_ptr<Node> parse(const std::string& text) { return Parser(text).run(); }

std::unique_ptr<Node> parse_file(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("File not found: " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return parse(ss.str());
}

}  // namespace mcxml
