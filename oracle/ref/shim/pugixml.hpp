// pugixml-compatible subset over the project's XML DOM (mcxml).
//
// TEST INFRASTRUCTURE ONLY: lets the reference's own sources compile here
// without the pugixml library.  It implements only what the reference
// calls (xml_node::child/attribute/child_value/first_child/next_sibling/
// name/value/parent/root/path/find_child_by_attribute/select_node, node
// iteration, xml_attribute::as_*/empty, xml_document::load_file), with
// pugixml's documented semantics for those calls.  No pugixml source is
// used.
#pragma once

#include "mc_xml.hpp"

#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

namespace pugi {

class xml_attribute {
 public:
  xml_attribute() = default;
  xml_attribute(const std::string* name, const std::string* value) : n_(name), v_(value) {}
  explicit operator bool() const { return v_ != nullptr; }
  bool operator!() const { return v_ == nullptr; }
  bool empty() const { return v_ == nullptr; }
  const char* name() const { return n_ ? n_->c_str() : ""; }
  const char* value() const { return v_ ? v_->c_str() : ""; }
  const char* as_string(const char* def = "") const { return v_ ? v_->c_str() : def; }
  double as_double(double def = 0) const { return v_ ? std::strtod(v_->c_str(), nullptr) : def; }
  float as_float(float def = 0) const { return v_ ? std::strtof(v_->c_str(), nullptr) : def; }
  int as_int(int def = 0) const { return v_ ? static_cast<int>(std::strtol(v_->c_str(), nullptr, 0)) : def; }
  unsigned int as_uint(unsigned int def = 0) const {
    return v_ ? static_cast<unsigned int>(std::strtoul(v_->c_str(), nullptr, 0)) : def;
  }
  unsigned long long as_ullong(unsigned long long def = 0) const {
    return v_ ? std::strtoull(v_->c_str(), nullptr, 0) : def;
  }
  bool as_bool(bool def = false) const {
    if (!v_ || v_->empty()) return def;
    const char c = (*v_)[0];
    return c == '1' || c == 't' || c == 'T' || c == 'y' || c == 'Y';
  }

 private:
  const std::string* n_ = nullptr;
  const std::string* v_ = nullptr;
};

class xml_node;

class xml_node_iterator {
 public:
  xml_node_iterator(const mcxml::Node* parent, size_t i) : p_(parent), i_(i) {}
  xml_node operator*() const;
  xml_node_iterator& operator++() {
    ++i_;
    return *this;
  }
  bool operator!=(const xml_node_iterator& o) const { return i_ != o.i_ || p_ != o.p_; }
  bool operator==(const xml_node_iterator& o) const { return !(*this != o); }

 private:
  const mcxml::Node* p_;
  size_t i_;
};

class xpath_node;

class xml_node {
 public:
  xml_node() = default;
  explicit xml_node(const mcxml::Node* n) : n_(n) {}
  explicit operator bool() const { return n_ != nullptr; }
  bool operator!() const { return n_ == nullptr; }
  bool operator==(const xml_node& o) const { return n_ == o.n_; }
  bool operator!=(const xml_node& o) const { return n_ != o.n_; }
  bool empty() const { return n_ == nullptr; }
  const char* name() const { return n_ && n_->kind == mcxml::Node::Kind::element ? n_->name.c_str() : ""; }
  const char* value() const { return n_ && n_->kind == mcxml::Node::Kind::pcdata ? n_->value.c_str() : ""; }
  xml_node child(const char* name) const {
    if (!n_) return {};
    for (const auto& c : n_->children)
      if (c->kind == mcxml::Node::Kind::element && c->name == name) return xml_node(c.get());
    return {};
  }
  xml_attribute attribute(const char* name) const {
    if (!n_) return {};
    for (const auto& a : n_->attributes)
      if (a.first == name) return xml_attribute(&a.first, &a.second);
    return {};
  }
  const char* child_value() const {
    if (!n_) return "";
    for (const auto& c : n_->children)
      if (c->kind == mcxml::Node::Kind::pcdata) return c->value.c_str();
    return "";
  }
  const char* child_value(const char* name) const { return child(name).child_value(); }
  xml_node first_child() const { return n_ && !n_->children.empty() ? xml_node(n_->children.front().get()) : xml_node(); }
  xml_node next_sibling() const {
    if (!n_ || !n_->parent) return {};
    const auto& sib = n_->parent->children;
    for (size_t i = 0; i + 1 < sib.size(); i++)
      if (sib[i].get() == n_) return xml_node(sib[i + 1].get());
    return {};
  }
  xml_node parent() const { return n_ && n_->parent ? xml_node(n_->parent) : xml_node(); }
  xml_node root() const {
    if (!n_) return {};
    const mcxml::Node* r = n_;
    while (r->parent) r = r->parent;
    return xml_node(r);
  }
  // "/a/b/c" from the document
  std::string path(char delimiter = '/') const {
    if (!n_) return "";
    std::string out;
    for (const mcxml::Node* c = n_; c && c->kind != mcxml::Node::Kind::document; c = c->parent)
      out = std::string(1, delimiter) + c->name + out;
    return out;
  }
  xml_node find_child_by_attribute(const char* attr_name, const char* attr_value) const {
    if (!n_) return {};
    for (const auto& c : n_->children) {
      if (c->kind != mcxml::Node::Kind::element) continue;
      for (const auto& a : c->attributes)
        if (a.first == attr_name && a.second == attr_value) return xml_node(c.get());
    }
    return {};
  }
  // location paths of element names separated by '/' (relative, or from the
  // document with a leading '/'); the first match
  xpath_node select_node(const char* query) const;
  xml_node_iterator begin() const { return xml_node_iterator(n_, 0); }
  xml_node_iterator end() const { return xml_node_iterator(n_, n_ ? n_->children.size() : 0); }
  const mcxml::Node* internal() const { return n_; }

 protected:
  const mcxml::Node* n_ = nullptr;
};

inline xml_node xml_node_iterator::operator*() const { return xml_node(p_->children[i_].get()); }

class xpath_node {
 public:
  xpath_node() = default;
  explicit xpath_node(xml_node n) : n_(n) {}
  xml_node node() const { return n_; }
  explicit operator bool() const { return static_cast<bool>(n_); }

 private:
  xml_node n_;
};

inline xpath_node xml_node::select_node(const char* query) const {
  std::string q(query);
  xml_node cur = *this;
  size_t pos = 0;
  if (!q.empty() && q[0] == '/') {
    cur = root();
    pos = 1;
  }
  while (cur && pos <= q.size()) {
    const size_t next = q.find('/', pos);
    const std::string step = q.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
    if (!step.empty()) cur = cur.child(step.c_str());
    if (next == std::string::npos) break;
    pos = next + 1;
  }
  return xpath_node(cur);
}

struct xml_parse_result {
  bool ok = false;
  std::string message;
  explicit operator bool() const { return ok; }
  const char* description() const { return message.c_str(); }
};

class xml_document : public xml_node {
 public:
  xml_document() = default;
  xml_document(const xml_document&) = delete;
  xml_document(xml_document&& o) noexcept : xml_node(), doc_(std::move(o.doc_)) {
    n_ = doc_.get();
    o.n_ = nullptr;
  }
  xml_parse_result load_file(const char* path) {
    xml_parse_result r;
    try {
      doc_ = mcxml::parse_file(path);
      n_ = doc_.get();
      r.ok = true;
    }
    catch (const std::exception& e) {
      r.message = e.what();
    }
    return r;
  }
  xml_parse_result load_string(const char* text) {
    xml_parse_result r;
    try {
      doc_ = mcxml::parse(text);
      n_ = doc_.get();
      r.ok = true;
    }
    catch (const std::exception& e) {
      r.message = e.what();
    }
    return r;
  }

 private:
  std::unique_ptr<mcxml::Node> doc_;
};

}  // namespace pugi
