// Replacement for the reference's src/XMLDocument.cpp (its only Xerces-C++
// user): loads the document without XSD validation.
// TEST INFRASTRUCTURE ONLY.
#include "XMLDocument.hpp"

#include <stdexcept>
#include <string>

XMLDocument::XMLDocument(const std::filesystem::path& xml_filepath) : doc{ValidateXML(xml_filepath)} {}

pugi::xml_document XMLDocument::ValidateXML(const std::filesystem::path& xml_filepath) {
  pugi::xml_document doc{};
  if (auto result = doc.load_file(xml_filepath.c_str()); !result)
    throw std::runtime_error(xml_filepath.string() + ": " + result.description());
  return doc;
}
