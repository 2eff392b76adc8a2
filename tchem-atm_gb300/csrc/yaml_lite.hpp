// Minimal YAML reader for NCAR-format kinetic-model and scenario files.
//
// The reference reads these files with yaml-cpp (src/core/TChem_KineticModelData.cpp:64-78,
// src/core/TChem_AtmosphericChemistry.cpp:440-446). yaml-cpp is not a dependency of this
// engine, so this reader covers the subset of YAML the mechanism files use: block mappings
// and sequences (including sequences indented at the level of their parent key), flow
// sequences and flow mappings, single/double quoted scalars, multi-line plain scalars,
// comments, anchors (&id) and aliases (*id). Mapping order is preserved, which matters
// because species and reactions are numbered in file order.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace tchem_gb {
namespace yaml {

struct Node;
using NodePtr = std::shared_ptr<Node>;

struct Node {
  enum Kind { Null, Scalar, Seq, Map };
  Kind kind = Null;
  std::string scalar;
  std::vector<NodePtr> seq;
  std::vector<std::pair<std::string, NodePtr>> map;

  bool is_null() const { return kind == Null; }
  bool is_scalar() const { return kind == Scalar; }
  bool is_seq() const { return kind == Seq; }
  bool is_map() const { return kind == Map; }

  // Mapping lookup; returns nullptr when the key is absent (yaml-cpp's falsy node).
  const Node* get(const std::string& key) const;
  // Number of children of a sequence or mapping, 0 otherwise (yaml-cpp Node::size()).
  size_t size() const;

  std::string as_string() const;
  double as_double() const;
  long as_int() const;
};

class ParseError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

NodePtr parse_string(const std::string& text);
NodePtr parse_file(const std::string& path);

}  // namespace yaml
}  // namespace tchem_gb
