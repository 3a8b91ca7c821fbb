// A reader for the subset of YAML that Ajisai scene files use (the
// reference parses them with yaml-cpp, factory/creator/*.cpp): block
// mappings and sequences by indentation, flow sequences [..] and flow
// mappings {..} (also across lines), plain / single- / double-quoted
// scalars, comments, a leading "---".  Anchors, tags, multi-document
// streams and block scalars (| >) are not supported and raise an error.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ajh {

struct YamlError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class Node {
 public:
  enum Kind { kUndefined, kNull, kScalar, kSequence, kMap };

  Kind kind = kUndefined;
  std::string scalar;
  std::vector<Node> items;                          // sequence
  std::vector<std::pair<std::string, Node>> entries;  // mapping, in order
  int line = 0;  // 1-based source line (0: synthesised)

  bool IsDefined() const { return kind != kUndefined; }
  bool IsNull() const { return kind == kNull; }
  bool IsScalar() const { return kind == kScalar; }
  bool IsSequence() const { return kind == kSequence; }
  bool IsMap() const { return kind == kMap; }
  explicit operator bool() const { return IsDefined() && !IsNull(); }
  size_t size() const {
    return kind == kSequence ? items.size()
                             : (kind == kMap ? entries.size() : 0);
  }

  // A missing key or index gives an undefined node (like yaml-cpp).
  const Node& operator[](const std::string& key) const;
  const Node& operator[](size_t i) const;

  // Conversions; throw YamlError naming the line on a mismatch.
  std::string AsString() const;
  double AsDouble() const;
  float AsFloat() const;  // decimal straight to float, as yaml-cpp reads it
  int64_t AsInt() const;
  bool AsBool() const;
  std::vector<float> AsFloats(size_t n) const;  // a sequence of n numbers

  std::string AsString(const std::string& def) const {
    return IsDefined() ? AsString() : def;
  }
  float AsFloat(float def) const { return IsDefined() ? AsFloat() : def; }
  int64_t AsInt(int64_t def) const { return IsDefined() ? AsInt() : def; }
  bool AsBool(bool def) const { return IsDefined() ? AsBool() : def; }
};

Node ParseYaml(const std::string& text);
Node LoadYamlFile(const std::string& path);

}  // namespace ajh
