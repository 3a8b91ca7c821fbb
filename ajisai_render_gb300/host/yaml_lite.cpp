#include "yaml_lite.h"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace ajh {
namespace {

const Node& undefined_node() {
  static const Node n;
  return n;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t')) --b;
  return s.substr(a, b - a);
}

[[noreturn]] void fail(int line, const std::string& what) {
  throw YamlError("YAML line " + std::to_string(line) + ": " + what);
}

struct Line {
  int indent;
  std::string text;
  int no;
};

// Removes a comment (a '#' at the start or after a blank, outside quotes)
// and returns the bracket depth change of the remaining text.
std::string strip_comment(const std::string& s, int* depth) {
  char quote = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (quote) {
      if (c == '\\' && quote == '"' && i + 1 < s.size()) {
        ++i;
      } else if (c == quote) {
        quote = 0;
      }
      continue;
    }
    if (c == '\'' || c == '"') {
      quote = c;
    } else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) {
      return s.substr(0, i);
    } else if (c == '[' || c == '{') {
      ++*depth;
    } else if (c == ']' || c == '}') {
      --*depth;
    }
  }
  return s;
}

std::vector<Line> lex(const std::string& text) {
  std::vector<Line> out;
  std::istringstream in(text);
  std::string raw;
  int no = 0;
  int depth = 0;
  while (std::getline(in, raw)) {
    ++no;
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    int d = 0;
    std::string s = strip_comment(raw, &d);
    // indentation: spaces only
    size_t ind = 0;
    while (ind < s.size() && s[ind] == ' ') ++ind;
    if (ind < s.size() && s[ind] == '\t') fail(no, "tab in indentation");
    std::string body = trim(s);
    if (depth > 0) {  // continuation of a flow collection
      if (!out.empty()) out.back().text += " " + body;
      depth += d;
      continue;
    }
    if (body.empty() || body == "---" || body == "...") continue;
    if (body.rfind("%", 0) == 0) continue;  // directives
    out.push_back(Line{(int)ind, body, no});
    depth = d;
    if (depth < 0) fail(no, "unbalanced brackets");
  }
  if (depth > 0) fail(no, "unterminated flow collection");
  return out;
}

bool is_seq_item(const std::string& t) {
  return t == "-" || (t.size() >= 2 && t[0] == '-' && t[1] == ' ');
}

// Position of the ':' that ends a mapping key (followed by a blank or the
// end), outside quotes and brackets; npos when the text is no entry.
size_t key_colon(const std::string& t) {
  if (t.empty() || t[0] == '[' || t[0] == '{') return std::string::npos;
  char quote = 0;
  int depth = 0;
  for (size_t i = 0; i < t.size(); ++i) {
    const char c = t[i];
    if (quote) {
      if (c == '\\' && quote == '"') {
        ++i;
      } else if (c == quote) {
        quote = 0;
      }
      continue;
    }
    if (c == '\'' || c == '"') {
      if (i == 0) quote = c;  // quoted keys only at the start
    } else if (c == '[' || c == '{') {
      ++depth;
    } else if (c == ']' || c == '}') {
      --depth;
    } else if (c == ':' && depth == 0 &&
               (i + 1 == t.size() || t[i + 1] == ' ')) {
      return i;
    }
  }
  return std::string::npos;
}

std::string unquote(const std::string& s, int line) {
  if (s.size() >= 2 && s[0] == '\'' && s.back() == '\'') {
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      out += s[i];
      if (s[i] == '\'' && i + 2 < s.size() && s[i + 1] == '\'') ++i;
    }
    return out;
  }
  if (s.size() >= 2 && s[0] == '"' && s.back() == '"') {
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      char c = s[i];
      if (c == '\\' && i + 2 < s.size()) {
        const char e = s[++i];
        c = e == 'n' ? '\n' : e == 't' ? '\t' : e == '0' ? '\0' : e;
      }
      out += c;
    }
    return out;
  }
  if (!s.empty() && (s[0] == '\'' || s[0] == '"'))
    fail(line, "unterminated quoted scalar");
  return s;
}

Node scalar_node(const std::string& raw, int line) {
  Node n;
  n.line = line;
  const std::string t = trim(raw);
  if (!t.empty() && (t[0] == '&' || t[0] == '*' || t[0] == '!' ||
                     t[0] == '|' || t[0] == '>'))
    fail(line, "anchors, aliases, tags and block scalars are not supported");
  if (t.empty() || t == "~" || t == "null" || t == "Null" || t == "NULL") {
    n.kind = Node::kNull;
    return n;
  }
  n.kind = Node::kScalar;
  n.scalar = unquote(t, line);
  return n;
}

struct Flow {
  const std::string& s;
  int line;
  size_t i = 0;

  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
  }
  std::string token(const char* stops) {
    ws();
    if (i < s.size() && (s[i] == '\'' || s[i] == '"')) {
      const char q = s[i];
      const size_t a = i++;
      while (i < s.size() && s[i] != q) {
        if (s[i] == '\\' && q == '"') ++i;
        ++i;
      }
      if (i >= s.size()) fail(line, "unterminated quoted scalar");
      ++i;
      return s.substr(a, i - a);
    }
    const size_t a = i;
    while (i < s.size()) {
      const char c = s[i];
      bool stop = false;
      for (const char* p = stops; *p; ++p) stop |= c == *p;
      // a ':' ends a key only when a blank or a closer follows
      if (c == ':' && !(i + 1 == s.size() || s[i + 1] == ' ' ||
                        s[i + 1] == ',' || s[i + 1] == '}'))
        stop = false;
      if (stop) break;
      ++i;
    }
    return trim(s.substr(a, i - a));
  }
  Node value() {
    ws();
    if (i < s.size() && (s[i] == '[' || s[i] == '{')) return collection();
    return scalar_node(token(",]}"), line);
  }
  Node collection() {
    Node n;
    n.line = line;
    const char open = s[i++];
    const char close = open == '[' ? ']' : '}';
    n.kind = open == '[' ? Node::kSequence : Node::kMap;
    ws();
    if (i < s.size() && s[i] == close) {
      ++i;
      return n;
    }
    for (;;) {
      if (open == '[') {
        n.items.push_back(value());
      } else {
        const std::string key = unquote(token(":,}"), line);
        ws();
        if (i >= s.size() || s[i] != ':') fail(line, "expected ':' in {..}");
        ++i;
        n.entries.emplace_back(key, value());
      }
      ws();
      if (i < s.size() && s[i] == ',') {
        ++i;
        continue;
      }
      if (i < s.size() && s[i] == close) {
        ++i;
        return n;
      }
      fail(line, std::string("expected ',' or '") + close + "'");
    }
  }
};

Node inline_node(const std::string& text, int line) {
  const std::string t = trim(text);
  if (!t.empty() && (t[0] == '[' || t[0] == '{')) {
    Flow f{t, line};
    Node n = f.collection();
    f.ws();
    if (f.i != t.size()) fail(line, "text after a flow collection");
    return n;
  }
  return scalar_node(t, line);
}

struct Parser {
  std::vector<Line> lines;
  size_t pos = 0;

  Node block(int indent) {
    return is_seq_item(lines[pos].text) ? seq(indent) : map(indent);
  }

  Node seq(int indent) {
    Node n;
    n.kind = Node::kSequence;
    n.line = lines[pos].no;
    while (pos < lines.size() && lines[pos].indent == indent &&
           is_seq_item(lines[pos].text)) {
      Line& l = lines[pos];
      const std::string rest =
          l.text == "-" ? std::string() : trim(l.text.substr(1));
      const int rest_indent =
          indent + (int)(l.text.size() - rest.size());
      if (rest.empty()) {
        ++pos;
        if (pos < lines.size() && lines[pos].indent > indent)
          n.items.push_back(block(lines[pos].indent));
        else
          n.items.push_back(scalar_node("", l.no));
      } else if (is_seq_item(rest) || key_colon(rest) != std::string::npos) {
        // "- - x" or "- key: value": the item is a block at the column of
        // its first entry
        l = Line{rest_indent, rest, l.no};
        n.items.push_back(block(rest_indent));
      } else {
        n.items.push_back(inline_node(rest, l.no));
        ++pos;
      }
    }
    return n;
  }

  Node map(int indent) {
    Node n;
    n.kind = Node::kMap;
    n.line = lines[pos].no;
    while (pos < lines.size() && lines[pos].indent == indent &&
           !is_seq_item(lines[pos].text)) {
      const Line l = lines[pos];
      const size_t c = key_colon(l.text);
      if (c == std::string::npos) fail(l.no, "expected 'key: value'");
      const std::string key = unquote(trim(l.text.substr(0, c)), l.no);
      const std::string value = trim(l.text.substr(c + 1));
      ++pos;
      Node child;
      if (!value.empty()) {
        child = inline_node(value, l.no);
      } else if (pos < lines.size() && lines[pos].indent > indent) {
        child = block(lines[pos].indent);
      } else if (pos < lines.size() && lines[pos].indent == indent &&
                 is_seq_item(lines[pos].text)) {
        child = seq(indent);  // "key:" then "- item" at the key's column
      } else {
        child = scalar_node("", l.no);
      }
      for (auto& e : n.entries)
        if (e.first == key) fail(l.no, "duplicate key '" + key + "'");
      n.entries.emplace_back(key, std::move(child));
    }
    if (pos < lines.size() && lines[pos].indent > indent)
      fail(lines[pos].no, "unexpected indentation");
    return n;
  }
};

}  // namespace

const Node& Node::operator[](const std::string& key) const {
  if (kind != kMap) return undefined_node();
  for (const auto& e : entries)
    if (e.first == key) return e.second;
  return undefined_node();
}

const Node& Node::operator[](size_t i) const {
  if (kind != kSequence || i >= items.size()) return undefined_node();
  return items[i];
}

std::string Node::AsString() const {
  if (kind != kScalar) fail(line, "expected a scalar");
  return scalar;
}

double Node::AsDouble() const {
  const std::string s = AsString();
  if (s == ".inf" || s == ".Inf" || s == "+.inf") return HUGE_VAL;
  if (s == "-.inf" || s == "-.Inf") return -HUGE_VAL;
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') fail(line, "'" + s + "' is no number");
  return v;
}

float Node::AsFloat() const {
  const std::string s = AsString();
  if (s == ".inf" || s == ".Inf" || s == "+.inf") return HUGE_VALF;
  if (s == "-.inf" || s == "-.Inf") return -HUGE_VALF;
  char* end = nullptr;
  const float v = std::strtof(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') fail(line, "'" + s + "' is no number");
  return v;
}

int64_t Node::AsInt() const {
  const std::string s = AsString();
  char* end = nullptr;
  const long long v = std::strtoll(s.c_str(), &end, 0);
  if (end == s.c_str() || *end != '\0')
    fail(line, "'" + s + "' is no integer");
  return (int64_t)v;
}

bool Node::AsBool() const {
  const std::string s = AsString();
  if (s == "true" || s == "True" || s == "TRUE" || s == "yes" || s == "Yes" ||
      s == "on" || s == "On" || s == "y" || s == "Y")
    return true;
  if (s == "false" || s == "False" || s == "FALSE" || s == "no" ||
      s == "No" || s == "off" || s == "Off" || s == "n" || s == "N")
    return false;
  fail(line, "'" + s + "' is no boolean");
}

std::vector<float> Node::AsFloats(size_t n) const {
  if (kind != kSequence || items.size() != n)
    fail(line, "expected a sequence of " + std::to_string(n) + " numbers");
  std::vector<float> out;
  for (const Node& x : items) out.push_back(x.AsFloat());
  return out;
}

Node ParseYaml(const std::string& text) {
  Parser p;
  p.lines = lex(text);
  if (p.lines.empty()) {
    Node n;
    n.kind = Node::kNull;
    return n;
  }
  Node root = p.block(p.lines[0].indent);
  if (p.pos != p.lines.size())
    fail(p.lines[p.pos].no, "unexpected indentation");
  return root;
}

Node LoadYamlFile(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw YamlError("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ParseYaml(ss.str());
}

}  // namespace ajh
