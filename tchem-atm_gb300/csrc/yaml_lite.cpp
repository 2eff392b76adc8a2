// Minimal YAML reader; see yaml_lite.hpp for the supported subset.
#include "yaml_lite.hpp"

#include <cerrno>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>

namespace tchem_gb {
namespace yaml {

const Node* Node::get(const std::string& key) const {
  if (kind != Map) return nullptr;
  for (const auto& kv : map)
    if (kv.first == key) return kv.second.get();
  return nullptr;
}

size_t Node::size() const {
  if (kind == Seq) return seq.size();
  if (kind == Map) return map.size();
  return 0;
}

std::string Node::as_string() const {
  if (kind == Scalar) return scalar;
  if (kind == Null) return "";
  throw ParseError("yaml: node is not a scalar");
}

double Node::as_double() const {
  if (kind != Scalar) throw ParseError("yaml: expected a number, found a non-scalar node");
  const char* s = scalar.c_str();
  char* end = nullptr;
  errno = 0;
  double v = std::strtod(s, &end);
  while (end && (*end == ' ' || *end == '\t')) ++end;
  if (end == s || (end && *end != '\0'))
    throw ParseError("yaml: bad conversion of '" + scalar + "' to a floating-point value");
  return v;
}

long Node::as_int() const {
  if (kind != Scalar) throw ParseError("yaml: expected an integer, found a non-scalar node");
  const char* s = scalar.c_str();
  char* end = nullptr;
  long v = std::strtol(s, &end, 10);
  while (end && (*end == ' ' || *end == '\t')) ++end;
  if (end == s || (end && *end != '\0'))
    throw ParseError("yaml: bad conversion of '" + scalar + "' to an integer");
  return v;
}

namespace {

struct Line {
  int indent;
  std::string text;
  int lineno;
};

std::string rtrim(const std::string& s) {
  size_t e = s.size();
  while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r')) --e;
  return s.substr(0, e);
}

std::string ltrim(const std::string& s) {
  size_t b = 0;
  while (b < s.size() && (s[b] == ' ' || s[b] == '\t')) ++b;
  return s.substr(b);
}

std::string trim(const std::string& s) { return ltrim(rtrim(s)); }

// Removes a trailing comment: '#' at the start or after whitespace, outside quotes.
std::string strip_comment(const std::string& s) {
  char q = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (q) {
      if (c == q) {
        if (q == '\'' && i + 1 < s.size() && s[i + 1] == '\'') { ++i; continue; }
        q = 0;
      } else if (q == '"' && c == '\\') {
        ++i;
      }
      continue;
    }
    if ((c == '\'' || c == '"') && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t' ||
                                    s[i - 1] == '[' || s[i - 1] == '{' || s[i - 1] == ',' ||
                                    s[i - 1] == ':' || s[i - 1] == '-')) {
      q = c;
      continue;
    }
    if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
  }
  return s;
}

bool is_seq_item(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && (t[1] == ' ' || t[1] == '\t')); }

// Finds the ':' that ends a mapping key on this line; returns npos when the line is not a key line.
size_t find_key_colon(const std::string& t) {
  if (t.empty()) return std::string::npos;
  size_t i = 0;
  if (t[0] == '\'' || t[0] == '"') {
    const char q = t[0];
    i = 1;
    while (i < t.size()) {
      if (t[i] == q) {
        if (q == '\'' && i + 1 < t.size() && t[i + 1] == '\'') { i += 2; continue; }
        break;
      }
      if (q == '"' && t[i] == '\\') ++i;
      ++i;
    }
    ++i;
    while (i < t.size() && (t[i] == ' ' || t[i] == '\t')) ++i;
    if (i < t.size() && t[i] == ':' && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) return i;
    return std::string::npos;
  }
  if (t[0] == '[' || t[0] == '{' || t[0] == '&' || t[0] == '*' || t[0] == '|' || t[0] == '>') return std::string::npos;
  for (; i < t.size(); ++i) {
    if (t[i] == ':' && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) return i;
  }
  return std::string::npos;
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && s[0] == '\'' && s.back() == '\'') {
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      if (s[i] == '\'' && i + 2 < s.size() && s[i + 1] == '\'') { out += '\''; ++i; }
      else out += s[i];
    }
    return out;
  }
  if (s.size() >= 2 && s[0] == '"' && s.back() == '"') {
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      if (s[i] == '\\' && i + 2 < s.size()) {
        const char c = s[++i];
        switch (c) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case '\\': out += '\\'; break;
          case '"': out += '"'; break;
          default: out += c; break;
        }
      } else {
        out += s[i];
      }
    }
    return out;
  }
  return s;
}

NodePtr make_scalar(const std::string& raw) {
  auto n = std::make_shared<Node>();
  const std::string t = trim(raw);
  if (t.empty() || t == "~" || t == "null" || t == "Null" || t == "NULL") {
    n->kind = Node::Null;
    return n;
  }
  n->kind = Node::Scalar;
  n->scalar = unquote(t);
  return n;
}

class Parser {
 public:
  explicit Parser(const std::string& text) {
    std::istringstream in(text);
    std::string raw;
    int lineno = 0;
    while (std::getline(in, raw)) {
      ++lineno;
      std::string s = rtrim(strip_comment(rtrim(raw)));
      if (s.find('\t') != std::string::npos) {
        // Tabs only appear inside scalars in the supported files; normalise leading ones to a space.
        size_t k = 0;
        while (k < s.size() && (s[k] == ' ' || s[k] == '\t')) { if (s[k] == '\t') s[k] = ' '; ++k; }
      }
      size_t ind = 0;
      while (ind < s.size() && s[ind] == ' ') ++ind;
      if (ind == s.size()) continue;
      const std::string body = s.substr(ind);
      if (body == "---" || body == "..." || body.rfind("%YAML", 0) == 0) continue;
      lines_.push_back({static_cast<int>(ind), body, lineno});
    }
  }

  NodePtr parse() {
    pos_ = 0;
    if (lines_.empty()) return std::make_shared<Node>();
    NodePtr root = parse_block(lines_[0].indent);
    if (pos_ < lines_.size())
      fail("unexpected content (indentation does not match an open block)");
    return root;
  }

 private:
  std::vector<Line> lines_;
  size_t pos_ = 0;
  std::map<std::string, NodePtr> anchors_;

  [[noreturn]] void fail(const std::string& what) const {
    const int ln = pos_ < lines_.size() ? lines_[pos_].lineno : (lines_.empty() ? 0 : lines_.back().lineno);
    throw ParseError("yaml: line " + std::to_string(ln) + ": " + what);
  }

  NodePtr parse_block(int indent) {
    const std::string& t = lines_[pos_].text;
    if (is_seq_item(t)) return parse_seq(indent);
    if (find_key_colon(t) != std::string::npos) return parse_map(indent);
    // A scalar or a flow collection standing alone on its line(s).
    std::string text = t;
    ++pos_;
    return parse_inline(text, indent - 1);
  }

  NodePtr parse_map(int indent) {
    auto node = std::make_shared<Node>();
    node->kind = Node::Map;
    while (pos_ < lines_.size() && lines_[pos_].indent == indent && !is_seq_item(lines_[pos_].text)) {
      const std::string t = lines_[pos_].text;
      const size_t c = find_key_colon(t);
      if (c == std::string::npos) fail("expected 'key: value'");
      const std::string key = unquote(trim(t.substr(0, c)));
      const std::string rest = trim(t.substr(c + 1));
      ++pos_;
      node->map.emplace_back(key, parse_value(indent, rest));
    }
    if (pos_ < lines_.size() && lines_[pos_].indent > indent) fail("bad indentation in mapping");
    return node;
  }

  NodePtr parse_seq(int indent) {
    auto node = std::make_shared<Node>();
    node->kind = Node::Seq;
    while (pos_ < lines_.size() && lines_[pos_].indent == indent && is_seq_item(lines_[pos_].text)) {
      Line& ln = lines_[pos_];
      size_t off = 1;
      while (off < ln.text.size() && (ln.text[off] == ' ' || ln.text[off] == '\t')) ++off;
      const std::string rest = ln.text.substr(off);
      if (rest.empty()) {
        ++pos_;
        if (pos_ < lines_.size() && lines_[pos_].indent > indent)
          node->seq.push_back(parse_block(lines_[pos_].indent));
        else
          node->seq.push_back(std::make_shared<Node>());
      } else if (is_seq_item(rest) || find_key_colon(rest) != std::string::npos) {
        // A nested block that starts on the item line: re-read the remainder at its own column.
        ln.indent = indent + static_cast<int>(off);
        ln.text = rest;
        node->seq.push_back(parse_block(ln.indent));
      } else {
        ++pos_;
        node->seq.push_back(parse_value(indent, rest));
      }
    }
    if (pos_ < lines_.size() && lines_[pos_].indent > indent) fail("bad indentation in sequence");
    return node;
  }

  // Value after "key:" (or after "- " for scalar items). parent_indent is the indentation of the key.
  NodePtr parse_value(int parent_indent, std::string rest) {
    std::string anchor;
    if (!rest.empty() && rest[0] == '&') {
      size_t e = rest.find_first_of(" \t");
      anchor = rest.substr(1, e == std::string::npos ? std::string::npos : e - 1);
      rest = e == std::string::npos ? std::string() : trim(rest.substr(e));
    }
    if (!rest.empty() && rest[0] == '*') {
      const std::string name = trim(rest.substr(1));
      auto it = anchors_.find(name);
      if (it == anchors_.end()) fail("unknown alias *" + name);
      return it->second;
    }
    NodePtr v;
    if (rest.empty()) {
      if (pos_ < lines_.size() && lines_[pos_].indent > parent_indent)
        v = parse_block(lines_[pos_].indent);
      else if (pos_ < lines_.size() && lines_[pos_].indent == parent_indent && is_seq_item(lines_[pos_].text))
        v = parse_seq(parent_indent);
      else
        v = std::make_shared<Node>();
    } else {
      v = parse_inline(rest, parent_indent);
    }
    if (!anchor.empty()) anchors_[anchor] = v;
    return v;
  }

  // Inline value: flow collection or scalar; consumes continuation lines indented deeper than parent_indent.
  NodePtr parse_inline(std::string text, int parent_indent) {
    if (text[0] == '[' || text[0] == '{') {
      while (!flow_closed(text)) {
        if (pos_ >= lines_.size() || lines_[pos_].indent <= parent_indent) fail("unterminated flow collection");
        text += " " + lines_[pos_].text;
        ++pos_;
      }
      size_t i = 0;
      NodePtr n = parse_flow(text, i);
      skip_ws(text, i);
      if (i != text.size()) fail("trailing characters after flow collection");
      return n;
    }
    if (text[0] == '\'' || text[0] == '"') {
      while (!quote_closed(text)) {
        if (pos_ >= lines_.size()) fail("unterminated quoted scalar");
        text += " " + lines_[pos_].text;
        ++pos_;
      }
      return make_scalar(text);
    }
    if (text == "|" || text == ">" || text == "|-" || text == ">-") fail("block scalars are not supported");
    // Plain multi-line scalar: fold deeper-indented continuation lines with single spaces.
    while (pos_ < lines_.size() && lines_[pos_].indent > parent_indent) {
      text += " " + lines_[pos_].text;
      ++pos_;
    }
    return make_scalar(text);
  }

  static bool quote_closed(const std::string& t) {
    const char q = t[0];
    for (size_t i = 1; i < t.size(); ++i) {
      if (t[i] == q) {
        if (q == '\'' && i + 1 < t.size() && t[i + 1] == '\'') { ++i; continue; }
        return true;
      }
      if (q == '"' && t[i] == '\\') ++i;
    }
    return false;
  }

  static bool flow_closed(const std::string& t) {
    int depth = 0;
    char q = 0;
    for (size_t i = 0; i < t.size(); ++i) {
      const char c = t[i];
      if (q) {
        if (c == q) q = 0;
        continue;
      }
      if (c == '\'' || c == '"') q = c;
      else if (c == '[' || c == '{') ++depth;
      else if (c == ']' || c == '}') { if (--depth == 0) return true; }
    }
    return false;
  }

  static void skip_ws(const std::string& t, size_t& i) {
    while (i < t.size() && (t[i] == ' ' || t[i] == '\t')) ++i;
  }

  std::string flow_scalar(const std::string& t, size_t& i) {
    skip_ws(t, i);
    if (i < t.size() && (t[i] == '\'' || t[i] == '"')) {
      const char q = t[i];
      size_t j = i + 1;
      while (j < t.size()) {
        if (t[j] == q) {
          if (q == '\'' && j + 1 < t.size() && t[j + 1] == '\'') { j += 2; continue; }
          break;
        }
        if (q == '"' && t[j] == '\\') ++j;
        ++j;
      }
      if (j >= t.size()) fail("unterminated quoted scalar in flow collection");
      std::string s = t.substr(i, j - i + 1);
      i = j + 1;
      return s;
    }
    size_t j = i;
    while (j < t.size() && t[j] != ',' && t[j] != ']' && t[j] != '}') {
      if (t[j] == ':' && (j + 1 == t.size() || t[j + 1] == ' ')) break;
      ++j;
    }
    std::string s = trim(t.substr(i, j - i));
    i = j;
    return s;
  }

  NodePtr parse_flow(const std::string& t, size_t& i) {
    skip_ws(t, i);
    auto node = std::make_shared<Node>();
    if (t[i] == '[') {
      node->kind = Node::Seq;
      ++i;
      skip_ws(t, i);
      if (i < t.size() && t[i] == ']') { ++i; return node; }
      while (true) {
        skip_ws(t, i);
        if (i < t.size() && (t[i] == '[' || t[i] == '{')) node->seq.push_back(parse_flow(t, i));
        else node->seq.push_back(make_scalar(flow_scalar(t, i)));
        skip_ws(t, i);
        if (i >= t.size()) fail("unterminated flow sequence");
        if (t[i] == ',') { ++i; skip_ws(t, i); if (i < t.size() && t[i] == ']') { ++i; break; } continue; }
        if (t[i] == ']') { ++i; break; }
        fail("expected ',' or ']' in flow sequence");
      }
      return node;
    }
    if (t[i] == '{') {
      node->kind = Node::Map;
      ++i;
      skip_ws(t, i);
      if (i < t.size() && t[i] == '}') { ++i; return node; }
      while (true) {
        const std::string key = unquote(flow_scalar(t, i));
        skip_ws(t, i);
        NodePtr val;
        if (i < t.size() && t[i] == ':') {
          ++i;
          skip_ws(t, i);
          if (i < t.size() && (t[i] == '[' || t[i] == '{')) val = parse_flow(t, i);
          else val = make_scalar(flow_scalar(t, i));
        } else {
          val = std::make_shared<Node>();
        }
        node->map.emplace_back(key, val);
        skip_ws(t, i);
        if (i >= t.size()) fail("unterminated flow mapping");
        if (t[i] == ',') { ++i; continue; }
        if (t[i] == '}') { ++i; break; }
        fail("expected ',' or '}' in flow mapping");
      }
      return node;
    }
    fail("expected a flow collection");
  }
};

}  // namespace

NodePtr parse_string(const std::string& text) {
  Parser p(text);
  return p.parse();
}

NodePtr parse_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw ParseError("yaml: cannot open file '" + path + "'");
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_string(ss.str());
}

}  // namespace yaml
}  // namespace tchem_gb
