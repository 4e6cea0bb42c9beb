// Small DOM JSON reader for MACE model files (tens to hundreds of MB of numbers).
//
// Values live in one flat arena; arrays and objects store index ranges into it,
// so parsing a 170 MB model file allocates a handful of large vectors rather than
// millions of small nodes.  Numbers are parsed with std::from_chars.
#pragma once

#include <charconv>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

namespace smx {

class JsonDoc {
 public:
  enum Kind : uint8_t { kNull, kBool, kNum, kStr, kArr, kObj };
  struct Node {
    Kind kind;
    bool b;
    double num;
    uint32_t first, count;  // children range in kids_ (arrays/objects) or chars_ (strings)
  };

  explicit JsonDoc(std::string text) : text_(std::move(text)) {
    p_ = text_.data();
    end_ = p_ + text_.size();
    nodes_.reserve(text_.size() / 8 + 16);
    root_ = parse_value();
    ws();
    if (p_ != end_) fail("trailing characters");
  }

  uint32_t root() const { return root_; }
  const Node& node(uint32_t i) const { return nodes_[i]; }

  // object member lookup; returns UINT32_MAX if absent
  uint32_t find(uint32_t obj, std::string_view key) const {
    const Node& n = nodes_[obj];
    if (n.kind != kObj) throw std::runtime_error("model file: expected an object");
    for (uint32_t q = 0; q < n.count; ++q) {
      const uint32_t k = kids_[n.first + 2 * q];
      if (str(k) == key) return kids_[n.first + 2 * q + 1];
    }
    return UINT32_MAX;
  }
  uint32_t at(uint32_t obj, std::string_view key) const {
    uint32_t v = find(obj, key);
    if (v == UINT32_MAX) throw std::runtime_error("model file: missing key '" + std::string(key) + "'");
    return v;
  }
  uint32_t size(uint32_t i) const {
    const Node& n = nodes_[i];
    if (n.kind != kArr && n.kind != kObj) throw std::runtime_error("model file: expected an array");
    return n.count;
  }
  uint32_t elem(uint32_t arr, uint32_t q) const {
    const Node& n = nodes_[arr];
    if (n.kind != kArr || q >= n.count) throw std::runtime_error("model file: bad array access");
    return kids_[n.first + q];
  }
  // q-th member of an object: key node and value node
  std::pair<uint32_t, uint32_t> member(uint32_t obj, uint32_t q) const {
    const Node& n = nodes_[obj];
    return {kids_[n.first + 2 * q], kids_[n.first + 2 * q + 1]};
  }
  std::string_view str(uint32_t i) const {
    const Node& n = nodes_[i];
    if (n.kind != kStr) throw std::runtime_error("model file: expected a string");
    return std::string_view(text_.data() + n.first, n.count);
  }
  double num(uint32_t i) const {
    const Node& n = nodes_[i];
    if (n.kind == kNum) return n.num;
    if (n.kind == kBool) return n.b ? 1.0 : 0.0;
    throw std::runtime_error("model file: expected a number");
  }
  bool boolean(uint32_t i) const {
    const Node& n = nodes_[i];
    if (n.kind != kBool) throw std::runtime_error("model file: expected a boolean");
    return n.b;
  }
  // flatten a (nested) numeric array in row-major order, checking a rectangular shape
  void flatten(uint32_t i, std::vector<double>& out, std::vector<uint32_t>* shape = nullptr) const {
    out.clear();
    std::vector<uint32_t> sh;
    uint32_t cur = i;
    while (nodes_[cur].kind == kArr) {
      sh.push_back(nodes_[cur].count);
      if (nodes_[cur].count == 0) break;
      cur = kids_[nodes_[cur].first];
    }
    size_t total = 1;
    for (auto s : sh) total *= s;
    out.reserve(total);
    flatten_rec(i, 0, sh, out);
    if (out.size() != total) throw std::runtime_error("model file: ragged array");
    if (shape) *shape = sh;
  }

 private:
  std::string text_;
  const char* p_;
  const char* end_;
  std::vector<Node> nodes_;
  std::vector<uint32_t> kids_;
  uint32_t root_;

  [[noreturn]] void fail(const char* what) const {
    throw std::runtime_error(std::string("model file is not valid JSON: ") + what);
  }
  void ws() {
    while (p_ < end_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) ++p_;
  }
  uint32_t add(Node n) {
    nodes_.push_back(n);
    return static_cast<uint32_t>(nodes_.size() - 1);
  }
  uint32_t parse_string() {
    ++p_;
    const char* s = p_;
    while (p_ < end_ && *p_ != '"') {
      if (*p_ == '\\') ++p_;  // keys here are plain; escapes are skipped, not decoded
      ++p_;
    }
    if (p_ >= end_) fail("unterminated string");
    Node n{kStr, false, 0.0, static_cast<uint32_t>(s - text_.data()), static_cast<uint32_t>(p_ - s)};
    ++p_;
    return add(n);
  }
  uint32_t parse_value() {
    ws();
    if (p_ >= end_) fail("unexpected end of input");
    const char c = *p_;
    if (c == '[' || c == '{') {
      const bool obj = c == '{';
      ++p_;
      std::vector<uint32_t> local;
      ws();
      if (p_ < end_ && *p_ == (obj ? '}' : ']')) {
        ++p_;
      } else {
        while (true) {
          ws();
          if (obj) {
            if (p_ >= end_ || *p_ != '"') fail("expected key");
            local.push_back(parse_string());
            ws();
            if (p_ >= end_ || *p_ != ':') fail("expected ':'");
            ++p_;
          }
          local.push_back(parse_value());
          ws();
          if (p_ < end_ && *p_ == ',') {
            ++p_;
            continue;
          }
          if (p_ < end_ && *p_ == (obj ? '}' : ']')) {
            ++p_;
            break;
          }
          fail("expected ',' or a closing bracket");
        }
      }
      Node n{obj ? kObj : kArr, false, 0.0, static_cast<uint32_t>(kids_.size()),
             static_cast<uint32_t>(obj ? local.size() / 2 : local.size())};
      kids_.insert(kids_.end(), local.begin(), local.end());
      return add(n);
    }
    if (c == '"') return parse_string();
    if (c == 't' && end_ - p_ >= 4 && std::string_view(p_, 4) == "true") {
      p_ += 4;
      return add(Node{kBool, true, 0.0, 0, 0});
    }
    if (c == 'f' && end_ - p_ >= 5 && std::string_view(p_, 5) == "false") {
      p_ += 5;
      return add(Node{kBool, false, 0.0, 0, 0});
    }
    if (c == 'n' && end_ - p_ >= 4 && std::string_view(p_, 4) == "null") {
      p_ += 4;
      return add(Node{kNull, false, 0.0, 0, 0});
    }
    double d = 0.0;
    auto res = std::from_chars(p_, end_, d);
    if (res.ec != std::errc()) fail("bad number");
    p_ = res.ptr;
    return add(Node{kNum, false, d, 0, 0});
  }
  void flatten_rec(uint32_t i, size_t depth, const std::vector<uint32_t>& sh, std::vector<double>& out) const {
    const Node& n = nodes_[i];
    if (depth == sh.size()) {
      out.push_back(num(i));
      return;
    }
    if (n.kind != kArr || n.count != sh[depth]) throw std::runtime_error("model file: ragged array");
    for (uint32_t q = 0; q < n.count; ++q) flatten_rec(kids_[n.first + q], depth + 1, sh, out);
  }
};

}  // namespace smx
