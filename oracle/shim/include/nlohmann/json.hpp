// Minimal stand-in for the nlohmann::json subset that libsymmetrix's model loader
// uses (libsymmetrix/source/mace.cpp:905-1030).  The real header lives in the
// un-vendored git submodule libsymmetrix/external/json (nlohmann/json, version
// not pinned in the reference tree), which is empty here.
//
// Test infrastructure only: this header lets the oracle build the reference's own
// evaluator sources and the oracle's restatement read the same model files.
//
// Supported: json::parse(std::istream&), operator[](key), implicit conversion to
// arithmetic types, and get<T>() for bool / int / double / std::string and any
// nesting of std::vector<...> and std::map<std::string, ...> of those.
#pragma once

#include <charconv>
#include <cstdint>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace nlohmann {

class json {
 public:
  enum class kind { null, boolean, number, string, array, object };

  struct parse_error : std::runtime_error {
    explicit parse_error(const std::string& m) : std::runtime_error(m) {}
  };
  struct type_error : std::runtime_error {
    explicit type_error(const std::string& m) : std::runtime_error(m) {}
  };

  json() = default;

  static json parse(std::istream& in) {
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (text.empty())
      throw parse_error("[json.exception.parse_error.101] parse error: empty input");
    const char* p = text.data();
    const char* end = p + text.size();
    json v = parse_value(p, end);
    skip_ws(p, end);
    if (p != end) throw parse_error("[json.exception.parse_error.101] trailing characters");
    return v;
  }

  json& operator[](const std::string& key) {
    if (k_ != kind::object) throw type_error("operator[] on a non-object");
    auto it = obj_->find(key);
    if (it == obj_->end()) throw type_error("missing key '" + key + "'");
    return it->second;
  }
  json& operator[](const char* key) { return (*this)[std::string(key)]; }
  const json& operator[](const std::string& key) const {
    if (k_ != kind::object) throw type_error("operator[] on a non-object");
    auto it = obj_->find(key);
    if (it == obj_->end()) throw type_error("missing key '" + key + "'");
    return it->second;
  }

  bool contains(const std::string& key) const {
    return k_ == kind::object && obj_->count(key) != 0;
  }

  template <typename T>
  T get() const {
    T out{};
    from(*this, out);
    return out;
  }

  template <typename T, typename = std::enable_if_t<std::is_arithmetic_v<T>>>
  operator T() const {
    return get<T>();
  }

  kind type() const { return k_; }
  size_t size() const {
    if (k_ == kind::array) return arr_->size();
    if (k_ == kind::object) return obj_->size();
    return 0;
  }

 private:
  kind k_ = kind::null;
  bool b_ = false;
  double num_ = 0.0;
  std::shared_ptr<std::string> str_;
  std::shared_ptr<std::vector<json>> arr_;
  std::shared_ptr<std::map<std::string, json>> obj_;

  static void skip_ws(const char*& p, const char* end) {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  static std::string parse_string(const char*& p, const char* end) {
    if (p >= end || *p != '"') throw parse_error("[json.exception.parse_error.101] expected string");
    ++p;
    std::string s;
    while (p < end && *p != '"') {
      if (*p == '\\') {
        ++p;
        if (p >= end) break;
        switch (*p) {
          case 'n': s += '\n'; break;
          case 't': s += '\t'; break;
          case 'r': s += '\r'; break;
          case 'b': s += '\b'; break;
          case 'f': s += '\f'; break;
          default: s += *p;
        }
        ++p;
      } else {
        s += *p++;
      }
    }
    if (p >= end) throw parse_error("[json.exception.parse_error.101] unterminated string");
    ++p;
    return s;
  }
  static json parse_value(const char*& p, const char* end) {
    skip_ws(p, end);
    if (p >= end) throw parse_error("[json.exception.parse_error.101] unexpected end of input");
    json v;
    const char c = *p;
    if (c == '{') {
      ++p;
      v.k_ = kind::object;
      v.obj_ = std::make_shared<std::map<std::string, json>>();
      skip_ws(p, end);
      if (p < end && *p == '}') { ++p; return v; }
      while (true) {
        skip_ws(p, end);
        std::string key = parse_string(p, end);
        skip_ws(p, end);
        if (p >= end || *p != ':') throw parse_error("[json.exception.parse_error.101] expected ':'");
        ++p;
        (*v.obj_)[key] = parse_value(p, end);
        skip_ws(p, end);
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; break; }
        throw parse_error("[json.exception.parse_error.101] expected ',' or '}'");
      }
    } else if (c == '[') {
      ++p;
      v.k_ = kind::array;
      v.arr_ = std::make_shared<std::vector<json>>();
      skip_ws(p, end);
      if (p < end && *p == ']') { ++p; return v; }
      while (true) {
        v.arr_->push_back(parse_value(p, end));
        skip_ws(p, end);
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; break; }
        throw parse_error("[json.exception.parse_error.101] expected ',' or ']'");
      }
    } else if (c == '"') {
      v.k_ = kind::string;
      v.str_ = std::make_shared<std::string>(parse_string(p, end));
    } else if (c == 't' && end - p >= 4 && std::string(p, 4) == "true") {
      v.k_ = kind::boolean; v.b_ = true; p += 4;
    } else if (c == 'f' && end - p >= 5 && std::string(p, 5) == "false") {
      v.k_ = kind::boolean; v.b_ = false; p += 5;
    } else if (c == 'n' && end - p >= 4 && std::string(p, 4) == "null") {
      v.k_ = kind::null; p += 4;
    } else {
      double d = 0.0;
      auto res = std::from_chars(p, end, d);
      if (res.ec != std::errc()) throw parse_error("[json.exception.parse_error.101] syntax error");
      p = res.ptr;
      v.k_ = kind::number;
      v.num_ = d;
    }
    return v;
  }

  static void from(const json& j, bool& out) {
    if (j.k_ != kind::boolean) throw type_error("type must be boolean");
    out = j.b_;
  }
  template <typename T, std::enable_if_t<std::is_arithmetic_v<T> && !std::is_same_v<T, bool>, int> = 0>
  static void from(const json& j, T& out) {
    if (j.k_ == kind::number) out = static_cast<T>(j.num_);
    else if (j.k_ == kind::boolean) out = static_cast<T>(j.b_);
    else throw type_error("type must be number");
  }
  static void from(const json& j, std::string& out) {
    if (j.k_ != kind::string) throw type_error("type must be string");
    out = *j.str_;
  }
  template <typename T>
  static void from(const json& j, std::vector<T>& out) {
    if (j.k_ != kind::array) throw type_error("type must be array");
    out.clear();
    out.reserve(j.arr_->size());
    for (const auto& e : *j.arr_) {
      T x{};
      from(e, x);
      out.push_back(std::move(x));
    }
  }
  template <typename T>
  static void from(const json& j, std::map<std::string, T>& out) {
    if (j.k_ != kind::object) throw type_error("type must be object");
    out.clear();
    for (const auto& [k, e] : *j.obj_) {
      T x{};
      from(e, x);
      out.emplace(k, std::move(x));
    }
  }
};

}  // namespace nlohmann
