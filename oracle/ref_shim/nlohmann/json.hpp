// Minimal stand-in for the parts of nlohmann::json that painty's mixer/src/Serialization.cxx
// uses, written for this repository so that file compiles unmodified in the oracle build (the
// JSON library is not installed here): null, booleans, numbers, strings, arrays and objects;
// parsing from a stream (numbers as nlohmann reads them: integers as 64-bit integers, other
// numbers by strtod), operator[] / at(), iteration over an array's elements, get<T>() and
// construction from T through the caller's from_json / to_json, and writing to a stream (numbers
// with 17 significant digits, which read back to the same double).
#pragma once
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <initializer_list>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace nlohmann {

class json {
 public:
  enum class kind { null, boolean, integer, real, string, array, object };

  json() = default;
  json(std::nullptr_t) {}
  json(bool b) : k_(kind::boolean), b_(b) {}
  json(int v) : k_(kind::integer), i_(v) {}
  json(int64_t v) : k_(kind::integer), i_(v) {}
  json(unsigned v) : k_(kind::integer), i_(static_cast<int64_t>(v)) {}
  json(double v) : k_(kind::real), d_(v) {}
  json(const char* s) : k_(kind::string), s_(s) {}
  json(const std::string& s) : k_(kind::string), s_(s) {}
  json(std::initializer_list<json> items) : k_(kind::array), a_(items) {}
  // anything else: through the caller's to_json(json&, const T&), found by argument lookup
  template <typename T,
            typename = std::enable_if_t<!std::is_arithmetic<std::decay_t<T>>::value &&
                                        !std::is_same<std::decay_t<T>, json>::value>>
  json(const T& v) {
    to_json(*this, v);
  }

  static json array() {
    json j;
    j.k_ = kind::array;
    return j;
  }

  json& operator=(std::initializer_list<json> items) {
    *this = json(items);
    return *this;
  }

  // object member, created as null when missing (an object is made from null)
  json& operator[](const std::string& key) {
    if (k_ == kind::null) k_ = kind::object;
    if (k_ != kind::object) throw std::domain_error("json: not an object");
    return o_[key];
  }
  const json& at(const std::string& key) const {
    if (k_ != kind::object) throw std::domain_error("json: not an object");
    auto it = o_.find(key);
    if (it == o_.end()) throw std::out_of_range("json: key not found: " + key);
    return it->second;
  }
  const json& at(size_t index) const {
    if (k_ != kind::array) throw std::domain_error("json: not an array");
    return a_.at(index);
  }

  void push_back(const json& v) {
    if (k_ == kind::null) k_ = kind::array;
    if (k_ != kind::array) throw std::domain_error("json: not an array");
    a_.push_back(v);
  }

  // iteration visits an array's elements (an object's values in key order)
  class iterator {
   public:
    iterator(json* owner, size_t i) : owner_(owner), i_(i) {}
    json& operator*() const { return owner_->element(i_); }
    iterator& operator++() {
      ++i_;
      return *this;
    }
    bool operator!=(const iterator& o) const { return i_ != o.i_ || owner_ != o.owner_; }

   private:
    json* owner_;
    size_t i_;
  };
  iterator begin() { return iterator(this, 0); }
  iterator end() { return iterator(this, size()); }
  size_t size() const {
    return k_ == kind::array ? a_.size() : k_ == kind::object ? o_.size() : k_ == kind::null ? 0 : 1;
  }

  operator double() const {
    if (k_ == kind::real) return d_;
    if (k_ == kind::integer) return static_cast<double>(i_);
    throw std::domain_error("json: not a number");
  }

  template <typename T>
  T get() const {
    T v{};
    from_json(*this, v);
    return v;
  }

  friend std::istream& operator>>(std::istream& in, json& j) {
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    j = parse_value(text, pos);
    skip_ws(text, pos);
    if (pos != text.size()) throw std::invalid_argument("json: trailing characters");
    return in;
  }

  friend std::ostream& operator<<(std::ostream& out, const json& j) {
    j.write(out);
    return out;
  }

 private:
  kind k_ = kind::null;
  bool b_ = false;
  int64_t i_ = 0;
  double d_ = 0.0;
  std::string s_;
  std::vector<json> a_;
  std::map<std::string, json> o_;

  json& element(size_t i) {
    if (k_ == kind::array) return a_[i];
    auto it = o_.begin();
    std::advance(it, static_cast<long>(i));
    return it->second;
  }

  static void skip_ws(const std::string& t, size_t& p) {
    while (p < t.size() && std::isspace(static_cast<unsigned char>(t[p]))) p++;
  }

  static std::string parse_string(const std::string& t, size_t& p) {
    if (t[p] != '"') throw std::invalid_argument("json: string expected");
    std::string s;
    for (p++; p < t.size() && t[p] != '"'; p++) {
      if (t[p] == '\\') {
        p++;
        if (p >= t.size()) break;
        const char c = t[p];
        s += c == 'n' ? '\n' : c == 't' ? '\t' : c == 'r' ? '\r' : c == 'b' ? '\b' : c == 'f' ? '\f' : c;
      } else {
        s += t[p];
      }
    }
    if (p >= t.size()) throw std::invalid_argument("json: unterminated string");
    p++;
    return s;
  }

  static json parse_value(const std::string& t, size_t& p) {
    skip_ws(t, p);
    if (p >= t.size()) throw std::invalid_argument("json: value expected");
    const char c = t[p];
    if (c == '[') {
      json j = array();
      p++;
      skip_ws(t, p);
      if (p < t.size() && t[p] == ']') {
        p++;
        return j;
      }
      for (;;) {
        j.a_.push_back(parse_value(t, p));
        skip_ws(t, p);
        if (p < t.size() && t[p] == ',') {
          p++;
          continue;
        }
        if (p < t.size() && t[p] == ']') {
          p++;
          return j;
        }
        throw std::invalid_argument("json: ',' or ']' expected");
      }
    }
    if (c == '{') {
      json j;
      j.k_ = kind::object;
      p++;
      skip_ws(t, p);
      if (p < t.size() && t[p] == '}') {
        p++;
        return j;
      }
      for (;;) {
        skip_ws(t, p);
        const std::string key = parse_string(t, p);
        skip_ws(t, p);
        if (p >= t.size() || t[p] != ':') throw std::invalid_argument("json: ':' expected");
        p++;
        j.o_[key] = parse_value(t, p);
        skip_ws(t, p);
        if (p < t.size() && t[p] == ',') {
          p++;
          continue;
        }
        if (p < t.size() && t[p] == '}') {
          p++;
          return j;
        }
        throw std::invalid_argument("json: ',' or '}' expected");
      }
    }
    if (c == '"') return json(parse_string(t, p));
    if (t.compare(p, 4, "true") == 0) {
      p += 4;
      return json(true);
    }
    if (t.compare(p, 5, "false") == 0) {
      p += 5;
      return json(false);
    }
    if (t.compare(p, 4, "null") == 0) {
      p += 4;
      return json();
    }
    // a number: integers without fraction or exponent stay integers
    size_t q = p;
    bool integral = true;
    if (q < t.size() && (t[q] == '-' || t[q] == '+')) q++;
    while (q < t.size() && (std::isdigit(static_cast<unsigned char>(t[q])) || t[q] == '.' ||
                            t[q] == 'e' || t[q] == 'E' || t[q] == '-' || t[q] == '+')) {
      if (t[q] == '.' || t[q] == 'e' || t[q] == 'E') integral = false;
      q++;
    }
    if (q == p) throw std::invalid_argument("json: unexpected character");
    const std::string tok = t.substr(p, q - p);
    p = q;
    if (integral) return json(static_cast<int64_t>(std::strtoll(tok.c_str(), nullptr, 10)));
    return json(std::strtod(tok.c_str(), nullptr));
  }

  void write(std::ostream& out) const {
    switch (k_) {
      case kind::null: out << "null"; break;
      case kind::boolean: out << (b_ ? "true" : "false"); break;
      case kind::integer: out << i_; break;
      case kind::real: {
        char buf[40];
        std::snprintf(buf, sizeof(buf), "%.17g", d_);
        out << buf;
        break;
      }
      case kind::string: out << '"' << s_ << '"'; break;
      case kind::array: {
        out << '[';
        for (size_t i = 0; i < a_.size(); i++) {
          if (i) out << ',';
          a_[i].write(out);
        }
        out << ']';
        break;
      }
      case kind::object: {
        out << '{';
        bool first = true;
        for (const auto& kv : o_) {
          if (!first) out << ',';
          first = false;
          out << '"' << kv.first << "\":";
          kv.second.write(out);
        }
        out << '}';
        break;
      }
    }
  }
};

}  // namespace nlohmann
