// Stand-in for nlohmann::json (an absent submodule of the reference), for
// the host build of the reference's scene.cpp.  Test infrastructure only.
//
// It restates the documented behaviour of nlohmann/json 3.x that
// parseScene relies on, written from its documentation:
//  * operator[] on a non-const value: a null value becomes an object (string
//    key) or an array (index); a missing key is inserted as null; an index
//    past the end extends the array with nulls; any other type throws
//    type_error (305).
//  * implicit conversions: to bool only from a boolean; to an arithmetic type
//    from an integer, a floating-point number or a boolean (static_cast);
//    to std::string only from a string; anything else throws type_error
//    (302).
//  * iteration: the elements of an array, the values of an object, nothing
//    for null, the value itself for a primitive.
//  * operator>> parses a whole JSON text; malformed input throws
//    parse_error (101).  Numbers with a fraction or an exponent are floating
//    point, others integers.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <exception>
#include <istream>
#include <iterator>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json {
 public:
  enum class value_t { null, boolean, number_integer, number_float, string, array, object };

  class exception : public std::exception {
   public:
    int id = 0;
    std::string msg;
    exception() = default;
    exception(int i, std::string m) : id(i), msg(std::move(m)) {}
    const char* what() const noexcept override { return msg.c_str(); }
  };
  class type_error : public exception {
   public:
    using exception::exception;
  };
  class parse_error : public exception {
   public:
    using exception::exception;
  };

  json() = default;

  value_t type() const { return t_; }
  bool is_null() const { return t_ == value_t::null; }

  json& operator[](const char* key) {
    if (t_ == value_t::null) t_ = value_t::object;
    if (t_ != value_t::object) throw type_error(305, "cannot use operator[] with a string argument");
    for (auto& kv : o_)
      if (kv.first == key) return kv.second;
    o_.emplace_back(key, json());
    return o_.back().second;
  }
  json& operator[](const std::string& key) { return (*this)[key.c_str()]; }
  json& operator[](int idx) {
    if (t_ == value_t::null) t_ = value_t::array;
    if (t_ != value_t::array) throw type_error(305, "cannot use operator[] with a numeric argument");
    if ((size_t)idx >= a_.size()) a_.resize((size_t)idx + 1);
    return a_[(size_t)idx];
  }

  template <class T>
  struct convertible
      : std::integral_constant<bool, std::is_same<T, bool>::value || std::is_same<T, int>::value ||
                                         std::is_same<T, unsigned>::value || std::is_same<T, long>::value ||
                                         std::is_same<T, long long>::value || std::is_same<T, float>::value ||
                                         std::is_same<T, double>::value || std::is_same<T, std::string>::value> {};
  template <class T, typename std::enable_if<convertible<T>::value, int>::type = 0>
  operator T() const {
    T v;
    get_to(v);
    return v;
  }

  // iteration over copies of the elements
  std::vector<json> items() const {
    if (t_ == value_t::array) return a_;
    if (t_ == value_t::object) {
      std::vector<json> r;
      for (auto& kv : o_) r.push_back(kv.second);
      return r;
    }
    if (t_ == value_t::null) return {};
    return {*this};
  }
  // range-for over a json: `for (auto d : j)` binds to begin()/end() of j;
  // the elements are snapshotted on begin()
  std::vector<json>::iterator begin() {
    iter_ = items();
    return iter_.begin();
  }
  std::vector<json>::iterator end() { return iter_.end(); }

  friend std::istream& operator>>(std::istream& is, json& j) {
    std::string text((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    j = parse_value(text, pos);
    skip_ws(text, pos);
    if (pos != text.size()) throw parse_error(101, "syntax error: trailing characters");
    return is;
  }

 private:
  value_t t_ = value_t::null;
  bool b_ = false;
  long long i_ = 0;
  double d_ = 0.0;
  std::string s_;
  std::vector<json> a_;
  std::vector<std::pair<std::string, json>> o_;
  std::vector<json> iter_;

  void get_to(bool& v) const {
    if (t_ != value_t::boolean) throw type_error(302, "type must be boolean");
    v = b_;
  }
  void get_to(std::string& v) const {
    if (t_ != value_t::string) throw type_error(302, "type must be string");
    v = s_;
  }
  template <class A>
  void get_to(A& v) const {
    switch (t_) {
      case value_t::number_integer: v = static_cast<A>(i_); break;
      case value_t::number_float: v = static_cast<A>(d_); break;
      case value_t::boolean: v = static_cast<A>(b_); break;
      default: throw type_error(302, "type must be number");
    }
  }

  static void skip_ws(const std::string& s, size_t& p) {
    while (p < s.size() && (s[p] == ' ' || s[p] == '\t' || s[p] == '\n' || s[p] == '\r')) ++p;
  }
  static void expect(const std::string& s, size_t& p, const char* word) {
    for (const char* c = word; *c; ++c, ++p)
      if (p >= s.size() || s[p] != *c) throw parse_error(101, "syntax error: invalid literal");
  }
  static std::string parse_string(const std::string& s, size_t& p) {
    if (p >= s.size() || s[p] != '"') throw parse_error(101, "syntax error: expected string");
    ++p;
    std::string r;
    while (p < s.size() && s[p] != '"') {
      char c = s[p++];
      if (c == '\\') {
        if (p >= s.size()) break;
        const char e = s[p++];
        switch (e) {
          case 'n': r += '\n'; break;
          case 't': r += '\t'; break;
          case 'r': r += '\r'; break;
          case 'b': r += '\b'; break;
          case 'f': r += '\f'; break;
          case 'u': {  // basic multilingual plane code point, as UTF-8
            if (p + 4 > s.size()) throw parse_error(101, "syntax error: bad \\u escape");
            const unsigned cp = (unsigned)strtoul(s.substr(p, 4).c_str(), nullptr, 16);
            p += 4;
            if (cp < 0x80) {
              r += (char)cp;
            } else if (cp < 0x800) {
              r += (char)(0xC0 | (cp >> 6));
              r += (char)(0x80 | (cp & 0x3F));
            } else {
              r += (char)(0xE0 | (cp >> 12));
              r += (char)(0x80 | ((cp >> 6) & 0x3F));
              r += (char)(0x80 | (cp & 0x3F));
            }
            break;
          }
          default: r += e;  // \" \\ \/
        }
      } else {
        r += c;
      }
    }
    if (p >= s.size()) throw parse_error(101, "syntax error: unterminated string");
    ++p;
    return r;
  }
  static json parse_value(const std::string& s, size_t& p) {
    skip_ws(s, p);
    if (p >= s.size()) throw parse_error(101, "syntax error: unexpected end of input");
    json j;
    const char c = s[p];
    if (c == '{') {
      j.t_ = value_t::object;
      ++p;
      skip_ws(s, p);
      if (p < s.size() && s[p] == '}') return ++p, j;
      for (;;) {
        skip_ws(s, p);
        std::string key = parse_string(s, p);
        skip_ws(s, p);
        if (p >= s.size() || s[p] != ':') throw parse_error(101, "syntax error: expected ':'");
        ++p;
        json v = parse_value(s, p);
        bool found = false;
        for (auto& kv : j.o_)
          if (kv.first == key) kv.second = v, found = true;  // the last duplicate wins
        if (!found) j.o_.emplace_back(key, v);
        skip_ws(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == '}') { ++p; break; }
        throw parse_error(101, "syntax error: expected ',' or '}'");
      }
    } else if (c == '[') {
      j.t_ = value_t::array;
      ++p;
      skip_ws(s, p);
      if (p < s.size() && s[p] == ']') return ++p, j;
      for (;;) {
        j.a_.push_back(parse_value(s, p));
        skip_ws(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == ']') { ++p; break; }
        throw parse_error(101, "syntax error: expected ',' or ']'");
      }
    } else if (c == '"') {
      j.t_ = value_t::string;
      j.s_ = parse_string(s, p);
    } else if (c == 't') {
      expect(s, p, "true");
      j.t_ = value_t::boolean;
      j.b_ = true;
    } else if (c == 'f') {
      expect(s, p, "false");
      j.t_ = value_t::boolean;
      j.b_ = false;
    } else if (c == 'n') {
      expect(s, p, "null");
    } else {
      size_t q = p;
      bool fp = false;
      if (q < s.size() && (s[q] == '-' || s[q] == '+')) ++q;
      while (q < s.size() && ((s[q] >= '0' && s[q] <= '9') || s[q] == '.' || s[q] == 'e' || s[q] == 'E' ||
                              ((s[q] == '-' || s[q] == '+') && (s[q - 1] == 'e' || s[q - 1] == 'E')))) {
        if (s[q] == '.' || s[q] == 'e' || s[q] == 'E') fp = true;
        ++q;
      }
      if (q == p) throw parse_error(101, "syntax error: unexpected character");
      const std::string num = s.substr(p, q - p);
      p = q;
      if (fp) {
        j.t_ = value_t::number_float;
        j.d_ = strtod(num.c_str(), nullptr);
      } else {
        j.t_ = value_t::number_integer;
        j.i_ = strtoll(num.c_str(), nullptr, 10);
      }
    }
    return j;
  }
};

}  // namespace nlohmann
