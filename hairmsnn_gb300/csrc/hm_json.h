// Minimal JSON reader for the library's two input formats: the scene config
// (parsed by the reference's parseScene, scene.cpp:119-339) and the
// tiny-cuda-nn style network config (tcnn_hairmsnn.json).  Recursive descent
// over RFC 8259 values; numbers are doubles; errors throw hm::JsonError,
// which the C ABI turns into HM_EPARSE.
#pragma once
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace hm {

struct JsonError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  bool is_null() const { return kind == Null; }
  bool is_number() const { return kind == Number; }
  bool is_string() const { return kind == String; }
  bool is_array() const { return kind == Array; }
  bool is_object() const { return kind == Object; }
  bool has(const std::string& k) const {
    if (kind != Object) return false;
    for (auto& kv : obj)
      if (kv.first == k) return true;
    return false;
  }
  const Json& operator[](const std::string& k) const {
    static const Json null_value;
    if (kind != Object) return null_value;
    for (auto& kv : obj)
      if (kv.first == k) return kv.second;
    return null_value;
  }
  const Json& operator[](size_t i) const {
    if (kind != Array || i >= arr.size()) throw JsonError("json: array index out of range");
    return arr[i];
  }
  size_t size() const { return kind == Array ? arr.size() : (kind == Object ? obj.size() : 0); }
  double as_number() const {
    if (kind == Number) return num;
    if (kind == Bool) return b ? 1.0 : 0.0;
    throw JsonError("json: expected a number");
  }
  bool as_bool() const {
    if (kind == Bool) return b;
    if (kind == Number) return num != 0.0;
    throw JsonError("json: expected a boolean");
  }
  const std::string& as_string() const {
    if (kind != String) throw JsonError("json: expected a string");
    return str;
  }
  double number_or(const std::string& k, double d) const { return has(k) ? (*this)[k].as_number() : d; }
  bool bool_or(const std::string& k, bool d) const { return has(k) ? (*this)[k].as_bool() : d; }
  std::string string_or(const std::string& k, const std::string& d) const {
    return has(k) && (*this)[k].is_string() ? (*this)[k].str : d;
  }
};

class JsonParser {
 public:
  explicit JsonParser(const char* text) : p_(text), begin_(text) {}
  Json parse() {
    Json v = value();
    ws();
    if (*p_) fail("trailing characters");
    return v;
  }

 private:
  const char* p_;
  const char* begin_;
  int depth_ = 0;

  [[noreturn]] void fail(const char* what) {
    throw JsonError(std::string("json: ") + what + " at offset " + std::to_string(p_ - begin_));
  }
  void ws() {
    while (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r') ++p_;
  }
  bool lit(const char* s) {
    size_t n = strlen(s);
    if (strncmp(p_, s, n) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }
  Json value() {
    ws();
    if (++depth_ > 256) fail("nesting too deep");
    Json v;
    char c = *p_;
    if (c == '{') {
      v.kind = Json::Object;
      ++p_;
      ws();
      if (*p_ == '}') {
        ++p_;
      } else {
        for (;;) {
          ws();
          if (*p_ != '"') fail("expected a key");
          std::string k = string();
          ws();
          if (*p_ != ':') fail("expected ':'");
          ++p_;
          v.obj.emplace_back(std::move(k), value());
          ws();
          if (*p_ == ',') { ++p_; continue; }
          if (*p_ == '}') { ++p_; break; }
          fail("expected ',' or '}'");
        }
      }
    } else if (c == '[') {
      v.kind = Json::Array;
      ++p_;
      ws();
      if (*p_ == ']') {
        ++p_;
      } else {
        for (;;) {
          v.arr.push_back(value());
          ws();
          if (*p_ == ',') { ++p_; continue; }
          if (*p_ == ']') { ++p_; break; }
          fail("expected ',' or ']'");
        }
      }
    } else if (c == '"') {
      v.kind = Json::String;
      v.str = string();
    } else if (lit("true")) {
      v.kind = Json::Bool;
      v.b = true;
    } else if (lit("false")) {
      v.kind = Json::Bool;
      v.b = false;
    } else if (lit("null")) {
      v.kind = Json::Null;
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      char* end = nullptr;
      v.kind = Json::Number;
      v.num = strtod(p_, &end);
      if (end == p_) fail("bad number");
      p_ = end;
    } else {
      fail("unexpected character");
    }
    --depth_;
    return v;
  }
  std::string string() {
    std::string s;
    ++p_;  // opening quote
    for (;;) {
      char c = *p_++;
      if (c == '\0') fail("unterminated string");
      if (c == '"') break;
      if (c == '\\') {
        char e = *p_++;
        switch (e) {
          case '"': s += '"'; break;
          case '\\': s += '\\'; break;
          case '/': s += '/'; break;
          case 'b': s += '\b'; break;
          case 'f': s += '\f'; break;
          case 'n': s += '\n'; break;
          case 'r': s += '\r'; break;
          case 't': s += '\t'; break;
          case 'u': {
            unsigned cp = 0;
            for (int i = 0; i < 4; ++i) {
              char h = *p_++;
              cp <<= 4;
              if (h >= '0' && h <= '9') cp |= h - '0';
              else if (h >= 'a' && h <= 'f') cp |= h - 'a' + 10;
              else if (h >= 'A' && h <= 'F') cp |= h - 'A' + 10;
              else fail("bad \\u escape");
            }
            if (cp < 0x80) s += (char)cp;
            else if (cp < 0x800) { s += (char)(0xC0 | (cp >> 6)); s += (char)(0x80 | (cp & 0x3F)); }
            else { s += (char)(0xE0 | (cp >> 12)); s += (char)(0x80 | ((cp >> 6) & 0x3F)); s += (char)(0x80 | (cp & 0x3F)); }
            break;
          }
          default: fail("bad escape");
        }
      } else {
        s += c;
      }
    }
    return s;
  }
};

inline Json json_parse(const char* text) {
  if (!text) throw JsonError("json: NULL text");
  return JsonParser(text).parse();
}

}  // namespace hm
