// json.hpp -- a small strict JSON reader for the microlc driver's input file.
//
// The reference reads its input with jsoncpp (src/driver.cpp:31-35), which is not a
// dependency of this library.  This reader accepts RFC 8259 JSON plus the // and /* */
// comments that jsoncpp's default reader allows, and reports the first error with its
// line and column.  Values are a plain tree; object member order is kept.  Lookups of a
// missing member or element give a shared null value (as jsoncpp's operator[] does), and
// the typed getters of the driver (microlc.cpp) turn that into an error naming the key.
#ifndef MLC_DRIVER_JSON_HPP
#define MLC_DRIVER_JSON_HPP

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace mlcjson {

struct Value {
  enum Type { Null, Bool, Number, String, Array, Object };
  Type type = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  static const Value& null() {
    static const Value v;
    return v;
  }
  bool is_null() const { return type == Null; }
  bool has(const std::string& k) const {
    if (type != Object) return false;
    for (const auto& m : obj)
      if (m.first == k) return true;
    return false;
  }
  const Value& operator[](const std::string& k) const {
    if (type == Object)
      for (const auto& m : obj)
        if (m.first == k) return m.second;
    return null();
  }
  const Value& operator[](size_t i) const { return (type == Array && i < arr.size()) ? arr[i] : null(); }
  size_t size() const { return type == Array ? arr.size() : type == Object ? obj.size() : 0; }
  static const char* type_name(Type t) {
    switch (t) {
      case Null: return "null";
      case Bool: return "a boolean";
      case Number: return "a number";
      case String: return "a string";
      case Array: return "an array";
      default: return "an object";
    }
  }
};

struct ParseError : std::runtime_error {
  int line, col;
  ParseError(const std::string& what, int l, int c)
      : std::runtime_error("line " + std::to_string(l) + ", column " + std::to_string(c) + ": " + what),
        line(l),
        col(c) {}
};

class Parser {
 public:
  explicit Parser(const std::string& text) : s_(text) {}

  Value parse_document() {
    Value v = value(0);
    skip();
    if (p_ != s_.size()) fail("unexpected text after the top-level value");
    return v;
  }

 private:
  static constexpr int kMaxDepth = 200;
  const std::string& s_;
  size_t p_ = 0;

  [[noreturn]] void fail(const std::string& what) const {
    int line = 1, col = 1;
    for (size_t i = 0; i < p_ && i < s_.size(); i++) {
      if (s_[i] == '\n') {
        line++;
        col = 1;
      } else {
        col++;
      }
    }
    throw ParseError(what, line, col);
  }
  bool at_end() const { return p_ >= s_.size(); }
  char peek() const { return at_end() ? '\0' : s_[p_]; }

  void skip() {
    while (!at_end()) {
      const char c = s_[p_];
      if (c == ' ' || c == '\t' || c == '\n' || c == '\r') {
        p_++;
      } else if (c == '/' && p_ + 1 < s_.size() && s_[p_ + 1] == '/') {
        while (!at_end() && s_[p_] != '\n') p_++;
      } else if (c == '/' && p_ + 1 < s_.size() && s_[p_ + 1] == '*') {
        const size_t e = s_.find("*/", p_ + 2);
        if (e == std::string::npos) fail("unterminated comment");
        p_ = e + 2;
      } else {
        break;
      }
    }
  }

  void expect_word(const char* w) {
    for (const char* q = w; *q; q++, p_++)
      if (peek() != *q) fail(std::string("invalid literal (expected '") + w + "')");
  }

  Value value(int depth) {
    if (depth > kMaxDepth) fail("nesting deeper than 200 levels");
    skip();
    if (at_end()) fail("unexpected end of input (expected a value)");
    Value v;
    const char c = peek();
    if (c == '{') {
      v.type = Value::Object;
      p_++;
      skip();
      if (peek() == '}') {
        p_++;
        return v;
      }
      for (;;) {
        skip();
        if (peek() != '"') fail("expected a member name in double quotes");
        std::string key = string_body();
        for (const auto& m : v.obj)
          if (m.first == key) fail("duplicate member \"" + key + "\"");
        skip();
        if (peek() != ':') fail("expected ':' after a member name");
        p_++;
        v.obj.emplace_back(std::move(key), value(depth + 1));
        skip();
        if (peek() == ',') {
          p_++;
          continue;
        }
        if (peek() == '}') {
          p_++;
          return v;
        }
        fail(at_end() ? "unexpected end of input (object not closed)" : "expected ',' or '}' in an object");
      }
    }
    if (c == '[') {
      v.type = Value::Array;
      p_++;
      skip();
      if (peek() == ']') {
        p_++;
        return v;
      }
      for (;;) {
        v.arr.push_back(value(depth + 1));
        skip();
        if (peek() == ',') {
          p_++;
          continue;
        }
        if (peek() == ']') {
          p_++;
          return v;
        }
        fail(at_end() ? "unexpected end of input (array not closed)" : "expected ',' or ']' in an array");
      }
    }
    if (c == '"') {
      v.type = Value::String;
      v.str = string_body();
      return v;
    }
    if (c == 't') {
      expect_word("true");
      v.type = Value::Bool;
      v.b = true;
      return v;
    }
    if (c == 'f') {
      expect_word("false");
      v.type = Value::Bool;
      return v;
    }
    if (c == 'n') {
      expect_word("null");
      return v;
    }
    if (c == '-' || (c >= '0' && c <= '9')) {
      v.type = Value::Number;
      v.num = number();
      return v;
    }
    fail(std::string("unexpected character '") + c + "'");
  }

  // RFC 8259 number grammar, converted with strtod (the C locale's '.').
  double number() {
    const size_t b = p_;
    auto digits = [&] {
      const size_t d = p_;
      while (peek() >= '0' && peek() <= '9') p_++;
      return p_ - d;
    };
    if (peek() == '-') p_++;
    if (peek() == '0') {
      p_++;
    } else if (digits() == 0) {
      fail("invalid number");
    }
    if (peek() == '.') {
      p_++;
      if (digits() == 0) fail("invalid number (digits expected after '.')");
    }
    if (peek() == 'e' || peek() == 'E') {
      p_++;
      if (peek() == '+' || peek() == '-') p_++;
      if (digits() == 0) fail("invalid number (exponent digits expected)");
    }
    const std::string tok = s_.substr(b, p_ - b);
    const double x = std::strtod(tok.c_str(), nullptr);
    if (!std::isfinite(x)) {
      p_ = b;
      fail("number out of range: " + tok);
    }
    return x;
  }

  unsigned hex4() {
    unsigned u = 0;
    for (int i = 0; i < 4; i++, p_++) {
      const char h = peek();
      u <<= 4;
      if (h >= '0' && h <= '9') u |= (unsigned)(h - '0');
      else if (h >= 'a' && h <= 'f') u |= (unsigned)(h - 'a' + 10);
      else if (h >= 'A' && h <= 'F') u |= (unsigned)(h - 'A' + 10);
      else fail("invalid \\u escape");
    }
    return u;
  }

  static void put_utf8(std::string& o, unsigned cp) {
    if (cp < 0x80) {
      o += (char)cp;
    } else if (cp < 0x800) {
      o += (char)(0xC0 | (cp >> 6));
      o += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      o += (char)(0xE0 | (cp >> 12));
      o += (char)(0x80 | ((cp >> 6) & 0x3F));
      o += (char)(0x80 | (cp & 0x3F));
    } else {
      o += (char)(0xF0 | (cp >> 18));
      o += (char)(0x80 | ((cp >> 12) & 0x3F));
      o += (char)(0x80 | ((cp >> 6) & 0x3F));
      o += (char)(0x80 | (cp & 0x3F));
    }
  }

  std::string string_body() {
    p_++;  // opening quote
    std::string o;
    for (;;) {
      if (at_end()) fail("unterminated string");
      const unsigned char c = (unsigned char)s_[p_];
      if (c == '"') {
        p_++;
        return o;
      }
      if (c < 0x20) fail("control character in a string");
      if (c != '\\') {
        o += (char)c;
        p_++;
        continue;
      }
      p_++;
      const char e = peek();
      p_++;
      switch (e) {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u': {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00) {
            if (peek() != '\\' || p_ + 1 >= s_.size() || s_[p_ + 1] != 'u') fail("unpaired surrogate in \\u escape");
            p_ += 2;
            const unsigned lo = hex4();
            if (lo < 0xDC00 || lo >= 0xE000) fail("invalid low surrogate in \\u escape");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          } else if (cp >= 0xDC00 && cp < 0xE000) {
            fail("unpaired surrogate in \\u escape");
          }
          put_utf8(o, cp);
          break;
        }
        default:
          p_--;
          fail("invalid escape in a string");
      }
    }
  }
};

inline Value parse(const std::string& text) { return Parser(text).parse_document(); }

}  // namespace mlcjson

#endif
