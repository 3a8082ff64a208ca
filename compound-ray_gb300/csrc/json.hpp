// Minimal JSON reader for glTF 2.0 ASCII files.
//
// Only what a .gltf scene needs: objects, arrays, strings (with \uXXXX escapes
// folded to UTF-8), numbers (kept as double), booleans and null.  Parse errors
// throw std::runtime_error with the byte offset; the C ABI turns them into a
// status code and an error string.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cr {

class Json {
 public:
  enum Type { Null, Bool, Number, String, Array, Object };

  Json() = default;
  Type type() const { return type_; }
  bool isNull() const { return type_ == Null; }
  bool isBool() const { return type_ == Bool; }
  bool isNumber() const { return type_ == Number; }
  bool isString() const { return type_ == String; }
  bool isArray() const { return type_ == Array; }
  bool isObject() const { return type_ == Object; }

  bool asBool() const { return b_; }
  double asNumber() const { return n_; }
  const std::string& asString() const { return s_; }
  const std::vector<Json>& items() const { return a_; }
  const std::map<std::string, Json>& members() const { return o_; }
  size_t size() const { return type_ == Array ? a_.size() : (type_ == Object ? o_.size() : 0); }

  // Member lookup; returns a shared null value when absent or not an object.
  const Json& operator[](const std::string& key) const {
    if (type_ != Object) return nullValue();
    auto it = o_.find(key);
    return it == o_.end() ? nullValue() : it->second;
  }
  const Json& operator[](size_t i) const {
    if (type_ != Array || i >= a_.size()) return nullValue();
    return a_[i];
  }
  bool has(const std::string& key) const { return type_ == Object && o_.count(key) != 0; }

  double num(const std::string& key, double dflt) const {
    const Json& v = (*this)[key];
    return v.isNumber() ? v.n_ : dflt;
  }
  int integer(const std::string& key, int dflt) const {
    const Json& v = (*this)[key];
    return v.isNumber() ? static_cast<int>(v.n_) : dflt;
  }
  std::string str(const std::string& key, const std::string& dflt = "") const {
    const Json& v = (*this)[key];
    return v.isString() ? v.s_ : dflt;
  }

  static Json parse(const std::string& text) {
    Parser p{text, 0};
    p.skipWs();
    Json v = p.value(0);
    p.skipWs();
    if (p.pos != text.size()) p.fail("trailing characters after JSON document");
    return v;
  }

 private:
  static const Json& nullValue() {
    static const Json n;
    return n;
  }

  Type type_ = Null;
  bool b_ = false;
  double n_ = 0.0;
  std::string s_;
  std::vector<Json> a_;
  std::map<std::string, Json> o_;

  struct Parser {
    const std::string& t;
    size_t pos;

    [[noreturn]] void fail(const char* what) const {
      throw std::runtime_error(std::string("JSON parse error at byte ") + std::to_string(pos) + ": " + what);
    }
    void skipWs() {
      while (pos < t.size() && (t[pos] == ' ' || t[pos] == '\n' || t[pos] == '\r' || t[pos] == '\t')) ++pos;
    }
    bool consume(const char* lit) {
      size_t n = 0;
      while (lit[n]) ++n;
      if (t.compare(pos, n, lit) == 0) {
        pos += n;
        return true;
      }
      return false;
    }
    Json value(int depth) {
      if (depth > 512) fail("nesting too deep");
      if (pos >= t.size()) fail("unexpected end of input");
      Json v;
      const char c = t[pos];
      if (c == '{') {
        v.type_ = Object;
        ++pos;
        skipWs();
        if (pos < t.size() && t[pos] == '}') {
          ++pos;
          return v;
        }
        for (;;) {
          skipWs();
          if (pos >= t.size() || t[pos] != '"') fail("expected object key");
          std::string key = string();
          skipWs();
          if (pos >= t.size() || t[pos] != ':') fail("expected ':'");
          ++pos;
          skipWs();
          v.o_[key] = value(depth + 1);
          skipWs();
          if (pos < t.size() && t[pos] == ',') {
            ++pos;
            continue;
          }
          if (pos < t.size() && t[pos] == '}') {
            ++pos;
            return v;
          }
          fail("expected ',' or '}'");
        }
      }
      if (c == '[') {
        v.type_ = Array;
        ++pos;
        skipWs();
        if (pos < t.size() && t[pos] == ']') {
          ++pos;
          return v;
        }
        for (;;) {
          skipWs();
          v.a_.push_back(value(depth + 1));
          skipWs();
          if (pos < t.size() && t[pos] == ',') {
            ++pos;
            continue;
          }
          if (pos < t.size() && t[pos] == ']') {
            ++pos;
            return v;
          }
          fail("expected ',' or ']'");
        }
      }
      if (c == '"') {
        v.type_ = String;
        v.s_ = string();
        return v;
      }
      if (consume("true")) {
        v.type_ = Bool;
        v.b_ = true;
        return v;
      }
      if (consume("false")) {
        v.type_ = Bool;
        v.b_ = false;
        return v;
      }
      if (consume("null")) return v;
      if (c == '-' || (c >= '0' && c <= '9')) {
        const char* begin = t.c_str() + pos;
        char* end = nullptr;
        v.type_ = Number;
        v.n_ = std::strtod(begin, &end);
        if (end == begin) fail("bad number");
        pos += static_cast<size_t>(end - begin);
        return v;
      }
      fail("unexpected character");
    }
    static void appendUtf8(std::string& out, uint32_t cp) {
      if (cp < 0x80) {
        out += static_cast<char>(cp);
      } else if (cp < 0x800) {
        out += static_cast<char>(0xC0 | (cp >> 6));
        out += static_cast<char>(0x80 | (cp & 0x3F));
      } else if (cp < 0x10000) {
        out += static_cast<char>(0xE0 | (cp >> 12));
        out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
        out += static_cast<char>(0x80 | (cp & 0x3F));
      } else {
        out += static_cast<char>(0xF0 | (cp >> 18));
        out += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
        out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
        out += static_cast<char>(0x80 | (cp & 0x3F));
      }
    }
    uint32_t hex4() {
      if (pos + 4 > t.size()) fail("short \\u escape");
      uint32_t v = 0;
      for (int i = 0; i < 4; ++i) {
        const char h = t[pos++];
        v <<= 4;
        if (h >= '0' && h <= '9') v |= static_cast<uint32_t>(h - '0');
        else if (h >= 'a' && h <= 'f') v |= static_cast<uint32_t>(h - 'a' + 10);
        else if (h >= 'A' && h <= 'F') v |= static_cast<uint32_t>(h - 'A' + 10);
        else fail("bad hex digit");
      }
      return v;
    }
    std::string string() {
      ++pos;  // opening quote
      std::string out;
      while (pos < t.size()) {
        const char c = t[pos++];
        if (c == '"') return out;
        if (c != '\\') {
          out += c;
          continue;
        }
        if (pos >= t.size()) break;
        const char e = t[pos++];
        switch (e) {
          case '"': out += '"'; break;
          case '\\': out += '\\'; break;
          case '/': out += '/'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'n': out += '\n'; break;
          case 'r': out += '\r'; break;
          case 't': out += '\t'; break;
          case 'u': {
            uint32_t cp = hex4();
            if (cp >= 0xD800 && cp < 0xDC00 && pos + 1 < t.size() && t[pos] == '\\' && t[pos + 1] == 'u') {
              pos += 2;
              const uint32_t lo = hex4();
              cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            }
            appendUtf8(out, cp);
            break;
          }
          default: fail("bad escape");
        }
      }
      fail("unterminated string");
    }
  };
};

}  // namespace cr
