// Minimal JSON DOM for the reference's scene files (the reference reads them
// with nlohmann-json through ConfigNode, rad.core/include/rad/core/config_node.h).
// Errors carry line:column and raise JsonError (mapped to RAD_ERR_JSON).
#pragma once
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace rad {

struct JsonError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Wrong type / missing key in a well-formed document (RadArgumentException in
// the reference's ConfigNode).
struct ConfigError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct JValue {
  enum Type { kNull, kBool, kNum, kStr, kArr, kObj } type = kNull;
  bool b = false;
  double n = 0;
  std::string s;
  std::vector<JValue> a;
  std::vector<std::pair<std::string, JValue>> o;

  const JValue* get(const char* key) const {
    if (type != kObj) return nullptr;
    for (const auto& kv : o)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  bool has(const char* key) const { return get(key) != nullptr; }
  bool isNum() const { return type == kNum; }
  bool isArr() const { return type == kArr; }
  bool isObj() const { return type == kObj; }
  bool isStr() const { return type == kStr; }
};

class JsonReader {
 public:
  static JValue Parse(const std::string& text) {
    JsonReader r(text);
    JValue v = r.Value(0);
    r.Skip();
    if (r.pos_ != text.size()) r.Fail("unexpected trailing characters");
    return v;
  }

 private:
  explicit JsonReader(const std::string& t) : t_(t) {}
  const std::string& t_;
  size_t pos_ = 0;

  [[noreturn]] void Fail(const std::string& what) const {
    size_t line = 1, col = 1;
    for (size_t i = 0; i < pos_ && i < t_.size(); i++) {
      if (t_[i] == '\n') {
        line++;
        col = 1;
      } else {
        col++;
      }
    }
    throw JsonError("json " + std::to_string(line) + ":" + std::to_string(col) + ": " + what);
  }
  void Skip() {
    while (pos_ < t_.size()) {
      char c = t_[pos_];
      if (c == ' ' || c == '\n' || c == '\r' || c == '\t') {
        pos_++;
      } else {
        break;
      }
    }
  }
  bool Lit(const char* w) {
    size_t n = std::char_traits<char>::length(w);
    if (t_.compare(pos_, n, w) == 0) {
      pos_ += n;
      return true;
    }
    return false;
  }
  JValue Value(int depth) {
    if (depth > 256) Fail("nesting too deep");
    Skip();
    if (pos_ >= t_.size()) Fail("unexpected end of input");
    JValue v;
    char c = t_[pos_];
    if (c == '{') {
      v.type = JValue::kObj;
      pos_++;
      Skip();
      if (pos_ < t_.size() && t_[pos_] == '}') {
        pos_++;
        return v;
      }
      for (;;) {
        Skip();
        if (pos_ >= t_.size() || t_[pos_] != '"') Fail("expected a key string");
        std::string key = Str();
        Skip();
        if (pos_ >= t_.size() || t_[pos_] != ':') Fail("expected ':'");
        pos_++;
        v.o.emplace_back(std::move(key), Value(depth + 1));
        Skip();
        if (pos_ < t_.size() && t_[pos_] == ',') {
          pos_++;
          continue;
        }
        if (pos_ < t_.size() && t_[pos_] == '}') {
          pos_++;
          break;
        }
        Fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      v.type = JValue::kArr;
      pos_++;
      Skip();
      if (pos_ < t_.size() && t_[pos_] == ']') {
        pos_++;
        return v;
      }
      for (;;) {
        v.a.push_back(Value(depth + 1));
        Skip();
        if (pos_ < t_.size() && t_[pos_] == ',') {
          pos_++;
          continue;
        }
        if (pos_ < t_.size() && t_[pos_] == ']') {
          pos_++;
          break;
        }
        Fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      v.type = JValue::kStr;
      v.s = Str();
    } else if (Lit("true")) {
      v.type = JValue::kBool;
      v.b = true;
    } else if (Lit("false")) {
      v.type = JValue::kBool;
      v.b = false;
    } else if (Lit("null")) {
      v.type = JValue::kNull;
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      const char* begin = t_.c_str() + pos_;
      char* end = nullptr;
      v.n = std::strtod(begin, &end);
      if (end == begin) Fail("malformed number");
      v.type = JValue::kNum;
      pos_ += size_t(end - begin);
    } else {
      Fail(std::string("unexpected character '") + c + "'");
    }
    return v;
  }
  std::string Str() {
    std::string out;
    pos_++;
    while (pos_ < t_.size() && t_[pos_] != '"') {
      char c = t_[pos_++];
      if (c == '\\') {
        if (pos_ >= t_.size()) Fail("unterminated escape");
        char e = t_[pos_++];
        switch (e) {
          case 'n': out.push_back('\n'); break;
          case 't': out.push_back('\t'); break;
          case 'r': out.push_back('\r'); break;
          case 'b': out.push_back('\b'); break;
          case 'f': out.push_back('\f'); break;
          case 'u': {
            if (pos_ + 4 > t_.size()) Fail("bad \\u escape");
            unsigned cp = (unsigned)std::strtoul(t_.substr(pos_, 4).c_str(), nullptr, 16);
            pos_ += 4;
            if (cp < 0x80) {
              out.push_back((char)cp);
            } else if (cp < 0x800) {
              out.push_back((char)(0xc0 | (cp >> 6)));
              out.push_back((char)(0x80 | (cp & 0x3f)));
            } else {
              out.push_back((char)(0xe0 | (cp >> 12)));
              out.push_back((char)(0x80 | ((cp >> 6) & 0x3f)));
              out.push_back((char)(0x80 | (cp & 0x3f)));
            }
            break;
          }
          default: out.push_back(e); break;
        }
      } else {
        out.push_back(c);
      }
    }
    if (pos_ >= t_.size()) Fail("unterminated string");
    pos_++;
    return out;
  }
};

}  // namespace rad
