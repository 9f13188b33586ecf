// Minimal JSON reader (RFC 8259) shared by the glTF importer and the replay
// keyframe parser.  Values are kept as a tree; objects keep member order.
#pragma once
#include <charconv>
#include <cstdlib>
#include <cstring>
#include <string>
#include <system_error>
#include <utility>
#include <vector>

namespace gbr {

struct Json {
  enum Type { Null, Bool, Number, String, Array, Object } type = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  const Json* get(const char* key) const {
    if (type != Object) return nullptr;
    for (auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  double numberOr(const char* key, double def) const {
    const Json* j = get(key);
    return j && j->type == Number ? j->num : def;
  }
  const Json& operator[](size_t i) const { return arr[i]; }
  size_t size() const { return type == Array ? arr.size() : 0; }
};

struct JsonParser {
  const char* p;
  const char* end;
  std::string err;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  bool fail(const char* m) {
    if (err.empty()) err = m;
    return false;
  }
  bool parseString(std::string& s) {
    if (p >= end || *p != '"') return fail("expected string");
    ++p;
    while (p < end && *p != '"') {
      // Runs without escapes are appended whole.
      const char* q = p;
      while (q < end && *q != '"' && *q != '\\') ++q;
      s.append(p, q);
      p = q;
      if (p >= end || *p == '"') break;
      ++p;  // the backslash
      if (p >= end) return fail("bad escape");
      const char c = *p++;
      switch (c) {
        case 'n': s += '\n'; break;
        case 't': s += '\t'; break;
        case 'r': s += '\r'; break;
        case 'b': s += '\b'; break;
        case 'f': s += '\f'; break;
        case 'u': {
          if (end - p < 4) return fail("bad unicode escape");
          unsigned cp = 0;
          for (int k = 0; k < 4; ++k, ++p) {
            const char h = *p;
            const int d = h >= '0' && h <= '9' ? h - '0'
                          : h >= 'a' && h <= 'f' ? h - 'a' + 10
                          : h >= 'A' && h <= 'F' ? h - 'A' + 10 : -1;
            if (d < 0) return fail("bad unicode escape");
            cp = cp * 16 + unsigned(d);
          }
          if (cp < 0x80) {
            s += char(cp);
          } else if (cp < 0x800) {
            s += char(0xC0 | (cp >> 6));
            s += char(0x80 | (cp & 63));
          } else {
            s += char(0xE0 | (cp >> 12));
            s += char(0x80 | ((cp >> 6) & 63));
            s += char(0x80 | (cp & 63));
          }
          break;
        }
        default: s += c;
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
  bool parse(Json& j, int depth = 0) {
    if (depth > 256) return fail("nesting too deep");
    ws();
    if (p >= end) return fail("unexpected end");
    char c = *p;
    if (c == '{') {
      j.type = Json::Object;
      ++p;
      ws();
      if (p < end && *p == '}') { ++p; return true; }
      j.obj.reserve(4);
      for (;;) {
        ws();
        std::string key;
        if (!parseString(key)) return false;
        ws();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        j.obj.emplace_back(std::move(key), Json{});
        if (!parse(j.obj.back().second, depth + 1)) return false;
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      j.type = Json::Array;
      ++p;
      ws();
      if (p < end && *p == ']') { ++p; return true; }
      j.arr.reserve(4);
      for (;;) {
        j.arr.emplace_back();
        if (!parse(j.arr.back(), depth + 1)) return false;
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') {
      j.type = Json::String;
      return parseString(j.str);
    }
    if (end - p >= 4 && !std::strncmp(p, "true", 4)) { j.type = Json::Bool; j.b = true; p += 4; return true; }
    if (end - p >= 5 && !std::strncmp(p, "false", 5)) { j.type = Json::Bool; p += 5; return true; }
    if (end - p >= 4 && !std::strncmp(p, "null", 4)) { p += 4; return true; }
    const char* s = p;
    while (p < end && ((*p >= '0' && *p <= '9') || *p == '-' || *p == '+' || *p == '.' || *p == 'e' ||
                       *p == 'E'))
      ++p;
    if (s == p) return fail("unexpected character");
    j.type = Json::Number;
    // Correctly rounded and independent of the process's locale.
    const std::from_chars_result r = std::from_chars(s, p, j.num);
    if (r.ec == std::errc::result_out_of_range) {
      j.num = std::strtod(std::string(s, p).c_str(), nullptr);  // overflow / underflow
      return true;
    }
    if (r.ec != std::errc() || r.ptr != p) return fail("bad number");
    return true;
  }
};

}  // namespace gbr
