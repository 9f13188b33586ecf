// Native unit test of the JSON reader shared by the glTF importer and the
// replay keyframe parser: numbers are read correctly rounded and without the
// process locale, escapes decode, and malformed documents fail.
#include <clocale>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "json.h"

using gbr::Json;
using gbr::JsonParser;

static int failures = 0;
#define CHECK(c)                                                                   \
  do {                                                                             \
    if (!(c)) {                                                                    \
      std::fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                                  \
    }                                                                              \
  } while (0)

static bool parse(const std::string& s, Json& j, std::string* err = nullptr) {
  JsonParser p{s.data(), s.data() + s.size(), {}};
  const bool ok = p.parse(j);
  if (err) *err = p.err;
  return ok;
}

int main() {
  // A locale with a decimal comma must not change how numbers read.
  std::setlocale(LC_NUMERIC, "de_DE.UTF-8");
  Json j;
  CHECK(parse("[0.1, -2.5e-3, 1e400, -1e400, 4.9e-324, 123456789012345678, -0.0, 3]", j));
  CHECK(j.type == Json::Array && j.size() == 8);
  if (j.size() == 8) {
    CHECK(j[0].num == 0.1);
    CHECK(j[1].num == -2.5e-3);
    CHECK(std::isinf(j[2].num) && j[2].num > 0);
    CHECK(std::isinf(j[3].num) && j[3].num < 0);
    CHECK(j[4].num == 4.9e-324);
    CHECK(j[5].num == 123456789012345678.0);
    CHECK(j[6].num == 0.0 && std::signbit(j[6].num));
    CHECK(j[7].num == 3.0);
  }
  CHECK(parse("{\"a\\u0041\\n\\\"b\": \"x\\\\y\\u00e9\", \"k\": [true, false, null]}", j));
  CHECK(j.type == Json::Object && j.obj.size() == 2);
  if (j.obj.size() == 2) {
    CHECK(j.obj[0].first == "aA\n\"b");
    CHECK(j.obj[0].second.str == "x\\y\xc3\xa9");
    const Json* k = j.get("k");
    CHECK(k && k->size() == 3 && (*k)[0].b && !(*k)[1].b && (*k)[2].type == Json::Null);
  }
  std::string err;
  Json bad;
  CHECK(!parse("[1.2.3]", bad, &err) && err == "bad number");
  CHECK(!parse("{\"a\": [1, 2}", bad));
  CHECK(!parse("\"unterminated", bad, &err) && err == "unterminated string");
  CHECK(!parse("\"\\u12\"", bad));
  CHECK(!parse("", bad, &err) && err == "unexpected end");
  std::string deep(300, '[');
  CHECK(!parse(deep, bad, &err) && err == "nesting too deep");
  // An embedded NUL is not part of a number.
  const std::string nul("[1\0]", 4);
  CHECK(!parse(nul, bad));
  if (failures) {
    std::fprintf(stderr, "%d failures\n", failures);
    return 1;
  }
  std::puts("json ok");
  return 0;
}
