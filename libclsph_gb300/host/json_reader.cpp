#include "json_reader.h"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace clsph_host {

namespace {

struct Parser {
  std::istream& in;

  int peek_nonspace() {
    int c;
    while ((c = in.peek()) != EOF && std::isspace(c)) in.get();
    return c;
  }
  [[noreturn]] void error(const std::string& what) {
    throw std::runtime_error("JSON parse error: " + what);
  }
  void expect(char c) {
    if (peek_nonspace() != c) error(std::string("expected '") + c + "'");
    in.get();
  }
  void literal(const char* word) {
    for (const char* p = word; *p; ++p)
      if (in.get() != *p) error(std::string("bad literal, expected ") + word);
  }

  std::string string_body() {
    expect('"');
    std::string out;
    for (;;) {
      int c = in.get();
      if (c == EOF) error("unterminated string");
      if (c == '"') break;
      if (c == '\\') {
        int e = in.get();
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
            char hex[5] = {0};
            for (int i = 0; i < 4; ++i) hex[i] = (char)in.get();
            unsigned code = (unsigned)std::strtoul(hex, nullptr, 16);
            if (code < 0x80) out += (char)code;
            else if (code < 0x800) { out += (char)(0xC0 | (code >> 6)); out += (char)(0x80 | (code & 0x3F)); }
            else { out += (char)(0xE0 | (code >> 12)); out += (char)(0x80 | ((code >> 6) & 0x3F)); out += (char)(0x80 | (code & 0x3F)); }
            break;
          }
          default: error("bad escape");
        }
      } else {
        out += (char)c;
      }
    }
    return out;
  }

  JsonValue value() {
    JsonValue v;
    int c = peek_nonspace();
    if (c == '{') {
      in.get();
      v.kind = JsonValue::Object;
      if (peek_nonspace() == '}') { in.get(); return v; }
      for (;;) {
        std::string key = string_body();
        expect(':');
        v.fields[key] = value();
        int d = peek_nonspace();
        in.get();
        if (d == '}') break;
        if (d != ',') error("expected ',' or '}' in object");
      }
    } else if (c == '[') {
      in.get();
      v.kind = JsonValue::Array;
      if (peek_nonspace() == ']') { in.get(); return v; }
      for (;;) {
        v.items.push_back(value());
        int d = peek_nonspace();
        in.get();
        if (d == ']') break;
        if (d != ',') error("expected ',' or ']' in array");
      }
    } else if (c == '"') {
      v.kind = JsonValue::String;
      v.text = string_body();
    } else if (c == 't') {
      literal("true");
      v.kind = JsonValue::Bool;
      v.boolean = true;
    } else if (c == 'f') {
      literal("false");
      v.kind = JsonValue::Bool;
    } else if (c == 'n') {
      literal("null");
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      std::string num;
      while ((c = in.peek()) != EOF && (std::isdigit(c) || c == '-' || c == '+' || c == '.' || c == 'e' || c == 'E'))
        num += (char)in.get();
      char* end = nullptr;
      v.number = std::strtod(num.c_str(), &end);
      if (end == num.c_str() || *end != '\0') error("bad number '" + num + "'");
      v.kind = JsonValue::Number;
    } else {
      error(c == EOF ? "unexpected end of input" : std::string("unexpected character '") + (char)c + "'");
    }
    return v;
  }
};

}  // namespace

const JsonValue& JsonValue::at(const std::string& key) const {
  if (kind != Object) throw std::runtime_error("JSON value is not an object (looking up '" + key + "')");
  auto it = fields.find(key);
  if (it == fields.end()) throw std::runtime_error("missing JSON key '" + key + "'");
  return it->second;
}

double JsonValue::as_number(const std::string& what) const {
  if (kind != Number) throw std::runtime_error("JSON key '" + what + "' is not a number");
  return number;
}

bool JsonValue::as_bool(const std::string& what) const {
  if (kind != Bool) throw std::runtime_error("JSON key '" + what + "' is not a boolean");
  return boolean;
}

JsonValue parse_json(std::istream& in) {
  Parser p{in};
  return p.value();
}

JsonValue parse_json_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open property file '" + path + "'");
  return parse_json(f);
}

}  // namespace clsph_host
