// Minimal JSON reader for libclsph's property files (fluid_properties/*.json,
// simulation_properties/*.json). Reads the first JSON value of a stream and
// ignores what follows it (the files end with `};`), like the stream parse of
// the picojson the reference uses in sph_simulation.cpp:409-488.
#pragma once

#include <istream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace clsph_host {

struct JsonValue {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool boolean = false;
  double number = 0.0;
  std::string text;
  std::vector<JsonValue> items;
  std::map<std::string, JsonValue> fields;

  // Object member; throws std::runtime_error naming the key when absent.
  const JsonValue& at(const std::string& key) const;
  double as_number(const std::string& what) const;
  bool as_bool(const std::string& what) const;
};

JsonValue parse_json(std::istream& in);
JsonValue parse_json_file(const std::string& path);

}  // namespace clsph_host
