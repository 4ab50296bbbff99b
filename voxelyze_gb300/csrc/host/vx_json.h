// Minimal JSON document model, parser and pretty writer for the *.vxl.json scene format of
// CVoxelyze::loadJSON / saveJSON (src/Voxelyze.cpp:61-241, src/VX_Material.cpp:75-160).
//
// The reference parses and writes with rapidjson (a header-only dependency vendored in its tree).
// Its reader tests value kinds with rapidjson's rules, which this model keeps: a number written
// with a fraction or an exponent is a double, otherwise an integer (is_double() is false for an
// integer literal, as rapidjson's IsDouble()); get_double() converts either.  The writer emits the
// layout of rapidjson's PrettyWriter with its default settings (four-space indent, one array
// element per line, "key": value, "[]" and "{}" for empty containers) and doubles in the shortest
// form that reads back to the same double, laid out by the rule rapidjson's dtoa applies (plain
// decimal with at least one fractional digit for decimal exponents -6 < e <= 21, else d.ddde±x).
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace vxjson {

struct Value {
  enum Kind { NUL, BOOL, INT, DOUBLE, STRING, ARRAY, OBJECT };
  Kind kind = NUL;
  bool b = false;
  long long i = 0;    // INT
  double d = 0;       // DOUBLE
  std::string s;      // STRING
  std::vector<Value> a;                              // ARRAY
  std::vector<std::pair<std::string, Value>> o;      // OBJECT, in file order

  bool is_object() const { return kind == OBJECT; }
  bool is_array() const { return kind == ARRAY; }
  bool is_string() const { return kind == STRING; }
  bool is_bool() const { return kind == BOOL; }
  bool is_double() const { return kind == DOUBLE; }
  // an integer that fits a 32-bit int (rapidjson's IsInt)
  bool is_int() const { return kind == INT && i >= INT32_MIN && i <= INT32_MAX; }
  bool is_number() const { return kind == INT || kind == DOUBLE; }
  double get_double() const { return kind == DOUBLE ? d : (double)i; }
  int get_int() const { return kind == INT ? (int)i : (int)d; }
  bool get_bool() const { return b; }
  size_t size() const { return kind == ARRAY ? a.size() : o.size(); }
  const Value* member(const char* key) const;  // nullptr when absent or not an object
};

// Parses a complete JSON text; returns false (with a message) on a syntax error.
bool parse(const std::string& text, Value& out, std::string* error = nullptr);

// Writer with the layout described above.  Calls mirror rapidjson's Writer interface.
class Writer {
 public:
  void start_object() { prefix(); out_ += '{'; stack_.push_back({false, 0}); }
  void end_object() { close('}'); }
  void start_array() { prefix(); out_ += '['; stack_.push_back({true, 0}); }
  void end_array() { close(']'); }
  void key(const char* k);
  void value_double(double v);
  void value_int(long long v);
  void value_bool(bool v);
  void value_string(const std::string& v);
  const std::string& str() const { return out_; }

 private:
  struct Level {
    bool array;
    int count;  // values (arrays) or keys + values (objects) written so far
  };
  void prefix();
  void close(char c);
  void indent() { out_.append(4 * stack_.size(), ' '); }
  void quoted(const std::string& v);
  std::string out_;
  std::vector<Level> stack_;
};

// The shortest decimal form of v that reads back to v, laid out as the writer emits it.
std::string format_double(double v);

}  // namespace vxjson
