// JSON model, parser and writer for the *.vxl.json scene format (see vx_json.h).
#include "vx_json.h"

#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace vxjson {

const Value* Value::member(const char* key) const {
  if (kind != OBJECT) return nullptr;
  for (const auto& kv : o)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

// ---------------------------------------------------------------------------------------------
// parser: recursive descent over RFC 8259 JSON
namespace {

struct Parser {
  const char* p;
  const char* end;
  std::string err;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  }
  bool fail(const char* what) {
    if (err.empty()) err = what;
    return false;
  }
  bool lit(const char* w) {
    size_t n = std::strlen(w);
    if ((size_t)(end - p) < n || std::memcmp(p, w, n) != 0) return fail("invalid literal");
    p += n;
    return true;
  }
  static void utf8(std::string& s, unsigned cp) {
    if (cp < 0x80) {
      s += (char)cp;
    } else if (cp < 0x800) {
      s += (char)(0xC0 | (cp >> 6));
      s += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      s += (char)(0xE0 | (cp >> 12));
      s += (char)(0x80 | ((cp >> 6) & 0x3F));
      s += (char)(0x80 | (cp & 0x3F));
    } else {
      s += (char)(0xF0 | (cp >> 18));
      s += (char)(0x80 | ((cp >> 12) & 0x3F));
      s += (char)(0x80 | ((cp >> 6) & 0x3F));
      s += (char)(0x80 | (cp & 0x3F));
    }
  }
  bool hex4(unsigned& cp) {
    if (end - p < 4) return fail("truncated \\u escape");
    cp = 0;
    for (int k = 0; k < 4; ++k) {
      char c = *p++;
      cp <<= 4;
      if (c >= '0' && c <= '9') cp |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') cp |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') cp |= (unsigned)(c - 'A' + 10);
      else return fail("bad \\u escape");
    }
    return true;
  }
  bool str(std::string& s) {
    if (p >= end || *p != '"') return fail("expected a string");
    ++p;
    while (p < end && *p != '"') {
      unsigned char c = (unsigned char)*p++;
      if (c < 0x20) return fail("control character in a string");
      if (c != '\\') {
        s += (char)c;
        continue;
      }
      if (p >= end) return fail("truncated escape");
      char e = *p++;
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
          unsigned cp;
          if (!hex4(cp)) return false;
          if (cp >= 0xD800 && cp < 0xDC00) {  // surrogate pair
            unsigned lo;
            if (end - p < 2 || p[0] != '\\' || p[1] != 'u') return fail("lone surrogate");
            p += 2;
            if (!hex4(lo) || lo < 0xDC00 || lo > 0xDFFF) return fail("bad surrogate pair");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          utf8(s, cp);
          break;
        }
        default: return fail("bad escape");
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
  bool number(Value& v) {
    const char* b = p;
    bool is_dbl = false;
    if (p < end && *p == '-') ++p;
    if (p >= end || !(*p >= '0' && *p <= '9')) return fail("bad number");
    if (*p == '0') ++p;
    else while (p < end && *p >= '0' && *p <= '9') ++p;
    if (p < end && *p == '.') {
      is_dbl = true;
      ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("bad fraction");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    if (p < end && (*p == 'e' || *p == 'E')) {
      is_dbl = true;
      ++p;
      if (p < end && (*p == '+' || *p == '-')) ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("bad exponent");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    std::string t(b, p);
    if (!is_dbl) {
      errno = 0;
      char* e = nullptr;
      long long x = std::strtoll(t.c_str(), &e, 10);
      if (errno == 0) {
        v.kind = Value::INT;
        v.i = x;
        return true;
      }
      // beyond 64 bits: a double, as rapidjson parses it
    }
    v.kind = Value::DOUBLE;
    v.d = std::strtod(t.c_str(), nullptr);
    return true;
  }
  bool value(Value& v, int depth) {
    if (depth > 512) return fail("nesting too deep");
    ws();
    if (p >= end) return fail("unexpected end");
    char c = *p;
    if (c == '{') {
      ++p;
      v.kind = Value::OBJECT;
      ws();
      if (p < end && *p == '}') { ++p; return true; }
      for (;;) {
        ws();
        std::string k;
        if (!str(k)) return false;
        ws();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        v.o.emplace_back(std::move(k), Value());
        if (!value(v.o.back().second, depth + 1)) return false;
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++p;
      v.kind = Value::ARRAY;
      ws();
      if (p < end && *p == ']') { ++p; return true; }
      for (;;) {
        v.a.emplace_back();
        if (!value(v.a.back(), depth + 1)) return false;
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v.kind = Value::STRING; return str(v.s); }
    if (c == 't') { v.kind = Value::BOOL; v.b = true; return lit("true"); }
    if (c == 'f') { v.kind = Value::BOOL; v.b = false; return lit("false"); }
    if (c == 'n') { v.kind = Value::NUL; return lit("null"); }
    return number(v);
  }
};

}  // namespace

bool parse(const std::string& text, Value& out, std::string* error) {
  Parser P{text.data(), text.data() + text.size(), {}};
  out = Value();
  bool ok = P.value(out, 0);
  if (ok) {
    P.ws();
    if (P.p != P.end) ok = P.fail("trailing characters");
  }
  if (!ok && error) *error = P.err + " at byte " + std::to_string(P.p - text.data());
  return ok;
}

// ---------------------------------------------------------------------------------------------
// number formatting: shortest round-trip digits (std::to_chars), then the layout rule
std::string format_double(double v) {
  if (std::isnan(v) || std::isinf(v)) return "null";  // not representable in JSON
  std::string sign = std::signbit(v) ? "-" : "";
  double a = std::fabs(v);
  if (a == 0.0) return sign + "0.0";
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), a, std::chars_format::scientific);
  std::string sci(buf, r.ptr);  // d[.ddd]e±XX
  size_t epos = sci.find('e');
  std::string digits;
  for (size_t k = 0; k < epos; ++k)
    if (sci[k] != '.') digits += sci[k];
  int e10 = std::atoi(sci.c_str() + epos + 1);
  // value = 0.d1d2...dn * 10^kk with kk = e10 + 1
  const int n = (int)digits.size();
  const int kk = e10 + 1;
  std::string out;
  if (kk >= n && kk <= 21) {  // integer: digits, zeros, ".0"
    out = digits + std::string(kk - n, '0') + ".0";
  } else if (kk > 0 && kk <= 21) {  // point inside the digits
    out = digits.substr(0, kk) + "." + digits.substr(kk);
  } else if (kk > -6 && kk <= 0) {  // 0.000ddd
    out = "0." + std::string(-kk, '0') + digits;
  } else {  // scientific d[.ddd]e±x
    out = digits.substr(0, 1);
    if (n > 1) out += "." + digits.substr(1);
    out += "e" + std::to_string(kk - 1);
  }
  return sign + out;
}

// ---------------------------------------------------------------------------------------------
// writer
void Writer::prefix() {
  if (stack_.empty()) return;  // the root value
  Level& L = stack_.back();
  if (L.array || L.count % 2 == 0) {  // an array element, or a key
    out_ += L.count ? ",\n" : "\n";
    indent();
  } else {  // the value after a key
    out_ += ": ";
  }
  L.count++;
}

void Writer::close(char c) {
  bool empty = stack_.back().count == 0;
  stack_.pop_back();
  if (!empty) {
    out_ += '\n';
    indent();
  }
  out_ += c;
}

void Writer::quoted(const std::string& v) {
  out_ += '"';
  for (unsigned char c : v) {
    switch (c) {
      case '"': out_ += "\\\""; break;
      case '\\': out_ += "\\\\"; break;
      case '\b': out_ += "\\b"; break;
      case '\f': out_ += "\\f"; break;
      case '\n': out_ += "\\n"; break;
      case '\r': out_ += "\\r"; break;
      case '\t': out_ += "\\t"; break;
      default:
        if (c < 0x20) {
          char h[8];
          std::snprintf(h, sizeof(h), "\\u%04X", (unsigned)c);
          out_ += h;
        } else {
          out_ += (char)c;
        }
    }
  }
  out_ += '"';
}

void Writer::key(const char* k) {
  prefix();
  quoted(k);
}
void Writer::value_double(double v) {
  prefix();
  out_ += format_double(v);
}
void Writer::value_int(long long v) {
  prefix();
  out_ += std::to_string(v);
}
void Writer::value_bool(bool v) {
  prefix();
  out_ += v ? "true" : "false";
}
void Writer::value_string(const std::string& v) {
  prefix();
  quoted(v);
}

}  // namespace vxjson
