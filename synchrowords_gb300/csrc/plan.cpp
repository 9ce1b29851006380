// JSON plan reader and C++-semantics expression evaluator (see plan.hpp).
#include "plan.hpp"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>

namespace sw {

// ===========================================================================
// JSON
// ===========================================================================
const Json* Json::get(const std::string& key) const {
  if (type != Object) return nullptr;
  for (auto& kv : obj)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

namespace {
struct JsonParser {
  const std::string& s;
  size_t p = 0;
  explicit JsonParser(const std::string& t) : s(t) {}
  [[noreturn]] void fail(const char* what) {
    throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(p));
  }
  void ws() {
    while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
  }
  bool lit(const char* w) {
    size_t L = std::strlen(w);
    if (s.compare(p, L, w) == 0) {
      p += L;
      return true;
    }
    return false;
  }
  std::string str() {
    if (s[p] != '"') fail("expected string");
    ++p;
    std::string out;
    while (p < s.size() && s[p] != '"') {
      char c = s[p++];
      if (c == '\\') {
        if (p >= s.size()) fail("bad escape");
        char e = s[p++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            if (p + 4 > s.size()) fail("bad \\u escape");
            unsigned v = std::stoul(s.substr(p, 4), nullptr, 16);
            p += 4;
            if (v < 0x80) out += (char)v;
            else if (v < 0x800) {
              out += (char)(0xC0 | (v >> 6));
              out += (char)(0x80 | (v & 0x3F));
            } else {
              out += (char)(0xE0 | (v >> 12));
              out += (char)(0x80 | ((v >> 6) & 0x3F));
              out += (char)(0x80 | (v & 0x3F));
            }
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (p >= s.size()) fail("unterminated string");
    ++p;
    return out;
  }
  Json value() {
    ws();
    if (p >= s.size()) fail("unexpected end");
    Json j;
    char c = s[p];
    if (c == '{') {
      ++p;
      j.type = Json::Object;
      ws();
      if (s[p] == '}') {
        ++p;
        return j;
      }
      while (true) {
        ws();
        std::string key = str();
        ws();
        if (s[p] != ':') fail("expected ':'");
        ++p;
        j.obj.emplace_back(key, value());
        ws();
        if (s[p] == ',') {
          ++p;
          continue;
        }
        if (s[p] == '}') {
          ++p;
          break;
        }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      ++p;
      j.type = Json::Array;
      ws();
      if (s[p] == ']') {
        ++p;
        return j;
      }
      while (true) {
        j.arr.push_back(value());
        ws();
        if (s[p] == ',') {
          ++p;
          continue;
        }
        if (s[p] == ']') {
          ++p;
          break;
        }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      j.type = Json::String;
      j.str = str();
    } else if (lit("true")) {
      j.type = Json::Bool;
      j.b = true;
    } else if (lit("false")) {
      j.type = Json::Bool;
      j.b = false;
    } else if (lit("null")) {
      j.type = Json::Null;
    } else {
      size_t st = p;
      if (s[p] == '-' || s[p] == '+') ++p;
      bool is_int = true;
      while (p < s.size() && (std::isdigit((unsigned char)s[p]) || s[p] == '.' || s[p] == 'e' || s[p] == 'E' ||
                              s[p] == '-' || s[p] == '+')) {
        if (s[p] == '.' || s[p] == 'e' || s[p] == 'E') is_int = false;
        ++p;
      }
      if (st == p) fail("unexpected character");
      std::string t = s.substr(st, p - st);
      j.type = Json::Number;
      j.num = std::stod(t);
      j.num_is_int = is_int;
      if (is_int) j.num_int = std::stoll(t);
    }
    return j;
  }
};
}  // namespace

Json Json::parse(const std::string& text) {
  JsonParser P(text);
  Json j = P.value();
  P.ws();
  if (P.p != text.size()) P.fail("trailing characters");
  return j;
}

// ===========================================================================
// C++ expression evaluation
// ===========================================================================
double CValue::as_double() const {
  switch (kind) {
    case Double: return d;
    case UInt:
    case ULL: return (double)u;
    default: return (double)i;
  }
}
uint64_t CValue::as_u64() const {
  switch (kind) {
    case Double:
      if (d <= -1.0) return (uint64_t)(int64_t)d;
      return (uint64_t)d;
    case UInt:
    case ULL: return u;
    default: return (uint64_t)i;
  }
}
int64_t CValue::as_i64() const {
  switch (kind) {
    case Double: return (int64_t)d;
    case UInt:
    case ULL: return (int64_t)u;
    default: return i;
  }
}
bool CValue::as_bool() const {
  switch (kind) {
    case Double: return d != 0.0;
    case UInt:
    case ULL: return u != 0;
    default: return i != 0;
  }
}

namespace {

CValue mk_int(int64_t v) {
  CValue r;
  r.kind = CValue::Int;
  r.i = (int64_t)(int32_t)(uint32_t)(uint64_t)v;
  return r;
}
CValue mk_uint(uint64_t v) {
  CValue r;
  r.kind = CValue::UInt;
  r.u = (uint32_t)v;
  return r;
}
CValue mk_ll(int64_t v) {
  CValue r;
  r.kind = CValue::LL;
  r.i = v;
  return r;
}
CValue mk_ull(uint64_t v) {
  CValue r;
  r.kind = CValue::ULL;
  r.u = v;
  return r;
}
CValue mk_dbl(double v) {
  CValue r;
  r.kind = CValue::Double;
  r.d = v;
  return r;
}
CValue mk_bool(bool v) {
  CValue r;
  r.kind = CValue::Bool;
  r.i = v ? 1 : 0;
  return r;
}

// Integer promotion: bool -> int.
CValue promote(CValue v) {
  if (v.kind == CValue::Bool) return mk_int(v.i);
  return v;
}

int rank_of(CValue::Kind k) { return (k == CValue::Int || k == CValue::UInt) ? 1 : 2; }
bool is_unsigned(CValue::Kind k) { return k == CValue::UInt || k == CValue::ULL; }

// Usual arithmetic conversions for two promoted integer operands.
CValue::Kind common_int(CValue::Kind a, CValue::Kind b) {
  if (a == b) return a;
  int ra = rank_of(a), rb = rank_of(b);
  bool ua = is_unsigned(a), ub = is_unsigned(b);
  if (ua == ub) return ra >= rb ? a : b;
  CValue::Kind uk = ua ? a : b, sk = ua ? b : a;
  if (rank_of(uk) >= rank_of(sk)) return uk;
  // signed type has greater rank: long long can hold every unsigned int
  return sk;
}

CValue convert(CValue v, CValue::Kind k) {
  v = promote(v);
  switch (k) {
    case CValue::Int: return mk_int(v.as_i64());
    case CValue::UInt: return mk_uint(v.as_u64());
    case CValue::LL: return mk_ll(v.as_i64());
    case CValue::ULL: return mk_ull(v.as_u64());
    case CValue::Double: return mk_dbl(v.as_double());
    case CValue::Bool: return mk_bool(v.as_bool());
  }
  return v;
}

struct ExprParser {
  const std::string& s;
  size_t p = 0;
  uint32_t n, k;
  ExprParser(const std::string& e, uint32_t n_, uint32_t k_) : s(e), n(n_), k(k_) {}

  [[noreturn]] void fail(const std::string& what) {
    throw std::runtime_error("config expression \"" + s + "\": " + what);
  }
  void ws() {
    while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
  }
  bool eat(const char* tok) {
    ws();
    size_t L = std::strlen(tok);
    if (s.compare(p, L, tok) == 0) {
      // do not split "<<" into "<" or "&&" into "&" etc.
      if (L == 1 && p + 1 < s.size()) {
        char c = tok[0], d = s[p + 1];
        if ((c == '<' && (d == '<' || d == '=')) || (c == '>' && (d == '>' || d == '=')) ||
            (c == '&' && d == '&') || (c == '|' && d == '|') || (c == '=' && d == '=') || (c == '!' && d == '='))
          return false;
      }
      p += L;
      return true;
    }
    return false;
  }

  static CValue arith(char op, CValue a, CValue b) {
    a = promote(a);
    b = promote(b);
    if (a.kind == CValue::Double || b.kind == CValue::Double) {
      double x = a.as_double(), y = b.as_double();
      switch (op) {
        case '+': return mk_dbl(x + y);
        case '-': return mk_dbl(x - y);
        case '*': return mk_dbl(x * y);
        case '/': return mk_dbl(x / y);
        default: throw std::runtime_error("invalid operands to binary operator");
      }
    }
    CValue::Kind kk = common_int(a.kind, b.kind);
    if (is_unsigned(kk)) {
      uint64_t x = convert(a, kk).u, y = convert(b, kk).u;
      uint64_t r;
      switch (op) {
        case '+': r = x + y; break;
        case '-': r = x - y; break;
        case '*': r = x * y; break;
        case '/':
          if (!y) throw std::runtime_error("division by zero");
          r = x / y;
          break;
        case '%':
          if (!y) throw std::runtime_error("division by zero");
          r = x % y;
          break;
        case '&': r = x & y; break;
        case '|': r = x | y; break;
        case '^': r = x ^ y; break;
        default: throw std::runtime_error("bad operator");
      }
      return kk == CValue::UInt ? mk_uint(r) : mk_ull(r);
    }
    int64_t x = convert(a, kk).i, y = convert(b, kk).i;
    int64_t r;
    switch (op) {
      case '+': r = (int64_t)((uint64_t)x + (uint64_t)y); break;
      case '-': r = (int64_t)((uint64_t)x - (uint64_t)y); break;
      case '*': r = (int64_t)((uint64_t)x * (uint64_t)y); break;
      case '/':
        if (!y) throw std::runtime_error("division by zero");
        r = x / y;
        break;
      case '%':
        if (!y) throw std::runtime_error("division by zero");
        r = x % y;
        break;
      case '&': r = x & y; break;
      case '|': r = x | y; break;
      case '^': r = x ^ y; break;
      default: throw std::runtime_error("bad operator");
    }
    return kk == CValue::Int ? mk_int(r) : mk_ll(r);
  }

  static bool compare(const std::string& op, CValue a, CValue b) {
    a = promote(a);
    b = promote(b);
    int c;
    if (a.kind == CValue::Double || b.kind == CValue::Double) {
      double x = a.as_double(), y = b.as_double();
      c = x < y ? -1 : (x > y ? 1 : 0);
    } else {
      CValue::Kind kk = common_int(a.kind, b.kind);
      if (is_unsigned(kk)) {
        uint64_t x = convert(a, kk).u, y = convert(b, kk).u;
        c = x < y ? -1 : (x > y ? 1 : 0);
      } else {
        int64_t x = convert(a, kk).i, y = convert(b, kk).i;
        c = x < y ? -1 : (x > y ? 1 : 0);
      }
    }
    if (op == "<") return c < 0;
    if (op == "<=") return c <= 0;
    if (op == ">") return c > 0;
    if (op == ">=") return c >= 0;
    if (op == "==") return c == 0;
    return c != 0;
  }

  CValue number() {
    ws();
    size_t st = p;
    bool is_float = false;
    bool hex = false;
    if (s.compare(p, 2, "0x") == 0 || s.compare(p, 2, "0X") == 0) {
      hex = true;
      p += 2;
      while (p < s.size() && std::isxdigit((unsigned char)s[p])) ++p;
    } else {
      while (p < s.size() && (std::isdigit((unsigned char)s[p]) || s[p] == '.')) {
        if (s[p] == '.') is_float = true;
        ++p;
      }
      if (p < s.size() && (s[p] == 'e' || s[p] == 'E')) {
        is_float = true;
        ++p;
        if (p < s.size() && (s[p] == '+' || s[p] == '-')) ++p;
        while (p < s.size() && std::isdigit((unsigned char)s[p])) ++p;
      }
    }
    std::string body = s.substr(st, p - st);
    std::string suf;
    while (p < s.size() && std::isalpha((unsigned char)s[p])) suf += (char)std::tolower((unsigned char)s[p++]);
    if (is_float) {
      if (!suf.empty() && suf != "f" && suf != "l") fail("bad float suffix");
      return mk_dbl(std::stod(body));
    }
    uint64_t v = std::stoull(body, nullptr, hex ? 16 : 10);
    bool u = suf.find('u') != std::string::npos;
    size_t ls = 0;
    for (char c : suf)
      if (c == 'l') ++ls;
    if (u) {
      if (ls == 0 && v <= 0xffffffffULL) return mk_uint(v);
      return mk_ull(v);
    }
    if (ls == 0 && v <= 0x7fffffffULL) return mk_int((int64_t)v);
    if (ls == 0 && hex && v <= 0xffffffffULL) return mk_uint(v);
    if (v <= 0x7fffffffffffffffULL) return mk_ll((int64_t)v);
    return mk_ull(v);  // (the compiler would diagnose this; accept it)
  }

  CValue call(const std::string& fn, const std::vector<CValue>& a) {
    auto need = [&](size_t c) {
      if (a.size() != c) fail("wrong number of arguments to " + fn);
    };
    auto d0 = [&]() { return a[0].as_double(); };
    if (fn == "log2") { need(1); return mk_dbl(std::log2(d0())); }
    if (fn == "log") { need(1); return mk_dbl(std::log(d0())); }
    if (fn == "log10") { need(1); return mk_dbl(std::log10(d0())); }
    if (fn == "sqrt") { need(1); return mk_dbl(std::sqrt(d0())); }
    if (fn == "cbrt") { need(1); return mk_dbl(std::cbrt(d0())); }
    if (fn == "exp") { need(1); return mk_dbl(std::exp(d0())); }
    if (fn == "floor") { need(1); return mk_dbl(std::floor(d0())); }
    if (fn == "ceil") { need(1); return mk_dbl(std::ceil(d0())); }
    if (fn == "round") { need(1); return mk_dbl(std::round(d0())); }
    if (fn == "pow") { need(2); return mk_dbl(std::pow(a[0].as_double(), a[1].as_double())); }
    if (fn == "abs" || fn == "fabs") {
      need(1);
      CValue v = promote(a[0]);
      if (v.kind == CValue::Double || fn == "fabs") return mk_dbl(std::fabs(v.as_double()));
      if (is_unsigned(v.kind)) return v;
      return v.kind == CValue::Int ? mk_int(v.i < 0 ? -v.i : v.i) : mk_ll(v.i < 0 ? -v.i : v.i);
    }
    if (fn == "min" || fn == "max") {
      need(2);
      bool lt = compare("<", a[0], a[1]);
      return (fn == "min") == lt ? a[0] : a[1];
    }
    fail("unknown function " + fn);
  }

  CValue cast_to(const std::string& ty, CValue v) {
    if (ty == "int") return convert(v, CValue::Int);
    if (ty == "unsigned" || ty == "unsigned int" || ty == "uint" || ty == "uint32_t") return convert(v, CValue::UInt);
    if (ty == "long" || ty == "long long" || ty == "int64_t" || ty == "ssize_t") return convert(v, CValue::LL);
    if (ty == "unsigned long" || ty == "unsigned long long" || ty == "uint64_t" || ty == "size_t")
      return convert(v, CValue::ULL);
    if (ty == "double" || ty == "float" || ty == "long double") return convert(v, CValue::Double);
    if (ty == "bool") return convert(v, CValue::Bool);
    fail("unknown type " + ty);
  }

  std::string ident() {
    ws();
    size_t st = p;
    while (p < s.size() && (std::isalnum((unsigned char)s[p]) || s[p] == '_' || s[p] == ':')) ++p;
    return s.substr(st, p - st);
  }

  std::string type_name() {
    std::string t = ident();
    ws();
    while (p < s.size() && std::isalpha((unsigned char)s[p])) {
      size_t save = p;
      std::string more = ident();
      if (more == "int" || more == "long" || more == "double") {
        t += " " + more;
      } else {
        p = save;
        break;
      }
      ws();
    }
    return t;
  }

  CValue primary() {
    ws();
    if (p >= s.size()) fail("unexpected end");
    char c = s[p];
    if (c == '(') {
      // C-style cast "(type)expr" or parenthesised expression
      size_t save = p;
      ++p;
      ws();
      size_t q = p;
      std::string maybe = type_name();
      ws();
      static const char* types[] = {"int", "unsigned", "unsigned int", "long", "long long", "unsigned long",
                                    "unsigned long long", "double", "float", "bool", "size_t", "uint64_t",
                                    "int64_t", "uint32_t", "uint", "long double"};
      bool is_type = false;
      for (auto t : types)
        if (maybe == t) is_type = true;
      if (is_type && p < s.size() && s[p] == ')') {
        ++p;
        return cast_to(maybe, unary());
      }
      p = q;
      (void)save;
      CValue v = ternary();
      if (!eat(")")) fail("expected ')'");
      return v;
    }
    if (std::isdigit((unsigned char)c) || c == '.') return number();
    std::string id = ident();
    if (id.empty()) fail(std::string("unexpected character '") + c + "'");
    std::string base = id.rfind("std::", 0) == 0 ? id.substr(5) : id;
    if (base == "AUT_N") return mk_int(n);
    if (base == "AUT_K") return mk_int(k);
    if (base == "true") return mk_bool(true);
    if (base == "false") return mk_bool(false);
    if (base == "static_cast") {
      if (!eat("<")) fail("expected '<'");
      std::string ty = type_name();
      if (!eat(">")) fail("expected '>'");
      if (!eat("(")) fail("expected '('");
      CValue v = ternary();
      if (!eat(")")) fail("expected ')'");
      return cast_to(ty, v);
    }
    if (!eat("(")) fail("unknown identifier " + id);
    std::vector<CValue> args;
    if (!eat(")")) {
      while (true) {
        args.push_back(ternary());
        if (eat(")")) break;
        if (!eat(",")) fail("expected ',' or ')'");
      }
    }
    return call(base, args);
  }

  CValue unary() {
    if (eat("-")) {
      CValue v = promote(unary());
      if (v.kind == CValue::Double) return mk_dbl(-v.d);
      if (v.kind == CValue::UInt) return mk_uint((uint64_t)(-(int64_t)v.u));
      if (v.kind == CValue::ULL) return mk_ull(~v.u + 1);
      return v.kind == CValue::Int ? mk_int(-v.i) : mk_ll(-v.i);
    }
    if (eat("+")) return promote(unary());
    if (eat("!")) return mk_bool(!unary().as_bool());
    if (eat("~")) {
      CValue v = promote(unary());
      if (v.kind == CValue::Double) fail("~ on double");
      if (v.kind == CValue::UInt) return mk_uint(~v.u);
      if (v.kind == CValue::ULL) return mk_ull(~v.u);
      return v.kind == CValue::Int ? mk_int(~v.i) : mk_ll(~v.i);
    }
    return primary();
  }

  CValue mul() {
    CValue v = unary();
    while (true) {
      if (eat("*")) v = arith('*', v, unary());
      else if (eat("/")) v = arith('/', v, unary());
      else if (eat("%")) v = arith('%', v, unary());
      else return v;
    }
  }
  CValue add() {
    CValue v = mul();
    while (true) {
      if (eat("+")) v = arith('+', v, mul());
      else if (eat("-")) v = arith('-', v, mul());
      else return v;
    }
  }
  CValue shift() {
    CValue v = add();
    while (true) {
      bool left;
      if (eat("<<")) left = true;
      else if (eat(">>")) left = false;
      else return v;
      CValue r = promote(add());
      CValue a = promote(v);
      if (a.kind == CValue::Double) fail("shift of double");
      unsigned sh = (unsigned)r.as_u64();
      if (a.kind == CValue::Int) v = mk_int(left ? (int64_t)((uint32_t)a.i << sh) : (a.i >> sh));
      else if (a.kind == CValue::UInt) v = mk_uint(left ? (a.u << sh) : (a.u >> sh));
      else if (a.kind == CValue::LL) v = mk_ll(left ? (int64_t)((uint64_t)a.i << sh) : (a.i >> sh));
      else v = mk_ull(left ? (a.u << sh) : (a.u >> sh));
    }
  }
  CValue rel() {
    CValue v = shift();
    while (true) {
      const char* ops[] = {"<=", ">=", "<", ">"};
      bool any = false;
      for (auto op : ops)
        if (eat(op)) {
          v = mk_bool(compare(op, v, shift()));
          any = true;
          break;
        }
      if (!any) return v;
    }
  }
  CValue equality() {
    CValue v = rel();
    while (true) {
      if (eat("==")) v = mk_bool(compare("==", v, rel()));
      else if (eat("!=")) v = mk_bool(compare("!=", v, rel()));
      else return v;
    }
  }
  CValue bitand_() {
    CValue v = equality();
    while (eat("&")) v = arith('&', v, equality());
    return v;
  }
  CValue bitxor_() {
    CValue v = bitand_();
    while (eat("^")) v = arith('^', v, bitand_());
    return v;
  }
  CValue bitor_() {
    CValue v = bitxor_();
    while (eat("|")) v = arith('|', v, bitxor_());
    return v;
  }
  CValue logand() {
    CValue v = bitor_();
    while (eat("&&")) {
      CValue r = bitor_();
      v = mk_bool(v.as_bool() && r.as_bool());
    }
    return v;
  }
  CValue logor() {
    CValue v = logand();
    while (eat("||")) {
      CValue r = logand();
      v = mk_bool(v.as_bool() || r.as_bool());
    }
    return v;
  }
  CValue ternary() {
    CValue c = logor();
    if (eat("?")) {
      CValue a = ternary();
      if (!eat(":")) fail("expected ':'");
      CValue b = ternary();
      // result type: common type of the branches
      CValue pa = promote(a), pb = promote(b);
      CValue::Kind kk;
      if (pa.kind == CValue::Double || pb.kind == CValue::Double) kk = CValue::Double;
      else kk = common_int(pa.kind, pb.kind);
      return convert(c.as_bool() ? a : b, kk);
    }
    return c;
  }
};

}  // namespace

CValue eval_cxx_expr(const std::string& expr, uint32_t n, uint32_t k) {
  ExprParser P(expr, n, k);
  CValue v = P.ternary();
  P.ws();
  if (P.p != expr.size()) P.fail("trailing characters");
  return v;
}

// ===========================================================================
// Plan evaluation (the reference's config classes + app/jit.hpp defaults).
// ===========================================================================
namespace {

// get_str_int / get_str_bool / get_str_float (synchrolib/algorithm/config.hpp:26-55):
// a string is a C++ expression; a JSON number or bool is printed the way the
// reference prints it (std::to_string of long long / "%f" of long double /
// "true"/"false") and then read back as that literal.
enum class Key { Int, Bool, Float };

CValue value_of(const Json* cfg, const char* key, const char* def, uint32_t n, uint32_t k, Key kind = Key::Int) {
  const Json* v = cfg ? cfg->get(key) : nullptr;
  if (!v) return eval_cxx_expr(def, n, k);
  if (v->type == Json::String) return eval_cxx_expr(v->str, n, k);
  switch (kind) {
    case Key::Int:
      if (v->type == Json::Number) return eval_cxx_expr(std::to_string(v->num_is_int ? v->num_int : (int64_t)v->num), n, k);
      break;
    case Key::Bool:
      if (v->type == Json::Bool) return mk_bool(v->b);
      break;
    case Key::Float:
      if (v->type == Json::Number) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%f", v->num);
        return eval_cxx_expr(buf, n, k);
      }
      break;
  }
  throw std::runtime_error(std::string("config key ") + key + " has an unsupported type");
}

void copy_name(char* dst, const std::string& s) {
  std::memset(dst, 0, SW_NAME_LEN);
  std::strncpy(dst, s.c_str(), SW_NAME_LEN - 1);
}

}  // namespace

void plan_from_json(const std::string& text, uint32_t n, uint32_t k, sw_plan* out) {
  Json root = Json::parse(text);
  if (root.type != Json::Object) throw std::runtime_error("plan must be a JSON object");
  std::memset(out, 0, sizeof(*out));
  // app/jit.hpp:117-127
  out->upper_bound = value_of(&root, "upper_bound", "1ULL * AUT_N * AUT_N * AUT_N / 6", n, k).as_u64();
  {
    const Json* g = root.get("gpu");
    out->gpu = (g && g->type == Json::Bool) ? (g->b ? 1 : 0) : 0;
    const Json* t = root.get("threads");
    int64_t threads = 1;
    if (t) {
      if (t->type != Json::Number || !t->num_is_int) throw std::runtime_error("threads must be an integer literal");
      threads = t->num_int;
    }
    if (threads < 1 || threads > 64) throw std::runtime_error("threads must belong to range [1, 64]");
    out->threads = (uint32_t)threads;
  }
  out->gpu_max_memory_mb = value_of(&root, "gpu_max_memory_mb", "1024 * 2", n, k).as_u64();
  const Json* algos = root.get("algorithms");
  if (!algos || algos->type != Json::Array || algos->arr.empty())
    throw std::runtime_error("Need at least one algorithm");
  if (algos->arr.size() > SW_MAX_ALGORITHMS) throw std::runtime_error("too many algorithms in the plan");
  for (auto& a : algos->arr) {
    const Json* nm = a.get("name");
    if (!nm || nm->type != Json::String) throw std::runtime_error("algorithm entry without a name");
    const Json* cfg = a.get("config");
    sw_algorithm& alg = out->algorithms[out->n_algorithms++];
    copy_name(alg.name, nm->str);
    const std::string& name = nm->str;
    if (name == "Exact") {  // synchrolib/algorithm/exact/config.hpp:24-46
      alg.kind = SW_ALGO_EXACT;
      alg.exact.dfs_shortcut = value_of(cfg, "dfs_shortcut", "true", n, k, Key::Bool).as_bool();
      alg.exact.dfs = value_of(cfg, "dfs", "true", n, k, Key::Bool).as_bool();
      alg.exact.strict_memory_limit = value_of(cfg, "strict_memory_limit", "false", n, k, Key::Bool).as_bool();
      alg.exact.max_memory_mb = value_of(cfg, "max_memory_mb", "2048", n, k).as_u64();
      alg.exact.dfs_min_list_size = value_of(cfg, "dfs_min_list_size", "10000", n, k).as_u64();
      alg.exact.bfs_small_list_size = value_of(cfg, "bfs_small_list_size", "AUT_N * 16", n, k).as_u64();
      std::string red = "auto";
      if (cfg && cfg->get("reductions")) {
        const Json* r = cfg->get("reductions");
        if (r->type != Json::String) throw std::runtime_error("reductions value not in [auto, always, memory]");
        red = r->str;
      }
      if (red == "auto")
        alg.exact.reductions = SW_REDUCE_AUTO;
      else if (red == "always")
        alg.exact.reductions = SW_REDUCE_ALWAYS;
      else if (red == "memory")
        alg.exact.reductions = SW_REDUCE_MEMORY;
      else
        throw std::runtime_error("reductions value not in [auto, always, memory]");
    } else if (name == "Beam") {  // synchrolib/algorithm/beam/config.hpp:23-44
      alg.kind = SW_ALGO_BEAM;
      alg.beam.beam_size = (uint32_t)value_of(cfg, "beam_size", "std::log2(AUT_N)", n, k).as_u64();
      alg.beam.dynamic = value_of(cfg, "dynamic", "false", n, k, Key::Bool).as_bool();
      alg.beam.min_beam_size = (uint32_t)value_of(cfg, "min_beam_size", "AUT_N * std::log2(AUT_N)", n, k).as_u64();
      alg.beam.max_beam_size =
          (uint32_t)value_of(cfg, "max_beam_size", "AUT_N * AUT_N * std::log2(AUT_N)", n, k).as_u64();
      alg.beam.beam_exact_ratio = value_of(cfg, "beam_exact_ratio", "0.01", n, k, Key::Float).as_double();
      alg.beam.max_iter = value_of(cfg, "max_iter", "-1", n, k).as_i64();
      std::string presort = "none";
      if (cfg && cfg->get("presort")) {
        const Json* ps = cfg->get("presort");
        if (ps->type != Json::String) throw std::runtime_error("presort value not in [none, indeg]");
        presort = ps->str;
      }
      if (presort != "none" && presort != "indeg") throw std::runtime_error("presort value not in [none, indeg]");
      alg.beam.presort_indeg = presort == "indeg";
    } else if (name == "Brute") {  // synchrolib/algorithm/brute/config.hpp:23-27
      alg.kind = SW_ALGO_BRUTE;
      alg.brute.max_n = value_of(cfg, "max_n", "20", n, k).as_u64();
    } else if (name == "Eppstein") {  // synchrolib/algorithm/eppstein/config.hpp:23-31
      alg.kind = SW_ALGO_EPPSTEIN;
      alg.eppstein.transition_tables = value_of(cfg, "transition_tables", "false", n, k, Key::Bool).as_bool();
      alg.eppstein.find_word = value_of(cfg, "find_word", "false", n, k, Key::Bool).as_bool();
    } else if (name == "Reduce") {  // synchrolib/algorithm/reduce/config.hpp:24-32
      alg.kind = SW_ALGO_REDUCE;
      alg.reduce.min_n = value_of(cfg, "min_n", "80", n, k).as_u64();
      alg.reduce.list_size_threshold = value_of(cfg, "list_size_threshold", "AUT_N * 16", n, k).as_u64();
    } else if (name == "LearnedBeam") {  // no reference counterpart
      alg.kind = SW_ALGO_LEARNED_BEAM;
      alg.learned_beam.beam_size = value_of(cfg, "beam_size", "4096", n, k).as_u64();
      alg.learned_beam.max_iter = value_of(cfg, "max_iter", "-1", n, k).as_i64();
      std::string order = "model";
      if (cfg && cfg->get("order")) {
        const Json* o = cfg->get("order");
        if (o->type != Json::String) throw std::runtime_error("order value not in [model, size, size_model]");
        order = o->str;
      }
      if (order == "model")
        alg.learned_beam.order = SW_ORDER_MODEL;
      else if (order == "size")
        alg.learned_beam.order = SW_ORDER_SIZE;
      else if (order == "size_model")
        alg.learned_beam.order = SW_ORDER_SIZE_MODEL;
      else
        throw std::runtime_error("order value not in [model, size, size_model]");
      if (alg.learned_beam.beam_size == 0) throw std::runtime_error("LearnedBeam: beam_size must be positive");
    } else {
      throw std::runtime_error("Unknown algorithm: " + name);  // synchrolib.hpp:205
    }
  }
}

}  // namespace sw
