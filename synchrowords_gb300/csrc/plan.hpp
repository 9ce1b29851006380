// Plan (config JSON) model and evaluation.
//
// The reference turns every plan value into a `#define` and lets the C++
// compiler evaluate it at JIT time (synchrolib/algorithm/config.hpp:13-55,
// app/jit.hpp:112-141; docs/config.md:7-13: "Integer and boolean parameters
// can appear ... as a string containing a valid C++ expression ... using
// <cmath> functions and AUT_N, AUT_K").  This library dispatches on runtime
// n, so it evaluates those expressions itself with C++ semantics: int /
// unsigned / long long / unsigned long long / double / bool values, the usual
// arithmetic conversions, truncating integer division and 32-bit wrap-around
// for int arithmetic.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/synchrowords.h"

namespace sw {

// ----- minimal JSON value -------------------------------------------------
struct Json {
  enum Type { Null, Bool, Number, String, Array, Object } type = Null;
  bool b = false;
  double num = 0;
  bool num_is_int = false;
  int64_t num_int = 0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;
  const Json* get(const std::string& key) const;
  static Json parse(const std::string& text);  // throws std::runtime_error
};

// ----- C++ expression evaluation ------------------------------------------
struct CValue {
  enum Kind { Bool, Int, UInt, LL, ULL, Double } kind = Int;
  int64_t i = 0;   // Bool/Int/LL (sign-extended)
  uint64_t u = 0;  // UInt/ULL
  double d = 0;    // Double
  double as_double() const;
  uint64_t as_u64() const;  // C++ conversion to uint64_t (double truncates toward zero)
  int64_t as_i64() const;
  bool as_bool() const;
};

// Evaluates `expr` with AUT_N = n and AUT_K = k as `int`.  Throws on syntax
// errors or unknown identifiers.
CValue eval_cxx_expr(const std::string& expr, uint32_t n, uint32_t k);

// Parses a plan and evaluates it for one automaton size (n, k).  Mirrors the
// defaults of the reference's config classes.  Throws std::runtime_error.
void plan_from_json(const std::string& json, uint32_t n, uint32_t k, sw_plan* out);

}  // namespace sw
