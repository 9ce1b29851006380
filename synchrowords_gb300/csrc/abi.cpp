// C ABI (include/synchrowords.h).  Every entry point catches exceptions and
// turns them into status codes with a thread-local message, where the
// reference exits or throws across dlopen (app/jit.hpp:61-83).
#include <chrono>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../../include/synchrowords.h"
#include "automaton.hpp"
#include "exact.hpp"
#include "plan.hpp"

struct sw_context {
  std::unique_ptr<sw::Solver> solver;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    g_last_error.clear();
    return f();
  } catch (const sw::CudaError& e) {
    return fail(SW_ERR_CUDA, e.what());
  } catch (const std::invalid_argument& e) {
    return fail(SW_ERR_INVALID_ARGUMENT, e.what());
  } catch (const std::bad_alloc&) {
    return fail(SW_ERR_CAPACITY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(SW_ERR_INTERNAL, e.what());
  } catch (...) {
    return fail(SW_ERR_INTERNAL, "unknown exception");
  }
}

void set_name(char* dst, const char* src) {
  std::memset(dst, 0, SW_NAME_LEN);
  std::strncpy(dst, src, SW_NAME_LEN - 1);
}

}  // namespace

extern "C" {

const char* sw_version(void) { return "synchrowords-gb300 0.1.0 (sm_103a)"; }

const char* sw_last_error(void) { return g_last_error.c_str(); }

int sw_plan_from_json(const char* json, uint32_t n, uint32_t k, sw_plan* out) {
  if (!json || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  try {
    g_last_error.clear();
    sw::plan_from_json(json, n, k, out);
    return SW_OK;
  } catch (const std::exception& e) {
    return fail(SW_ERR_CONFIG, e.what());
  }
}

int sw_eval_expression(const char* expr, uint32_t n, uint32_t k, uint64_t* as_u64, double* as_double) {
  if (!expr) return fail(SW_ERR_INVALID_ARGUMENT, "NULL expression");
  try {
    g_last_error.clear();
    sw::CValue v = sw::eval_cxx_expr(expr, n, k);
    if (as_u64) *as_u64 = v.as_u64();
    if (as_double) *as_double = v.as_double();
    return SW_OK;
  } catch (const std::exception& e) {
    return fail(SW_ERR_CONFIG, e.what());
  }
}

int sw_context_create(int device, sw_context** out) {
  if (!out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL out");
  *out = nullptr;
  return guarded([&] {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
      return fail(SW_ERR_NO_DEVICE, std::string("no CUDA device available (this library has no CPU path): ") +
                                        cudaGetErrorString(e));
    if (device < 0 || device >= count) return fail(SW_ERR_INVALID_ARGUMENT, "device index out of range");
    auto ctx = std::make_unique<sw_context>();
    ctx->solver = std::make_unique<sw::Solver>(device);
    *out = ctx.release();
    return SW_OK;
  });
}

void sw_context_destroy(sw_context* ctx) { delete ctx; }

int sw_solve(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const sw_plan* plan, sw_result* r) {
  if (!ctx || !plan || !r) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    sw::Automaton A = sw::make_automaton(delta, n, k);
    uint32_t* word_buf = r->word;
    uint32_t word_cap = r->word_capacity;
    std::memset(r, 0, sizeof(*r));
    r->word = word_buf;
    r->word_capacity = word_cap;
    // jit/jitmain.cpp:21-32 — bounds start at [0, min(UPPER_BOUND, max)]
    sw::Bounds b;
    b.lower = 0;
    b.upper = plan->upper_bound;
    if (plan->n_algorithms > SW_MAX_ALGORITHMS) return fail(SW_ERR_CONFIG, "too many algorithms");
    for (uint32_t i = 0; i < plan->n_algorithms; ++i) {
      const sw_algorithm& alg = plan->algorithms[i];
      auto t0 = std::chrono::steady_clock::now();
      switch (alg.kind) {
        case SW_ALGO_EXACT:
          ctx->solver->exact(A, alg.exact, b, r->stats);
          break;
        case SW_ALGO_BEAM:
          ctx->solver->beam(A, alg.beam, b, r->stats);
          break;
        default:
          return fail(SW_ERR_UNSUPPORTED, std::string("algorithm ") + alg.name +
                                              " is outside this library's scope (supported: Exact, Beam)");
      }
      auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
      set_name(r->runs[r->n_runs].name, alg.name);
      r->runs[r->n_runs].ms = (uint64_t)ms;
      r->n_runs++;
    }
    r->non_synchro = b.non_synchro ? 1 : 0;
    r->mlsw_lower_bound = b.lower;
    r->mlsw_upper_bound = b.upper;
    if (b.has_word && b.word.size() == b.upper && !b.non_synchro) {
      r->has_word = 1;
      r->word_len = (uint32_t)b.word.size();
      if (r->word) {
        if (r->word_capacity < b.word.size()) return fail(SW_ERR_CAPACITY, "word buffer too small");
        std::memcpy(r->word, b.word.data(), sizeof(uint32_t) * b.word.size());
      }
    }
    return SW_OK;
  });
}

int sw_solve_json(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const char* plan_json,
                  sw_result* r) {
  sw_plan plan;
  int rc = sw_plan_from_json(plan_json, n, k, &plan);
  if (rc != SW_OK) return rc;
  return sw_solve(ctx, delta, n, k, &plan, r);
}

int sw_apply_transition(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, uint32_t letter,
                        int32_t inverse, const uint64_t* from, uint64_t* to, uint64_t count) {
  if (!ctx || (count && (!from || !to))) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    sw::Automaton A = sw::make_automaton(delta, n, k);
    ctx->solver->apply_transition(A, letter, inverse != 0, from, to, count);
    return SW_OK;
  });
}

int sw_subsets_check(sw_context* ctx, uint32_t n, const uint64_t* sets, uint64_t set_count, const uint64_t* checks,
                     uint64_t check_count, int32_t proper, uint8_t* results) {
  if (!ctx || (set_count && !sets) || (check_count && (!checks || !results)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    ctx->solver->subsets_check(n, sets, set_count, checks, check_count, proper != 0, results);
    return SW_OK;
  });
}

int sw_sort_unique(sw_context* ctx, uint32_t n, uint64_t* sets, uint64_t count, uint64_t* out_count) {
  if (!ctx || !out_count || (count && !sets)) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    *out_count = ctx->solver->sort_unique(n, sets, count);
    return SW_OK;
  });
}

}  // extern "C"
