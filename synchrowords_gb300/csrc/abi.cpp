// C ABI (include/synchrowords.h).  Every entry point catches exceptions and
// turns them into status codes with a thread-local message, where the
// reference exits or throws across dlopen (app/jit.hpp:61-83).
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>
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
  std::vector<std::unique_ptr<sw::Solver>> workers;  // extra streams for sw_solve_batch
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

namespace sw {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace sw

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

namespace {

// Runs a plan on one automaton with one solver (jit/jitmain.cpp:11-49).
// Returns SW_OK or an error code; throws on device errors (caught by callers).
int run_plan(sw::Solver& solver, const uint32_t* delta, uint32_t n, uint32_t k, const sw_plan* plan, sw_result* r,
             std::string& err) {
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
  if (plan->n_algorithms > SW_MAX_ALGORITHMS) {
    err = "too many algorithms";
    return SW_ERR_CONFIG;
  }
  // After a successful Reduce the remaining algorithms see the reduced
  // automaton (app/main.cpp:60-68, jit/jitmain.cpp:21-45); only Exact can use
  // it, the others refuse and leave the bounds alone (beam.hpp:48-52,
  // brute.hpp:38-42, eppstein.hpp:38-42, reduce.hpp:34-38).
  sw::ReduceState red;
  for (uint32_t i = 0; i < plan->n_algorithms; ++i) {
    const sw_algorithm& alg = plan->algorithms[i];
    auto t0 = std::chrono::steady_clock::now();
    if (red.active && alg.kind != SW_ALGO_EXACT) {
      if (alg.kind < SW_ALGO_EXACT || alg.kind > SW_ALGO_LEARNED_BEAM) {
        err = std::string("algorithm ") + alg.name + " is outside this library's scope";
        return SW_ERR_UNSUPPORTED;
      }
    } else {
      switch (alg.kind) {
        case SW_ALGO_EXACT:
          if (red.active)
            solver.exact(red.reduced, alg.exact, b, r->stats, &red);
          else
            solver.exact(A, alg.exact, b, r->stats);
          break;
        case SW_ALGO_BEAM:
          solver.beam(A, alg.beam, b, r->stats);
          break;
        case SW_ALGO_EPPSTEIN:
          solver.eppstein(A, alg.eppstein, b, r->stats);
          break;
        case SW_ALGO_BRUTE:
          solver.brute(A, alg.brute, b, r->stats);
          break;
        case SW_ALGO_REDUCE:
          solver.reduce(A, alg.reduce, b, r->stats, red);
          break;
        case SW_ALGO_LEARNED_BEAM:
          solver.learned_beam(A, alg.learned_beam, b, r->stats);
          break;
        default:
          err = std::string("algorithm ") + alg.name + " is outside this library's scope";
          return SW_ERR_UNSUPPORTED;
      }
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
      if (r->word_capacity < b.word.size()) {
        err = "word buffer too small";
        return SW_ERR_CAPACITY;
      }
      std::memcpy(r->word, b.word.data(), sizeof(uint32_t) * b.word.size());
    }
  }
  return SW_OK;
}

}  // namespace

int sw_solve(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const sw_plan* plan, sw_result* r) {
  if (!ctx || !plan || !r) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    std::string err;
    int rc = run_plan(*ctx->solver, delta, n, k, plan, r, err);
    return rc == SW_OK ? SW_OK : fail(rc, err);
  });
}

int sw_solve_batch(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                   const char* plan_json, sw_result* results, uint32_t workers) {
  if (!ctx || !plan_json || (count && (!deltas || !ns || !ks || !results)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    if (count == 0) return SW_OK;
    std::vector<size_t> off(count + 1, 0);
    for (uint32_t i = 0; i < count; ++i) off[i + 1] = off[i] + (size_t)ns[i] * ks[i];
    if (workers == 0) workers = std::min<uint32_t>(count, 16);
    workers = std::max<uint32_t>(1, std::min<uint32_t>(workers, count));
    while (ctx->workers.size() + 1 < workers)
      ctx->workers.push_back(std::make_unique<sw::Solver>(ctx->solver->device()));
    if (ctx->solver->has_model()) {  // every worker scores with the context's distance model
      std::vector<float> model(SW_MLP_PARAMS);
      ctx->solver->get_model(model.data());
      for (uint32_t w = 1; w < workers; ++w) ctx->workers[w - 1]->set_model(model.data());
    }
    std::atomic<uint32_t> next{0};
    std::atomic<int> first_rc{SW_OK};
    std::mutex err_mu;
    std::string first_err;
    auto work = [&](sw::Solver& solver) {
      uint32_t i;
      while ((i = next++) < count && first_rc.load() == SW_OK) {
        int rc;
        std::string err;
        try {
          sw_plan plan;
          sw::plan_from_json(plan_json, ns[i], ks[i], &plan);
          rc = run_plan(solver, deltas + off[i], ns[i], ks[i], &plan, &results[i], err);
        } catch (const sw::CudaError& e) {
          rc = SW_ERR_CUDA;
          err = e.what();
        } catch (const std::invalid_argument& e) {
          rc = SW_ERR_INVALID_ARGUMENT;
          err = e.what();
        } catch (const std::exception& e) {
          rc = SW_ERR_INTERNAL;
          err = e.what();
        }
        if (rc != SW_OK) {
          std::lock_guard<std::mutex> g(err_mu);
          if (first_rc.load() == SW_OK) {
            first_rc = rc;
            first_err = "instance " + std::to_string(i) + ": " + err;
          }
        }
      }
    };
    std::vector<std::thread> th;
    for (uint32_t w = 1; w < workers; ++w) th.emplace_back(work, std::ref(*ctx->workers[w - 1]));
    work(*ctx->solver);
    for (auto& t : th) t.join();
    if (first_rc.load() != SW_OK) return fail(first_rc.load(), first_err);
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

int sw_profile_begin(sw_context* ctx) {
  if (!ctx) return fail(SW_ERR_INVALID_ARGUMENT, "NULL context");
  return guarded([&] {
    ctx->solver->profile_begin();
    return SW_OK;
  });
}

int sw_profile_end(sw_context* ctx, sw_kernel_profile out[SW_PROFILE_CLASSES]) {
  if (!ctx || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    ctx->solver->profile_end(out);
    return SW_OK;
  });
}

void* sw_context_stream(sw_context* ctx) { return ctx ? ctx->solver->stream() : nullptr; }

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

// ---- learned distance model --------------------------------------------------
int sw_context_set_model(sw_context* ctx, const float* params, uint32_t count) {
  if (!ctx || !params) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (count != SW_MLP_PARAMS) return fail(SW_ERR_INVALID_ARGUMENT, "model must have SW_MLP_PARAMS floats");
  return guarded([&] {
    ctx->solver->set_model(params);
    return SW_OK;
  });
}

int sw_context_get_model(sw_context* ctx, float* params, uint32_t count) {
  if (!ctx || !params) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (count != SW_MLP_PARAMS) return fail(SW_ERR_INVALID_ARGUMENT, "model must have SW_MLP_PARAMS floats");
  return guarded([&] {
    ctx->solver->get_model(params);
    return SW_OK;
  });
}

int sw_state_features(const uint32_t* delta, uint32_t n, uint32_t k, float* out) {
  if (!delta || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    const std::vector<float> f = sw::state_features(sw::make_automaton(delta, n, k));
    std::memcpy(out, f.data(), sizeof(float) * f.size());
    return SW_OK;
  });
}

int sw_distance_pairs(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, uint32_t per_layer,
                      uint64_t max_inverse_sets, uint64_t* sets, float* labels, uint32_t* depths, uint64_t capacity,
                      uint64_t* count, uint32_t* length) {
  if (!ctx || !delta || !count || !length || (capacity && (!sets || !labels)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    std::vector<uint64_t> s;
    std::vector<float> l;
    std::vector<uint32_t> dep;
    *length = ctx->solver->distance_pairs(sw::make_automaton(delta, n, k), per_layer, max_inverse_sets, s, l, dep);
    *count = l.size();
    if (l.size() > capacity) return fail(SW_ERR_CAPACITY, "pair buffer too small");
    std::memcpy(sets, s.data(), sizeof(uint64_t) * s.size());
    std::memcpy(labels, l.data(), sizeof(float) * l.size());
    if (depths) std::memcpy(depths, dep.data(), sizeof(uint32_t) * dep.size());
    return SW_OK;
  });
}

int sw_mlp_forward(sw_context* ctx, const float* params, const uint32_t* delta, uint32_t n, uint32_t k,
                   const uint64_t* sets, uint64_t count, float* out) {
  if (!ctx || !params || !delta || (count && (!sets || !out))) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    ctx->solver->set_model(params);
    ctx->solver->mlp_forward(sw::make_automaton(delta, n, k), sets, count, out);
    return SW_OK;
  });
}

int sw_mlp_gradient(sw_context* ctx, const float* params, const uint32_t* delta, uint32_t n, uint32_t k,
                    const uint64_t* sets, const float* labels, uint64_t count, float* grad, float* loss) {
  if (!ctx || !params || !delta || !sets || !labels || !grad || !loss || !count)
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  return guarded([&] {
    ctx->solver->set_model(params);
    *loss = ctx->solver->mlp_gradient(sw::make_automaton(delta, n, k), sets, labels, count, grad);
    return SW_OK;
  });
}

int sw_mlp_train(sw_context* ctx, float* params, uint32_t automata, const uint32_t* deltas, const uint32_t* ns,
                 const uint32_t* ks, const uint64_t* offsets, const uint64_t* sets, const float* labels,
                 uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* loss) {
  if (!ctx || !params || !deltas || !ns || !ks || !offsets || !sets || !labels || !loss)
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    std::vector<sw::Automaton> autos;
    size_t off = 0;
    for (uint32_t i = 0; i < automata; ++i) {
      autos.push_back(sw::make_automaton(deltas + off, ns[i], ks[i]));
      off += (size_t)ns[i] * ks[i];
      if (offsets[i + 1] < offsets[i]) throw std::invalid_argument("pair offsets must not decrease");
    }
    ctx->solver->set_model(params);
    *loss = ctx->solver->mlp_train(autos, offsets, sets, labels, epochs, batch, lr, seed);
    ctx->solver->get_model(params);
    return SW_OK;
  });
}

}  // extern "C"
