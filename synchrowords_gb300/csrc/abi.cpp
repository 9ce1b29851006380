// C ABI (include/synchrowords.h).  Every entry point catches exceptions and
// turns them into status codes with a thread-local message, where the
// reference exits or throws across dlopen (app/jit.hpp:61-83).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <thread>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../../include/synchrowords.h"
#include "automaton.hpp"
#include "algos.cuh"
#include "exact.hpp"
#include "plan.hpp"

// Device state of the batched launches (batch_small.cu, batch_cluster.cu).
struct SmallBatchState {
  cudaStream_t stream = nullptr;
  sw::DevBuf inst, delta, seeds, results, words, origins, visited, counter;
  // cluster launch: tag counter, control blocks and per-cluster regions; the
  // regions' hash tables must start zero-filled (tag 0 = empty slot)
  sw::DevBuf c_scratch, c_stats;
  size_t c_zeroed = 0;       // bytes of c_scratch zero-filled since its allocation
  uint64_t c_tags_used = 0;  // upper bound on the tags taken since the last zero fill
  sw_batch_profile last{};
  // CUDA graphs of recent device rounds, keyed by everything their launches
  // bake in (buffers, per-width counts, cluster geometry): a batch of a shape
  // seen before replays its round with one graph launch
  std::vector<std::pair<std::vector<uint64_t>, cudaGraphExec_t>> graphs;
  ~SmallBatchState() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct sw_context {
  std::unique_ptr<sw::Solver> solver;
  std::vector<std::unique_ptr<sw::Solver>> workers;  // extra streams for sw_solve_batch
  SmallBatchState small;
  sw_batch_tuning tuning{0, 104.0, 0, 160.0};  // sw_autotune_batch / sw_set_batch_tuning
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
  } catch (const std::length_error& e) {
    return fail(SW_ERR_CAPACITY, e.what());
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

namespace {

// One device round of sw_solve_batch: the automata of `small` (shared-memory
// launch) and `cluster` (cluster launch), each by set width, uploaded once and
// launched per width on the batch stream; finish_round() waits for it.
struct DeviceRound {
  std::vector<uint32_t> order;  // slot -> instance
  std::vector<uint8_t> engine;  // per slot: 0 shared-memory launch, 1 cluster launch
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  int launches = 0;
  uint32_t word_stride = 1024;
  bool active = false;
  bool replayed = false;  // launched from a graph captured for an earlier batch of the same shape
};

void start_round(sw_context* ctx, DeviceRound& D, const std::vector<uint32_t> small[4],
                 const std::vector<uint32_t> cluster[4], const uint32_t* deltas, const std::vector<size_t>& off,
                 const uint32_t* ns, const uint32_t* ks, const std::vector<std::vector<uint32_t>>& seeds,
                 const std::vector<uint32_t>& max_len) {
  SmallBatchState& S = ctx->small;
  size_t total = 0;
  for (int c = 0; c < 4; ++c) total += small[c].size() + cluster[c].size();
  if (!total) return;
  SW_CUDA(cudaSetDevice(ctx->solver->device()));
  if (!S.stream) SW_CUDA(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
  std::vector<sw::SmallInstance> inst;
  std::vector<uint8_t> dpool, spool;
  size_t class_start[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < 8; ++c) {
    class_start[c] = inst.size();
    for (uint32_t i : (c < 4 ? small[c] : cluster[c - 4])) {
      sw::SmallInstance I{ns[i], ks[i], (uint32_t)dpool.size(), (uint32_t)spool.size(), (uint32_t)seeds[i].size(),
                          std::min<uint32_t>(max_len[i], D.word_stride)};
      for (size_t e = 0; e < (size_t)ns[i] * ks[i]; ++e) dpool.push_back((uint8_t)deltas[off[i] + e]);
      for (uint32_t q : seeds[i]) spool.push_back((uint8_t)q);
      inst.push_back(I);
      D.order.push_back(i);
      D.engine.push_back(c < 4 ? 0 : 1);
    }
  }
  class_start[8] = inst.size();
  S.inst.reserve(sizeof(sw::SmallInstance) * inst.size());
  S.delta.reserve(std::max<size_t>(dpool.size(), 1));
  S.seeds.reserve(std::max<size_t>(spool.size(), 1));
  S.results.reserve(sizeof(sw::SmallResult) * inst.size());
  S.words.reserve((size_t)D.word_stride * inst.size());
  S.counter.reserve(sizeof(uint32_t) * 2);
  const uint32_t blocks = (uint32_t)sw::small_batch_blocks();
  size_t ow = 0, vw = 0;
  for (int c = 0; c < 4; ++c)
    if (!small[c].empty()) {
      ow = std::max(ow, sw::small_batch_origin_words(c + 1, blocks));
      vw = std::max(vw, sw::small_batch_visited_words(c + 1, blocks));
    }
  if (ow) S.origins.reserve(sizeof(uint32_t) * ow);
  if (vw) S.visited.reserve(sizeof(uint64_t) * vw);
  // cluster launch geometry and scratch
  const int cs = ctx->tuning.cluster_size > 0 ? std::min<int>(ctx->tuning.cluster_size, 16) : 8;
  const sw::ClusterCaps caps = sw::cluster_default_caps();
  uint32_t clusters[4] = {0, 0, 0, 0};
  uint32_t max_clusters = 0;
  for (int c = 0; c < 4; ++c)
    if (!cluster[c].empty()) {
      clusters[c] = std::min<uint32_t>({(uint32_t)cluster[c].size(), sw::cluster_batch_max_clusters(c + 1, cs),
                                        sw::cluster_max_clusters_supported()});
      if (!clusters[c]) throw std::runtime_error("cluster launch: no cluster of this size fits on the device");
      max_clusters = std::max(max_clusters, clusters[c]);
    }
  if (max_clusters) {
    const size_t need = sw::cluster_scratch_bytes(max_clusters, caps);
    uint64_t tags = 0;
    for (int c = 0; c < 4; ++c) tags += sw::cluster_tags_per_launch((uint32_t)cluster[c].size());
    if (S.c_scratch.cap < need) {
      S.c_scratch.reserve(need);
      S.c_zeroed = 0;
    }
    if (S.c_zeroed < S.c_scratch.cap || S.c_tags_used + tags >= 0xF0000000ull) {
      // new memory, or the tag counter could wrap: every slot back to "empty"
      SW_CUDA(cudaMemsetAsync(S.c_scratch.p, 0, S.c_scratch.cap, S.stream));
      S.c_zeroed = S.c_scratch.cap;
      S.c_tags_used = 0;
    }
    S.c_tags_used += tags;
    S.c_stats.reserve(sizeof(uint64_t) * 9);
  }
  SW_CUDA(cudaMemcpyAsync(S.inst.p, inst.data(), sizeof(sw::SmallInstance) * inst.size(), cudaMemcpyHostToDevice,
                          S.stream));
  SW_CUDA(cudaMemcpyAsync(S.delta.p, dpool.data(), dpool.size(), cudaMemcpyHostToDevice, S.stream));
  SW_CUDA(cudaMemcpyAsync(S.seeds.p, spool.data(), spool.size(), cudaMemcpyHostToDevice, S.stream));
  SW_CUDA(cudaEventCreate(&D.t0));
  SW_CUDA(cudaEventCreate(&D.t1));
  // the round's device work: the cluster statistics reset and one persistent
  // launch per non-empty class
  auto issue = [&] {
    if (max_clusters) SW_CUDA(cudaMemsetAsync(S.c_stats.p, 0, sizeof(uint64_t) * 9, S.stream));
    for (int c = 0; c < 8; ++c) {
      const size_t a = class_start[c], b = class_start[c + 1];
      if (a == b) continue;
      const int W = c % 4 + 1;
      if (c < 4)
        sw::launch_small_batch(W, S.inst.as<sw::SmallInstance>() + a, (uint32_t)(b - a), S.delta.as<uint8_t>(),
                               S.seeds.as<uint8_t>(), S.results.as<sw::SmallResult>() + a,
                               S.words.as<uint8_t>() + a * D.word_stride, D.word_stride, S.origins.as<uint32_t>(),
                               S.visited.as<sw::u64>(), blocks, S.counter.as<uint32_t>(), S.stream);
      else
        sw::launch_cluster_batch(W, cs, clusters[c - 4], S.inst.as<sw::SmallInstance>() + a, (uint32_t)(b - a),
                                 S.delta.as<uint8_t>(), S.seeds.as<uint8_t>(), S.results.as<sw::SmallResult>() + a,
                                 S.words.as<uint8_t>() + a * D.word_stride, D.word_stride, S.c_scratch.p, caps,
                                 S.counter.as<uint32_t>(), S.c_stats.as<sw::u64>(), S.stream);
    }
  };
  for (int c = 0; c < 8; ++c) D.launches += class_start[c] != class_start[c + 1];
  std::vector<uint64_t> key{(uint64_t)cs, blocks, D.word_stride, (uint64_t)(uintptr_t)S.inst.p,
                            (uint64_t)(uintptr_t)S.delta.p, (uint64_t)(uintptr_t)S.seeds.p,
                            (uint64_t)(uintptr_t)S.results.p, (uint64_t)(uintptr_t)S.words.p,
                            (uint64_t)(uintptr_t)S.origins.p, (uint64_t)(uintptr_t)S.visited.p,
                            (uint64_t)(uintptr_t)S.counter.p, (uint64_t)(uintptr_t)S.c_scratch.p,
                            (uint64_t)(uintptr_t)S.c_stats.p};
  for (int c = 0; c < 9; ++c) key.push_back(class_start[c]);
  for (int c = 0; c < 4; ++c) key.push_back(clusters[c]);
  cudaGraphExec_t exec = nullptr;
  for (auto& g : S.graphs)
    if (g.first == key) exec = g.second;
  if (!exec) {
    // the kernels' attributes are set before the capture (not a stream operation)
    sw::small_batch_prepare();
    cudaGraph_t graph = nullptr;
    SW_CUDA(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
    try {
      issue();
    } catch (...) {
      cudaStreamEndCapture(S.stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    SW_CUDA(cudaStreamEndCapture(S.stream, &graph));
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    SW_CUDA(e);
    if (S.graphs.size() >= 4) {  // keep the four most recent shapes
      cudaGraphExecDestroy(S.graphs.front().second);
      S.graphs.erase(S.graphs.begin());
    }
    S.graphs.emplace_back(std::move(key), exec);
  } else {
    D.replayed = true;
  }
  SW_CUDA(cudaEventRecord(D.t0, S.stream));
  SW_CUDA(cudaGraphLaunch(exec, S.stream));
  SW_CUDA(cudaEventRecord(D.t1, S.stream));
  D.active = true;
}

// Waits for a round, verifies and stores what it solved; returns the
// instances it did not finish (those of the shared-memory launch go to
// *unfinished_small when given).
std::vector<uint32_t> finish_round(sw_context* ctx, DeviceRound& D, const uint32_t* deltas,
                                   const std::vector<size_t>& off, const uint32_t* ns, const uint32_t* ks,
                                   const std::map<std::pair<uint32_t, uint32_t>, sw_plan>& plans, sw_result* results,
                                   std::vector<uint32_t>* unfinished_small, bool verbose) {
  std::vector<uint32_t> again;
  if (!D.active) return again;
  SmallBatchState& S = ctx->small;
  const size_t m = D.order.size();
  std::vector<sw::SmallResult> R(m);
  std::vector<uint8_t> words((size_t)D.word_stride * m);
  uint64_t cst[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  SW_CUDA(cudaMemcpyAsync(R.data(), S.results.p, sizeof(sw::SmallResult) * m, cudaMemcpyDeviceToHost, S.stream));
  SW_CUDA(cudaMemcpyAsync(words.data(), S.words.p, words.size(), cudaMemcpyDeviceToHost, S.stream));
  const bool any_cluster = std::find(D.engine.begin(), D.engine.end(), 1) != D.engine.end();
  if (any_cluster) SW_CUDA(cudaMemcpyAsync(cst, S.c_stats.p, sizeof(cst), cudaMemcpyDeviceToHost, S.stream));
  SW_CUDA(cudaStreamSynchronize(S.stream));
  float ms = 0;
  SW_CUDA(cudaEventElapsedTime(&ms, D.t0, D.t1));
  cudaEventDestroy(D.t0);
  cudaEventDestroy(D.t1);
  D.active = false;
  sw_batch_profile& P = S.last;
  P.device_ms += ms;
  P.launches += (uint32_t)D.launches;
  P.graph_replays += D.replayed ? 1u : 0u;
  P.meet_pairs += cst[0];
  P.children += cst[1];
  P.staged_bytes += cst[2];
  P.steps += cst[3];
  bool first = true;
  size_t st[2][3] = {{0, 0, 0}, {0, 0, 0}};
  std::map<std::pair<int, uint32_t>, size_t> over;  // (engine, capacity) -> automata
  for (size_t t = 0; t < m; ++t) {
    const uint32_t i = D.order[t];
    st[D.engine[t]][std::min<uint32_t>(R[t].status, 2)]++;
    if (R[t].status != 0) {
      if (R[t].status == 1) over[{D.engine[t], R[t].why & 255u}]++;
      if (D.engine[t] == 0 && unfinished_small)
        unfinished_small->push_back(i);
      else
        again.push_back(i);
      continue;
    }
    sw_result* r = &results[i];
    uint32_t* wb = r->word;
    const uint32_t cap = r->word_capacity;
    std::memset(r, 0, sizeof(*r));
    r->word = wb;
    r->word_capacity = cap;
    std::vector<uint32_t> word(words.begin() + t * D.word_stride,
                               words.begin() + t * D.word_stride + R[t].word_len);
    const sw::Automaton A = sw::make_automaton(deltas + off[i], ns[i], ks[i]);
    if (word.size() != R[t].length || sw::apply_word(A, word).size() != 1)
      throw std::runtime_error("internal: batched word does not synchronize");
    r->mlsw_lower_bound = r->mlsw_upper_bound = R[t].length;
    r->has_word = 1;
    r->word_len = R[t].length;
    if (wb) {
      if (cap < word.size()) throw std::length_error("instance " + std::to_string(i) + ": word buffer too small");
      std::memcpy(wb, word.data(), sizeof(uint32_t) * word.size());
    }
    const sw_plan& p = plans.at(std::make_pair(ns[i], ks[i]));
    std::strncpy(r->runs[0].name, p.algorithms[0].name, SW_NAME_LEN - 1);
    r->runs[0].ms = 0;
    r->n_runs = 1;
    r->stats.device_ms = ms / (double)m;
    if (first) {
      r->stats.kernel_launches = (uint64_t)D.launches;  // the round's launches, counted once
      r->stats.meet_pairs = cst[0];
      r->stats.subsets_expanded = cst[1];
    }
    first = false;
    if (D.engine[t] == 0)
      P.small_solved++;
    else
      P.cluster_solved++;
  }
  if (verbose) {
    for (const auto& kv : over)
      std::fprintf(stderr, "[sw] %s launch: capacity %u: %zu automata\n", kv.first.first ? "cluster" : "batched",
                   kv.first.second, kv.second);
    std::fprintf(stderr,
                 "[sw] device round: %zu automata in %d launches, %.3f ms; batched launch %zu solved / %zu over "
                 "capacity / %zu unfinished; cluster launch %zu / %zu / %zu\n",
                 m, D.launches, (double)ms, st[0][0], st[0][1], st[0][2], st[1][0], st[1][1], st[1][2]);
    if (any_cluster)
      std::fprintf(stderr, "[sw] cluster launch cycles (rank 0, summed over automata): expand %.3g, dedup %.3g, "
                   "visited insert %.3g, meet %.3g, result %.3g\n", (double)cst[4], (double)cst[5],
                   (double)cst[6], (double)cst[7], (double)cst[8]);
  }
  return again;
}

}  // namespace

int sw_solve_batch(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                   const char* plan_json, sw_result* results, uint32_t workers) {
  if (!ctx || !plan_json || (count && (!deltas || !ns || !ks || !results)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    ctx->small.last = sw_batch_profile{};
    if (count == 0) return SW_OK;
    std::vector<size_t> off(count + 1, 0);
    for (uint32_t i = 0; i < count; ++i) off[i + 1] = off[i] + (size_t)ns[i] * ks[i];
    if (workers == 0) workers = ctx->tuning.workers ? ctx->tuning.workers : std::min<uint32_t>(count, 16);
    workers = std::max<uint32_t>(1, std::min<uint32_t>(workers, count));
    using clk = std::chrono::steady_clock;
    const bool verbose = std::getenv("SYNCHRO_BATCH_VERBOSE") != nullptr;
    const auto h0 = clk::now();
    auto since = [&](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
    // every worker that runs an instance scores with the context's distance model (copied on first use)
    bool model_copied = !ctx->solver->has_model();
    auto copy_model = [&](uint32_t nw) {
      if (model_copied) return;
      std::vector<float> model(SW_MLP_PARAMS);
      ctx->solver->get_model(model.data());
      for (uint32_t w = 1; w < nw; ++w) ctx->workers[w - 1]->set_model(model.data());
      model_copied = true;
    };
    // Automata whose plan is a plain Exact run are searched on the device
    // without host round trips: the smallest by the shared-memory launch
    // (batch_small.cu), the others by the cluster launch (batch_cluster.cu).
    // What neither finishes, and every other automaton, runs on the worker
    // streams.
    const bool cluster_on = ctx->tuning.cluster_size >= 0;
    std::vector<uint32_t> streamed, small[4], cluster[4];
    std::map<std::pair<uint32_t, uint32_t>, sw_plan> plans;
    std::vector<std::vector<uint32_t>> seeds(count);
    std::vector<uint32_t> max_len(count, 0);
    for (uint32_t i = 0; i < count; ++i) {
      const uint32_t n = ns[i], k = ks[i];
      bool ok = n >= 2 && n <= 256 && k >= 1 && k <= 16 && n * k <= 4096;
      if (ok) {
        auto key = std::make_pair(n, k);
        auto it = plans.find(key);
        if (it == plans.end()) {
          sw_plan p;
          sw::plan_from_json(plan_json, n, k, &p);
          it = plans.emplace(key, p).first;
        }
        const sw_plan& p = it->second;
        ok = p.n_algorithms == 1 && p.algorithms[0].kind == SW_ALGO_EXACT && p.upper_bound >= 1;
        if (ok) {
          // No synchronisation test here: the device searches report a length
          // only when their two sides meet, which proves a reset word; an
          // automaton without one ends over capacity or unfinished and the
          // streamed path settles it.
          const sw::Automaton A = sw::make_automaton(deltas + off[i], n, k);
          seeds[i] = sw::backward_seeds(A);
          std::sort(seeds[i].begin(), seeds[i].end());
          ok = !seeds[i].empty();
          // plain Exact with no word behind the bound searches lengths up to the bound
          max_len[i] = (uint32_t)std::min<uint64_t>(p.upper_bound, 1024);
        }
      }
      const bool small_ok = ok && k <= 4 && (double)n * std::log2((double)k) <= ctx->tuning.batched_limit;
      if (small_ok)
        small[(n - 1) / 64].push_back(i);
      else if (ok && cluster_on && (double)n * std::log2((double)std::max(k, 2u)) <= ctx->tuning.cluster_limit)
        cluster[(n - 1) / 64].push_back(i);
      else
        streamed.push_back(i);
    }
    const double ms_classify = since(h0);
    DeviceRound round1;
    start_round(ctx, round1, small, cluster, deltas, off, ns, ks, seeds, max_len);
    std::atomic<int> first_rc{SW_OK};
    std::mutex err_mu;
    std::string first_err;
    auto run_pool = [&](const std::vector<uint32_t>& todo) {
      if (todo.empty()) return;
      const uint32_t nw = std::min<uint32_t>(workers, (uint32_t)todo.size());
      while (ctx->workers.size() + 1 < nw) ctx->workers.push_back(std::make_unique<sw::Solver>(ctx->solver->device()));
      for (auto& w : ctx->workers) w->set_scan_shapes(ctx->solver->scan_shapes());
      ctx->small.last.streamed += (uint32_t)todo.size();
      std::atomic<size_t> next{0};
      auto work = [&](sw::Solver& solver) {
        size_t t;
        while ((t = next++) < todo.size() && first_rc.load() == SW_OK) {
          const uint32_t i = todo[t];
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
      copy_model(nw);
      std::vector<std::thread> th;
      for (uint32_t w = 1; w < nw; ++w) th.emplace_back(work, std::ref(*ctx->workers[w - 1]));
      work(*ctx->solver);
      for (auto& t : th) t.join();
    };
    const double ms_launch = since(h0) - ms_classify;
    const auto h1 = clk::now();
    run_pool(streamed);
    const double ms_streamed = since(h1);
    const auto h2 = clk::now();
    // what the shared-memory launch leaves gets a cluster round before the streams
    std::vector<uint32_t> small_left;
    std::vector<uint32_t> again = finish_round(ctx, round1, deltas, off, ns, ks, plans, results,
                                               cluster_on ? &small_left : nullptr, verbose);
    if (!small_left.empty()) {
      std::vector<uint32_t> none[4], second[4];
      for (uint32_t i : small_left) second[(ns[i] - 1) / 64].push_back(i);
      DeviceRound round2;
      start_round(ctx, round2, none, second, deltas, off, ns, ks, seeds, max_len);
      std::vector<uint32_t> left = finish_round(ctx, round2, deltas, off, ns, ks, plans, results, nullptr, verbose);
      again.insert(again.end(), left.begin(), left.end());
    }
    const double ms_device = since(h2);
    if (verbose)
      std::fprintf(stderr, "[sw] batch of %u: host classify %.3f ms, upload+launch %.3f ms, streamed %.3f ms, "
                   "device rounds %.3f ms, %zu left for the streams\n", count, ms_classify, ms_launch, ms_streamed,
                   ms_device, again.size());
    run_pool(again);
    if (first_rc.load() != SW_OK) return fail(first_rc.load(), first_err);
    return SW_OK;
  });
}

int sw_batch_last_profile(sw_context* ctx, sw_batch_profile* out) {
  if (!ctx || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = ctx->small.last;
  return SW_OK;
}

int sw_get_batch_tuning(sw_context* ctx, sw_batch_tuning* out) {
  if (!ctx || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = ctx->tuning;
  return SW_OK;
}

int sw_set_batch_tuning(sw_context* ctx, const sw_batch_tuning* in) {
  if (!ctx || !in) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  ctx->tuning = *in;
  return SW_OK;
}

int sw_autotune_batch(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                      const char* plan_json, sw_result* results, const uint32_t* worker_candidates,
                      uint32_t n_workers, const double* limit_candidates, uint32_t n_limits, uint32_t reps,
                      double* ms, sw_batch_tuning* best) {
  if (!ctx || !plan_json || (count && (!deltas || !ns || !ks || !results)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (count == 0) return fail(SW_ERR_INVALID_ARGUMENT, "empty batch");
  static const uint32_t kWorkers[4] = {8, 12, 16, 24};
  static const double kLimits[3] = {-1.0, 104.0, 1024.0};
  if (!worker_candidates) {
    worker_candidates = kWorkers;
    n_workers = 4;
  }
  if (!limit_candidates) {
    limit_candidates = kLimits;
    n_limits = 3;
  }
  if (n_workers == 0 || n_limits == 0) return fail(SW_ERR_INVALID_ARGUMENT, "empty candidate list");
  reps = std::max<uint32_t>(reps, 1);
  const sw_batch_tuning saved = ctx->tuning;
  // wall-clock time of the batch under tuning t (best of reps)
  auto run = [&](const sw_batch_tuning& t, double& out) -> int {
    ctx->tuning = t;
    for (uint32_t r = 0; r < reps; ++r) {
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = sw_solve_batch(ctx, count, deltas, ns, ks, plan_json, results, 0);
      if (rc != SW_OK) return rc;
      const double ms_run = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (r == 0 || ms_run < out) out = ms_run;
    }
    return SW_OK;
  };
  sw_batch_tuning cur = saved, top = saved;
  double top_ms = 0;
  bool have = false;
  for (uint32_t c = 0; c < n_workers; ++c) {
    cur.workers = std::max<uint32_t>(1, std::min<uint32_t>(worker_candidates[c], count));
    double t = 0;
    const int rc = run(cur, t);
    if (rc != SW_OK) {
      ctx->tuning = saved;
      return rc;
    }
    if (ms) ms[c] = t;
    if (!have || t < top_ms) {
      top_ms = t;
      top = cur;
      have = true;
    }
  }
  cur = top;
  const sw_batch_tuning first = top;
  const double first_ms = top_ms;
  for (uint32_t c = 0; c < n_limits; ++c) {
    cur.batched_limit = limit_candidates[c];
    if (cur.batched_limit == first.batched_limit) {  // measured in the first pass
      if (ms) ms[n_workers + c] = first_ms;
      continue;
    }
    double t = 0;
    const int rc = run(cur, t);
    if (rc != SW_OK) {
      ctx->tuning = saved;
      return rc;
    }
    if (ms) ms[n_workers + c] = t;
    if (t < top_ms) {
      top_ms = t;
      top = cur;
    }
  }
  ctx->tuning = top;
  if (best) *best = top;
  return SW_OK;
}

int sw_autotune_cluster(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                        const char* plan_json, sw_result* results, const int32_t* size_candidates, uint32_t n_sizes,
                        const double* limit_candidates, uint32_t n_limits, uint32_t reps, double* ms,
                        sw_batch_tuning* best) {
  if (!ctx || !plan_json || (count && (!deltas || !ns || !ks || !results)))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (count == 0) return fail(SW_ERR_INVALID_ARGUMENT, "empty batch");
  static const int32_t kSizes[4] = {2, 4, 8, 16};
  static const double kLimits[4] = {-1.0, 128.0, 160.0, 200.0};
  if (!size_candidates) {
    size_candidates = kSizes;
    n_sizes = 4;
  }
  if (!limit_candidates) {
    limit_candidates = kLimits;
    n_limits = 4;
  }
  if (n_sizes == 0 || n_limits == 0) return fail(SW_ERR_INVALID_ARGUMENT, "empty candidate list");
  for (uint32_t c = 0; c < n_sizes; ++c)
    if (size_candidates[c] < 1 || size_candidates[c] > 16) return fail(SW_ERR_INVALID_ARGUMENT, "cluster size must be 1..16");
  reps = std::max<uint32_t>(reps, 1);
  const sw_batch_tuning saved = ctx->tuning;
  auto run = [&](const sw_batch_tuning& t, double& out) -> int {
    ctx->tuning = t;
    for (uint32_t r = 0; r < reps; ++r) {
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = sw_solve_batch(ctx, count, deltas, ns, ks, plan_json, results, 0);
      if (rc != SW_OK) return rc;
      const double ms_run = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (r == 0 || ms_run < out) out = ms_run;
    }
    return SW_OK;
  };
  // coordinate descent: cluster size with the current limit, then the limit
  sw_batch_tuning cur = saved, top = saved;
  double top_ms = 0;
  bool have = false;
  for (uint32_t c = 0; c < n_sizes; ++c) {
    cur.cluster_size = size_candidates[c];
    double t = 0;
    const int rc = run(cur, t);
    if (rc != SW_OK) {
      ctx->tuning = saved;
      return rc;
    }
    if (ms) ms[c] = t;
    if (!have || t < top_ms) {
      top_ms = t;
      top = cur;
      have = true;
    }
  }
  cur = top;
  const double first_limit = top.cluster_limit, first_ms = top_ms;
  for (uint32_t c = 0; c < n_limits; ++c) {
    cur.cluster_limit = limit_candidates[c];
    if (cur.cluster_limit == first_limit) {  // measured in the first pass
      if (ms) ms[n_sizes + c] = first_ms;
      continue;
    }
    double t = 0;
    const int rc = run(cur, t);
    if (rc != SW_OK) {
      ctx->tuning = saved;
      return rc;
    }
    if (ms) ms[n_sizes + c] = t;
    if (t < top_ms) {
      top_ms = t;
      top = cur;
    }
  }
  ctx->tuning = top;
  if (best) *best = top;
  return SW_OK;
}

int sw_solve_json(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const char* plan_json,
                  sw_result* r) {
  sw_plan plan;
  int rc = sw_plan_from_json(plan_json, n, k, &plan);
  if (rc != SW_OK) return rc;
  return sw_solve(ctx, delta, n, k, &plan, r);
}

namespace {
constexpr int kKeys = 8 * sw::kScanSizeClasses;  // (words - 1) * size classes + size class
bool to_shape(const sw_scan_shape& in, sw::ScanShape& out) {
  out.tile_rows = in.tile_rows;
  out.warps = in.warps;
  out.tiles_per_super = in.tiles_per_super;
  out.grid_factor = in.grid_factor;
  return true;
}
sw_scan_shape from_shape(const sw::ScanShape& s) {
  sw_scan_shape o;
  o.tile_rows = s.tile_rows;
  o.warps = s.warps;
  o.tiles_per_super = s.tiles_per_super;
  o.grid_factor = s.grid_factor;
  return o;
}
void set_shapes(sw_context* ctx, const sw::ScanShapes& s) {
  ctx->solver->set_scan_shapes(s);
  for (auto& w : ctx->workers) w->set_scan_shapes(s);
}
}  // namespace

int sw_get_scan_shape(sw_context* ctx, uint32_t words, uint32_t size_class, sw_scan_shape* out) {
  if (!ctx || !out) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (words < 1 || words > 8 || size_class >= SW_SCAN_SIZE_CLASSES)
    return fail(SW_ERR_INVALID_ARGUMENT, "words must be 1..8 and size_class 0..1");
  *out = from_shape(ctx->solver->scan_shapes().s[words - 1][size_class]);
  return SW_OK;
}

int sw_scan_shape_check(uint32_t words, const sw_scan_shape* shape) {
  if (!shape) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (words < 1 || words > 8) return fail(SW_ERR_INVALID_ARGUMENT, "words must be 1..8");
  sw::ScanShape sh;
  to_shape(*shape, sh);
  if (!sw::scan_shape_valid((int)words, sh))
    return fail(SW_ERR_INVALID_ARGUMENT,
                "scan shape: tile_rows 32/64/128, warps 4/8/16, tiles_per_super 4/8/16/32, grid_factor 1..64, "
                "and two tiles per warp within the shared-memory limit");
  g_last_error.clear();
  return SW_OK;
}

int sw_set_scan_shape(sw_context* ctx, uint32_t words, uint32_t size_class, const sw_scan_shape* in) {
  if (!ctx || !in) return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (words < 1 || words > 8 || size_class >= SW_SCAN_SIZE_CLASSES)
    return fail(SW_ERR_INVALID_ARGUMENT, "words must be 1..8 and size_class 0..1");
  const int rc = sw_scan_shape_check(words, in);
  if (rc != SW_OK) return rc;
  sw::ScanShape sh;
  to_shape(*in, sh);
  sw::ScanShapes all = ctx->solver->scan_shapes();
  all.s[words - 1][size_class] = sh;
  set_shapes(ctx, all);
  return SW_OK;
}

int sw_autotune_scan(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                     const char* plan_json, uint32_t reps, sw_scan_tuned* out, uint32_t out_cap,
                     uint32_t* out_count) {
  if (!ctx || (count && (!deltas || !ns || !ks)) || (out_cap && !out))
    return fail(SW_ERR_INVALID_ARGUMENT, "NULL argument");
  if (count == 0) return fail(SW_ERR_INVALID_ARGUMENT, "empty batch");
  if (out_count) *out_count = 0;
  reps = std::max<uint32_t>(reps, 1);
  const char* json = plan_json ? plan_json : "{\"algorithms\": [{\"name\": \"Exact\"}]}";
  std::vector<sw_plan> plans(count);
  std::vector<size_t> off(count + 1, 0);
  for (uint32_t i = 0; i < count; ++i) {
    const int rc = sw_plan_from_json(json, ns[i], ks[i], &plans[i]);
    if (rc != SW_OK) return rc;
    off[i + 1] = off[i] + (size_t)ns[i] * ks[i];
  }
  const sw::ScanShapes start = ctx->solver->scan_shapes();
  bool profiling = false;
  // a failed tuning leaves the context as it found it: its starting shapes,
  // profiling off
  auto restore = [&] {
    set_shapes(ctx, start);
    if (profiling) {
      profiling = false;
      try {
        sw_kernel_profile drop[SW_PROFILE_CLASSES];
        ctx->solver->profile_end(drop);
      } catch (...) {
      }
    }
  };
  return guarded([&] {
    try {
      // one timed pass: every automaton through the context's solver with the
      // subset checks timed per key; per key the best of `reps` passes
      auto pass = [&](double ms[kKeys], uint64_t checks[kKeys]) -> int {
        for (int i = 0; i < kKeys; ++i) ms[i] = -1;
        for (uint32_t r = 0; r < reps; ++r) {
          ctx->solver->profile_begin();
          profiling = true;
          for (uint32_t i = 0; i < count; ++i) {
            sw_result res{};
            std::string err;
            const int rc = run_plan(*ctx->solver, deltas + off[i], ns[i], ks[i], &plans[i], &res, err);
            if (rc != SW_OK) {
              restore();
              return fail(rc, err);
            }
          }
          sw_kernel_profile prof[SW_PROFILE_CLASSES];
          profiling = false;
          ctx->solver->profile_end(prof);
          double t[kKeys];
          ctx->solver->last_scan_profile(t, checks);
          for (int i = 0; i < kKeys; ++i)
            if (ms[i] < 0 || t[i] < ms[i]) ms[i] = t[i];
        }
        return SW_OK;
      };
      double base[kKeys];
      uint64_t checks[kKeys];
      int rc = pass(base, checks);
      if (rc != SW_OK) return rc;
      double best[kKeys];
      for (int i = 0; i < kKeys; ++i) best[i] = base[i];
      sw::ScanShapes top = start;
      // coordinate descent, every key at once: a knob's candidate value is set
      // for every key (where the shape stays valid) and each key keeps its
      // fastest value; a value must beat the key's best by 2% to replace it
      static const int kTile[3] = {32, 64, 128}, kWarps[3] = {4, 8, 16}, kTps[4] = {4, 8, 16, 32},
                       kGrid[5] = {4, 8, 16, 32, 64};
      struct Knob {
        const int* vals;
        int n;
        int sw::ScanShape::*field;
      };
      const Knob knobs[4] = {{kTile, 3, &sw::ScanShape::tile_rows},
                             {kWarps, 3, &sw::ScanShape::warps},
                             {kTps, 4, &sw::ScanShape::tiles_per_super},
                             {kGrid, 5, &sw::ScanShape::grid_factor}};
      for (const Knob& kn : knobs) {
        const sw::ScanShapes before = top;
        for (int v = 0; v < kn.n; ++v) {
          sw::ScanShapes trial = before;
          bool any = false;
          for (int key = 0; key < kKeys; ++key) {
            if (!checks[key]) continue;
            sw::ScanShape sh = before.s[key / sw::kScanSizeClasses][key % sw::kScanSizeClasses];
            if (sh.*kn.field == kn.vals[v]) continue;  // already timed
            sh.*kn.field = kn.vals[v];
            if (!sw::scan_shape_valid(key / sw::kScanSizeClasses + 1, sh)) continue;
            trial.s[key / sw::kScanSizeClasses][key % sw::kScanSizeClasses] = sh;
            any = true;
          }
          if (!any) continue;
          set_shapes(ctx, trial);
          double t[kKeys];
          uint64_t c2[kKeys];
          rc = pass(t, c2);
          if (rc != SW_OK) return rc;  // pass() restored the context
          for (int key = 0; key < kKeys; ++key) {
            const int w = key / sw::kScanSizeClasses, c = key % sw::kScanSizeClasses;
            if (!checks[key] || !(trial.s[w][c].*kn.field == kn.vals[v]) || before.s[w][c].*kn.field == kn.vals[v])
              continue;
            if (t[key] < 0.98 * best[key]) {
              best[key] = t[key];
              top.s[w][c] = trial.s[w][c];
            }
          }
        }
      }
      set_shapes(ctx, top);
      uint32_t n_out = 0;
      for (int key = 0; key < kKeys; ++key) {
        if (!checks[key]) continue;
        if (n_out < out_cap) {
          sw_scan_tuned& o = out[n_out];
          o.words = (uint32_t)(key / sw::kScanSizeClasses + 1);
          o.size_class = (uint32_t)(key % sw::kScanSizeClasses);
          o.checks = checks[key];
          o.ms_start = base[key];
          o.ms_best = best[key];
          o.shape = from_shape(top.s[key / sw::kScanSizeClasses][key % sw::kScanSizeClasses]);
        }
        ++n_out;
      }
      if (out_count) *out_count = n_out;
      return SW_OK;
    } catch (...) {
      restore();
      throw;
    }
  });
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
  return sw_mlp_train_ranked(ctx, params, automata, deltas, ns, ks, offsets, sets, labels, nullptr, 0.0f, epochs,
                             batch, lr, seed, loss);
}

int sw_mlp_train_ranked(sw_context* ctx, float* params, uint32_t automata, const uint32_t* deltas,
                        const uint32_t* ns, const uint32_t* ks, const uint64_t* offsets, const uint64_t* sets,
                        const float* labels, const uint32_t* groups, float rank_weight, uint32_t epochs,
                        uint32_t batch, float lr, uint64_t seed, float* loss) {
  if (rank_weight < 0.0f || (rank_weight > 0.0f && !groups))
    return fail(SW_ERR_INVALID_ARGUMENT, "a ranking weight needs a group per pair");
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
    *loss = ctx->solver->mlp_train(autos, offsets, sets, labels, epochs, batch, lr, seed, groups, rank_weight);
    ctx->solver->get_model(params);
    return SW_OK;
  });
}

}  // extern "C"
