// GPU exact shortest-reset-word search (the reference's `Exact`,
// synchrolib/algorithm/exact/exact.cpp:37-97 with meet_in_the_middle.cpp and
// dfs.cpp) and the GPU `Beam` upper bound (synchrolib/algorithm/beam/beam.hpp).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "../../include/synchrowords.h"
#include "automaton.hpp"
#include "common.cuh"
#include "kernels.cuh"

namespace sw {

struct Bounds {
  bool non_synchro = false;
  uint64_t lower = 0, upper = UINT64_MAX;
  bool has_word = false;
  std::vector<uint32_t> word;  // verified reset word of length `upper` when has_word
};

class Engine;  // device state, defined in exact.cu

// What a successful Reduce hands to the algorithms after it
// (synchrolib/algorithm/algorithm.hpp:29-34 ReduceData, reduce.hpp:75-90).
struct ReduceState {
  bool active = false;    // the automaton was reduced (the reference's reduce->done)
  uint64_t bfs_steps = 0; // BFS steps the reduction took (added back by Exact)
  Automaton original;     // the automaton before reduction (words are checked on it)
  Automaton reduced;      // restriction to the states reachable from the BFS list
  std::vector<std::vector<uint32_t>> seeds;   // BFS list, as state lists in reduced labels
  std::vector<std::vector<uint32_t>> prefix;  // word taking the full set to each seed
};

class Solver {
 public:
  explicit Solver(int device);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  // Exact::run semantics on `b` (in/out).
  // With `red`, A is the reduced automaton and the search starts from the
  // reduced BFS list (exact.cpp:130-146, 83-87).
  void exact(const Automaton& A, const sw_exact_config& cfg, Bounds& b, sw_stats& st,
             const ReduceState* red = nullptr);
  // Reduce::run semantics: short dominance-pruned BFS from the full set; on
  // success `red` describes the reduced automaton and the bounds are shifted.
  void reduce(const Automaton& A, const sw_reduce_config& cfg, Bounds& b, sw_stats& st, ReduceState& red);
  // Beam::run semantics on `b` (in/out); also records a verified word.
  void beam(const Automaton& A, const sw_beam_config& cfg, Bounds& b, sw_stats& st);
  // Eppstein::run semantics (greedy pair-merging upper bound and its word).
  void eppstein(const Automaton& A, const sw_eppstein_config& cfg, Bounds& b, sw_stats& st);
  // Brute::run semantics (power-set BFS, n <= 32): exact length and a word.
  void brute(const Automaton& A, const sw_brute_config& cfg, Bounds& b, sw_stats& st);

  // Forward beam scored by the loaded distance model (or by set size).
  void learned_beam(const Automaton& A, const sw_learned_beam_config& cfg, Bounds& b, sw_stats& st);

  // Learned distance model (sets in the 8-word reference layout).
  void set_model(const float* params);
  void get_model(float* params);
  bool has_model() const;
  // Labelled forward-layer sets; returns the reset length (0 if none found).
  uint32_t distance_pairs(const Automaton& A, uint32_t per_layer, uint64_t max_inverse_sets,
                          std::vector<uint64_t>& sets, std::vector<float>& labels, std::vector<uint32_t>& depths);
  void mlp_forward(const Automaton& A, const uint64_t* sets, uint64_t count, float* out);
  float mlp_gradient(const Automaton& A, const uint64_t* sets, const float* labels, uint64_t count, float* grad);
  // groups (optional): a group id per pair; with rank_w > 0 the loss adds a
  // pairwise ranking term within each group of a batch.
  float mlp_train(const std::vector<Automaton>& autos, const uint64_t* offsets, const uint64_t* sets,
                  const float* labels, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                  const uint32_t* groups = nullptr, float rank_w = 0.0f);

  // Kernel-level helpers (reference bitset layout on the host).
  void apply_transition(const Automaton& A, uint32_t letter, bool inverse, const uint64_t* from, uint64_t* to,
                        uint64_t count);
  void subsets_check(uint32_t n, const uint64_t* sets, uint64_t set_count, const uint64_t* checks,
                     uint64_t check_count, bool proper, uint8_t* results);
  uint64_t sort_unique(uint32_t n, uint64_t* sets, uint64_t count);

  int device() const { return device_; }
  void* stream() const;  // the cudaStream_t every kernel of this solver runs on
  // Per-kernel-class CUDA-event timing of everything launched in between.
  void profile_begin();
  void profile_end(sw_kernel_profile out[4]);
  // Launch shapes of the subset check per row width and list size class.
  void set_scan_shapes(const ScanShapes& s);
  const ScanShapes& scan_shapes() const;
  // CUDA-event milliseconds and count of the subset checks (mask build plus
  // scan) of the last profiled interval, per (W - 1) * kScanSizeClasses + size class.
  void last_scan_profile(double ms[8 * kScanSizeClasses], uint64_t checks[8 * kScanSizeClasses]) const;

 private:
  int device_;
  std::unique_ptr<Engine> eng_;
};

}  // namespace sw
