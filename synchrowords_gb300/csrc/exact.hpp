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

namespace sw {

struct Bounds {
  bool non_synchro = false;
  uint64_t lower = 0, upper = UINT64_MAX;
  bool has_word = false;
  std::vector<uint32_t> word;  // verified reset word of length `upper` when has_word
};

class Engine;  // device state, defined in exact.cu

class Solver {
 public:
  explicit Solver(int device);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  // Exact::run semantics on `b` (in/out).
  void exact(const Automaton& A, const sw_exact_config& cfg, Bounds& b, sw_stats& st);
  // Beam::run semantics on `b` (in/out); also records a verified word.
  void beam(const Automaton& A, const sw_beam_config& cfg, Bounds& b, sw_stats& st);

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

 private:
  int device_;
  std::unique_ptr<Engine> eng_;
};

}  // namespace sw
