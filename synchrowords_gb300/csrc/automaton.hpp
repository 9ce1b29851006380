// Host-side automaton utilities: validation, sink component, backward seeds,
// state relabelling and the per-letter tables the expansion kernel stages in
// shared memory.
#pragma once
#include <cstdint>
#include <vector>

namespace sw {

struct Automaton {
  uint32_t n = 0, k = 0;
  std::vector<uint32_t> t;  // t[q*k + a]  (synchrolib/data_structures/automaton/automaton.hpp:14-33)
  uint32_t at(uint32_t q, uint32_t a) const { return t[(size_t)q * k + a]; }
};

// Throws std::invalid_argument on n/k out of range or an entry >= n
// (app/io.hpp:38-52 validate()).
Automaton make_automaton(const uint32_t* delta, uint32_t n, uint32_t k);

// States of the sink strongly connected component reached by the DFS from
// state 0 (synchrolib/utils/connectivity.cpp:105-160).
std::vector<char> sink_states(const Automaton& A);

// Backward seeds: sink states with some letter of in-degree > 1
// (synchrolib/algorithm/exact/exact.cpp:149-164; beam.hpp:104-115).
std::vector<uint32_t> backward_seeds(const Automaton& A);

// Relabel states: new label of q is order[q] (automaton.hpp:54-64).
Automaton permute(const Automaton& A, const std::vector<uint32_t>& order);

// True iff every pair of states can be merged by some word (pair-graph
// reachability to the diagonal).  An automaton failing this has no reset
// word; the search would otherwise run to its upper bound.
bool is_synchronizing(const Automaton& A);

// Per-state feature vectors of the learned distance model (n rows of
// `kStateFeatures` floats): structural quantities that mean the same thing in
// automata of any size (in-degrees, stationary mass of a random-letter walk,
// sink membership, collisions, shortest merge lengths with the other states),
// standardised over the states, plus a
// constant one and 64 / n, so one trained model scores sets of any automaton.
constexpr int kStateFeatures = 16;
std::vector<float> state_features(const Automaton& A);

// Per-letter device tables (u16): delta[a*n + q]; inverse CSR inv_beg[a*(n+1) + t],
// inv_src[a*n + e].
struct HostTables {
  std::vector<uint16_t> delta, inv_beg, inv_src;
};
HostTables build_tables(const Automaton& A);

// Reference-layout (LSB-first, ceil(n/64) words) <-> device MSB-first rows of W words.
void to_device_rows(const uint64_t* ref, uint64_t count, uint32_t n, int W, unsigned long long* out);
void from_device_rows(const unsigned long long* rows, uint64_t count, uint32_t n, int W, uint64_t* out);

// Image of the full state set under a word (the word check).
std::vector<uint32_t> apply_word(const Automaton& A, const std::vector<uint32_t>& word);

}  // namespace sw
