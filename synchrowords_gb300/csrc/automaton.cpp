#include "automaton.hpp"

#include <algorithm>
#include <deque>
#include <stdexcept>
#include <string>

#include "common.cuh"

namespace sw {

Automaton make_automaton(const uint32_t* delta, uint32_t n, uint32_t k) {
  if (!delta) throw std::invalid_argument("delta is NULL");
  if (n == 0 || k == 0) throw std::invalid_argument("N and K must be greater than 0");
  if (n > (uint32_t)kMaxStates) throw std::invalid_argument("n exceeds " + std::to_string(kMaxStates));
  if (k > (uint32_t)kMaxLetters) throw std::invalid_argument("k exceeds " + std::to_string(kMaxLetters));
  Automaton A;
  A.n = n;
  A.k = k;
  A.t.assign(delta, delta + (size_t)n * k);
  for (size_t i = 0; i < A.t.size(); ++i)
    if (A.t[i] >= n)
      throw std::invalid_argument("Expected integer in range [0, " + std::to_string(n - 1) + "], found " +
                                  std::to_string(A.t[i]));
  return A;
}

std::vector<char> sink_states(const Automaton& A) {
  // Iterative form of the reference's recursive low-link DFS from state 0: the
  // first vertex whose low-link equals its own index closes a sink component.
  std::vector<uint32_t> idx(A.n, 0), low(A.n, 0), next_letter(A.n, 0);
  std::vector<uint32_t> stack{0};
  uint32_t counter = 1, sink = 0;
  idx[0] = low[0] = counter++;
  bool done = false;
  while (!stack.empty() && !done) {
    uint32_t v = stack.back();
    if (next_letter[v] < A.k) {
      uint32_t w = A.at(v, next_letter[v]++);
      if (idx[w]) {
        low[v] = std::min(low[v], idx[w]);
      } else {
        idx[w] = low[w] = counter++;
        stack.push_back(w);
      }
      continue;
    }
    if (low[v] == idx[v]) {
      sink = v;
      done = true;
      break;
    }
    stack.pop_back();
    uint32_t parent = stack.back();
    low[parent] = std::min(low[parent], low[v]);
  }
  std::vector<char> r(A.n, 0);
  std::vector<uint32_t> st{sink};
  r[sink] = 1;
  while (!st.empty()) {
    uint32_t q = st.back();
    st.pop_back();
    for (uint32_t a = 0; a < A.k; ++a) {
      uint32_t p = A.at(q, a);
      if (!r[p]) {
        r[p] = 1;
        st.push_back(p);
      }
    }
  }
  return r;
}

std::vector<uint32_t> backward_seeds(const Automaton& A) {
  std::vector<char> sink = sink_states(A);
  std::vector<uint32_t> indeg((size_t)A.n * A.k, 0);
  for (uint32_t q = 0; q < A.n; ++q)
    for (uint32_t a = 0; a < A.k; ++a) indeg[(size_t)A.at(q, a) * A.k + a]++;
  std::vector<uint32_t> out;
  for (uint32_t q = 0; q < A.n; ++q) {
    if (!sink[q]) continue;
    for (uint32_t a = 0; a < A.k; ++a)
      if (indeg[(size_t)q * A.k + a] > 1) {
        out.push_back(q);
        break;
      }
  }
  return out;
}

Automaton permute(const Automaton& A, const std::vector<uint32_t>& order) {
  Automaton R;
  R.n = A.n;
  R.k = A.k;
  R.t.assign(A.t.size(), 0);
  for (uint32_t q = 0; q < A.n; ++q)
    for (uint32_t a = 0; a < A.k; ++a) R.t[(size_t)order[q] * A.k + a] = order[A.at(q, a)];
  return R;
}

bool is_synchronizing(const Automaton& A) {
  // Backward BFS in the pair graph from the diagonal: every pair must reach it.
  const uint32_t n = A.n;
  if (n <= 1) return true;
  std::vector<std::vector<uint32_t>> pre((size_t)n * A.k);
  for (uint32_t q = 0; q < n; ++q)
    for (uint32_t a = 0; a < A.k; ++a) pre[(size_t)A.at(q, a) * A.k + a].push_back(q);
  auto id = [n](uint32_t p, uint32_t q) { return (size_t)std::min(p, q) * n + std::max(p, q); };
  std::vector<char> seen((size_t)n * n, 0);
  std::deque<std::pair<uint32_t, uint32_t>> dq;
  for (uint32_t q = 0; q < n; ++q) {
    seen[id(q, q)] = 1;
    dq.push_back({q, q});
  }
  size_t reached = n;
  while (!dq.empty()) {
    auto [p, q] = dq.front();
    dq.pop_front();
    for (uint32_t a = 0; a < A.k; ++a)
      for (uint32_t x : pre[(size_t)p * A.k + a])
        for (uint32_t y : pre[(size_t)q * A.k + a]) {
          size_t i = id(x, y);
          if (!seen[i]) {
            seen[i] = 1;
            ++reached;
            dq.push_back({x, y});
          }
        }
  }
  return reached == (size_t)n * (n + 1) / 2;
}

HostTables build_tables(const Automaton& A) {
  HostTables T;
  const uint32_t n = A.n, k = A.k;
  T.delta.resize((size_t)k * n);
  T.inv_beg.assign((size_t)k * (n + 1), 0);
  T.inv_src.resize((size_t)k * n);
  for (uint32_t a = 0; a < k; ++a) {
    std::vector<uint32_t> cnt(n + 1, 0);
    for (uint32_t q = 0; q < n; ++q) {
      T.delta[(size_t)a * n + q] = (uint16_t)A.at(q, a);
      cnt[A.at(q, a) + 1]++;
    }
    for (uint32_t t = 0; t < n; ++t) cnt[t + 1] += cnt[t];
    for (uint32_t t = 0; t <= n; ++t) T.inv_beg[(size_t)a * (n + 1) + t] = (uint16_t)cnt[t];
    std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
    for (uint32_t q = 0; q < n; ++q) T.inv_src[(size_t)a * n + fill[A.at(q, a)]++] = (uint16_t)q;
  }
  return T;
}

void to_device_rows(const uint64_t* ref, uint64_t count, uint32_t n, int W, unsigned long long* out) {
  const uint32_t rw = (n + 63) / 64;
  for (uint64_t i = 0; i < count; ++i) {
    unsigned long long* o = out + i * W;
    for (int w = 0; w < W; ++w) o[w] = 0;
    for (uint32_t q = 0; q < n; ++q)
      if ((ref[i * rw + q / 64] >> (q % 64)) & 1ULL) o[q >> 6] |= state_bit((int)q);
  }
}

void from_device_rows(const unsigned long long* rows, uint64_t count, uint32_t n, int W, uint64_t* out) {
  const uint32_t rw = (n + 63) / 64;
  for (uint64_t i = 0; i < count; ++i) {
    uint64_t* o = out + i * rw;
    for (uint32_t w = 0; w < rw; ++w) o[w] = 0;
    for (uint32_t q = 0; q < n; ++q)
      if (rows[i * W + (q >> 6)] & state_bit((int)q)) o[q / 64] |= 1ULL << (q % 64);
  }
}

std::vector<uint32_t> apply_word(const Automaton& A, const std::vector<uint32_t>& word) {
  std::vector<char> cur(A.n, 1), nxt(A.n);
  for (uint32_t a : word) {
    std::fill(nxt.begin(), nxt.end(), 0);
    for (uint32_t q = 0; q < A.n; ++q)
      if (cur[q]) nxt[A.at(q, a)] = 1;
    cur.swap(nxt);
  }
  std::vector<uint32_t> out;
  for (uint32_t q = 0; q < A.n; ++q)
    if (cur[q]) out.push_back(q);
  return out;
}

}  // namespace sw
