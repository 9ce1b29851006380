#include "automaton.hpp"

#include <algorithm>
#include <cmath>
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
  const uint32_t n = A.n, k = A.k;
  if (n <= 1) return true;
  // preimages of (state, letter) as one flat list
  std::vector<uint32_t> start((size_t)n * k + 1, 0), pre((size_t)n * k);
  for (uint32_t q = 0; q < n; ++q)
    for (uint32_t a = 0; a < k; ++a) start[(size_t)A.at(q, a) * k + a + 1]++;
  for (size_t i = 0; i < (size_t)n * k; ++i) start[i + 1] += start[i];
  {
    std::vector<uint32_t> pos(start.begin(), start.end() - 1);
    for (uint32_t q = 0; q < n; ++q)
      for (uint32_t a = 0; a < k; ++a) pre[pos[(size_t)A.at(q, a) * k + a]++] = q;
  }
  // unordered pair {p, q}, p <= q, as p * n + q
  std::vector<char> seen((size_t)n * n, 0);
  std::vector<uint32_t> queue;
  queue.reserve((size_t)n * (n + 1) / 2);
  for (uint32_t q = 0; q < n; ++q) {
    seen[(size_t)q * n + q] = 1;
    queue.push_back(q * n + q);
  }
  for (size_t h = 0; h < queue.size(); ++h) {
    const uint32_t p = queue[h] / n, q = queue[h] % n;
    for (uint32_t a = 0; a < k; ++a) {
      const size_t pa = (size_t)p * k + a, qa = (size_t)q * k + a;
      for (uint32_t i = start[pa]; i < start[pa + 1]; ++i)
        for (uint32_t j = start[qa]; j < start[qa + 1]; ++j) {
          const uint32_t x = pre[i], y = pre[j];
          const uint32_t id = x <= y ? x * n + y : y * n + x;
          if (!seen[id]) {
            seen[id] = 1;
            queue.push_back(id);
          }
        }
    }
  }
  return queue.size() == (size_t)n * (n + 1) / 2;
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

std::vector<float> state_features(const Automaton& A) {
  const uint32_t n = A.n, k = A.k;
  std::vector<uint32_t> indeg((size_t)n * k, 0), total(n, 0);
  for (uint32_t q = 0; q < n; ++q)
    for (uint32_t a = 0; a < k; ++a) {
      indeg[(size_t)A.at(q, a) * k + a]++;
      total[A.at(q, a)]++;
    }
  // stationary mass of the walk that applies a uniformly random letter, with a
  // 1% restart anywhere (well defined for every automaton)
  std::vector<double> pi(n, 1.0 / n), nx(n);
  for (int it = 0; it < 100; ++it) {
    std::fill(nx.begin(), nx.end(), 0.01 / n);
    for (uint32_t q = 0; q < n; ++q)
      for (uint32_t a = 0; a < k; ++a) nx[A.at(q, a)] += 0.99 * pi[q] / k;
    pi.swap(nx);
  }
  std::vector<uint32_t> idx(n);
  for (uint32_t q = 0; q < n; ++q) idx[q] = q;
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return pi[x] > pi[y]; });
  std::vector<double> rank(n);
  for (uint32_t r = 0; r < n; ++r) rank[idx[r]] = n > 1 ? (double)r / (n - 1) : 0.0;
  const std::vector<char> sink = sink_states(A);
  // shortest merge length of every pair {p, q} (breadth first from the
  // diagonal over pairs of preimages); pairs that never merge get n * n
  std::vector<uint32_t> pair_len((size_t)n * n, 0);
  {
    std::vector<uint32_t> beg((size_t)k * (n + 1), 0), src((size_t)k * n);
    for (uint32_t a = 0; a < k; ++a) {
      for (uint32_t q = 0; q < n; ++q) beg[(size_t)a * (n + 1) + A.at(q, a) + 1]++;
      for (uint32_t t = 0; t < n; ++t) beg[(size_t)a * (n + 1) + t + 1] += beg[(size_t)a * (n + 1) + t];
      std::vector<uint32_t> fill(beg.begin() + (size_t)a * (n + 1), beg.begin() + (size_t)a * (n + 1) + n);
      for (uint32_t q = 0; q < n; ++q) src[(size_t)a * n + fill[A.at(q, a)]++] = q;
    }
    std::vector<uint32_t> queue;
    auto visit = [&](uint32_t p, uint32_t q, uint32_t len) {
      if (p == q || pair_len[(size_t)p * n + q]) return;
      pair_len[(size_t)p * n + q] = pair_len[(size_t)q * n + p] = len;
      queue.push_back(p * n + q);
    };
    for (uint32_t t = 0; t < n; ++t)
      for (uint32_t a = 0; a < k; ++a)
        for (uint32_t i = beg[(size_t)a * (n + 1) + t]; i < beg[(size_t)a * (n + 1) + t + 1]; ++i)
          for (uint32_t j = i + 1; j < beg[(size_t)a * (n + 1) + t + 1]; ++j)
            visit(src[(size_t)a * n + i], src[(size_t)a * n + j], 1);
    for (size_t h = 0; h < queue.size(); ++h) {
      const uint32_t v1 = queue[h] / n, v2 = queue[h] % n, l = pair_len[queue[h]] + 1;
      for (uint32_t a = 0; a < k; ++a)
        for (uint32_t i = beg[(size_t)a * (n + 1) + v1]; i < beg[(size_t)a * (n + 1) + v1 + 1]; ++i)
          for (uint32_t j = beg[(size_t)a * (n + 1) + v2]; j < beg[(size_t)a * (n + 1) + v2 + 1]; ++j)
            visit(src[(size_t)a * n + i], src[(size_t)a * n + j], l);
    }
  }
  std::vector<float> f((size_t)n * kStateFeatures, 0.0f);
  for (uint32_t q = 0; q < n; ++q) {
    float* x = &f[(size_t)q * kStateFeatures];
    uint32_t mn = UINT32_MAX, mx = 0, into_sink = 0, collide = 0, seed = 0;
    double img_in = 0.0, two_step = 0.0;
    for (uint32_t a = 0; a < k; ++a) {
      const uint32_t d = indeg[(size_t)q * k + a];
      mn = std::min(mn, d);
      mx = std::max(mx, d);
      seed |= sink[q] && d > 1;
      const uint32_t t = A.at(q, a);
      into_sink += sink[t] ? 1u : 0u;
      collide += indeg[(size_t)t * k + a] > 1;
      img_in += total[t];
    }
    for (uint32_t p = 0; p < n; ++p)
      for (uint32_t a = 0; a < k; ++a)
        if (A.at(p, a) == q) two_step += total[p];
    double pl_sum = 0;
    uint32_t pl_min = UINT32_MAX;
    for (uint32_t r = 0; r < n; ++r) {
      if (r == q) continue;
      const uint32_t l = pair_len[(size_t)q * n + r] ? pair_len[(size_t)q * n + r] : n * n;
      pl_sum += l;
      pl_min = std::min(pl_min, l);
    }
    x[0] = 1.0f;
    x[1] = (float)total[q] / k;
    x[2] = (float)mn;
    x[3] = (float)mx;
    x[4] = n > 1 ? (float)pl_min : 0.0f;  // closest merge partner
    x[5] = (float)(pi[q] * n);
    x[6] = sink[q] ? 1.0f : 0.0f;
    x[7] = n > 1 ? (float)(pl_sum / (n - 1)) : 0.0f;  // mean merge length with the other states
    x[8] = (float)(img_in / ((double)k * k));
    x[9] = (float)(two_step / ((double)k * k));
    x[10] = (float)collide / k;
    x[11] = (float)std::log2(1.0 + total[q]);
    x[12] = (float)rank[q];
    x[13] = 64.0f / (float)n;
    x[14] = seed ? 1.0f : 0.0f;
    x[15] = (float)into_sink / k;
  }
  // standardise every varying column over the states (zero mean, unit
  // deviation), so that the sum over a set carries the set's composition at
  // the scale of its size; columns 0 (one) and 13 (64 / n) stay as they are
  for (int j = 1; j < kStateFeatures; ++j) {
    if (j == 13) continue;
    double mean = 0, var = 0;
    for (uint32_t q = 0; q < n; ++q) mean += f[(size_t)q * kStateFeatures + j];
    mean /= n;
    for (uint32_t q = 0; q < n; ++q) {
      const double d = f[(size_t)q * kStateFeatures + j] - mean;
      var += d * d;
    }
    const double sd = std::sqrt(var / n);
    for (uint32_t q = 0; q < n; ++q) {
      float& v = f[(size_t)q * kStateFeatures + j];
      v = sd > 1e-6 ? (float)((v - mean) / sd) : 0.0f;
    }
  }
  return f;
}

}  // namespace sw
