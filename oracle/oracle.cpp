// ORACLE — test infrastructure, not product.
//
// A CPU restatement of SynchroLib 1.1.0's exact shortest-reset-word search
// (the `Exact` algorithm: bidirectional BFS with dominance pruning, the
// implicit-trie subset check, the long-double cost model and the
// memory-bounded inverse DFS) and of its `Beam` upper bound.  Every function
// cites the reference file:line whose behaviour it restates; the code itself
// is written from scratch for a runtime (n, k) instead of the reference's
// compile-time templates.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load this library, and only as the checker or the timed CPU baseline; the
// product (synchrowords_gb300) never calls it.
//
// Pinning: tests/test_oracle_pin.py compares this restatement's results and
// its per-step frontier sizes with the compiled reference (oracle/_ref, built
// by oracle/build_ref.py) and with committed golden vectors.
//
// Set layout (as the reference, subset.hpp:11-26): state q is bit q%64 of
// word q/64; W = ceil(n/64) words; tail bits are zero.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <utility>
#include <vector>

#include "oracle.h"

namespace orc {

using u64 = uint64_t;
using u32 = uint32_t;
using cost_t = long double;

struct OutOfMemory {};

// Bit reversal of a 64-bit word (standard swap ladder).  The reference orders
// sets lexicographically with state 0 most significant by comparing
// bit-reversed words (subset.hpp:71-77, bits.hpp:88-96).
static inline u64 rev64(u64 v) {
  v = ((v >> 1) & 0x5555555555555555ULL) | ((v & 0x5555555555555555ULL) << 1);
  v = ((v >> 2) & 0x3333333333333333ULL) | ((v & 0x3333333333333333ULL) << 2);
  v = ((v >> 4) & 0x0F0F0F0F0F0F0F0FULL) | ((v & 0x0F0F0F0F0F0F0F0FULL) << 4);
  v = ((v >> 8) & 0x00FF00FF00FF00FFULL) | ((v & 0x00FF00FF00FF00FFULL) << 8);
  v = ((v >> 16) & 0x0000FFFF0000FFFFULL) | ((v & 0x0000FFFF0000FFFFULL) << 16);
  return (v >> 32) | (v << 32);
}

template <int W>
struct Set {
  u64 v[W];
  bool has(u32 q) const { return (v[q >> 6] >> (q & 63)) & 1ULL; }
  void put(u32 q) { v[q >> 6] |= 1ULL << (q & 63); }
  u32 card() const {
    u32 c = 0;
    for (int b = 0; b < W; ++b) c += (u32)__builtin_popcountll(v[b]);
    return c;
  }
  bool operator==(const Set& o) const {
    for (int b = 0; b < W; ++b)
      if (v[b] != o.v[b]) return false;
    return true;
  }
  bool operator!=(const Set& o) const { return !(*this == o); }
  // subset.hpp:71-77 — lexicographic by state index, state 0 first.
  bool operator<(const Set& o) const {
    for (int b = 0; b < W; ++b)
      if (v[b] != o.v[b]) return rev64(v[b]) < rev64(o.v[b]);
    return false;
  }
  // `this ⊇ s` (subset.hpp:206-211 names it is_subset(s)).
  bool contains(const Set& s) const {
    for (int b = 0; b < W; ++b)
      if ((s.v[b] & v[b]) != s.v[b]) return false;
    return true;
  }
  bool contains_proper(const Set& s) const { return *this != s && contains(s); }
};

// subset.hpp:78-84 — raw word order.
template <int W>
static bool comp_fast(const Set<W>& a, const Set<W>& b) {
  for (int i = 0; i < W; ++i)
    if (a.v[i] != b.v[i]) return a.v[i] < b.v[i];
  return false;
}

template <int W>
struct Ctx {
  u32 n, k;
  u64 tail_mask;  // mask of valid bits in the last word
  Set<W> empty() const {
    Set<W> s;
    std::fill(s.v, s.v + W, 0ULL);
    return s;
  }
  Set<W> singleton(u32 q) const {
    Set<W> s = empty();
    s.put(q);
    return s;
  }
  Set<W> complete() const {
    Set<W> s;
    std::fill(s.v, s.v + W, ~0ULL);
    s.v[W - 1] &= tail_mask;
    return s;
  }
  // subset.hpp:104-115
  void negate(Set<W>& s) const {
    for (int b = 0; b < W; ++b) s.v[b] = ~s.v[b];
    s.v[W - 1] &= tail_mask;
  }
  // subset.hpp:55-61
  Set<W> permute(const Set<W>& s, const std::vector<u32>& order) const {
    Set<W> r = empty();
    for (u32 i = 0; i < n; ++i)
      if (s.has(i)) r.put(order[i]);
    return r;
  }
};

template <int W>
using List = std::vector<Set<W>>;

// vector.hpp:13-27
template <int W>
static void sort_unique(List<W>& l) {
  std::sort(l.begin(), l.end());
  l.erase(std::unique(l.begin(), l.end()), l.end());
}

// ---------------------------------------------------------------------------
// Automaton helpers.
// ---------------------------------------------------------------------------
struct Aut {
  u32 n, k;
  std::vector<u32> t;  // t[q*k + a]  (automaton.hpp:14-33)
  u32 at(u32 q, u32 a) const { return t[(size_t)q * k + a]; }
};

// inverse_automaton.hpp:152-177 — per-letter CSR of preimages.
struct InvAut {
  u32 n, k;
  std::vector<u32> edges, begin, end;  // [a*n + ...]
  explicit InvAut(const Aut& A) : n(A.n), k(A.k), edges(A.n * A.k), begin(A.n * A.k), end(A.n * A.k, 0) {
    for (u32 a = 0; a < k; ++a)
      for (u32 q = 0; q < n; ++q) end[a * n + A.at(q, a)]++;
    for (u32 a = 0; a < k; ++a) {
      begin[a * n] = 0;
      for (u32 q = 1; q < n; ++q) begin[a * n + q] = begin[a * n + q - 1] + end[a * n + q - 1];
      for (u32 q = 0; q < n; ++q) end[a * n + q] = begin[a * n + q];
    }
    for (u32 a = 0; a < k; ++a)
      for (u32 q = 0; q < n; ++q) edges[a * n + end[a * n + A.at(q, a)]++] = q;
  }
  u32 indeg(u32 q, u32 a) const { return end[a * n + q] - begin[a * n + q]; }
};

// automaton.hpp:54-64 — relabel states: q -> order[q].
static Aut permute_aut(const Aut& A, const std::vector<u32>& order) {
  Aut R{A.n, A.k, std::vector<u32>(A.t.size())};
  for (u32 q = 0; q < A.n; ++q)
    for (u32 a = 0; a < A.k; ++a) R.t[(size_t)order[q] * A.k + a] = order[A.at(q, a)];
  return R;
}

// connectivity.cpp:105-140 — DFS from state 0; the first strongly connected
// component to close is a sink component; return its root.
static u32 sink_component_vertex(const Aut& A) {
  std::vector<u32> idx(A.n, 0);
  u32 counter = 1, sink = 0;
  // Recursive formulation as in the reference: returns 0 when the DFS is done.
  struct Rec {
    const Aut& A;
    std::vector<u32>& idx;
    u32& counter;
    u32& sink;
    u32 go(u32 v) {
      u32 low = idx[v] = counter++;
      for (u32 a = 0; a < A.k; ++a) {
        u32 w = A.at(v, a);
        if (idx[w]) {
          if (idx[w] < low) low = idx[w];
        } else {
          u32 l2 = go(w);
          if (!l2) return 0;
          if (l2 < low) low = l2;
        }
      }
      if (idx[v] == low) {
        sink = v;
        return 0;
      }
      return low;
    }
  } rec{A, idx, counter, sink};
  rec.go(0);
  return sink;
}

// connectivity.cpp:142-160
static std::vector<char> reachable_from(const Aut& A, u32 v) {
  std::vector<char> r(A.n, 0);
  std::vector<u32> st{v};
  r[v] = 1;
  while (!st.empty()) {
    u32 q = st.back();
    st.pop_back();
    for (u32 a = 0; a < A.k; ++a) {
      u32 p = A.at(q, a);
      if (!r[p]) {
        r[p] = 1;
        st.push_back(p);
      }
    }
  }
  return r;
}

static std::vector<char> sink_states(const Aut& A) { return reachable_from(A, sink_component_vertex(A)); }

// distribution.cpp:5-51 — in-place inverse of a square matrix by LU
// decomposition (Doolittle-style: unit-diagonal U after normalising row 0).
static void invert_lu(std::vector<double>& d, u32 N) {
  auto at = [&](u32 r, u32 c) -> double& { return d[(size_t)r * N + c]; };
  for (u32 i = 1; i < N; ++i) d[i] /= d[0];
  for (u32 i = 1; i < N; ++i) {
    for (u32 j = i; j < N; ++j) {
      double s = 0.0;
      for (u32 q = 0; q < i; ++q) s += at(j, q) * at(q, i);
      at(j, i) -= s;
    }
    if (i == N - 1) continue;
    for (u32 j = i + 1; j < N; ++j) {
      double s = 0.0;
      for (u32 q = 0; q < i; ++q) s += at(i, q) * at(q, j);
      at(i, j) = (at(i, j) - s) / at(i, i);
    }
  }
  for (u32 i = 0; i < N; ++i)
    for (u32 j = i; j < N; ++j) {
      double x = 1.0;
      if (i != j) {
        x = 0.0;
        for (u32 q = i; q < j; ++q) x -= at(j, q) * at(q, i);
      }
      at(j, i) = x / at(j, j);
    }
  for (u32 i = 0; i < N; ++i)
    for (u32 j = i; j < N; ++j) {
      if (i == j) continue;
      double s = 0.0;
      for (u32 q = i; q < j; ++q) s += at(q, j) * ((i == q) ? 1.0 : at(i, q));
      at(i, j) = -s;
    }
  for (u32 i = 0; i < N; ++i)
    for (u32 j = 0; j < N; ++j) {
      double s = 0.0;
      for (u32 q = (i > j ? i : j); q < N; ++q) s += ((j == q) ? 1.0 : at(j, q)) * at(q, i);
      at(j, i) = s;
    }
}

// distribution.cpp:53-88 — stationary distribution of the lazy random walk
// pi = u (I - P + U)^{-1}.
static std::vector<double> stationary(const Aut& R) {
  const u32 N = R.n, K = R.k;
  std::vector<double> prob((size_t)N * N);
  for (u32 q = 0; q < N; ++q) {
    double w = 1.0 / (N * N * K * (1.0 / (N * K) + 1.0));
    for (u32 m = 0; m < N; ++m) prob[(size_t)q * N + m] = w;
    w = 1.0 / (K * (1.0 / (N * K) + 1.0));
    for (u32 a = 0; a < K; ++a) prob[(size_t)q * N + R.at(q, a)] += w;
  }
  std::vector<double> mat((size_t)N * N);
  for (u32 a = 0; a < N; ++a) {
    for (u32 b = 0; b < N; ++b) mat[(size_t)a * N + b] = 1.0 / N - prob[(size_t)a * N + b];
    mat[(size_t)a * N + a] += 1.0;
  }
  std::vector<double> pi(N);
  if (N == 1) {
    pi[0] = 1.0;
    return pi;
  }
  invert_lu(mat, N);
  for (u32 a = 0; a < N; ++a) {
    pi[a] = 0.0;
    for (u32 b = 0; b < N; ++b) pi[a] += mat[(size_t)b * N + a];
    pi[a] /= N;
  }
  return pi;
}

// automaton.hpp:30-45 — order[i] = rank of weights[i] (ascending, ties by index).
static std::vector<u32> order_ascending(const std::vector<double>& w) {
  std::vector<std::pair<double, u32>> v(w.size());
  for (u32 i = 0; i < w.size(); ++i) v[i] = {w[i], i};
  std::sort(v.begin(), v.end());
  std::vector<u32> order(w.size());
  for (u32 i = 0; i < w.size(); ++i) order[v[i].second] = i;
  return order;
}

// exact.cpp:108-127 — sink states by stationary mass, others by 1 + in-degree.
static std::vector<u32> exact_state_order(const Aut& A, const InvAut& inv) {
  std::vector<char> sink = sink_states(A);
  std::vector<u32> tr(A.n);
  u32 rn = 0;
  for (u32 q = 0; q < A.n; ++q)
    if (sink[q]) tr[q] = rn++;
  Aut R{rn, A.k, std::vector<u32>((size_t)rn * A.k)};
  for (u32 q = 0; q < A.n; ++q)
    if (sink[q])
      for (u32 a = 0; a < A.k; ++a) R.t[(size_t)tr[q] * A.k + a] = tr[A.at(q, a)];
  std::vector<double> rpi = stationary(R);
  std::vector<double> pi(A.n);
  u32 c = 0;
  for (u32 q = 0; q < A.n; ++q) {
    if (sink[q]) {
      pi[q] = rpi[c++];
    } else {
      pi[q] = 1.0;
      for (u32 a = 0; a < A.k; ++a) pi[q] += inv.indeg(q, a);
    }
  }
  return order_ascending(pi);
}

// exact.cpp:149-164 and beam.hpp:104-115 — backward seeds: singletons of sink
// states that have some letter with in-degree > 1.
static std::vector<u32> backward_seeds(const Aut& A, const InvAut& inv) {
  std::vector<char> sink = sink_states(A);
  std::vector<u32> out;
  for (u32 q = 0; q < A.n; ++q) {
    if (!sink[q]) continue;
    for (u32 a = 0; a < A.k; ++a)
      if (inv.indeg(q, a) > 1) {
        out.push_back(q);
        break;
      }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Slice look-up transition (preprocessed_transition.hpp:13-49,
// preprocessed_transitions.cpp:15-50): for each 8-state slice and each byte
// value, the image (or preimage union) of those states under one letter.
// ---------------------------------------------------------------------------
template <int W>
struct SliceLut {
  u32 slices = 0;
  std::vector<Set<W>> t;  // [slice*256 + byte]
  void build_forward(const Ctx<W>& c, const Aut& A, u32 a) {
    slices = (c.n + 7) / 8;
    t.assign((size_t)slices * 256, c.empty());
    for (u32 i = 0; i < slices; ++i)
      for (u32 b = 0; b < 256; ++b) {
        Set<W> s = c.empty();
        for (u32 j = 0; j < 8; ++j) {
          u32 q = 8 * i + j;
          if (q >= c.n) break;
          if ((b >> j) & 1) s.put(A.at(q, a));
        }
        t[(size_t)i * 256 + b] = s;
      }
  }
  void build_inverse(const Ctx<W>& c, const InvAut& I, u32 a) {
    slices = (c.n + 7) / 8;
    t.assign((size_t)slices * 256, c.empty());
    for (u32 i = 0; i < slices; ++i)
      for (u32 b = 0; b < 256; ++b) {
        Set<W> s = c.empty();
        for (u32 j = 0; j < 8; ++j) {
          u32 q = 8 * i + j;
          if (q >= c.n) break;
          if ((b >> j) & 1)
            for (u32 e = I.begin[a * I.n + q]; e < I.end[a * I.n + q]; ++e) s.put(I.edges[a * I.n + e]);
        }
        t[(size_t)i * 256 + b] = s;
      }
  }
  inline void apply(const Set<W>& from, Set<W>& to) const {
    for (int b = 0; b < W; ++b) to.v[b] = 0;
    u32 slice = 0;
    for (int w = 0; w < W && slice < slices; ++w)
      for (u32 sh = 0; sh < 64 && slice < slices; sh += 8, ++slice) {
        const Set<W>& e = t[(size_t)slice * 256 + ((from.v[w] >> sh) & 255)];
        for (int b = 0; b < W; ++b) to.v[b] |= e.v[b];
      }
  }
  // preprocessed_transitions.cpp:56-93 (threaded over chunks when asked).
  void apply_many(const Set<W>* from, Set<W>* to, size_t cnt, u32 threads) const {
    if (threads > 1 && cnt > 256) {
      std::vector<std::thread> th;
      for (u32 t = 0; t < threads; ++t) {
        size_t lo = cnt * t / threads, hi = cnt * (t + 1) / threads;
        th.emplace_back([=] {
          for (size_t i = lo; i < hi; ++i) apply(from[i], to[i]);
        });
      }
      for (auto& x : th) x.join();
    } else {
      for (size_t i = 0; i < cnt; ++i) apply(from[i], to[i]);
    }
  }
  size_t bytes() const { return (size_t)slices * 256 * sizeof(Set<W>); }
};

// ---------------------------------------------------------------------------
// Implicit trie (subsets_implicit_trie.hpp:24-267).  `check_contains_subset(S, C)`
// reorders C so that [it, end) holds exactly the c having some s in S with
// s ⊆ c (s ⊊ c when `proper`), and returns it.  S must be sorted and unique.
// ---------------------------------------------------------------------------
template <int W>
struct ImplicitTrie {
  using It = typename List<W>::iterator;
  static constexpr u32 M = 6;  // leaf size on the CPU path (:68-71)
  bool proper;

  // subsets_implicit_trie.hpp:151-163
  static It first_with_bit(It b, u32 d, size_t count) {
    while (count > 0) {
      size_t step = count / 2;
      It it = b + step;
      if (!it->has(d)) {
        b = it + 1;
        count -= step + 1;
      } else {
        count = step;
      }
    }
    return b;
  }

  // subsets_implicit_trie.hpp:166-266
  void rec(u32 d, It sb, It se, It cb, It& ce) {
    if (sb == se || cb == ce) return;
    if ((size_t)(se - sb) <= M) {
      for (It s = sb; s != se; ++s) {
        It it = cb;
        while (it != ce) {
          bool hit = proper ? it->contains_proper(*s) : it->contains(*s);
          if (hit) {
            --ce;
            std::swap(*it, *ce);
          } else {
            ++it;
          }
        }
      }
      return;
    }
    It lo = first_with_bit(sb, d, (size_t)(se - sb));
    if (sb != lo) rec(d + 1, sb, lo, cb, ce);
    if (lo == se || cb == ce) return;
    // Queries with bit d go to the back of [cb, ce).
    It p = std::partition(cb, ce, [d](const Set<W>& x) { return !x.has(d); });
    if (p != ce) rec(d + 1, lo, se, p, ce);
  }

  It run_single(List<W>& S, It cb, It ce) {
    It end = ce;
    rec(0, S.begin(), S.end(), cb, end);
    return end;
  }

  // :90-148 — split C into `threads` ranges, one std::thread each, then
  // compact the kept prefixes.
  It run(List<W>& S, List<W>& C, u32 threads) {
    if (threads <= 1 || std::max(S.size(), C.size()) < 256) return run_single(S, C.begin(), C.end());
    size_t cnt = C.size();
    std::vector<std::pair<size_t, size_t>> keep(threads);
    std::vector<std::thread> th;
    for (u32 t = 0; t < threads; ++t) {
      size_t lo = t * cnt / threads, hi = (t + 1) * cnt / threads;
      th.emplace_back([this, &S, &C, &keep, t, lo, hi] {
        ImplicitTrie<W> local{proper};
        It b = C.begin() + lo;
        It e = local.run_single(S, b, C.begin() + hi);
        keep[t] = {lo, (size_t)(e - C.begin())};
      });
    }
    for (auto& x : th) x.join();
    It out = C.begin();
    for (u32 t = 0; t < threads; ++t) {
      It b = C.begin() + keep[t].first, e = C.begin() + keep[t].second;
      if (b != out) out = std::move(b, e, out);
      else out = e;
    }
    return out;  // only the kept prefix [begin, out) is meaningful afterwards
  }
};

// SubsetsImplicitTrie::check_contains_subset with SortUniqueDone=false sorts
// and uniques both lists first (:29-44).
template <int W>
static typename List<W>::iterator contains_subset(List<W>& S, List<W>& C, bool proper, bool sort_done, u32 threads) {
  if (!sort_done) {
    sort_unique(S);
    sort_unique(C);
  }
  ImplicitTrie<W> t{proper};
  return t.run(S, C, threads);
}

// reduce(set): drop sets having a proper subset in the same list (:46-56).
template <int W>
static void reduce_self(List<W>& L, bool sort_done, u32 threads) {
  if (L.empty()) return;
  List<W> cpy = L;
  auto it = contains_subset(cpy, L, true, sort_done, threads);
  L.resize(it - L.begin());
}

// reduce(set, vec): drop from vec the sets having a (proper) subset in set (:58-64).
template <int W>
static void reduce_by(List<W>& S, List<W>& V, bool proper, bool sort_done, u32 threads) {
  if (V.empty()) return;
  auto it = contains_subset(S, V, proper, sort_done, threads);
  V.resize(it - V.begin());
}

// ---------------------------------------------------------------------------
// Explicit trie for the DFS phase (subsets_trie.hpp:18-518).
// ---------------------------------------------------------------------------
template <int W>
struct ExplicitTrie {
  struct Node {
    u32 zero = 0, one = 0, bit = 0, cnt = 0, pos = 0;
    u32 minpop = std::numeric_limits<u32>::max();
  };
  using It = typename List<W>::iterator;
  static constexpr u32 M = 10;  // :150
  u32 n = 0;
  u32 threads = 1;
  std::vector<Node> nodes;
  List<W> sets;

  size_t bytes() const { return nodes.size() * 24 + sets.size() * sizeof(Set<W>); }

  // :299-350 — most frequent bit that is neither constant 0 nor constant 1.
  u32 division_bit(It b, It e) {
    std::vector<long> cnt(n, 0);
    size_t all = e - b;
    for (It it = b; it != e; ++it)
      for (int w = 0; w < W; ++w) {
        u64 x = it->v[w];
        while (x) {
          cnt[w * 64 + __builtin_ctzll(x)]++;
          x &= x - 1;
        }
      }
    long best = -2;
    u32 arg = 0;
    for (u32 i = 0; i < n; ++i) {
      long c = (cnt[i] == (long)all || cnt[i] == 0) ? -1 : cnt[i];
      if (c > best) {
        best = c;
        arg = i;
      }
    }
    return arg;
  }

  // :236-297 (build_impl_swap)
  void build_rec(u32 v, It b, It e) {
    if (b == e) return;
    size_t all = e - b;
    if (all <= M) {
      nodes[v].pos = (u32)(b - sets.begin());
      for (; b != e; ++b) {
        nodes[v].cnt++;
        nodes[v].minpop = std::min(nodes[v].minpop, b->card());
      }
      return;
    }
    u32 bit = division_bit(b, e);
    nodes[v].bit = bit;
    It lo = std::partition(b, e, [bit](const Set<W>& x) { return !x.has(bit); });
    if ((size_t)(lo - b) <= M) {
      nodes[v].pos = (u32)(b - sets.begin());
      while (b != e && nodes[v].cnt < M) {
        nodes[v].cnt++;
        nodes[v].minpop = std::min(nodes[v].minpop, b->card());
        ++b;
      }
      if (lo < b) lo = b;
    }
    if (b != lo) {
      u32 z = (u32)nodes.size();
      nodes.emplace_back();
      nodes[v].zero = z;
      build_rec(z, b, lo);
      nodes[v].minpop = std::min(nodes[v].minpop, nodes[z].minpop);
    }
    if (lo != e) {
      u32 o = (u32)nodes.size();
      nodes.emplace_back();
      nodes[v].one = o;
      build_rec(o, lo, e);
      nodes[v].minpop = std::min(nodes[v].minpop, nodes[o].minpop);
    }
  }

  // :57-70
  void build(List<W>&& v) {
    nodes.assign(1, Node{});
    sets = std::move(v);
    sort_unique(sets);
    sets.shrink_to_fit();
    build_rec(0, sets.begin(), sets.end());
    nodes.shrink_to_fit();
  }

  // :353-468 — does some trie set fit inside some query in [b, e)?  All
  // queries have cardinality `card`.
  bool query(const Node& nd, It b, It e, u32 card) const {
    if (card < nd.minpop) return false;
    if (nd.zero) {
      if (query(nodes[nd.zero], b, e, card)) return true;
    } else {
      for (It it = b; it != e; ++it)
        for (u32 i = 0; i < nd.cnt; ++i)
          if (it->contains(sets[nd.pos + i])) return true;
      if (!nd.one) return false;
    }
    u32 bit = nd.bit;
    It lo = std::partition(b, e, [bit](const Set<W>& x) { return !x.has(bit); });
    return lo != e && query(nodes[nd.one], lo, e, card);
  }
  bool contains_subset_of(It b, It e) const {
    if (b == e) return false;
    return query(nodes[0], b, e, b->card());
  }
};

// ---------------------------------------------------------------------------
// Exact (exact.cpp, meet_in_the_middle.cpp, dfs.cpp).
// ---------------------------------------------------------------------------
template <int W>
struct Exact {
  Ctx<W> c;
  const oracle_exact_params& P;
  oracle_trace* trace;
  Aut aut;
  InvAut inv;
  std::vector<SliceLut<W>> fwd, bwd;
  List<W> bfs, ibfs;
  u64 rt = 0;           // reset_threshold
  size_t max_memory = 0;
  static constexpr size_t RESERVE = 16ull << 20;  // exact.hpp:52-53
  static constexpr size_t SZ = sizeof(Set<W>);

  Exact(const Aut& A, const oracle_exact_params& p, oracle_trace* tr) : P(p), trace(tr), aut(A), inv(A) {
    c.n = A.n;
    c.k = A.k;
    c.tail_mask = (A.n % 64) ? ((1ULL << (A.n % 64)) - 1) : ~0ULL;
  }

  void record(int phase, u64 len, size_t a, size_t b, int novisited) {
    if (!trace || trace->count >= trace->capacity) return;
    oracle_trace_step& s = trace->steps[trace->count++];
    s.phase = phase;
    s.len = len;
    s.list_bfs = a;
    s.list_invbfs = b;
    s.novisited = novisited;
  }

  size_t luts_bytes() const {
    size_t t = 0;
    for (auto& l : fwd) t += l.bytes();
    for (auto& l : bwd) t += l.bytes();
    return t;
  }

  void build_luts() {
    fwd.assign(c.k, SliceLut<W>{});
    bwd.assign(c.k, SliceLut<W>{});
    for (u32 a = 0; a < c.k; ++a) {
      fwd[a].build_forward(c, aut, a);
      bwd[a].build_inverse(c, inv, a);
    }
  }

  // ---------------- meet in the middle (meet_in_the_middle.cpp) ----------
  struct Hist {
    double dup = 0, vis = 0, self = 0;
  };
  struct Mitm {
    Exact& X;
    u64 max_rt;
    List<W> bvis, ivis;  // visited; the inverse one holds complements
    u64 last_red_bvis = 0, last_red_ivis = 0, last_bfs = 0, last_ibfs = 0, steps_b = 0, steps_i = 0;
    bool b_novis = false, i_novis = false;
    int phase = 0;  // 0 BFS, 1 IBFS, 2 IDFS
    Hist hb, hi;

    size_t mem() const {
      return (X.bfs.size() + X.ibfs.size() + bvis.size() + ivis.size()) * SZ + X.luts_bytes();
    }

    // :580-593
    bool oom_dfs(size_t list_size) const {
      if (!X.P.dfs) return false;
      size_t additional = list_size * (X.c.k - 1) * SZ;
      size_t taken = (size_t)X.P.dfs_min_list_size * SZ * (X.c.k + 1);
      if (additional <= taken) return false;
      return (size_t)X.P.dfs_min_list_size * SZ * (X.c.k + 1) * (max_rt - X.rt) + additional - taken > X.max_memory;
    }

    static u64 cards(const List<W>& l) {
      u64 s = 0;
      for (auto& x : l) s += x.card();
      return s;
    }

    // :572-577 (the reference returns double here)
    double trie_evn(cost_t m, cost_t p, cost_t q) const {
      cost_t e = ((1.0 + p) / p + 1.0 / (q - p * q)) * std::pow(m, std::log(1.0 + p) / std::log((1.0 + p) / (1.0 + p * q - q)));
      if (e >= 0 && e < m * X.c.n) return (double)e;
      return (double)(m * X.c.n);
    }

    static double reduction(size_t initial, size_t current) {
      if (current > initial) throw std::runtime_error("reduction made the list bigger");
      return static_cast<double>(initial - current) / initial;
    }

    // :347-551
    void decide() {
      const u32 N = X.c.n, K = X.c.k;
      const cost_t SET_COST = 512, MIN_RED = 0.001, CHECK_W = 0.25, SET_W = 0.25;
      const cost_t RED_OF_RED = 1.0 / K;
      auto& lb = X.bfs;
      auto& li = X.ibfs;
      if (lb.size() <= X.P.bfs_small_list_size || li.size() <= X.P.bfs_small_list_size || steps_b == 0 || steps_i == 0) {
        phase = lb.size() <= li.size() ? 0 : 1;
        return;
      }
      const u64 card_b = cards(lb), card_i = cards(li), card_bv = cards(bvis);
      const u64 card_iv = (u64)N * ivis.size() - cards(ivis);
      const cost_t dens_b = static_cast<cost_t>(card_b) / (N * lb.size());
      const cost_t dens_i = static_cast<cost_t>(card_i) / (N * li.size());
      if (hb.vis < MIN_RED) hb.vis = (double)MIN_RED;
      if (hi.vis < MIN_RED) hi.vis = (double)MIN_RED;

      cost_t br_bv = K * (1.0 - hb.dup);
      cost_t c_bv = SET_COST * K * lb.size();
      c_bv += br_bv * lb.size() *
              trie_evn(br_bv * lb.size() + bvis.size(), dens_b,
                       static_cast<cost_t>(br_bv * card_b + card_bv) / (N * (br_bv * lb.size() + bvis.size())));
      br_bv *= (1.0 - hb.vis);
      c_bv += li.size() * trie_evn(br_bv * lb.size(), dens_i, dens_b);

      cost_t br_bn = K * (1.0 - hb.dup);
      cost_t c_bn = SET_COST * K * lb.size();
      c_bn += br_bn * lb.size() *
              trie_evn(br_bn * lb.size(), dens_b, static_cast<cost_t>(br_bn * card_b) / (N * (br_bn * lb.size())));
      if (b_novis) br_bn *= (1.0 - hb.vis);
      c_bn += li.size() * trie_evn(br_bn * lb.size(), dens_i, dens_b);

      cost_t br_iv = K * (1.0 - hi.dup);
      cost_t c_iv = SET_COST * K * li.size();
      c_iv += br_iv * li.size() * trie_evn(br_iv * li.size(), 1.0 - dens_i, 1.0 - dens_i);
      br_iv *= (1.0 - hi.self);
      c_iv += br_iv * li.size() *
              trie_evn(ivis.size(), 1.0 - dens_i, 1.0 - static_cast<cost_t>(card_iv) / (N * ivis.size()));
      br_iv *= (1.0 - hi.vis);
      c_iv += br_iv * li.size() * trie_evn(lb.size(), dens_i, dens_b);

      cost_t br_in = K * (1.0 - hi.dup);
      cost_t c_in = SET_COST * K * li.size();
      c_in += br_in * li.size() * trie_evn(br_in * li.size(), 1.0 - dens_i, 1.0 - dens_i);
      br_in *= (1.0 - hi.self);
      c_in += br_in * li.size() * trie_evn(lb.size(), dens_i, dens_b);

      const size_t mu = mem();
      const size_t mbv = bvis.size() * SZ, miv = ivis.size() * SZ;
      u32 inf = 0;
      const cost_t INF = std::numeric_limits<cost_t>::infinity();
      if (b_novis || mu + mbv > X.max_memory || mu + 2 * SZ * lb.size() * K > X.max_memory || oom_dfs(lb.size())) {
        c_bv = INF;
        inf++;
      }
      if (mu - mbv + 2 * SZ * lb.size() * K > X.max_memory || oom_dfs(lb.size())) {
        c_bn = INF;
        inf++;
      }
      if (i_novis || mu + miv > X.max_memory || mu + 2 * SZ * li.size() * K > X.max_memory || oom_dfs(li.size())) {
        c_iv = INF;
        inf++;
      }
      if (mu - miv + SZ * li.size() * K > X.max_memory || oom_dfs(li.size())) {
        c_in = INF;
        inf++;
      }

      cost_t br_dfs = std::max(K * (1.0 - hi.dup * RED_OF_RED), static_cast<cost_t>(1.0));
      u64 remaining = max_rt - X.rt;
      // the reference takes a uint depth here
      auto total = [&](u32 depth) { return br_dfs * (std::pow(br_dfs, depth) - 1.0) / (br_dfs - 1.0); };
      const cost_t dfs_set = SET_COST * SET_W * K / br_dfs;
      cost_t p_bv = c_bv + li.size() * total(remaining - 1) * (dfs_set + CHECK_W * trie_evn(br_bv * lb.size(), dens_i, dens_b));
      cost_t p_bn = c_bn + li.size() * total(remaining - 1) * (dfs_set + CHECK_W * trie_evn(br_bn * lb.size(), dens_i, dens_b));
      cost_t p_iv = c_iv + br_iv * li.size() * total(remaining - 1) * (dfs_set + CHECK_W * trie_evn(lb.size(), dens_i, dens_b));
      cost_t p_in = c_in + br_in * li.size() * total(remaining - 1) * (dfs_set + CHECK_W * trie_evn(lb.size(), dens_i, dens_b));
      cost_t p_dfs = li.size() * total(remaining) * (dfs_set + CHECK_W * trie_evn(lb.size(), dens_i, dens_b));
      cost_t mn = std::min(std::min(p_bv, p_bn), std::min(p_iv, p_in));
      if (inf == 4) {
        phase = 2;
        return;
      }
      if (X.P.dfs_shortcut && p_dfs < mn) {
        phase = 2;
        return;
      }
      if (p_bv < p_bn && p_iv < p_in) {
        phase = (c_iv < c_bv) ? 1 : 0;
        return;
      }
      if (mn == p_bv) {
        phase = 0;
        return;
      }
      if (mn == p_bn) {
        b_novis = true;
        List<W>().swap(bvis);
        phase = 0;
        return;
      }
      if (mn == p_iv) {
        phase = 1;
        return;
      }
      if (mn == p_in) {
        i_novis = true;
        List<W>().swap(ivis);
        phase = 1;
        return;
      }
      throw std::runtime_error("Impossible");
    }

    // :179-242
    void bfs_step() {
      const u32 K = X.c.k;
      const u32 T = X.P.threads;
      auto& lb = X.bfs;
      const size_t next = lb.size() * K;
      if (mem() + SZ * next > X.max_memory || oom_dfs(lb.size())) throw OutOfMemory{};
      List<W> nx(next);
      for (u32 a = 0; a < K; ++a) X.fwd[a].apply_many(lb.data(), nx.data() + a * lb.size(), lb.size(), T);
      lb = std::move(nx);
      if (b_novis) {
        size_t s0 = lb.size();
        sort_unique(lb);
        hb.dup = reduction(s0, lb.size());
        if (mem() + lb.size() * SZ > X.max_memory) throw OutOfMemory{};
        size_t s1 = lb.size();
        reduce_self(lb, true, T);
        hb.vis = reduction(s1, lb.size());
      } else {
        if (mem() + lb.size() * SZ > X.max_memory) throw OutOfMemory{};
        sort_unique(bvis);
        size_t s0 = lb.size();
        sort_unique(lb);
        hb.dup = reduction(s0, lb.size());
        size_t old = bvis.size();
        bvis.reserve(old + lb.size());
        size_t j = 0;
        for (const auto& s : lb) {
          while (j < old && bvis[j] < s) ++j;
          if (j == old || bvis[j] != s) bvis.push_back(s);
        }
        lb.assign(bvis.begin() + old, bvis.end());
        std::sort(bvis.begin(), bvis.end());
        size_t s1 = lb.size();
        reduce_by(bvis, lb, true, true, T);
        hb.vis = reduction(s1, lb.size());
      }
    }

    // :245-344
    void ibfs_step() {
      const u32 K = X.c.k;
      const u32 T = X.P.threads;
      auto& li = X.ibfs;
      const size_t next = li.size() * K;
      if (mem() + SZ * next > X.max_memory || oom_dfs(li.size())) throw OutOfMemory{};
      List<W> nx(next);
      for (u32 a = 0; a < K; ++a) X.bwd[a].apply_many(li.data(), nx.data() + a * li.size(), li.size(), T);
      li = std::move(nx);
      auto neg_all = [&] {
        for (auto& s : li) X.c.negate(s);
      };
      if (i_novis) {
        hi.vis = 0;
        neg_all();
        size_t s0 = li.size();
        sort_unique(li);
        hi.dup = reduction(s0, li.size());
        size_t s1 = li.size();
        if (mem() + li.size() * SZ > X.max_memory) {
          neg_all();
          throw OutOfMemory{};
        }
        reduce_self(li, true, T);
        hi.self = reduction(s1, li.size());
        neg_all();
      } else {
        if (mem() + SZ * li.size() > X.max_memory) throw OutOfMemory{};
        neg_all();
        sort_unique(ivis);
        size_t s0 = li.size();
        sort_unique(li);
        hi.dup = reduction(s0, li.size());
        size_t s1 = li.size();
        if (mem() + li.size() * SZ > X.max_memory) {
          neg_all();
          throw OutOfMemory{};
        }
        reduce_self(li, true, T);
        hi.self = reduction(s1, li.size());
        std::sort(li.begin(), li.end());
        size_t s2 = li.size();
        reduce_by(ivis, li, false, true, T);
        hi.vis = reduction(s2, li.size());
        std::sort(li.begin(), li.end());
        ivis.insert(ivis.end(), li.begin(), li.end());
        neg_all();
      }
    }

    // :58-107
    bool run() {
      bool found = false;
      while (X.rt < max_rt) {
        if (mem() > X.max_memory) break;
        decide();
        if (phase == 2) break;
        X.rt++;
        try {
          if (phase == 0) {
            X.record(0, X.rt, X.bfs.size(), X.ibfs.size(), b_novis);
            steps_b++;
            bool red = !b_novis && (bvis.size() >= (u64)X.c.k * X.c.k * last_red_bvis);
            if (red) {
              u32 mx = 0;
              for (auto& s : X.bfs) mx = std::max(mx, s.card());
              bvis.erase(std::remove_if(bvis.begin(), bvis.end(), [mx](const Set<W>& s) { return s.card() > mx; }),
                         bvis.end());
              reduce_self(bvis, false, X.P.threads);
              last_red_bvis = bvis.size();
            }
            last_bfs = X.bfs.size();
            bfs_step();
          } else {
            X.record(1, X.rt, X.bfs.size(), X.ibfs.size(), i_novis);
            steps_i++;
            bool red = !i_novis && (ivis.size() >= (u64)X.c.k * X.c.k * last_red_ivis);
            if (red) {
              reduce_self(ivis, false, X.P.threads);
              last_red_ivis = ivis.size();
            }
            last_ibfs = X.ibfs.size();
            ibfs_step();
          }
          auto it = contains_subset(X.bfs, X.ibfs, false, false, X.P.threads);
          if (it != X.ibfs.end()) {
            found = true;
            break;
          }
        } catch (OutOfMemory&) {
          X.rt--;
          break;
        }
      }
      List<W>().swap(bvis);
      List<W>().swap(ivis);
      return found;
    }
  };

  // ---------------- inverse DFS (dfs.cpp) -------------------------------
  struct Dfs {
    Exact& X;
    u64 max_depth;
    size_t dfs_max = 0;
    ExplicitTrie<W> trie;
    List<W>& li;

    size_t mem() const { return (X.bfs.size() + li.size()) * SZ + trie.bytes() + X.luts_bytes(); }

    // dfs.cpp:350-373
    void update_max_list_size() {
      size_t mu = mem();
      if (X.max_memory < mu) {
        if (X.P.strict_memory_limit) throw OutOfMemory{};
      }
      mu -= li.size() * SZ;
      dfs_max = static_cast<size_t>((X.max_memory - mu) / (SZ * (X.c.k + 1) * (max_depth - X.rt)));
      if (dfs_max < X.P.dfs_min_list_size) {
        if (X.P.strict_memory_limit) throw OutOfMemory{};
        dfs_max = X.P.dfs_min_list_size;
      }
    }

    // dfs.cpp:102-159
    void prepare() {
      const u32 N = X.c.n;
      std::vector<double> w(N, 0.0);
      for (auto& s : X.bfs)
        for (u32 i = 0; i < N; ++i)
          if (s.has(i)) w[i]++;
      std::vector<std::pair<double, u32>> idx(N);
      for (u32 i = 0; i < N; ++i) idx[i] = {1.0 - w[i] / (X.bfs.size() * N), i};
      std::sort(idx.begin(), idx.end());
      std::vector<u32> order(N);
      for (u32 i = 0; i < N; ++i) order[idx[i].second] = i;
      for (auto& s : X.bfs) s = X.c.permute(s, order);
      for (auto& s : li) s = X.c.permute(s, order);
      X.aut = permute_aut(X.aut, order);
      X.inv = InvAut(X.aut);
      X.build_luts();
      trie.n = N;
      trie.threads = X.P.threads;
      trie.build(std::move(X.bfs));
      List<W>().swap(X.bfs);
      update_max_list_size();
    }

    // dfs.cpp:228-347
    std::tuple<bool, size_t, size_t> step(size_t b, size_t e, bool red_dup, size_t red_sub) {
      const u32 K = X.c.k, N = X.c.n;
      size_t nb = li.size();
      li.resize(li.size() + K * (e - b));
      size_t ne = li.size();
      for (u32 a = 0; a < K; ++a) X.bwd[a].apply_many(li.data() + b, li.data() + nb + a * (e - b), e - b, X.P.threads);
      if (red_sub) {
        List<W> vec(li.begin() + nb, li.begin() + ne);
        for (auto& s : vec) X.c.negate(s);
        List<W> red(vec.begin(), vec.begin() + std::min(vec.size(), red_sub));
        reduce_by(red, vec, true, false, X.P.threads);
        for (auto& s : vec) X.c.negate(s);
        std::copy(vec.begin(), vec.end(), li.begin() + nb);
        ne = nb + vec.size();
        li.resize(ne);
      }
      // subset_utils.hpp:58-110 — bucket by cardinality, descending.
      std::vector<std::pair<size_t, size_t>> seg(N + 1);
      {
        std::vector<size_t> cnt(N + 2, 0);
        for (size_t i = nb; i < ne; ++i) cnt[li[i].card()]++;
        std::vector<size_t> start(N + 1);
        size_t acc = nb;
        for (int cd = (int)N; cd >= 0; --cd) {
          start[cd] = acc;
          acc += cnt[cd];
        }
        List<W> tmp(li.begin() + nb, li.begin() + ne);
        std::vector<size_t> fill = start;
        for (auto& s : tmp) li[fill[s.card()]++] = s;
        for (u32 cd = 0; cd <= N; ++cd) {
          seg[cd] = {start[cd], fill[cd]};
          if (red_dup && start[cd] != fill[cd])
            std::sort(li.begin() + start[cd], li.begin() + fill[cd], comp_fast<W>);
        }
      }
      li.resize(seg[1].first);
      ne = li.size();
      if (red_dup) {
        ne = std::unique(li.begin() + nb, li.begin() + ne) - li.begin();
        li.resize(ne);
        size_t lo = nb;
        for (u32 sz = N; sz >= 2; --sz) {
          size_t hi = lo;
          while (hi != ne && li[hi].card() == sz) ++hi;
          seg[sz] = {lo, hi};
          lo = hi;
        }
      }
      if (X.P.threads > 1 && ne - nb > 32) {
        std::atomic<bool> ret{false};
        std::vector<std::thread> th;
        std::vector<u32> buckets;
        for (u32 sz = N; sz >= 2; --sz)
          if (seg[sz].first != seg[sz].second) buckets.push_back(sz);
        std::atomic<size_t> next{0};
        for (u32 t = 0; t < X.P.threads; ++t)
          th.emplace_back([&] {
            size_t i;
            while ((i = next++) < buckets.size()) {
              auto [lo, hi] = seg[buckets[i]];
              if (trie.contains_subset_of(li.begin() + lo, li.begin() + hi)) ret = true;
            }
          });
        for (auto& x : th) x.join();
        return {ret.load(), nb, ne};
      }
      for (u32 sz = N; sz >= 2; --sz) {
        auto [lo, hi] = seg[sz];
        if (lo == hi) continue;
        if (trie.contains_subset_of(li.begin() + lo, li.begin() + hi)) return {true, nb, ne};
      }
      return {false, nb, ne};
    }

    // dfs.cpp:161-218
    void process(size_t b, size_t e, u64 lsw, u64 depth) {
      size_t initial = li.size();
      size_t size = e - b;
      bool red_dup = (depth <= 3 || depth % 2 == 0) && lsw + 1 < max_depth;
      size_t red_sub = (depth % 3 == 0 && depth <= 6 && lsw + 10 < max_depth) ? 20000 : 0;
      auto [found, nb, ne] = step(b, e, red_dup, red_sub);
      if (found) {
        max_depth = lsw;
        if (max_depth > X.rt) update_max_list_size();
        if (X.trace) X.record(3, lsw + 1, 0, 0, 0);
        li.resize(initial);
        return;
      }
      if (lsw + 1 >= max_depth) {
        li.resize(initial);
        return;
      }
      size_t next = ne - nb;
      size_t part = dfs_max >= size / 2 ? dfs_max : size / 2;
      size_t pos = 0;
      while (pos + part < next) {
        process(nb + pos, nb + pos + part, lsw + 1, depth + 1);
        if (lsw + 1 >= max_depth) {
          li.resize(initial);
          return;
        }
        pos += part;
        part = dfs_max >= size / 2 ? dfs_max : size / 2;
      }
      process(nb + pos, ne, lsw + 1, depth + 1);
      li.resize(initial);
    }

    // dfs.cpp:63-91
    bool run() {
      if (X.rt == max_depth) return true;
      try {
        prepare();
        X.record(2, X.rt, trie.sets.size(), li.size(), 0);
        process(0, li.size(), X.rt, 0);
      } catch (OutOfMemory&) {
        return false;
      }
      X.rt = max_depth;
      return true;
    }
  };

  // exact.cpp:37-97 (bounds are in/out as in AlgoResult).
  void run(oracle_bounds& R) {
    if (R.non_synchro || R.lower == R.upper) return;
    if (c.n == 1) {
      R.lower = R.upper = 0;
      return;
    }
    rt = 0;
    // exact.cpp:167-175: below the reserve the reference only logs an error
    // and keeps the unreduced budget.
    max_memory = (size_t)P.max_memory_mb * 1024 * 1024;
    if (max_memory >= RESERVE) max_memory -= RESERVE;
    bfs.push_back(c.complete());
    for (u32 q : backward_seeds(aut, inv)) ibfs.push_back(c.singleton(q));
    std::vector<u32> order = exact_state_order(aut, inv);
    aut = permute_aut(aut, order);
    inv = InvAut(aut);
    for (auto& s : bfs) s = c.permute(s, order);
    for (auto& s : ibfs) s = c.permute(s, order);
    build_luts();

    Mitm m{*this, R.upper - 1};
    bool found = m.run();
    if (!found && P.dfs) {
      Dfs d{*this, R.upper - 1, 0, ExplicitTrie<W>{}, ibfs};
      if (d.run()) {
        rt++;
        found = true;
      }
    }
    if (!found) {
      rt++;
      if (rt == R.upper) found = true;
    }
    R.lower = std::max<u64>(R.lower, rt);
    if (found) R.upper = rt;
  }
};

// ---------------------------------------------------------------------------
// Beam (beam.hpp:31-188, 351-369).
// ---------------------------------------------------------------------------
template <int W>
struct Beam {
  Ctx<W> c;
  const oracle_beam_params& P;

  Beam(u32 n, u32 k, const oracle_beam_params& p) : P(p) {
    c.n = n;
    c.k = k;
    c.tail_mask = (n % 64) ? ((1ULL << (n % 64)) - 1) : ~0ULL;
  }

  // beam.hpp:98-188
  u64 cutoff(const Aut& A, const InvAut& I, u32 beam_size, u64 max_mlsw) {
    List<W> list, next;
    for (u32 q : backward_seeds(A, I)) list.push_back(c.singleton(q));
    std::vector<SliceLut<W>> luts(c.k);
    for (u32 a = 0; a < c.k; ++a) luts[a].build_inverse(c, I, a);
    for (u64 len = 1; len < max_mlsw; ++len) {
      if (P.max_iter >= 0 && (int64_t)len > P.max_iter) break;
      next.resize((size_t)c.k * list.size());
      for (u32 a = 0; a < c.k; ++a) luts[a].apply_many(list.data(), next.data() + a * list.size(), list.size(), 1);
      std::swap(list, next);
      // cardinality-descending buckets, each sorted by comp_fast
      std::vector<size_t> cnt(c.n + 2, 0);
      for (auto& s : list) cnt[s.card()]++;
      std::vector<size_t> start(c.n + 1);
      size_t acc = 0;
      for (int cd = (int)c.n; cd >= 0; --cd) {
        start[cd] = acc;
        acc += cnt[cd];
      }
      List<W> tmp(list);
      std::vector<size_t> fill = start;
      for (auto& s : tmp) list[fill[s.card()]++] = s;
      for (u32 cd = 0; cd <= c.n; ++cd)
        if (start[cd] != fill[cd]) std::sort(list.begin() + start[cd], list.begin() + fill[cd], comp_fast<W>);
      if (list[0].card() == c.n) return len;
      list.erase(std::unique(list.begin(), list.end()), list.end());
      if (list.size() > beam_size) list.resize(beam_size);
    }
    return max_mlsw;
  }

  void run(const Aut& A0, oracle_bounds& R) {
    if (R.non_synchro || R.lower == R.upper) return;
    if (c.n == 1) {
      R.lower = R.upper = 0;
      return;
    }
    std::vector<u32> perm(c.n);
    std::iota(perm.begin(), perm.end(), 0u);
    if (P.presort_indeg) {  // beam.hpp:351-369
      std::vector<std::pair<double, int>> d(c.n);
      for (u32 q = 0; q < c.n; ++q) d[q] = {0, (int)q};
      for (u32 q = 0; q < c.n; ++q)
        for (u32 a = 0; a < c.k; ++a) d[A0.at(q, a)].first++;
      std::sort(d.begin(), d.end());
      for (u32 q = 0; q < c.n; ++q) perm[d[q].second] = q;
    }
    Aut A = permute_aut(A0, perm);
    InvAut I(A);
    u32 bound;
    if (P.dynamic) {
      bound = (u32)cutoff(A, I, (u32)P.min_beam_size, R.upper);
      cost_t exact_cost = 2 * std::pow(static_cast<cost_t>(c.k), (bound + 1) / 2);
      cost_t proposed = std::round(exact_cost * (cost_t)P.beam_exact_ratio / bound);
      u32 bs = (u32)std::clamp<cost_t>(proposed, (cost_t)(u32)P.min_beam_size, (cost_t)(u32)P.max_beam_size);
      if (bs > (u32)P.min_beam_size) bound = (u32)cutoff(A, I, bs, bound);
    } else {
      bound = (u32)cutoff(A, I, (u32)P.beam_size, R.upper);
    }
    R.upper = bound;
  }
};

template <int W>
static int exact_w(const Aut& A, const oracle_exact_params* p, oracle_bounds* R, oracle_trace* tr) {
  Exact<W> X(A, *p, tr);
  X.run(*R);
  return 0;
}

template <int W>
static int beam_w(const Aut& A, const oracle_beam_params* p, oracle_bounds* R) {
  Beam<W> B(A.n, A.k, *p);
  B.run(A, *R);
  return 0;
}

}  // namespace orc

extern "C" {

int oracle_exact(const uint32_t* delta, uint32_t n, uint32_t k, const oracle_exact_params* p, oracle_bounds* r,
                 oracle_trace* trace) {
  if (!delta || !p || !r || n == 0 || k == 0 || n > 512) return -1;
  for (size_t i = 0; i < (size_t)n * k; ++i)
    if (delta[i] >= n) return -2;
  orc::Aut A{n, k, std::vector<uint32_t>(delta, delta + (size_t)n * k)};
  try {
    switch ((n + 63) / 64) {
      case 1: return orc::exact_w<1>(A, p, r, trace);
      case 2: return orc::exact_w<2>(A, p, r, trace);
      case 3: return orc::exact_w<3>(A, p, r, trace);
      case 4: return orc::exact_w<4>(A, p, r, trace);
      case 5: return orc::exact_w<5>(A, p, r, trace);
      case 6: return orc::exact_w<6>(A, p, r, trace);
      case 7: return orc::exact_w<7>(A, p, r, trace);
      case 8: return orc::exact_w<8>(A, p, r, trace);
    }
  } catch (std::exception&) {
    return -3;
  }
  return -1;
}

int oracle_beam(const uint32_t* delta, uint32_t n, uint32_t k, const oracle_beam_params* p, oracle_bounds* r) {
  if (!delta || !p || !r || n == 0 || k == 0 || n > 512) return -1;
  for (size_t i = 0; i < (size_t)n * k; ++i)
    if (delta[i] >= n) return -2;
  orc::Aut A{n, k, std::vector<uint32_t>(delta, delta + (size_t)n * k)};
  switch ((n + 63) / 64) {
    case 1: return orc::beam_w<1>(A, p, r);
    case 2: return orc::beam_w<2>(A, p, r);
    case 3: return orc::beam_w<3>(A, p, r);
    case 4: return orc::beam_w<4>(A, p, r);
    case 5: return orc::beam_w<5>(A, p, r);
    case 6: return orc::beam_w<6>(A, p, r);
    case 7: return orc::beam_w<7>(A, p, r);
    case 8: return orc::beam_w<8>(A, p, r);
  }
  return -1;
}

// Shortest reset length by plain power-set BFS over bit masks (n <= 24).
// Independent of every trick above; used to cross-check tiny automata
// (brute.hpp:88-122 does the same with a distance array).
int oracle_brute(const uint32_t* delta, uint32_t n, uint32_t k, int64_t* out) {
  if (!delta || !out || n == 0 || n > 24 || k == 0) return -1;
  if (n == 1) {
    *out = 0;
    return 0;
  }
  const uint32_t full = (n == 32) ? 0xFFFFFFFFu : ((1u << n) - 1);
  std::vector<uint8_t> seen((size_t)1 << n, 0);
  std::vector<uint32_t> cur{full}, nxt;
  seen[full] = 1;
  for (int64_t d = 0; !cur.empty(); ++d) {
    for (uint32_t s : cur)
      if (__builtin_popcount(s) == 1) {
        *out = d;
        return 0;
      }
    nxt.clear();
    for (uint32_t s : cur)
      for (uint32_t a = 0; a < k; ++a) {
        uint32_t t = 0;
        for (uint32_t x = s; x; x &= x - 1) t |= 1u << delta[(size_t)__builtin_ctz(x) * k + a];
        if (!seen[t]) {
          seen[t] = 1;
          nxt.push_back(t);
        }
      }
    cur.swap(nxt);
  }
  *out = -1;  // not synchronizing
  return 0;
}

// Eppstein's greedy bound (eppstein.hpp:82-114) over the pairs tree
// (pairs_tree.hpp:25-62), restated sequentially with the reference's FIFO
// queue so that every pair records the same first letter.  `r` in/out as
// AlgoResult; word (capacity word_cap) receives the greedy word.
// Returns 0, or -1 on bad arguments; *word_len = letters written.
int oracle_eppstein(const uint32_t* delta, uint32_t n, uint32_t k, oracle_bounds* r, uint32_t* word,
                    uint64_t word_cap, uint64_t* word_len) {
  if (!delta || !r || n == 0 || k == 0 || n > 512) return -1;
  for (size_t i = 0; i < (size_t)n * k; ++i)
    if (delta[i] >= n) return -1;
  if (word_len) *word_len = 0;
  if (r->non_synchro || r->lower == r->upper) return 0;  // eppstein.hpp:28-34
  orc::Aut A{n, k, std::vector<uint32_t>(delta, delta + (size_t)n * k)};
  orc::InvAut inv(A);
  const size_t N = n;
  std::vector<uint32_t> len(N * N, 0), let(N * N, 0);
  std::vector<std::pair<uint32_t, uint32_t>> queue;
  queue.reserve(N * (N - 1) / 2);
  for (uint32_t t = 0; t < n; ++t)
    for (uint32_t a = 0; a < k; ++a)
      for (uint32_t i1 = inv.begin[a * n + t]; i1 < inv.end[a * n + t]; ++i1)
        for (uint32_t i2 = i1 + 1; i2 < inv.end[a * n + t]; ++i2) {
          const uint32_t p = inv.edges[a * n + i1], q = inv.edges[a * n + i2];
          if (len[p * N + q]) continue;
          len[p * N + q] = len[q * N + p] = 1;
          let[p * N + q] = let[q * N + p] = a;
          queue.push_back({p, q});
        }
  for (size_t head = 0; head < queue.size() && queue.size() < N * (N - 1) / 2; ++head) {
    const uint32_t v1 = queue[head].first, v2 = queue[head].second;
    const uint32_t l = len[v1 * N + v2] + 1;
    for (uint32_t a = 0; a < k; ++a)
      for (uint32_t i1 = inv.begin[a * n + v1]; i1 < inv.end[a * n + v1]; ++i1)
        for (uint32_t i2 = inv.begin[a * n + v2]; i2 < inv.end[a * n + v2]; ++i2) {
          const uint32_t p = inv.edges[a * n + i1], q = inv.edges[a * n + i2];
          if (len[p * N + q]) continue;
          len[p * N + q] = len[q * N + p] = l;
          let[p * N + q] = let[q * N + p] = a;
          queue.push_back({p, q});
        }
  }
  if (queue.size() < N * (N - 1) / 2) {  // pairs_tree.hpp:95-100
    r->non_synchro = 1;
    return 0;
  }
  std::vector<char> cur(n, 1), nxt(n);
  uint64_t total = 0, wl = 0;
  size_t size = n;
  do {
    uint32_t p = 0, q = 0, l = n * n;
    for (uint32_t v1 = 0; v1 + 1 < n; ++v1)
      if (cur[v1])
        for (uint32_t v2 = v1 + 1; v2 < n; ++v2)
          if (cur[v2] && len[v1 * N + v2] < l) {
            p = v1;
            q = v2;
            l = len[v1 * N + v2];
          }
    total += l;
    if (total > r->upper) return 0;  // bound unchanged (eppstein.hpp:104-106)
    while (p != q) {
      const uint32_t a = let[p * N + q];
      if (word && wl < word_cap) word[wl] = a;
      ++wl;
      std::fill(nxt.begin(), nxt.end(), 0);
      for (uint32_t s = 0; s < n; ++s)
        if (cur[s]) nxt[A.at(s, a)] = 1;
      cur.swap(nxt);
      p = A.at(p, a);
      q = A.at(q, a);
    }
    size = 0;
    for (uint32_t s = 0; s < n; ++s) size += cur[s];
  } while (size > 1);
  r->upper = total;
  if (word_len) *word_len = wl;
  return 0;
}

}  // extern "C"
