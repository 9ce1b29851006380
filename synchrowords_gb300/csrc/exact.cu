// Host driver of the GPU exact search and beam (see exact.hpp).
//
// Exact (synchrolib/algorithm/exact/exact.cpp:37-97, meet_in_the_middle.cpp:58-344):
// two frontiers live on the device,
//   F: forward images  delta(Q, w), seeded with {Q}           (exact.cpp:130-146)
//   B: inverse preimages, seeded with sink singletons whose
//      state has some letter of in-degree > 1                (exact.cpp:149-164)
// B is stored as complements: the preimage of a complement is the complement
// of the preimage, so the same expansion, dedup and dominance code serves both
// sides.  One step expands the smaller side (meet_in_the_middle.cpp:355-358),
// sorts and deduplicates the children, drops every child that has a visited
// set inside it or a proper subset in its own layer
// (meet_in_the_middle.cpp:179-344 on complements for B), and then asks
// whether some F is disjoint from some B-complement (F ⊆ B,
// meet_in_the_middle.cpp:90).  Each kept child records (letter, parent) so the
// meeting pair yields a word, which is verified on the host before it is
// returned.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>

#include "algos.cuh"
#include "exact.hpp"
#include "kernels.cuh"
#include "learn.hpp"

namespace sw {

namespace {

struct Layer {
  DevBuf origin;        // per kept set: child position a*parent_count + parent
  u32 count = 0;
  u32 parent_count = 0;
};

struct Side {
  DevBuf rows, rows_alt;
  u32 count = 0;
  DevBuf vis, vis_alt;
  u32 vis_count = 0;
  std::vector<std::unique_ptr<Layer>> layers;
  std::vector<u64> seed_states;  // backward side: the state of each seed row
  double unique_growth = 0;      // distinct children per parent at the last step
  KeyMap keymap;                 // sort key of this side's layers and visited list
  bool keymap_chosen = false;
  // Layers of earlier solves, kept with their device buffers, so that a
  // solve's layers reuse them instead of allocating: a new layer takes the
  // spare whose origin buffer holds `origin_bytes` with the least room to
  // spare, else the largest (which then grows).
  std::vector<std::unique_ptr<Layer>> spare;
  std::unique_ptr<Layer> new_layer(size_t origin_bytes) {
    if (spare.empty()) return std::make_unique<Layer>();
    size_t best = 0;
    for (size_t i = 1; i < spare.size(); ++i) {
      const size_t c = spare[i]->origin.cap, cb = spare[best]->origin.cap;
      const bool fits = c >= origin_bytes, best_fits = cb >= origin_bytes;
      if (fits ? (!best_fits || c < cb) : (!best_fits && c > cb)) best = i;
    }
    std::unique_ptr<Layer> L = std::move(spare[best]);
    spare[best] = std::move(spare.back());
    spare.pop_back();
    L->count = L->parent_count = 0;
    return L;
  }
  void reset() {
    count = vis_count = 0;
    unique_growth = 0;
    keymap = KeyMap{};
    keymap_chosen = false;
    for (auto& L : layers) spare.push_back(std::move(L));
    layers.clear();
    seed_states.clear();
  }
};

// One level of the bounded inverse phase (a chunk of parents' children).
struct DLevel {
  DevBuf rows, origin;
  u32 count = 0;
  u32 chunk_off = 0, chunk_cnt = 0;  // parent slice this level was expanded from
};

}  // namespace

class Engine {
 public:
  explicit Engine(int device) {
    SW_CUDA(cudaSetDevice(device));
    SW_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    pinned.reserve(4096);
    SW_CUDA(cudaMalloc(&d_misc, 64 * sizeof(u32)));
    SW_CUDA(cudaMemset(d_misc, 0, 64 * sizeof(u32)));
    mlp = std::make_unique<MlpRunner>(stream);
  }
  ~Engine() {
    for (auto e : ev_pool) cudaEventDestroy(e);
    if (d_query_bytes) cudaFree(d_query_bytes);
    if (d_misc) cudaFree(d_misc);
    if (stream) cudaStreamDestroy(stream);
  }

  cudaStream_t stream = nullptr;
  HostPinned pinned;
  std::unique_ptr<MlpRunner> mlp;

  // ---- optional per-kernel-class timing (CUDA events on `stream`) ----
  // class 0: subset-query tree walks, 1: layer expansion, 2: radix sorts,
  // 3: everything else (unique/compaction/tree build/merge).
  struct ProfClass {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    u64 launches = 0;
    double bytes = 0;
  };
  bool prof_on = false;
  ProfClass prof[4];
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_next = 0;
  u64* d_query_bytes = nullptr;
  cudaEvent_t next_event() {
    if (ev_next == ev_pool.size()) {
      cudaEvent_t e;
      SW_CUDA(cudaEventCreate(&e));
      ev_pool.push_back(e);
    }
    return ev_pool[ev_next++];
  }
  template <class Fn>
  void timed(int cls, double bytes, Fn&& fn) {
    if (!prof_on) {
      fn();
      return;
    }
    cudaEvent_t a = next_event(), b = next_event();
    SW_CUDA(cudaEventRecord(a, stream));
    fn();
    SW_CUDA(cudaEventRecord(b, stream));
    prof[cls].ev.emplace_back(a, b);
    prof[cls].launches++;
    prof[cls].bytes += bytes;
  }
  void profile_begin() {
    if (!d_query_bytes) SW_CUDA(cudaMalloc(&d_query_bytes, sizeof(u64)));
    SW_CUDA(cudaMemsetAsync(d_query_bytes, 0, sizeof(u64), stream));
    for (auto& c : prof) c = ProfClass{};
    scan_ev.clear();
    ev_next = 0;
    prof_on = true;
  }
  void profile_end(sw_kernel_profile out[4]) {
    SW_CUDA(cudaStreamSynchronize(stream));
    u64 qb = 0;
    SW_CUDA(cudaMemcpy(&qb, d_query_bytes, sizeof(u64), cudaMemcpyDeviceToHost));
    prof[0].bytes += (double)qb;
    for (int c = 0; c < 4; ++c) {
      double ms = 0;
      for (auto& pr : prof[c].ev) {
        float t = 0;
        SW_CUDA(cudaEventElapsedTime(&t, pr.first, pr.second));
        ms += t;
      }
      out[c].launches = prof[c].launches;
      out[c].ms = ms;
      out[c].bytes = prof[c].bytes;
    }
    for (int i = 0; i < 8 * kScanSizeClasses; ++i) {
      scan_ms[i] = 0;
      scan_launches[i] = 0;
    }
    for (auto& kv : scan_ev) {
      float t = 0;
      SW_CUDA(cudaEventElapsedTime(&t, kv.second.first, kv.second.second));
      scan_ms[kv.first] += t;
      scan_launches[kv.first]++;
    }
    prof_on = false;
  }
  u32* d_misc = nullptr;  // [0..3] witness, [8] scan total, [kScanErrWord] bounded-wait timeouts
  static constexpr int kScanErrWord = 4;  // read back with the witness, never cleared by it
  // Throws if a launch reported a bounded wait that ran out: 1 = a subset
  // check's tile copy never arrived, 2 = a compaction tile's look-back never
  // saw its predecessor; `w` is the pinned copy of d_misc[kScanErrWord].
  static void check_scan_error(u32 w) {
    if (w == 2) throw CudaError("layer compaction: a look-back wait ran out");
    if (w) throw CudaError("subset check: a tile copy did not complete within its wait limit");
  }
  // Single-pass duplicate removal (launch_dedup_compact): its tile status
  // words (zero-filled when allocated), tile counter and launch epoch.
  DevBuf dc_status, dc_ctr;
  size_t dc_status_zeroed = 0;
  u32 dc_epoch = 0;
  u32 next_dc_epoch(u32 m) {
    const size_t words = dedup_compact_status_words(m);
    if (!dc_ctr.p) {
      dc_ctr.reserve(sizeof(u32));
      SW_CUDA(cudaMemsetAsync(dc_ctr.p, 0, sizeof(u32), stream));
    }
    if (++dc_epoch >= (1u << 30)) dc_epoch = 0;  // wrapped: every word back to "unpublished"
    if (dc_status.cap < sizeof(u64) * words || dc_epoch == 0) {
      dc_status.reserve(sizeof(u64) * std::max<size_t>(words, (size_t)1 << 16));
      SW_CUDA(cudaMemsetAsync(dc_status.p, 0, dc_status.cap, stream));
      if (dc_epoch == 0) dc_epoch = 1;
    }
    return dc_epoch;
  }
  // The compaction's count and the timeout word in one read-back.
  u32 read_total_checked() {
    SW_CUDA(cudaMemcpyAsync(pinned.p, d_misc + kScanErrWord, 5 * sizeof(u32), cudaMemcpyDeviceToHost, stream));
    SW_CUDA(cudaStreamSynchronize(stream));
    const u32* w = pinned.as<u32>();
    check_scan_error(w[0]);
    return w[8 - kScanErrWord];
  }
  // tables
  DevBuf t_delta, t_beg, t_src;
  TransTables tables;
  // scratch
  DevBuf ch_rows, ch_vals, alt_rows, alt_vals, uq_rows, uq_vals, new_vals;
  DevBuf epp_scratch, epp_word, br_visited, br_arena;
  DevBuf flags_a, flags_b, keep, pos, sort_tmp, scan_tmp, keys, keys_alt, sorted_rows;

  // Sort m rows in place by layer key (word 0, then a mix of the other words).
  void sort_by_layer_key(int W, u64* rows, u32 m, const KeyMap& map = KeyMap{}) {
    if (m < 2) return;
    keys.reserve(sizeof(u64) * 2 * m);
    ch_vals.reserve(sizeof(u32) * m);
    sorted_rows.reserve(sizeof(u64) * W * m);
    launch_layer_keys(W, rows, m, keys.as<u64>(), stream, map);
    launch_iota(ch_vals.as<u32>(), m, stream);
    sort_rows(2, keys.as<u64>(), ch_vals.as<u32>(), m);
    launch_gather_rows(W, rows, ch_vals.as<u32>(), m, sorted_rows.as<u64>(), stream);
    SW_CUDA(cudaMemcpyAsync(rows, sorted_rows.p, sizeof(u64) * W * m, cudaMemcpyDeviceToDevice, stream));
    count_launch(4);
  }
  Side F, B;
  sw_stats* st = nullptr;
  std::vector<std::unique_ptr<DLevel>> dlevel_pool;  // the bounded phase's per-depth levels
  // scratch of the learned beam and of Reduce, kept across calls
  DevBuf lb_counts, lb_scores, lb_keys, lb_vals, lb_alt_k, lb_alt_v, lb_sel_rows, lb_sel_origin, red_counts;

  void upload_tables(const Automaton& A) {
    HostTables h = build_tables(A);
    t_delta.reserve(h.delta.size() * 2);
    t_beg.reserve(h.inv_beg.size() * 2);
    t_src.reserve(h.inv_src.size() * 2);
    SW_CUDA(cudaMemcpyAsync(t_delta.p, h.delta.data(), h.delta.size() * 2, cudaMemcpyHostToDevice, stream));
    SW_CUDA(cudaMemcpyAsync(t_beg.p, h.inv_beg.data(), h.inv_beg.size() * 2, cudaMemcpyHostToDevice, stream));
    SW_CUDA(cudaMemcpyAsync(t_src.p, h.inv_src.data(), h.inv_src.size() * 2, cudaMemcpyHostToDevice, stream));
    SW_CUDA(cudaStreamSynchronize(stream));
    tables.delta = t_delta.as<uint16_t>();
    tables.inv_beg = t_beg.as<uint16_t>();
    tables.inv_src = t_src.as<uint16_t>();
    tables.n = (int)A.n;
    tables.k = (int)A.k;
  }

  u32 read_u32(const u32* dptr) {
    SW_CUDA(cudaMemcpyAsync(pinned.p, dptr, sizeof(u32), cudaMemcpyDeviceToHost, stream));
    SW_CUDA(cudaStreamSynchronize(stream));
    return *pinned.as<u32>();
  }

  void count_launch(u64 c = 1) {
    if (st) st->kernel_launches += c;
  }

  // Compact rows/vals by flags; returns kept count.
  u32 compact(int W, const u64* rows, const u32* vals, const u32* flags, u32 m, u64* out_rows, u32* out_vals) {
    pos.reserve(sizeof(u32) * (size_t)m);
    scan_tmp.reserve(scan_temp_bytes(m));
    u32* total = d_misc + 8;
    timed(3, (double)m * (4 + 4 + 4 + 8.0 * W + 4), [&] {
      launch_scan(flags, pos.as<u32>(), m, total, scan_tmp.p, stream);
      launch_compact(W, rows, vals, flags, pos.as<u32>(), m, out_rows, out_vals, stream);
    });
    count_launch(4);
    return read_u32(total);
  }

  void sort_rows(int R, u64* rows, u32* vals, u32 m) {
    alt_rows.reserve(sizeof(u64) * R * (size_t)m);
    alt_vals.reserve(sizeof(u32) * (size_t)m);
    sort_tmp.reserve(sort_temp_bytes(R, m));
    int launches = 0, passes = 0;
    // algorithmic bytes: every pass reads and writes each (row, payload) once
    timed(2, 0.0, [&] {
      launches =
          radix_sort_rows(R, rows, vals, alt_rows.as<u64>(), alt_vals.as<u32>(), m, sort_tmp.p, stream, &passes);
    });
    if (prof_on) prof[2].bytes += (double)m * passes * 2.0 * (8.0 * R + 4);
    count_launch(launches);
  }

  // Subset queries run on the tiled check (subset_check.cu), in the launch
  // shape the context holds for the row width and the list's size class.
  DevBuf tile_and;
  ScanShapes scan_shapes;
  // while profiling: events around each check's mask build + scan, keyed by
  // (W - 1) * kScanSizeClasses + size class
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> scan_ev;
  double scan_ms[8 * kScanSizeClasses] = {};
  u64 scan_launches[8 * kScanSizeClasses] = {};

  void query(int W, int mode, const u64* S, u32 m, const u64* Q, u32 q, int n, u32* flags, bool stop) {
    if (!m || !q) return;
    const ScanShape& sh = scan_shapes.pick(W, m);
    tile_and.reserve(subset_check_temp_bytes(W, m, sh));
    cudaEvent_t e0 = nullptr;
    if (prof_on) {
      e0 = next_event();
      SW_CUDA(cudaEventRecord(e0, stream));
    }
    timed(3, (double)m * 8.0 * W, [&] { launch_tile_and(W, S, m, tile_and.as<u64>(), sh, stream); });
    // algorithmic bytes: the query rows plus every S tile staged on chip
    timed(0, (double)q * 8.0 * W, [&] {
      launch_subset_check(W, mode, S, m, tile_and.as<u64>(), Q, q, n, flags, d_misc, stop, sh, stream,
                          prof_on ? d_query_bytes : nullptr, d_misc + kScanErrWord);
    });
    if (prof_on) {
      cudaEvent_t e1 = next_event();
      SW_CUDA(cudaEventRecord(e1, stream));
      scan_ev.push_back({(W - 1) * kScanSizeClasses + (m >= kScanLargeRows ? 1 : 0), {e0, e1}});
    }
    count_launch(2);
    if (st) {
      st->trie_queries += q;
      st->logical_pairs += (u64)m * q;
    }
  }

  // Step log on stderr when SYNCHRO_VERBOSE is set (synchronises per phase).
  const bool verbose = std::getenv("SYNCHRO_VERBOSE") != nullptr;
  double vclock() {
    if (!verbose) return 0.0;
    SW_CUDA(cudaStreamSynchronize(stream));
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }

  // One BFS layer on side X (forward = image, backward = preimage of complements).
  // With `dominance` false only duplicates are removed and the visited list is
  // left alone (the bounded inverse phase, see Solver::exact).
  // Dominance reductions (the reference's self and visited reductions).
  // self_check: drop children with a proper subset in their own layer;
  // visited_subsets: drop children containing a visited set (false: only
  // children equal to a visited set, by a sorted-membership search).
  // Solver::exact runs the full reductions only where they pay: each removes
  // ~15% of a layer for a layer-by-layer subset query, which repays itself
  // when the lists are large or feed the bounded phase.  Measured (ms per
  // DFA): n = 200 plain Exact 4.8 with duplicates only, 7.3 with the visited
  // subset check, 10.3 with both reductions; n = 320 Beam+Exact 949 without
  // the self reduction, 863 with both.  Lengths are the same either way:
  // every kept set is still a set of its layer and the meet check is exact.
  bool self_check = true;
  bool visited_subsets = true;

  void step(Side& X, bool forward, int W, int n, int k, bool dominance = true) {
    const u32 m = X.count;
    const u64 N = (u64)m * k;
    if (N > 0xffffffffULL) throw std::runtime_error("layer exceeds 2^32 children");
    const u32 Nc = (u32)N;
    ch_rows.reserve(sizeof(u64) * W * N);
    ch_vals.reserve(sizeof(u32) * N);
    uq_rows.reserve(sizeof(u64) * W * N);
    uq_vals.reserve(sizeof(u32) * N);
    flags_a.reserve(sizeof(u32) * N);
    flags_b.reserve(sizeof(u32) * N);
    keep.reserve(sizeof(u32) * N);
    const double t_step0 = vclock();
    keys.reserve(sizeof(u64) * 2 * N);
    sorted_rows.reserve(sizeof(u64) * W * N);
    // expansion reads each parent row and writes k child rows, each with its
    // layer key (2 words) and its index as the sort payload
    timed(1, (double)m * 8.0 * W * (1 + k) + (double)N * 20.0, [&] {
      launch_expand(W, forward, X.rows.as<u64>(), m, tables, ch_rows.as<u64>(), stream, keys.as<u64>(),
                    ch_vals.as<u32>(), X.keymap);
    });
    count_launch(1);
    if (st) st->subsets_expanded += N;
    // sort the children by layer key
    sort_rows(2, keys.as<u64>(), ch_vals.as<u32>(), Nc);
    if (dominance && !self_check && !visited_subsets) {
      // duplicates only: a child is dropped when it equals its predecessor in
      // the sorted layer or a visited set.  One launch flags the children in
      // sort order (rows read through the sort's permutation), counts the
      // kept ones before each tile by decoupled look-back, and gathers the
      // kept rows and their origins into the new layer.
      X.rows_alt.reserve(sizeof(u64) * W * (size_t)std::max<u32>(Nc, 1));
      std::unique_ptr<Layer> L = X.new_layer(sizeof(u32) * (size_t)std::max<u32>(Nc, 1));
      L->origin.reserve(sizeof(u32) * (size_t)std::max<u32>(Nc, 1));
      u32* total = d_misc + 8;
      const u32 epoch = next_dc_epoch(Nc);
      timed(3, (double)Nc * (4 + 16 + 8.0 * W) + (double)Nc * (8.0 * W + 4), [&] {
        launch_dedup_compact(W, ch_rows.as<u64>(), ch_vals.as<u32>(), keys.as<u64>(), Nc, X.vis.as<u64>(),
                             X.vis_count, X.keymap, X.rows_alt.as<u64>(), L->origin.as<u32>(), total,
                             dc_status.as<u64>(), dc_ctr.as<u32>(), epoch, d_misc + kScanErrWord, stream);
      });
      count_launch();
      const u32 f = read_total_checked();
      if (m) X.unique_growth = (double)f / m;
      if (verbose)
        std::fprintf(stderr, "[sw] %s parents=%u children=%u kept=%u (duplicates only) | %.3f ms\n",
                     forward ? "BFS " : "IBFS", m, Nc, f, vclock() - t_step0);
      finish_layer(X, W, n, m, f, std::move(L));
      return;
    }
    // the other reductions work on the rows in sorted order
    launch_gather_rows(W, ch_rows.as<u64>(), ch_vals.as<u32>(), Nc, sorted_rows.as<u64>(), stream);
    launch_unique_flags(W, sorted_rows.as<u64>(), Nc, flags_a.as<u32>(), stream);
    count_launch(2);
    const u32 u = compact(W, sorted_rows.as<u64>(), ch_vals.as<u32>(), flags_a.as<u32>(), Nc, uq_rows.as<u64>(),
                          uq_vals.as<u32>());
    if (m) X.unique_growth = (double)u / m;  // branching before dominance pruning
    if (!dominance) {
      // bounded phase: the deduplicated layer is the new frontier as is
      std::swap(X.rows.p, uq_rows.p);
      std::swap(X.rows.cap, uq_rows.cap);
      X.count = u;
      if (st) {
        st->subsets_kept += u;
        st->dfs_sets += u;
      }
      auto L = X.new_layer(sizeof(u32) * std::max<u32>(u, 1));
      L->origin.reserve(sizeof(u32) * std::max<u32>(u, 1));
      if (u) SW_CUDA(cudaMemcpyAsync(L->origin.p, uq_vals.p, sizeof(u32) * u, cudaMemcpyDeviceToDevice, stream));
      L->count = u;
      L->parent_count = m;
      X.layers.push_back(std::move(L));
      if (verbose)
        std::fprintf(stderr, "[sw] %s (bounded) parents=%u children=%u unique=%u | %.3f ms\n",
                     forward ? "BFS " : "IBFS", m, Nc, u, vclock() - t_step0);
      return;
    }
    // dominance: visited set inside the child, or a proper subset in the layer
    launch_fill_u32(flags_a.as<u32>(), 0, u, stream);
    launch_fill_u32(flags_b.as<u32>(), 0, u, stream);
    count_launch(2);
    const double t_sort = vclock();
    if (X.vis_count) {
      if (visited_subsets) {
        query(W, kQuerySubset, X.vis.as<u64>(), X.vis_count, uq_rows.as<u64>(), u, n, flags_a.as<u32>(), false);
      } else {
        timed(3, (double)u * 8.0 * W, [&] {
          launch_member_key(W, X.vis.as<u64>(), X.vis_count, uq_rows.as<u64>(), u, flags_a.as<u32>(), stream,
                            X.keymap);
        });
        count_launch();
      }
    }
    const double t_vis = vclock();
    if (self_check)
      query(W, kQueryProperSubset, uq_rows.as<u64>(), u, uq_rows.as<u64>(), u, n,
            flags_b.as<u32>(), false);
    const double t_self = vclock();
    if (verbose) {
      std::vector<u32> fa(u), fb(u);
      SW_CUDA(cudaMemcpy(fa.data(), flags_a.p, sizeof(u32) * u, cudaMemcpyDeviceToHost));
      SW_CUDA(cudaMemcpy(fb.data(), flags_b.p, sizeof(u32) * u, cudaMemcpyDeviceToHost));
      size_t cv = 0, cs = 0;
      for (u32 i = 0; i < u; ++i) {
        cv += fa[i] != 0;
        cs += fb[i] != 0;
      }
      std::fprintf(stderr,
                   "[sw] %s parents=%u children=%u unique=%u visited=%u dropped_by_visited=%zu dropped_by_self=%zu "
                   "| expand+sort+unique %.3f ms, visited check %.3f ms, self check %.3f ms\n",
                   forward ? "BFS " : "IBFS", m, Nc, u, X.vis_count, cv, cs, t_sort - t_step0, t_vis - t_sort,
                   t_self - t_vis);
    }
    launch_keep_flags(flags_a.as<u32>(), flags_b.as<u32>(), u, keep.as<u32>(), stream);
    count_launch();
    X.rows_alt.reserve(sizeof(u64) * W * (size_t)std::max<u32>(u, 1));
    new_vals.reserve(sizeof(u32) * (size_t)std::max<u32>(u, 1));
    const u32 f = compact(W, uq_rows.as<u64>(), uq_vals.as<u32>(), keep.as<u32>(), u, X.rows_alt.as<u64>(),
                          new_vals.as<u32>());
    finish_layer(X, W, n, m, f);
  }

  // The kept children (X.rows_alt, f of them) become the new layer of X:
  // recorded for word tracing and merged into the visited list.  Their origins
  // are in `L` when given, else in new_vals.
  void finish_layer(Side& X, int W, int n, u32 m, u32 f, std::unique_ptr<Layer> L = nullptr) {
    std::swap(X.rows.p, X.rows_alt.p);
    std::swap(X.rows.cap, X.rows_alt.cap);
    X.count = f;
    if (st) st->subsets_kept += f;
    if (!L) {
      L = X.new_layer(sizeof(u32) * std::max<u32>(f, 1));
      L->origin.reserve(sizeof(u32) * std::max<u32>(f, 1));
      if (f)
        SW_CUDA(cudaMemcpyAsync(L->origin.p, new_vals.p, sizeof(u32) * f, cudaMemcpyDeviceToDevice, stream));
    }
    L->count = f;
    L->parent_count = m;
    X.layers.push_back(std::move(L));
    // visited := visited ∪ layer (both sorted, disjoint)
    X.vis_alt.reserve(sizeof(u64) * W * ((size_t)X.vis_count + f + 1));
    timed(3, (double)(X.vis_count + f) * 8.0 * W * 2, [&] {
      launch_merge_key(W, X.vis.as<u64>(), X.vis_count, X.rows.as<u64>(), f, X.vis_alt.as<u64>(), stream,
                       X.keymap);
    });
    count_launch();
    std::swap(X.vis.p, X.vis_alt.p);
    std::swap(X.vis.cap, X.vis_alt.cap);
    X.vis_count += f;
    if (!X.keymap_chosen && X.count >= 2048) choose_keymap(X, W, n);
  }

  // Optionally, once a side's layers are large enough to matter, lead its
  // sort key with 64 chosen states of its current layer (for the backward
  // side, states of the complements) and re-sort its visited list.
  DevBuf d_counts;
  void choose_keymap(Side& X, int W, int n) {
    X.keymap_chosen = true;
    if (n <= 64) return;  // the identity map already covers every state
    // Measured on random binary DFAs (n = 200 and 320), re-keying made the
    // subset checks slower than the identity key, so it is opt-in:
    // SW_SORT_KEY=frequent or SW_SORT_KEY=balanced.
    static const char* opt = std::getenv("SW_SORT_KEY");
    if (!opt || (std::string(opt) != "frequent" && std::string(opt) != "balanced")) return;
    d_counts.reserve(sizeof(u32) * 64 * W);
    SW_CUDA(cudaMemsetAsync(d_counts.p, 0, sizeof(u32) * 64 * W, stream));
    launch_state_counts(W, X.rows.as<u64>(), X.count, d_counts.as<u32>(), stream);
    std::vector<u32> cnt(64 * W);
    SW_CUDA(cudaMemcpyAsync(cnt.data(), d_counts.p, sizeof(u32) * cnt.size(), cudaMemcpyDeviceToHost, stream));
    SW_CUDA(cudaStreamSynchronize(stream));
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    // column q of the device row holds state q (word q/64, bit 63 - q%64).
    // "balanced" leads with the states closest to half the layer (the most
    // even splits), "frequent" with the most frequent.
    if (std::string(opt) == "balanced") {
      const long long half = X.count / 2;
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int a, int b) { return std::llabs(cnt[a] - half) < std::llabs(cnt[b] - half); });
    } else {
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cnt[a] > cnt[b]; });
    }
    KeyMap km;
    km.identity = 0;
    for (int j = 0; j < 64; ++j) km.q[j] = (uint16_t)idx[j];
    X.keymap = km;
    sort_by_layer_key(W, X.vis.as<u64>(), X.vis_count, X.keymap);
    count_launch(2);
  }

  // Bounded phase helpers.  expand_dedup: preimages (complement rows) of m
  // parents, duplicates removed, into out_rows / out_origin (origin = letter *
  // m + parent) — no dominance, no visited update.
  void expand_dedup(const u64* parents, u32 m, int W, int k, DevBuf& out_rows, DevBuf& out_origin, u32& out_count) {
    const u64 N = (u64)m * k;
    if (N > 0xffffffffULL) throw std::runtime_error("level exceeds 2^32 children");
    const u32 Nc = (u32)N;
    ch_rows.reserve(sizeof(u64) * W * N);
    ch_vals.reserve(sizeof(u32) * N);
    flags_a.reserve(sizeof(u32) * N);
    keys.reserve(sizeof(u64) * 2 * N);
    sorted_rows.reserve(sizeof(u64) * W * N);
    out_rows.reserve(sizeof(u64) * W * std::max<u64>(N, 1));
    out_origin.reserve(sizeof(u32) * std::max<u64>(N, 1));
    const double t0 = vclock();
    timed(1, (double)m * 8.0 * W * (1 + k), [&] { launch_expand(W, false, parents, m, tables, ch_rows.as<u64>(), stream); });
    launch_iota(ch_vals.as<u32>(), Nc, stream);
    launch_layer_keys(W, ch_rows.as<u64>(), Nc, keys.as<u64>(), stream);
    sort_rows(2, keys.as<u64>(), ch_vals.as<u32>(), Nc);
    launch_gather_rows(W, ch_rows.as<u64>(), ch_vals.as<u32>(), Nc, sorted_rows.as<u64>(), stream);
    launch_unique_flags(W, sorted_rows.as<u64>(), Nc, flags_a.as<u32>(), stream);
    count_launch(5);
    if (st) st->subsets_expanded += N;
    out_count = compact(W, sorted_rows.as<u64>(), ch_vals.as<u32>(), flags_a.as<u32>(), Nc, out_rows.as<u64>(),
                        out_origin.as<u32>());
    if (verbose)
      std::fprintf(stderr, "[sw] IBFS (bounded) parents=%u children=%u unique=%u | %.3f ms\n", m, Nc, out_count,
                   vclock() - t0);
  }

  // Meet check of q complement rows against F; on a hit returns true with the
  // query index and the F index.
  bool meet(int W, int n, const u64* Q, u32 q, u32* qi, u32* si) {
    SW_CUDA(cudaMemsetAsync(d_misc, 0, 4 * sizeof(u32), stream));
    query(W, kQueryDisjoint, F.rows.as<u64>(), F.count, Q, q, n, nullptr, true);
    if (st) st->meet_pairs += (u64)F.count * q;
    SW_CUDA(cudaMemcpyAsync(pinned.p, d_misc, 5 * sizeof(u32), cudaMemcpyDeviceToHost, stream));  // witness + error
    SW_CUDA(cudaStreamSynchronize(stream));
    const u32* w = pinned.as<u32>();
    check_scan_error(w[4]);
    if (!w[0]) return false;
    *qi = w[1];
    *si = w[2];
    return true;
  }

  // Trace letters of set `idx` at the top layer of side X down to depth 0.
  std::vector<uint32_t> trace(const Side& X, u32 idx, u32* seed_index) {
    std::vector<uint32_t> letters;  // from the top layer down
    for (size_t d = X.layers.size(); d-- > 0;) {
      const Layer& L = *X.layers[d];
      u32 o = read_u32(L.origin.as<u32>() + idx);
      letters.push_back(o / L.parent_count);
      idx = o % L.parent_count;
    }
    if (seed_index) *seed_index = idx;
    return letters;
  }
};

// ---------------------------------------------------------------------------
// Bounded inverse phase with chunking (the reference's memory-bounded DFS,
// dfs.cpp:161-218, on device levels).  F is frozen; B levels are expanded
// with duplicate removal only and meet-checked against F.  A level whose
// children fit the budget is expanded whole (plain BFS); otherwise its
// parents are taken in chunks and each chunk's subtree is explored depth
// first.  A hit at length L makes every other branch search only lengths
// below L (dfs.cpp:179-189), so the smallest length found is the answer.
// ---------------------------------------------------------------------------
namespace {

struct BoundedSearch {
  Engine& E;
  const Automaton& A;
  int W, n, k;
  size_t budget, row_bytes;
  u64 min_chunk;
  u64 max_len;  // longest length still worth examining
  u64 best = 0;
  std::vector<uint32_t> best_tail;  // letters after the forward part, for the best hit
  u32 best_f = 0;
  std::vector<DLevel*> levels;                // levels[0] stands for E.B (nullptr)
  std::vector<std::unique_ptr<DLevel>> pool;  // one reusable level per depth
  sw_stats& st;

  size_t held() const {
    size_t s = (size_t)(E.F.count + E.F.vis_count + E.B.count + E.B.vis_count) * row_bytes;
    for (size_t i = 1; i < levels.size(); ++i) s += (size_t)levels[i]->count * (row_bytes + 4);
    return s;
  }

  const u64* level_rows(size_t li) const {
    return li == 0 ? E.B.rows.as<u64>() : levels[li]->rows.as<u64>();
  }

  // Letters from level `li` index x back to the B frontier, plus the MITM B trace.
  std::vector<uint32_t> tail_word(size_t li, u32 x) {
    std::vector<uint32_t> letters;
    for (size_t l = li; l >= 1; --l) {
      const DLevel& L = *levels[l];
      const u32 o = E.read_u32(L.origin.as<u32>() + x);
      letters.push_back(o / L.chunk_cnt);
      x = L.chunk_off + o % L.chunk_cnt;
    }
    std::vector<uint32_t> bw = E.trace(E.B, x, nullptr);
    letters.insert(letters.end(), bw.begin(), bw.end());
    return letters;
  }

  // Explore the children of parents [off, off+cnt) of level li (at length len).
  void explore(size_t li, u32 off, u32 cnt, u64 len) {
    if (len + 1 > max_len || cnt == 0) return;
    const double per_child = (double)k * (3.0 * row_bytes + 32) + (double)k * (row_bytes + 4);
    const size_t have = budget > held() ? budget - held() : 0;
    u64 chunk = (u64)((double)have / per_child);
    if (chunk < min_chunk) chunk = min_chunk;
    if (chunk > cnt) chunk = cnt;
    for (u32 pos = 0; pos < cnt && len + 1 <= max_len; pos += (u32)chunk) {
      const u32 c = (u32)std::min<u64>(chunk, cnt - pos);
      const size_t me = levels.size();
      while (pool.size() <= me) pool.push_back(std::make_unique<DLevel>());
      DLevel* L = pool[me].get();
      L->chunk_off = off + pos;
      L->chunk_cnt = c;
      E.expand_dedup(level_rows(li) + (size_t)(off + pos) * W, c, W, k, L->rows, L->origin, L->count);
      st.dfs_sets += L->count;
      levels.push_back(L);
      u32 q = 0, s = 0;
      if (E.meet(W, n, levels[me]->rows.as<u64>(), levels[me]->count, &q, &s)) {
        best = len + 1;
        best_f = s;
        best_tail = tail_word(me, q);
        max_len = len;  // only shorter words are of interest from now on
        if (E.verbose)
          std::fprintf(stderr, "[sw] bounded search: word of length %llu found; searching below\n",
                       (unsigned long long)best);
      } else if (len + 1 < max_len) {
        explore(me, 0, levels[me]->count, len + 1);
      }
      levels.pop_back();
    }
  }
};
}  // namespace

Solver::Solver(int device) : device_(device), eng_(new Engine(device)) {}
Solver::~Solver() = default;

void* Solver::stream() const { return (void*)eng_->stream; }
void Solver::profile_begin() {
  SW_CUDA(cudaSetDevice(device_));
  eng_->profile_begin();
}
void Solver::profile_end(sw_kernel_profile out[4]) {
  SW_CUDA(cudaSetDevice(device_));
  eng_->profile_end(out);
}
void Solver::set_scan_shapes(const ScanShapes& s) { eng_->scan_shapes = s; }
const ScanShapes& Solver::scan_shapes() const { return eng_->scan_shapes; }
void Solver::last_scan_profile(double ms[8 * kScanSizeClasses], uint64_t checks[8 * kScanSizeClasses]) const {
  for (int i = 0; i < 8 * kScanSizeClasses; ++i) {
    ms[i] = eng_->scan_ms[i];
    checks[i] = eng_->scan_launches[i];
  }
}

// ---------------------------------------------------------------------------
// Exact::run (exact.cpp:37-97) on the device.
// ---------------------------------------------------------------------------
// State order for the device search: states most likely to lie in forward
// images first (descending stationary mass of the random walk that applies a
// uniform random letter, with a 1% uniform restart).  Images are then most
// often separated by their first word, and the subset check's tile filter
// sees the shared states of a tile early.  The reference orders by stationary
// mass too (synchrolib/algorithm/exact/exact.cpp:108-127, ascending there, for
// its CPU trie); the order changes the work done, never the result.
static std::vector<uint32_t> image_frequency_order(const Automaton& A) {
  const uint32_t n = A.n, k = A.k;
  std::vector<double> pi(n, 1.0 / n), nx(n);
  for (int it = 0; it < 200; ++it) {
    std::fill(nx.begin(), nx.end(), 0.01 / n);
    for (uint32_t q = 0; q < n; ++q) {
      const double w = 0.99 * pi[q] / k;
      for (uint32_t a = 0; a < k; ++a) nx[A.at(q, a)] += w;
    }
    pi.swap(nx);
  }
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return pi[x] > pi[y]; });
  std::vector<uint32_t> order(n);
  for (uint32_t r = 0; r < n; ++r) order[idx[r]] = r;
  return order;
}

void Solver::exact(const Automaton& A0, const sw_exact_config& cfg, Bounds& b, sw_stats& st,
                   const ReduceState* red) {
  const std::vector<uint32_t> order = image_frequency_order(A0);
  const Automaton A = permute(A0, order);
  if (b.non_synchro || b.lower == b.upper) return;  // exact.cpp:45-47
  if (A.n == 1) {                                   // exact.cpp:49-53
    b.lower = b.upper = 0;
    b.has_word = true;
    b.word.clear();
    return;
  }
  if (!is_synchronizing(A)) {
    // The reference's Exact has no such check and runs until its bound; a
    // non-synchronizing automaton is reported as such instead.
    b.non_synchro = true;
    return;
  }
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  AllocScope alloc_scope(E.stream);  // buffer growth ordered on this solve's stream only
  E.st = &st;
  auto t0 = std::chrono::steady_clock::now();
  const int n = (int)A.n, k = (int)A.k, W = words_for(n);
  E.upload_tables(A);
  E.F.reset();
  E.B.reset();
  // seeds
  {
    std::vector<u64> full(W, 0);
    for (int q = 0; q < n; ++q) full[q >> 6] |= state_bit(q);
    std::vector<u64> fseeds;
    if (red) {
      // exact.cpp:130-146: the forward side starts from the reduced BFS list
      fseeds.assign((size_t)W * red->seeds.size(), 0);
      for (size_t i = 0; i < red->seeds.size(); ++i)
        for (uint32_t q : red->seeds[i]) fseeds[i * W + (order[q] >> 6)] |= state_bit((int)order[q]);
    } else {
      fseeds = full;
    }
    const u32 nf = (u32)(fseeds.size() / W);
    E.F.rows.reserve(sizeof(u64) * W * std::max<u32>(nf, 1));
    SW_CUDA(cudaMemcpyAsync(E.F.rows.p, fseeds.data(), sizeof(u64) * W * nf, cudaMemcpyHostToDevice, E.stream));
    E.F.count = nf;
    std::vector<uint32_t> seeds = backward_seeds(A);
    std::vector<u64> rows((size_t)W * std::max<size_t>(seeds.size(), 1), 0);
    for (size_t i = 0; i < seeds.size(); ++i) {
      for (int q = 0; q < n; ++q)
        if ((uint32_t)q != seeds[i]) rows[i * W + (q >> 6)] |= state_bit(q);  // complement of {seed}
      E.B.seed_states.push_back(seeds[i]);
    }
    E.B.rows.reserve(sizeof(u64) * rows.size());
    SW_CUDA(cudaMemcpyAsync(E.B.rows.p, rows.data(), sizeof(u64) * W * seeds.size(), cudaMemcpyHostToDevice,
                            E.stream));
    E.B.count = (u32)seeds.size();
    // visited starts with the seeds (the reference's visited lists start empty;
    // a seed can never be dominated by its own descendants' check either way)
    E.F.vis.reserve(sizeof(u64) * W);
    E.B.vis.reserve(sizeof(u64) * W * std::max<size_t>(seeds.size(), 1));
    SW_CUDA(cudaMemcpyAsync(E.F.vis.p, E.F.rows.p, sizeof(u64) * W, cudaMemcpyDeviceToDevice, E.stream));
    E.F.vis_count = red ? 0 : 1;  // a reduced list starts with an empty visited list, as the reference's does
    if (!seeds.empty()) {
      // seeds are already sorted ascending by state = descending by row value
      // for complements; sort them properly via the row sort.
      SW_CUDA(cudaMemcpyAsync(E.B.vis.p, E.B.rows.p, sizeof(u64) * W * seeds.size(), cudaMemcpyDeviceToDevice,
                              E.stream));
      E.sort_by_layer_key(W, E.B.vis.as<u64>(), (u32)seeds.size());
      E.B.vis_count = (u32)seeds.size();
    }
  }
  const size_t budget = (size_t)cfg.max_memory_mb * 1024 * 1024;
  const size_t row_bytes = sizeof(u64) * W;
  // exact.cpp:65 searches lengths below the upper bound; when no word backs
  // that bound (it came from the plan's upper_bound), length == bound is
  // searched too so that a word can be returned.
  const u64 max_rt = b.has_word ? b.upper - 1 : b.upper;
  u64 rt = 0;
  bool found = false, oom = false;
  u32 wit_q = 0, wit_s = 0;
  // Bounded inverse phase (the device counterpart of the reference's DFS
  // shortcut, dfs.cpp:64-218 and meet_in_the_middle.cpp:466-511): when the
  // upper bound is backed by a word, only lengths < bound remain to be
  // excluded.  F is then frozen and B is expanded level by level with
  // duplicate removal only, each level meet-checked against F.  The switch is
  // taken when the projected cost of those levels (measured per-query meet
  // time, B growing by the last observed branching) is below that of
  // continuing the dominance-pruned search (last step's time growing 1.6x per
  // step), and the widest projected level fits the memory budget.
  bool bounded = false;
  double t_iter_last = 0, t_meet_per_query = 0, b_growth = k * 0.95;
  while (rt < max_rt) {  // meet_in_the_middle.cpp:73
    const auto t_iter0 = std::chrono::steady_clock::now();
    const bool fwd = bounded ? false : E.F.count <= E.B.count;
    Side& X = fwd ? E.F : E.B;
    size_t live = (size_t)(E.F.count + E.F.vis_count + E.B.count + E.B.vis_count) * row_bytes;
    size_t next = (size_t)X.count * k * (3 * row_bytes + 4 * sizeof(u32));
    if (live + next > budget) {
      // meet_in_the_middle.cpp:98-101 + exact.cpp:139-145: out of memory, the
      // search continues in the memory-bounded inverse phase when DFS is
      // enabled and the remaining depth is bounded (word-backed bound or at
      // most 64 levels); otherwise only a lower bound results
      if (cfg.dfs && !bounded && E.B.count && (b.has_word || max_rt - rt <= 64)) {
        bounded = true;
        if (E.verbose)
          std::fprintf(stderr, "[sw] memory budget reached at length %llu: bounded phase\n", (unsigned long long)rt);
        break;
      }
      oom = true;
      break;
    }
    rt++;
    const u32 parents_before = X.count;
    // self reduction only where it pays: a word-backed bound (the bounded
    // phase expands B from its size at the switch) or lists past a quarter
    // of the memory budget
    const bool pressure = 4 * (live + next) > budget;
    E.self_check = E.visited_subsets = cfg.reductions == SW_REDUCE_ALWAYS ||
                                       (cfg.reductions == SW_REDUCE_AUTO && b.has_word) || pressure;
    E.step(X, fwd, W, n, k, /*dominance=*/!bounded);
    // projected branching of the bounded levels: distinct children per parent
    // before pruning, never below 1.5, plus 10% margin
    if (!fwd && parents_before) b_growth = std::max(1.2, E.B.unique_growth);
    if (fwd) {
      st.bfs_steps++;
    } else {
      st.ibfs_steps++;
    }
    // meet check: some F disjoint from some B-complement (F ⊆ B)
    const double t_meet0 = E.vclock();
    // the switch to the bounded phase prices the meet check per query: time it
    // alone (a synchronisation first) only while that switch is possible
    const bool time_meet = !bounded && b.has_word;
    if (time_meet) SW_CUDA(cudaStreamSynchronize(E.stream));
    const auto t_meet_host0 = std::chrono::steady_clock::now();
    SW_CUDA(cudaMemsetAsync(E.d_misc, 0, 4 * sizeof(u32), E.stream));
    E.query(W, kQueryDisjoint, E.F.rows.as<u64>(), E.F.count, E.B.rows.as<u64>(), E.B.count,
            n, nullptr, true);
    st.meet_pairs += (u64)E.F.count * E.B.count;
    SW_CUDA(cudaMemcpyAsync(E.pinned.p, E.d_misc, 5 * sizeof(u32), cudaMemcpyDeviceToHost, E.stream));  // witness + error
    SW_CUDA(cudaStreamSynchronize(E.stream));
    const auto t_end = std::chrono::steady_clock::now();
    const u32* w = E.pinned.as<u32>();
    Engine::check_scan_error(w[4]);
    t_iter_last = std::chrono::duration<double>(t_end - t_iter0).count();
    if (E.B.count)
      t_meet_per_query = std::chrono::duration<double>(t_end - t_meet_host0).count() / (double)E.B.count;
    if (!bounded && b.has_word && !w[0] && rt < max_rt && rt >= 4 && E.B.count) {
      const u64 R = max_rt - rt;  // levels still to exclude
      // per child: dedup (~1 ns measured at 10^7 rows) + the meet check's cost per query
      const double per_row = t_meet_per_query + 2e-9;
      double lvl = E.B.count, total = 0, mitm = 0, grow = 1.0;
      bool fits = true;
      for (u64 i = 1; i <= R && fits; ++i) {
        const double children = lvl * k;
        total += children * per_row;
        grow *= 1.35;  // both sides alternate: each side grows ~1.7x every other step
        mitm += t_iter_last * grow;
        // children rows + their sorted copy + the kept level, keys and payloads
        if (children * (3.0 * row_bytes + 32) + (lvl + (double)E.F.count) * row_bytes > (double)budget)
          fits = false;
        lvl *= b_growth;
      }
      // voluntary switch only when every projected level fits; chunking is the
      // safety net for an exhausted budget, not a plan
      if (fits && total < mitm) {
        bounded = true;
        if (E.verbose)
          std::fprintf(stderr, "[sw] bounded phase from length %llu: %llu levels left, |F|=%u |B|=%u, "
                       "projected %.1f ms vs %.1f ms\n", (unsigned long long)rt, (unsigned long long)R, E.F.count,
                       E.B.count, 1e3 * total, 1e3 * mitm);
      }
    }
    if (E.verbose)
      std::fprintf(stderr, "[sw] len %llu: |F|=%u |B|=%u meet check %.3f ms%s\n", (unsigned long long)rt, E.F.count,
                   E.B.count, E.vclock() - t_meet0, w[0] ? " -> found" : "");
    if (w[0]) {
      found = true;
      wit_q = w[1];
      wit_s = w[2];
      break;
    }
    if (E.F.count == 0 || E.B.count == 0) break;  // a side died out: no reset word within reach
    if (bounded) break;
  }
  std::vector<uint32_t> bounded_tail;
  if (bounded && !found) {
    BoundedSearch S{E, A, W, n, k, budget, row_bytes, std::max<u64>(cfg.dfs_min_list_size, 1), max_rt, 0, {}, 0,
                    {}, {}, st};
    S.pool.swap(E.dlevel_pool);  // levels (and their device buffers) kept across solves
    S.levels.push_back(nullptr);
    S.explore(0, 0, E.B.count, rt);
    E.dlevel_pool.swap(S.pool);
    if (S.best) {
      found = true;
      rt = S.best;
      wit_s = S.best_f;
      bounded_tail = S.best_tail;
    } else {
      rt = max_rt;  // every length up to the bound minus one is excluded
    }
  }
  if (red) {  // exact.cpp:83-87: lengths count the reduction's BFS steps
    rt += red->bfs_steps;
    b.lower += red->bfs_steps;
    b.upper += red->bfs_steps;
  }
  if (found) {
    // word = (reduction prefix) forward letters (depth 1..df) then backward
    // letters (depth db..1)
    u32 fseed = 0;
    std::vector<uint32_t> fw = E.trace(E.F, wit_s, &fseed);
    std::reverse(fw.begin(), fw.end());
    u32 seed_idx = 0;
    std::vector<uint32_t> bw = bounded_tail.empty() ? E.trace(E.B, wit_q, &seed_idx) : bounded_tail;
    std::vector<uint32_t> word;
    if (red) word = red->prefix.at(fseed);
    word.insert(word.end(), fw.begin(), fw.end());
    word.insert(word.end(), bw.begin(), bw.end());
    std::vector<uint32_t> img = apply_word(red ? red->original : A, word);
    if (img.size() != 1 || word.size() != rt)
      throw std::runtime_error("internal error: reconstructed word does not synchronize (length " +
                               std::to_string(word.size()) + ", image " + std::to_string(img.size()) + ")");
    b.lower = std::max<u64>(b.lower, rt);
    b.upper = rt;
    b.has_word = true;
    b.word = word;
  } else {
    // exact.cpp:148-164: every length <= rt is excluded; if that reaches the
    // upper bound, the bound is the answer (its word, if any, came from the
    // algorithm that set it).  Otherwise (memory budget) only a lower bound.
    (void)oom;
    if (rt + 1 >= b.upper) {
      b.lower = std::max<u64>(b.lower, b.upper);
    } else {
      b.lower = std::max<u64>(b.lower, rt + 1);
    }
  }
  st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  E.st = nullptr;
}

// ---------------------------------------------------------------------------
// Beam (beam.hpp:31-188): inverse BFS from the backward seeds keeping the
// `beam_size` largest sets, ties by the reference's raw word order.
// ---------------------------------------------------------------------------
namespace {
struct BeamRun {
  u64 bound = 0;
  bool has_word = false;
  std::vector<uint32_t> word;
};
}  // namespace

static BeamRun beam_cutoff(Engine& E, const Automaton& A, u32 beam_size, u64 max_mlsw, int64_t max_iter, sw_stats& st) {
  const int n = (int)A.n, k = (int)A.k, W = words_for(n);
  const int R = (n + 63) / 64 + 1;
  BeamRun out;
  out.bound = max_mlsw;
  std::vector<uint32_t> seeds = backward_seeds(A);
  Side& X = E.B;  // beam rows are plain (not complemented) preimages
  X.reset();
  std::vector<u64> rows((size_t)W * std::max<size_t>(seeds.size(), 1), 0);
  for (size_t i = 0; i < seeds.size(); ++i) rows[i * W + (seeds[i] >> 6)] |= state_bit((int)seeds[i]);
  X.rows.reserve(sizeof(u64) * rows.size());
  SW_CUDA(cudaMemcpyAsync(X.rows.p, rows.data(), sizeof(u64) * W * seeds.size(), cudaMemcpyHostToDevice, E.stream));
  X.count = (u32)seeds.size();
  if (X.count == 0 || beam_size == 0) return out;
  for (u64 len = 1; len < max_mlsw; ++len) {
    if (max_iter >= 0 && (int64_t)len > max_iter) break;
    const u32 m = X.count;
    const u64 N = (u64)m * k;
    if (N > 0xffffffffULL) throw std::runtime_error("beam layer exceeds 2^32 children");
    const u32 Nc = (u32)N;
    E.ch_rows.reserve(sizeof(u64) * W * N);
    E.keys.reserve(sizeof(u64) * R * N);
    E.ch_vals.reserve(sizeof(u32) * N);
    E.flags_a.reserve(sizeof(u32) * N);
    E.uq_vals.reserve(sizeof(u32) * N);
    E.keys_alt.reserve(sizeof(u64) * R * N);
    E.timed(1, (double)m * 8.0 * W * (1 + k), [&] {
      launch_expand(W, false, X.rows.as<u64>(), m, E.tables, E.ch_rows.as<u64>(), E.stream);
    });
    launch_beam_keys(W, E.ch_rows.as<u64>(), Nc, n, R, E.keys.as<u64>(), E.stream);
    launch_iota(E.ch_vals.as<u32>(), Nc, E.stream);
    E.count_launch(3);
    st.subsets_expanded += N;
    E.sort_rows(R, E.keys.as<u64>(), E.ch_vals.as<u32>(), Nc);
    // beam.hpp:173-177: the largest set is first; Q means done
    SW_CUDA(cudaMemcpyAsync(E.pinned.p, E.keys.p, sizeof(u64), cudaMemcpyDeviceToHost, E.stream));
    SW_CUDA(cudaStreamSynchronize(E.stream));
    if (*E.pinned.as<u64>() == 0) {
      u32 first_val = 0;
      SW_CUDA(cudaMemcpy(&first_val, E.ch_vals.p, sizeof(u32), cudaMemcpyDeviceToHost));
      // word: letters from this layer down to the first, applied in that order
      std::vector<uint32_t> letters;
      letters.push_back(first_val / m);
      u32 idx = first_val % m;
      for (size_t d = X.layers.size(); d-- > 0;) {
        const Layer& L = *X.layers[d];
        u32 o = E.read_u32(L.origin.as<u32>() + idx);
        letters.push_back(o / L.parent_count);
        idx = o % L.parent_count;
      }
      out.bound = len;
      out.word = letters;
      std::vector<uint32_t> img = apply_word(A, out.word);
      out.has_word = img.size() == 1 && out.word.size() == len;
      return out;
    }
    // keep_unique + truncate (beam.hpp:179-182)
    launch_unique_flags(R, E.keys.as<u64>(), Nc, E.flags_a.as<u32>(), E.stream);
    E.count_launch();
    E.uq_rows.reserve(sizeof(u64) * R * N);
    u32 u = E.compact(R, E.keys.as<u64>(), E.ch_vals.as<u32>(), E.flags_a.as<u32>(), Nc, E.uq_rows.as<u64>(),
                      E.uq_vals.as<u32>());
    u32 keep = std::min<u32>(u, beam_size);
    X.rows_alt.reserve(sizeof(u64) * W * std::max<u32>(keep, 1));
    launch_gather_rows(W, E.ch_rows.as<u64>(), E.uq_vals.as<u32>(), keep, X.rows_alt.as<u64>(), E.stream);
    E.count_launch();
    std::swap(X.rows.p, X.rows_alt.p);
    std::swap(X.rows.cap, X.rows_alt.cap);
    auto L = X.new_layer(sizeof(u32) * std::max<u32>(keep, 1));
    L->origin.reserve(sizeof(u32) * std::max<u32>(keep, 1));
    SW_CUDA(cudaMemcpyAsync(L->origin.p, E.uq_vals.p, sizeof(u32) * keep, cudaMemcpyDeviceToDevice, E.stream));
    L->count = keep;
    L->parent_count = m;
    X.layers.push_back(std::move(L));
    X.count = keep;
  }
  return out;
}

void Solver::beam(const Automaton& A0, const sw_beam_config& cfg, Bounds& b, sw_stats& st) {
  if (b.non_synchro || b.lower == b.upper) return;  // beam.hpp:34-40
  if (A0.n == 1) {                                  // beam.hpp:42-46
    b.lower = b.upper = 0;
    b.has_word = true;
    b.word.clear();
    return;
  }
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  AllocScope alloc_scope(E.stream);  // buffer growth ordered on this solve's stream only
  E.st = &st;
  auto t0 = std::chrono::steady_clock::now();
  // presort (beam.hpp:54-63, 351-369): states ordered by in-degree ascending
  std::vector<uint32_t> perm(A0.n);
  std::iota(perm.begin(), perm.end(), 0u);
  if (cfg.presort_indeg) {
    std::vector<std::pair<double, int>> d(A0.n);
    for (uint32_t q = 0; q < A0.n; ++q) d[q] = {0.0, (int)q};
    for (uint32_t q = 0; q < A0.n; ++q)
      for (uint32_t a = 0; a < A0.k; ++a) d[A0.at(q, a)].first++;
    std::sort(d.begin(), d.end());
    for (uint32_t q = 0; q < A0.n; ++q) perm[d[q].second] = q;
  }
  Automaton A = permute(A0, perm);
  E.upload_tables(A);
  BeamRun run;
  if (cfg.dynamic) {  // beam.hpp:66-86
    using cost_t = long double;
    const uint32_t minb = (uint32_t)cfg.min_beam_size, maxb = (uint32_t)cfg.max_beam_size;
    run = beam_cutoff(E, A, minb, b.upper, cfg.max_iter, st);
    uint32_t bound = (uint32_t)run.bound;
    cost_t exact_cost = 2 * std::pow(static_cast<cost_t>(A.k), (bound + 1) / 2);
    cost_t proposed = std::round(exact_cost * (cost_t)cfg.beam_exact_ratio / bound);
    uint32_t bs = (uint32_t)std::clamp<cost_t>(proposed, (cost_t)minb, (cost_t)maxb);
    if (bs > minb) {
      // the second run searches below the first bound; it returns that bound
      // unchanged (and no word) when it finds nothing shorter
      BeamRun second = beam_cutoff(E, A, bs, bound, cfg.max_iter, st);
      if (second.bound < bound) run = second;
    }
  } else {
    run = beam_cutoff(E, A, (uint32_t)cfg.beam_size, b.upper, cfg.max_iter, st);
  }
  const uint32_t bound = (uint32_t)run.bound;  // the reference stores the bound in a uint
  b.upper = bound;
  if (run.has_word && run.word.size() == bound) {
    b.has_word = true;
    b.word = run.word;
  } else if (b.has_word && b.word.size() != b.upper) {
    b.has_word = false;
  }
  st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  E.st = nullptr;
}

// ---------------------------------------------------------------------------
// Kernel-level helpers.
// ---------------------------------------------------------------------------
void Solver::apply_transition(const Automaton& A, uint32_t letter, bool inverse, const uint64_t* from, uint64_t* to,
                              uint64_t count) {
  if (letter >= A.k) throw std::invalid_argument("letter out of range");
  if (count == 0) return;
  if (count > 0xffffffffULL) throw std::invalid_argument("count exceeds 2^32");
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  const int n = (int)A.n, W = words_for(n);
  // single-letter automaton view so the kernel writes one block
  Automaton one;
  one.n = A.n;
  one.k = 1;
  one.t.resize(A.n);
  for (uint32_t q = 0; q < A.n; ++q) one.t[q] = A.at(q, letter);
  E.upload_tables(one);
  std::vector<u64> rows((size_t)W * count);
  to_device_rows(from, count, A.n, W, rows.data());
  E.uq_rows.reserve(sizeof(u64) * rows.size());
  E.ch_rows.reserve(sizeof(u64) * rows.size());
  SW_CUDA(cudaMemcpyAsync(E.uq_rows.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
  launch_expand(W, !inverse, E.uq_rows.as<u64>(), (u32)count, E.tables, E.ch_rows.as<u64>(), E.stream);
  SW_CUDA(cudaMemcpyAsync(rows.data(), E.ch_rows.p, sizeof(u64) * rows.size(), cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  from_device_rows(rows.data(), count, A.n, W, to);
}

void Solver::subsets_check(uint32_t n, const uint64_t* sets, uint64_t set_count, const uint64_t* checks,
                           uint64_t check_count, bool proper, uint8_t* results) {
  if (n == 0 || n > (uint32_t)kMaxStates) throw std::invalid_argument("n out of range");
  if (set_count > 0xffffffffULL || check_count > 0xffffffffULL) throw std::invalid_argument("count exceeds 2^32");
  std::fill(results, results + check_count, 0);
  if (!set_count || !check_count) return;
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  const int W = words_for((int)n);
  std::vector<u64> srows((size_t)W * set_count), qrows((size_t)W * check_count);
  to_device_rows(sets, set_count, n, W, srows.data());
  to_device_rows(checks, check_count, n, W, qrows.data());
  const u32 m = (u32)set_count, q = (u32)check_count;
  E.uq_rows.reserve(sizeof(u64) * srows.size());
  E.uq_vals.reserve(sizeof(u32) * m);
  E.ch_rows.reserve(sizeof(u64) * qrows.size());
  E.flags_a.reserve(sizeof(u32) * m);
  E.flags_b.reserve(sizeof(u32) * q);
  E.keys.reserve(sizeof(u64) * srows.size());
  SW_CUDA(cudaMemcpyAsync(E.uq_rows.p, srows.data(), sizeof(u64) * srows.size(), cudaMemcpyHostToDevice, E.stream));
  SW_CUDA(cudaMemcpyAsync(E.ch_rows.p, qrows.data(), sizeof(u64) * qrows.size(), cudaMemcpyHostToDevice, E.stream));
  // sort + unique the set list (check_contains_subset sorts both, :30-33)
  launch_iota(E.uq_vals.as<u32>(), m, E.stream);
  E.sort_rows(W, E.uq_rows.as<u64>(), E.uq_vals.as<u32>(), m);
  launch_unique_flags(W, E.uq_rows.as<u64>(), m, E.flags_a.as<u32>(), E.stream);
  u32 u = E.compact(W, E.uq_rows.as<u64>(), E.uq_vals.as<u32>(), E.flags_a.as<u32>(), m, E.keys.as<u64>(), nullptr);
  launch_fill_u32(E.flags_b.as<u32>(), 0, q, E.stream);
  E.query(W, proper ? kQueryProperSubset : kQuerySubset, E.keys.as<u64>(), u,
          E.ch_rows.as<u64>(), q, (int)n, E.flags_b.as<u32>(), false);
  std::vector<u32> flags(q);
  u32 scan_err = 0;
  SW_CUDA(cudaMemcpyAsync(flags.data(), E.flags_b.p, sizeof(u32) * q, cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaMemcpyAsync(&scan_err, E.d_misc + Engine::kScanErrWord, sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  Engine::check_scan_error(scan_err);
  for (u32 i = 0; i < q; ++i) results[i] = flags[i] ? 1 : 0;
}

uint64_t Solver::sort_unique(uint32_t n, uint64_t* sets, uint64_t count) {
  if (n == 0 || n > (uint32_t)kMaxStates) throw std::invalid_argument("n out of range");
  if (count > 0xffffffffULL) throw std::invalid_argument("count exceeds 2^32");
  if (count == 0) return 0;
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  const int W = words_for((int)n);
  std::vector<u64> rows((size_t)W * count);
  to_device_rows(sets, count, n, W, rows.data());
  const u32 m = (u32)count;
  E.uq_rows.reserve(sizeof(u64) * rows.size());
  E.uq_vals.reserve(sizeof(u32) * m);
  E.keys.reserve(sizeof(u64) * rows.size());
  E.flags_a.reserve(sizeof(u32) * m);
  SW_CUDA(cudaMemcpyAsync(E.uq_rows.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
  launch_iota(E.uq_vals.as<u32>(), m, E.stream);
  E.sort_rows(W, E.uq_rows.as<u64>(), E.uq_vals.as<u32>(), m);
  launch_unique_flags(W, E.uq_rows.as<u64>(), m, E.flags_a.as<u32>(), E.stream);
  u32 u = E.compact(W, E.uq_rows.as<u64>(), E.uq_vals.as<u32>(), E.flags_a.as<u32>(), m, E.keys.as<u64>(), nullptr);
  SW_CUDA(cudaMemcpyAsync(rows.data(), E.keys.p, sizeof(u64) * W * u, cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  from_device_rows(rows.data(), u, n, W, sets);
  return u;
}

// ---------------------------------------------------------------------------
// Eppstein (synchrolib/algorithm/eppstein/eppstein.hpp:26-76).
// ---------------------------------------------------------------------------
void Solver::eppstein(const Automaton& A, const sw_eppstein_config&, Bounds& b, sw_stats& st) {
  if (b.non_synchro || b.lower == b.upper) return;  // eppstein.hpp:28-34
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  auto t0 = std::chrono::steady_clock::now();
  E.upload_tables(A);
  const u64 n = A.n;
  E.epp_scratch.reserve(eppstein_scratch_bytes((int)n));
  // the greedy word is at most (n^3 - n) / 6 letters long (Eppstein 1990)
  const u64 cap = std::min<u64>(b.upper, n * n * n / 6 + n) + 1;
  E.epp_word.reserve(cap);
  u32* out = E.d_misc + 16;
  SW_CUDA(cudaMemsetAsync(out, 0, 8 * sizeof(u32), E.stream));
  launch_eppstein(E.tables, b.upper, E.epp_scratch.p, out, E.epp_word.as<uint8_t>(), cap, E.stream);
  ++st.kernel_launches;
  u32* h = E.pinned.as<u32>();
  SW_CUDA(cudaMemcpyAsync(h, out, 8 * sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  const u32 status = h[0];
  const u64 len = (u64)h[1] | ((u64)h[2] << 32);
  const u64 letters = h[3];
  st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (status == kEppNonSynchro) {  // eppstein.hpp:53-57
    b.non_synchro = true;
    return;
  }
  if (status == kEppOverBound) return;  // eppstein.hpp:60-62: bound unchanged
  if (status != kEppFound) throw std::runtime_error("internal: Eppstein word buffer too small");
  const u64 old_upper = b.upper;
  b.upper = len;
  if (letters == len) {
    std::vector<uint8_t> w8(letters);
    if (letters) SW_CUDA(cudaMemcpy(w8.data(), E.epp_word.p, letters, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> word(w8.begin(), w8.end());
    if (apply_word(A, word).size() != 1) throw std::runtime_error("internal: Eppstein word does not synchronize");
    if (!b.has_word || len < old_upper) {
      b.has_word = true;
      b.word = std::move(word);
    }
  }
  if (b.has_word && b.word.size() != b.upper) b.has_word = false;
}

// ---------------------------------------------------------------------------
// Brute (synchrolib/algorithm/brute/brute.hpp:28-71).
// ---------------------------------------------------------------------------
void Solver::brute(const Automaton& A, const sw_brute_config& cfg, Bounds& b, sw_stats& st) {
  if (b.non_synchro || b.lower == b.upper) return;  // brute.hpp:30-36
  if (cfg.max_n > 32) return;                       // brute.hpp:44-47: refused, bounds unchanged
  if (A.n > cfg.max_n) return;                      // brute.hpp:49-52
  if (A.n == 1) {
    b.lower = b.upper = 0;
    b.has_word = true;
    b.word.clear();
    return;
  }
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  auto t0 = std::chrono::steady_clock::now();
  E.upload_tables(A);
  const int n = (int)A.n, k = (int)A.k;
  const u64 space = 1ULL << n;  // masks; every level holds new masks only, so all levels fit in `space`
  const u32 full = n == 32 ? 0xffffffffu : ((1u << n) - 1u);
  E.br_visited.reserve(brute_visited_bytes(n));
  SW_CUDA(cudaMemsetAsync(E.br_visited.p, 0, brute_visited_bytes(n), E.stream));
  const u32 full_bit = 1u << (full & 31u);
  SW_CUDA(cudaMemcpyAsync(E.br_visited.as<u32>() + (full >> 5), &full_bit, sizeof(u32), cudaMemcpyHostToDevice,
                          E.stream));
  E.br_arena.reserve(sizeof(u32) * std::min<u64>(space, 1ULL << 20));
  SW_CUDA(cudaMemcpyAsync(E.br_arena.p, &full, sizeof(u32), cudaMemcpyHostToDevice, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  std::vector<u64> off{0, 1};  // level j = arena[off[j], off[j+1])
  u32* ctrl = E.d_misc + 24;   // [0] next count, [1] found, [2] singleton
  u32* h = E.pinned.as<u32>();
  u64 length = 0;
  u32 target = 0;
  for (u64 depth = 0;; ++depth) {
    const u64 begin = off[depth], end = off[depth + 1], count = end - begin;
    const u64 room = std::min<u64>(count * (u64)k, space - end);
    const size_t need = sizeof(u32) * (end + room);
    if (need > E.br_arena.cap) {  // grow, keeping the stored levels
      DevBuf bigger;
      bigger.reserve(std::max(need, 2 * E.br_arena.cap));
      SW_CUDA(cudaMemcpyAsync(bigger.p, E.br_arena.p, sizeof(u32) * end, cudaMemcpyDeviceToDevice, E.stream));
      SW_CUDA(cudaStreamSynchronize(E.stream));
      std::swap(bigger.p, E.br_arena.p);
      std::swap(bigger.cap, E.br_arena.cap);
    }
    u32* arena = E.br_arena.as<u32>();
    SW_CUDA(cudaMemsetAsync(ctrl, 0, 3 * sizeof(u32), E.stream));
    launch_brute_level(E.t_delta.as<uint16_t>(), n, k, arena + begin, (u32)count, E.br_visited.as<u32>(), arena + end,
                       (u32)room, ctrl, ctrl + 1, E.stream);
    ++st.kernel_launches;
    SW_CUDA(cudaMemcpyAsync(h, ctrl, 3 * sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
    SW_CUDA(cudaStreamSynchronize(E.stream));
    st.subsets_expanded += count * (u64)k;
    st.subsets_kept += h[0];
    if (h[0] > room) throw std::runtime_error("internal: Brute level overflow");
    if (h[1]) {
      length = depth + 1;
      target = h[2];
      break;
    }
    if (h[0] == 0) {  // brute.hpp:61-65: BFS exhausted without a singleton
      b.non_synchro = true;
      st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      return;
    }
    off.push_back(end + h[0]);
  }
  // walk back through the stored levels: a parent of `target` in level j
  std::vector<uint32_t> word(length);
  u64* best = reinterpret_cast<u64*>(E.d_misc + 32);
  for (u64 j = length; j-- > 0;) {
    const u64 begin = off[j], count = off[j + 1] - begin;
    SW_CUDA(cudaMemsetAsync(best, 0xff, sizeof(u64), E.stream));
    launch_brute_parent(E.t_delta.as<uint16_t>(), n, k, E.br_arena.as<u32>() + begin, (u32)count, target, best,
                        E.stream);
    ++st.kernel_launches;
    u64 hb = 0;
    SW_CUDA(cudaMemcpyAsync(h, best, sizeof(u64), cudaMemcpyDeviceToHost, E.stream));
    SW_CUDA(cudaStreamSynchronize(E.stream));
    std::memcpy(&hb, h, sizeof(u64));
    if (hb == ~0ULL) throw std::runtime_error("internal: Brute parent not found");
    word[j] = (uint32_t)(hb % (u64)k);
    SW_CUDA(cudaMemcpy(&target, E.br_arena.as<u32>() + begin + hb / (u64)k, sizeof(u32), cudaMemcpyDeviceToHost));
  }
  if (apply_word(A, word).size() != 1) throw std::runtime_error("internal: Brute word does not synchronize");
  b.lower = b.upper = length;  // brute.hpp:66-70
  b.has_word = true;
  b.word = std::move(word);
  st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ---------------------------------------------------------------------------
// Reduce (synchrolib/algorithm/reduce/reduce.hpp:31-91).  The BFS steps are
// the forward side of the exact search (expansion, duplicate removal, the two
// dominance checks, visited merge); the reachability closure and relabelling
// of the small final list are host bookkeeping.
// ---------------------------------------------------------------------------
void Solver::reduce(const Automaton& A, const sw_reduce_config& cfg, Bounds& b, sw_stats& st, ReduceState& red) {
  if (b.non_synchro || b.lower == b.upper) return;  // reduce.hpp:40-46
  if (A.n < cfg.min_n) return;                      // reduce.hpp:48-50
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  E.st = &st;
  auto t0 = std::chrono::steady_clock::now();
  const int n = (int)A.n, k = (int)A.k, W = words_for(n);
  E.upload_tables(A);
  E.self_check = E.visited_subsets = true;  // the reference's step (reduce.hpp:186-187): its list sizes decide the reduction
  E.F.reset();
  std::vector<u64> full(W, 0);
  for (int q = 0; q < n; ++q) full[q >> 6] |= state_bit(q);
  E.F.rows.reserve(sizeof(u64) * W);
  SW_CUDA(cudaMemcpyAsync(E.F.rows.p, full.data(), sizeof(u64) * W, cudaMemcpyHostToDevice, E.stream));
  E.F.count = 1;
  E.F.vis_count = 0;  // reduce.hpp:128: the visited list starts empty
  const u64 max_mlsw = b.upper - 1;
  u64 mlsw = 0;
  bool found = false;
  std::vector<uint32_t> word;
  DevBuf& counts = E.red_counts;
  auto done = [&] {
    st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    E.st = nullptr;
  };
  // reduce.hpp:96-109 (process_short_bfs) with bfs_step :171-198
  while (mlsw < max_mlsw) {
    if (E.F.count > cfg.list_size_threshold) break;
    mlsw++;
    st.bfs_steps++;
    if (E.F.count == 0) continue;  // an exhausted list stays empty up to the bound, as in the reference
    E.step(E.F, true, W, n, k, true);
    const u32 m = E.F.count;
    if (!m) continue;
    counts.reserve(sizeof(u32) * m);
    launch_popcount(W, E.F.rows.as<u64>(), m, counts.as<u32>(), E.stream);
    E.count_launch();
    std::vector<u32> pc(m);
    SW_CUDA(cudaMemcpyAsync(pc.data(), counts.p, sizeof(u32) * m, cudaMemcpyDeviceToHost, E.stream));
    SW_CUDA(cudaStreamSynchronize(E.stream));
    for (u32 i = 0; i < m; ++i)
      if (pc[i] == 1) {
        word = E.trace(E.F, i, nullptr);
        std::reverse(word.begin(), word.end());
        found = true;
        break;
      }
    if (found) break;
  }
  if (!found && mlsw == max_mlsw) {  // reduce.hpp:60-63: every shorter length is excluded
    mlsw++;
    if (b.has_word && b.word.size() != mlsw) b.has_word = false;
    b.lower = b.upper = mlsw;
    return done();
  }
  if (found) {  // reduce.hpp:65-70
    if (apply_word(A, word).size() != 1 || word.size() != mlsw)
      throw std::runtime_error("internal: Reduce word does not synchronize");
    b.lower = b.upper = mlsw;
    b.has_word = true;
    b.word = word;
    return done();
  }
  // reduce.hpp:112-143 (try_to_reduce): states reachable from the list
  const u32 m = E.F.count;
  std::vector<u64> rows((size_t)m * W);
  if (m) SW_CUDA(cudaMemcpyAsync(rows.data(), E.F.rows.p, sizeof(u64) * W * m, cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  std::vector<char> reach(n, 0);
  std::vector<uint32_t> stack;
  for (u32 i = 0; i < m; ++i)
    for (int q = 0; q < n; ++q)
      if ((rows[(size_t)i * W + (q >> 6)] & state_bit(q)) && !reach[q]) {
        reach[q] = 1;
        stack.push_back((uint32_t)q);
      }
  while (!stack.empty()) {  // reduce.hpp:145-169
    const uint32_t q = stack.back();
    stack.pop_back();
    for (int a = 0; a < k; ++a) {
      const uint32_t p = A.at(q, (uint32_t)a);
      if (!reach[p]) {
        reach[p] = 1;
        stack.push_back(p);
      }
    }
  }
  uint32_t rn = 0;
  std::vector<uint32_t> map(n, 0);
  for (int q = 0; q < n; ++q)
    if (reach[q]) map[q] = rn++;
  if (rn == (uint32_t)n || rn == 0) return done();  // reduce.hpp:72-75: skipping reduction
  red = ReduceState{};
  red.active = true;
  red.bfs_steps = mlsw;
  red.original = A;
  red.reduced.n = rn;
  red.reduced.k = A.k;
  red.reduced.t.assign((size_t)rn * A.k, 0);
  for (int q = 0; q < n; ++q)
    if (reach[q])
      for (uint32_t a = 0; a < A.k; ++a) red.reduced.t[(size_t)map[q] * A.k + a] = map[A.at((uint32_t)q, a)];
  // each list set and the word that produced it, traced on the host from the
  // per-layer origin arrays
  std::vector<std::vector<u32>> origin(E.F.layers.size());
  for (size_t d = 0; d < E.F.layers.size(); ++d) {
    const Layer& L = *E.F.layers[d];
    origin[d].resize(L.count);
    if (L.count)
      SW_CUDA(cudaMemcpyAsync(origin[d].data(), L.origin.p, sizeof(u32) * L.count, cudaMemcpyDeviceToHost,
                              E.stream));
  }
  SW_CUDA(cudaStreamSynchronize(E.stream));
  red.seeds.resize(m);
  red.prefix.resize(m);
  for (u32 i = 0; i < m; ++i) {
    for (int q = 0; q < n; ++q)
      if (rows[(size_t)i * W + (q >> 6)] & state_bit(q)) red.seeds[i].push_back(map[q]);
    std::vector<uint32_t>& w = red.prefix[i];
    u32 idx = i;
    for (size_t d = E.F.layers.size(); d-- > 0;) {
      const u32 o = origin[d][idx];
      w.push_back(o / E.F.layers[d]->parent_count);
      idx = o % E.F.layers[d]->parent_count;
    }
    std::reverse(w.begin(), w.end());
  }
  st.reduce_bfs_steps = mlsw;
  st.reduced_states = rn;
  // reduce.hpp:77-84: the remaining search works on reduced lengths
  b.lower = b.lower > mlsw ? b.lower - mlsw : 0;
  b.upper -= mlsw;
  done();
}

// ---------------------------------------------------------------------------
// Learned distance model: training pairs, scoring, training, learned beam.
// ---------------------------------------------------------------------------
namespace {
// 8-word reference layout (state q = bit q % 64 of word q / 64) <-> device rows
// of W words.
std::vector<u64> ref8_to_rows(const uint64_t* ref, uint64_t count, uint32_t n, int W) {
  std::vector<u64> out((size_t)count * W, 0);
  for (uint64_t i = 0; i < count; ++i)
    for (int w = 0; w < 8; ++w) {
      uint64_t v = ref[i * 8 + w];
      while (v) {
        const int q = w * 64 + __builtin_ctzll(v);
        v &= v - 1;
        if ((uint32_t)q < n) out[(size_t)i * W + (q >> 6)] |= state_bit(q);
      }
    }
  return out;
}
void rows_to_ref8(const u64* rows, uint64_t count, uint32_t n, int W, uint64_t* out) {
  for (uint64_t i = 0; i < count; ++i) {
    for (int w = 0; w < 8; ++w) out[i * 8 + w] = 0;
    for (uint32_t q = 0; q < n; ++q)
      if (rows[(size_t)i * W + (q >> 6)] & state_bit((int)q)) out[i * 8 + (q >> 6)] |= 1ULL << (q & 63);
  }
}
}  // namespace

void Solver::set_model(const float* params) {
  SW_CUDA(cudaSetDevice(device_));
  eng_->mlp->set_params(params);
}
void Solver::get_model(float* params) {
  if (!eng_->mlp->has_params()) throw std::runtime_error("no distance model loaded");
  SW_CUDA(cudaSetDevice(device_));
  eng_->mlp->get_params(params);
}
bool Solver::has_model() const { return eng_->mlp->has_params(); }

uint32_t Solver::distance_pairs(const Automaton& A, uint32_t per_layer, uint64_t max_inverse_sets,
                                std::vector<uint64_t>& sets, std::vector<float>& labels,
                                std::vector<uint32_t>& depths) {
  sets.clear();
  labels.clear();
  depths.clear();
  if (A.n < 2 || per_layer == 0) return 0;
  // the reset length bounds the depths worth labelling
  Bounds b;
  b.upper = std::max<u64>(1, (u64)A.n * A.n * A.n / 6);
  sw_exact_config cfg{1, 1, 0, 2048, 10000, (uint64_t)A.n * 16};
  sw_stats st0{};
  exact(A, cfg, b, st0);
  if (b.non_synchro || b.lower != b.upper) return 0;
  const u64 L = b.upper;
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  const int n = (int)A.n, k = (int)A.k, W = words_for(n);
  E.upload_tables(A);
  E.self_check = E.visited_subsets = true;  // labelled layers are the fully reduced ones
  // inverse layers (complements of the maximal preimage sets), depth 0..D
  E.B.reset();
  std::vector<uint32_t> seeds = backward_seeds(A);
  if (seeds.empty()) return 0;
  {
    std::vector<u64> rows((size_t)W * seeds.size(), 0);
    for (size_t i = 0; i < seeds.size(); ++i)
      for (int q = 0; q < n; ++q)
        if ((uint32_t)q != seeds[i]) rows[i * W + (q >> 6)] |= state_bit(q);
    E.B.rows.reserve(sizeof(u64) * rows.size());
    E.B.vis.reserve(sizeof(u64) * rows.size());
    SW_CUDA(cudaMemcpyAsync(E.B.rows.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
    SW_CUDA(cudaMemcpyAsync(E.B.vis.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
    E.B.count = E.B.vis_count = (u32)seeds.size();
    E.sort_by_layer_key(W, E.B.vis.as<u64>(), E.B.vis_count);
  }
  std::vector<std::unique_ptr<DevBuf>> inv;
  std::vector<u32> inv_count;
  u64 inv_total = 0;
  auto keep_layer = [&] {
    inv.push_back(std::make_unique<DevBuf>());
    inv.back()->reserve(sizeof(u64) * W * std::max<u32>(E.B.count, 1));
    SW_CUDA(cudaMemcpyAsync(inv.back()->p, E.B.rows.p, sizeof(u64) * W * E.B.count, cudaMemcpyDeviceToDevice,
                            E.stream));
    inv_count.push_back(E.B.count);
    inv_total += E.B.count;
  };
  keep_layer();
  for (u64 j = 1; j <= L && inv_total < max_inverse_sets; ++j) {
    E.step(E.B, false, W, n, k, true);
    if (!E.B.count) break;
    keep_layer();
  }
  const u32 D = (u32)inv.size() - 1;
  // forward layers, sampled and labelled
  E.F.reset();
  {
    std::vector<u64> full(W, 0);
    for (int q = 0; q < n; ++q) full[q >> 6] |= state_bit(q);
    E.F.rows.reserve(sizeof(u64) * W);
    E.F.vis.reserve(sizeof(u64) * W);
    SW_CUDA(cudaMemcpyAsync(E.F.rows.p, full.data(), sizeof(u64) * W, cudaMemcpyHostToDevice, E.stream));
    SW_CUDA(cudaMemcpyAsync(E.F.vis.p, full.data(), sizeof(u64) * W, cudaMemcpyHostToDevice, E.stream));
    E.F.count = E.F.vis_count = 1;
  }
  DevBuf idx_d, sample, flags;
  for (u64 i = 0; i <= L; ++i) {
    const u32 c = E.F.count;
    const u32 s = std::min<u32>(c, per_layer);
    std::vector<u32> idx(s);
    for (u32 t = 0; t < s; ++t) idx[t] = (u32)(((u64)t * c) / s);
    idx_d.reserve(sizeof(u32) * s);
    sample.reserve(sizeof(u64) * W * s);
    flags.reserve(sizeof(u32) * s);
    SW_CUDA(cudaMemcpyAsync(idx_d.p, idx.data(), sizeof(u32) * s, cudaMemcpyHostToDevice, E.stream));
    launch_gather_rows(W, E.F.rows.as<u64>(), idx_d.as<u32>(), s, sample.as<u64>(), E.stream);
    std::vector<float> lab(s, (float)(D + 1));
    std::vector<u32> fl(s);
    u32 open = s;
    for (u32 j = 0; j <= D && open; ++j) {
      launch_fill_u32(flags.as<u32>(), 0, s, E.stream);
      E.query(W, kQueryDisjoint, inv[j]->as<u64>(), inv_count[j], sample.as<u64>(), s, n, flags.as<u32>(), false);
      SW_CUDA(cudaMemcpyAsync(fl.data(), flags.p, sizeof(u32) * s, cudaMemcpyDeviceToHost, E.stream));
      SW_CUDA(cudaStreamSynchronize(E.stream));
      for (u32 t = 0; t < s; ++t)
        if (fl[t] && lab[t] > (float)j) {
          lab[t] = (float)j;
          --open;
        }
    }
    std::vector<u64> rows((size_t)s * W);
    SW_CUDA(cudaMemcpy(rows.data(), sample.p, sizeof(u64) * W * s, cudaMemcpyDeviceToHost));
    const size_t base = sets.size();
    sets.resize(base + (size_t)s * 8);
    rows_to_ref8(rows.data(), s, (uint32_t)n, W, sets.data() + base);
    labels.insert(labels.end(), lab.begin(), lab.end());
    depths.insert(depths.end(), s, (uint32_t)i);
    if (i == L) break;
    E.step(E.F, true, W, n, k, true);
    if (!E.F.count) break;
  }
  return (uint32_t)L;
}

void Solver::mlp_forward(const Automaton& A, const uint64_t* sets, uint64_t count, float* out) {
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  if (!count) return;
  const std::vector<u64> rows = ref8_to_rows(sets, count, A.n, 8);
  DevBuf d_rows, d_y;
  d_rows.reserve(sizeof(u64) * rows.size());
  d_y.reserve(sizeof(float) * count);
  SW_CUDA(cudaMemcpyAsync(d_rows.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
  E.mlp->prepare(A);
  E.mlp->forward(d_rows.as<u64>(), 8, (u32)count, d_y.as<float>());
  SW_CUDA(cudaMemcpyAsync(out, d_y.p, sizeof(float) * count, cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
}

float Solver::mlp_gradient(const Automaton& A, const uint64_t* sets, const float* labels, uint64_t count,
                           float* grad) {
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  if (!count) throw std::invalid_argument("empty batch");
  const std::vector<u64> rows = ref8_to_rows(sets, count, A.n, 8);
  DevBuf d_rows, d_y, d_t;
  d_rows.reserve(sizeof(u64) * rows.size());
  d_y.reserve(sizeof(float) * count);
  d_t.reserve(sizeof(float) * count);
  SW_CUDA(cudaMemcpyAsync(d_rows.p, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice, E.stream));
  SW_CUDA(cudaMemcpyAsync(d_t.p, labels, sizeof(float) * count, cudaMemcpyHostToDevice, E.stream));
  E.mlp->prepare(A);
  E.mlp->zero_grad();
  E.mlp->forward(d_rows.as<u64>(), 8, (u32)count, d_y.as<float>());
  E.mlp->backward(d_t.as<float>(), (u32)count);
  float loss = 0;
  SW_CUDA(cudaMemcpyAsync(grad, E.mlp->grad(), sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaMemcpyAsync(&loss, E.mlp->loss(), sizeof(float), cudaMemcpyDeviceToHost, E.stream));
  SW_CUDA(cudaStreamSynchronize(E.stream));
  return loss;
}

float Solver::mlp_train(const std::vector<Automaton>& autos, const uint64_t* offsets, const uint64_t* sets,
                        const float* labels, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                        const uint32_t* groups, float rank_w) {
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  const size_t A_n = autos.size();
  const uint64_t total = offsets[A_n];
  if (!total || !batch) throw std::invalid_argument("no training pairs");
  // all pairs resident on the device as 8-word rows
  DevBuf d_rows, d_lab, d_y;
  d_rows.reserve(sizeof(u64) * 8 * total);
  d_lab.reserve(sizeof(float) * total);
  d_y.reserve(sizeof(float) * batch);
  for (size_t a = 0; a < A_n; ++a) {
    const uint64_t o = offsets[a], c = offsets[a + 1] - o;
    if (!c) continue;
    const std::vector<u64> rows = ref8_to_rows(sets + o * 8, c, autos[a].n, 8);
    SW_CUDA(cudaMemcpy(d_rows.as<u64>() + o * 8, rows.data(), sizeof(u64) * rows.size(), cudaMemcpyHostToDevice));
  }
  SW_CUDA(cudaMemcpy(d_lab.p, labels, sizeof(float) * total, cudaMemcpyHostToDevice));
  DevBuf d_grp;
  if (groups && rank_w > 0.0f) {
    d_grp.reserve(sizeof(uint32_t) * total);
    SW_CUDA(cudaMemcpy(d_grp.p, groups, sizeof(uint32_t) * total, cudaMemcpyHostToDevice));
  }
  std::vector<size_t> order(A_n);
  for (size_t a = 0; a < A_n; ++a) order[a] = a;
  uint64_t state = seed;
  auto next = [&] {  // SplitMix64
    uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  double last = 0;
  for (uint32_t ep = 0; ep < epochs; ++ep) {
    for (size_t a = A_n; a > 1; --a) std::swap(order[a - 1], order[next() % a]);
    double sum = 0;
    uint64_t steps = 0;
    for (size_t oi = 0; oi < A_n; ++oi) {
      const size_t a = order[oi];
      for (uint64_t o = offsets[a]; o < offsets[a + 1]; o += batch) {
        const u32 c = (u32)std::min<uint64_t>(batch, offsets[a + 1] - o);
        E.mlp->prepare(autos[a]);
        E.mlp->zero_grad();
        E.mlp->forward(d_rows.as<u64>() + o * 8, 8, c, d_y.as<float>());
        E.mlp->backward(d_lab.as<float>() + o, c, d_grp.p ? d_grp.as<uint32_t>() + o : nullptr, rank_w);
        E.mlp->adam_step(lr);
        float l = 0;
        SW_CUDA(cudaMemcpyAsync(&l, E.mlp->loss(), sizeof(float), cudaMemcpyDeviceToHost, E.stream));
        SW_CUDA(cudaStreamSynchronize(E.stream));
        sum += l;
        ++steps;
      }
    }
    last = steps ? sum / steps : 0.0;
  }
  return (float)last;
}

void Solver::learned_beam(const Automaton& A, const sw_learned_beam_config& cfg, Bounds& b, sw_stats& st) {
  if (b.non_synchro || b.lower == b.upper) return;
  const bool use_model = cfg.order != SW_ORDER_SIZE;
  if (use_model && !has_model()) throw std::runtime_error("LearnedBeam: no distance model loaded");
  if (A.n == 1) {
    b.lower = b.upper = 0;
    b.has_word = true;
    b.word.clear();
    return;
  }
  SW_CUDA(cudaSetDevice(device_));
  Engine& E = *eng_;
  E.st = &st;
  auto t0 = std::chrono::steady_clock::now();
  const int n = (int)A.n, k = (int)A.k, W = words_for(n);
  E.upload_tables(A);
  if (use_model) E.mlp->prepare(A);
  E.F.reset();
  {
    std::vector<u64> full(W, 0);
    for (int q = 0; q < n; ++q) full[q >> 6] |= state_bit(q);
    E.F.rows.reserve(sizeof(u64) * W);
    SW_CUDA(cudaMemcpyAsync(E.F.rows.p, full.data(), sizeof(u64) * W, cudaMemcpyHostToDevice, E.stream));
    E.F.count = 1;
    E.F.vis_count = 0;
  }
  const u32 width = (u32)std::min<uint64_t>(cfg.beam_size, 1u << 26);
  // engine-owned, kept across calls: freeing device memory would synchronise the device
  DevBuf &counts = E.lb_counts, &scores = E.lb_scores, &keys = E.lb_keys, &vals = E.lb_vals;
  DevBuf &alt_k = E.lb_alt_k, &alt_v = E.lb_alt_v, &sel_rows = E.lb_sel_rows, &sel_origin = E.lb_sel_origin;
  std::vector<u32> pc;
  u64 found_len = 0;
  std::vector<uint32_t> word;
  for (u64 depth = 1; depth < b.upper && (cfg.max_iter < 0 || depth <= (u64)cfg.max_iter); ++depth) {
    E.step(E.F, true, W, n, k, /*dominance=*/false);  // children, duplicates removed, origins recorded
    const u32 m = E.F.count;
    if (!m) break;
    counts.reserve(sizeof(u32) * m);
    launch_popcount(W, E.F.rows.as<u64>(), m, counts.as<u32>(), E.stream);
    pc.resize(m);
    SW_CUDA(cudaMemcpyAsync(pc.data(), counts.p, sizeof(u32) * m, cudaMemcpyDeviceToHost, E.stream));
    SW_CUDA(cudaStreamSynchronize(E.stream));
    u32 hit = UINT32_MAX;
    for (u32 i = 0; i < m && hit == UINT32_MAX; ++i)
      if (pc[i] == 1) hit = i;
    if (hit != UINT32_MAX) {
      word = E.trace(E.F, hit, nullptr);
      std::reverse(word.begin(), word.end());
      found_len = depth;
      break;
    }
    if (m <= width) continue;
    // keep the `width` children with the smallest score (ties: child order)
    keys.reserve(sizeof(u64) * m);
    vals.reserve(sizeof(u32) * m);
    if (use_model) {
      scores.reserve(sizeof(float) * m);
      E.mlp->forward(E.F.rows.as<u64>(), W, m, scores.as<float>());
    }
    launch_score_keys(use_model ? scores.as<float>() : nullptr,
                      cfg.order != SW_ORDER_MODEL ? counts.as<u32>() : nullptr, m, keys.as<u64>(), E.stream);
    launch_iota(vals.as<u32>(), m, E.stream);
    E.sort_rows(1, keys.as<u64>(), vals.as<u32>(), m);
    sel_rows.reserve(sizeof(u64) * W * width);
    sel_origin.reserve(sizeof(u32) * width);
    launch_gather_rows(W, E.F.rows.as<u64>(), vals.as<u32>(), width, sel_rows.as<u64>(), E.stream);
    Layer& top = *E.F.layers.back();
    launch_gather_u32(top.origin.as<u32>(), vals.as<u32>(), width, sel_origin.as<u32>(), E.stream);
    SW_CUDA(cudaMemcpyAsync(E.F.rows.p, sel_rows.p, sizeof(u64) * W * width, cudaMemcpyDeviceToDevice, E.stream));
    SW_CUDA(cudaMemcpyAsync(top.origin.p, sel_origin.p, sizeof(u32) * width, cudaMemcpyDeviceToDevice, E.stream));
    top.count = width;
    E.F.count = width;
    E.count_launch(5);
  }
  if (found_len && found_len < b.upper) {
    if (apply_word(A, word).size() != 1 || word.size() != found_len)
      throw std::runtime_error("internal: learned beam word does not synchronize");
    b.upper = found_len;
    b.has_word = true;
    b.word = word;
  }
  st.device_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  E.st = nullptr;
}

}  // namespace sw
