/*
 * synchrowords GB300 — C ABI of the GPU exact shortest-reset-word search.
 *
 * Drop-in boundary for SynchroLib 1.1.0's plugin entry
 *   extern "C" void run(const std::string& aut_encoded,
 *                       const std::vector<std::string>& algorithms,
 *                       AlgoResult& result, Logger::LogLevel)
 * (jit/jitmain.cpp:11-49), which passes C++ objects and needs N, K at compile
 * time.  This ABI takes plain pointers and sizes, dispatches on the runtime
 * number of states n (1..512) and alphabet size k (1..16), returns status
 * codes (nothing throws across it) and keeps device buffers in an opaque
 * context between calls.
 *
 * Automaton layout (as the reference, synchrolib/data_structures/automaton/
 * automaton.hpp:14-33 and app/io.hpp:136-159): delta[q*k + a] is the state
 * reached from q by letter a, 0 <= delta[.] < n.
 *
 * Host bitset layout used by the kernel-level entry points (as the
 * reference's Subset<N>, synchrolib/data_structures/subset.hpp:11-26): a set
 * is ceil(n/64) uint64 words, state q is bit q%64 of word q/64, bits >= n are 0.
 */
#ifndef SYNCHROWORDS_H
#define SYNCHROWORDS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SW_OK 0
#define SW_ERR_INVALID_ARGUMENT (-1) /* bad pointer, size or automaton entry */
#define SW_ERR_CONFIG (-2)           /* plan JSON / expression error (app/jit.hpp:61-83 exit 4) */
#define SW_ERR_CUDA (-3)             /* CUDA runtime error (reference: checkCudaErrors + exit) */
#define SW_ERR_NO_DEVICE (-4)        /* no CUDA device: this library has no CPU fallback */
#define SW_ERR_UNSUPPORTED (-5)      /* algorithm outside this library's scope */
#define SW_ERR_INTERNAL (-6)         /* internal check failed (e.g. word verification) */
#define SW_ERR_CAPACITY (-7)         /* caller buffer too small */

#define SW_MAX_STATES 512
#define SW_MAX_LETTERS 16
#define SW_MAX_ALGORITHMS 16
#define SW_NAME_LEN 16

/* ---- plan (the reference's JSON config, evaluated for one (n, k)) -------- */
typedef enum {
  SW_ALGO_EXACT = 1,    /* synchrolib/algorithm/exact/ */
  SW_ALGO_BEAM = 2,     /* synchrolib/algorithm/beam/ */
  SW_ALGO_BRUTE = 3,    /* synchrolib/algorithm/brute/ */
  SW_ALGO_EPPSTEIN = 4, /* synchrolib/algorithm/eppstein/ */
  SW_ALGO_REDUCE = 5,   /* synchrolib/algorithm/reduce/ */
  SW_ALGO_LEARNED_BEAM = 6 /* no reference counterpart: forward beam scored by the learned model */
} sw_algo_kind;

/* Evaluated Exact defines (synchrolib/algorithm/exact/config.hpp:24-46). */
typedef struct {
  int32_t dfs;                  /* "dfs" (default true) */
  int32_t dfs_shortcut;         /* "dfs_shortcut" (default true) */
  int32_t strict_memory_limit;  /* "strict_memory_limit" (default false) */
  uint64_t max_memory_mb;       /* "max_memory_mb" (default 2048): device budget of the lists */
  uint64_t dfs_min_list_size;   /* "dfs_min_list_size" (default 10000) */
  uint64_t bfs_small_list_size; /* "bfs_small_list_size" (default AUT_N * 16) */
  /* "reductions" (no reference key; the reference always reduces): when the
   * device search drops sets dominated by a visited set or by a proper subset
   * in their layer (meet_in_the_middle.cpp:195-237, 264-337).  Lengths never
   * depend on it.  SW_REDUCE_AUTO ("auto", default): when the upper bound is
   * backed by a word or the lists pass a quarter of max_memory_mb;
   * SW_REDUCE_ALWAYS ("always"); SW_REDUCE_MEMORY ("memory"): only past a
   * quarter of max_memory_mb. */
  int32_t reductions;
} sw_exact_config;
#define SW_REDUCE_AUTO 0
#define SW_REDUCE_ALWAYS 1
#define SW_REDUCE_MEMORY 2

/* Evaluated Beam defines (synchrolib/algorithm/beam/config.hpp:23-44). */
typedef struct {
  uint64_t beam_size;      /* "beam_size" (default std::log2(AUT_N)) */
  int32_t dynamic;         /* "dynamic" (default false) */
  uint64_t min_beam_size;  /* "min_beam_size" (default AUT_N * std::log2(AUT_N)) */
  uint64_t max_beam_size;  /* "max_beam_size" (default AUT_N * AUT_N * std::log2(AUT_N)) */
  double beam_exact_ratio; /* "beam_exact_ratio" (default 0.01) */
  int64_t max_iter;        /* "max_iter" (default -1) */
  int32_t presort_indeg;   /* "presort": 0 = "none", 1 = "indeg" */
} sw_beam_config;

/* Evaluated Brute defines (synchrolib/algorithm/brute/config.hpp:23-27). */
typedef struct {
  uint64_t max_n; /* "max_n" (default 20; above 32 the algorithm refuses to run) */
} sw_brute_config;

/* Evaluated Eppstein defines (synchrolib/algorithm/eppstein/config.hpp:23-31).
 * Neither changes the bound; the word is returned whenever it is verified. */
typedef struct {
  int32_t transition_tables; /* "transition_tables" (default false) */
  int32_t find_word;         /* "find_word" (default false) */
} sw_eppstein_config;

/* Evaluated Reduce defines (synchrolib/algorithm/reduce/config.hpp:24-32). */
typedef struct {
  uint64_t min_n;               /* "min_n" (default 80) */
  uint64_t list_size_threshold; /* "list_size_threshold" (default AUT_N * 16) */
} sw_reduce_config;

/* "LearnedBeam" (no reference counterpart): a forward beam from the full set
 * that keeps the `beam_size` best children of each layer; the first
 * singleton gives an upper bound and its word.  "order" ranks children by
 * "model" (smallest predicted merge length, the context's distance model),
 * "size" (fewest states; no model needed) or "size_model" (fewest states,
 * ties by predicted merge length). */
#define SW_ORDER_MODEL 0
#define SW_ORDER_SIZE 1
#define SW_ORDER_SIZE_MODEL 2
typedef struct {
  uint64_t beam_size; /* "beam_size" (default 4096) */
  int64_t max_iter;   /* "max_iter" (default -1: up to the upper bound) */
  int32_t order;      /* "order" (default "model"): SW_ORDER_* */
} sw_learned_beam_config;

typedef struct {
  int32_t kind; /* sw_algo_kind */
  char name[SW_NAME_LEN];
  sw_exact_config exact;
  sw_beam_config beam;
  sw_brute_config brute;
  sw_eppstein_config eppstein;
  sw_reduce_config reduce;
  sw_learned_beam_config learned_beam;
} sw_algorithm;

/* Global plan keys (app/jit.hpp:112-141, docs/config.md:15-27). */
typedef struct {
  uint64_t upper_bound;       /* "upper_bound" (default 1ULL*AUT_N*AUT_N*AUT_N/6) */
  uint32_t threads;           /* "threads" (1..64; host threads of the CPU reference only) */
  int32_t gpu;                /* "gpu" (accepted; this library always runs on the GPU) */
  uint64_t gpu_max_memory_mb; /* "gpu_max_memory_mb" (default 2048) */
  uint32_t n_algorithms;
  sw_algorithm algorithms[SW_MAX_ALGORITHMS];
} sw_plan;

/* ---- result (synchrolib/algorithm/algorithm.hpp:19-42) ------------------ */
typedef struct {
  char name[SW_NAME_LEN];
  uint64_t ms;
} sw_algo_run;

typedef struct {
  uint64_t subsets_expanded;  /* children produced by layer expansion */
  uint64_t subsets_kept;      /* sets that survived dedup + dominance */
  uint64_t trie_queries;      /* subset queries issued against a radix tree */
  uint64_t logical_pairs;     /* sum over queries of the queried list size (|S| per query) */
  uint64_t meet_pairs;        /* logical (F, B) pairs covered by meet checks */
  uint64_t bfs_steps;         /* forward layers */
  uint64_t ibfs_steps;        /* inverse layers */
  uint64_t dfs_sets;          /* sets generated in the memory-bounded inverse DFS phase */
  uint64_t kernel_launches;   /* device kernels launched by the solve */
  double device_ms;           /* wall time of the solve spent in the GPU search */
  uint64_t reduce_bfs_steps;  /* BFS steps of a successful Reduce (0 if none) */
  uint64_t reduced_states;    /* states left after a successful Reduce (0 if none) */
} sw_stats;

typedef struct {
  int32_t non_synchro;
  uint64_t mlsw_lower_bound;
  uint64_t mlsw_upper_bound;
  int32_t has_word;       /* 1 if word[0..word_len) is a verified reset word */
  uint32_t word_len;
  uint32_t* word;         /* caller buffer, may be NULL */
  uint32_t word_capacity; /* entries available in `word` */
  uint32_t n_runs;
  sw_algo_run runs[SW_MAX_ALGORITHMS];
  sw_stats stats;
} sw_result;

typedef struct sw_context sw_context;

/* ---- library ------------------------------------------------------------ */
const char* sw_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* sw_last_error(void);

/* Parse a plan (the reference's config JSON, docs/config.md) and evaluate its
 * expressions for an automaton with n states and k letters.  Replaces
 * AlgoConfig::get_substs + the JIT's compile-time evaluation
 * (synchrolib/algorithm/config.hpp:57-60, app/jit.hpp:96-141). */
int sw_plan_from_json(const char* json, uint32_t n, uint32_t k, sw_plan* out);

/* Evaluate one C++ config expression (AUT_N = n, AUT_K = k) as the reference's
 * compiler would and convert it to uint64 / double.  For tests and tools. */
int sw_eval_expression(const char* expr, uint32_t n, uint32_t k, uint64_t* as_u64, double* as_double);

/* Context = one CUDA device + persistent device buffers.  Not thread-safe:
 * use one context per host thread (the reference is single-caller too). */
int sw_context_create(int device, sw_context** out);
void sw_context_destroy(sw_context* ctx);

/* Run every algorithm of `plan` in order on one automaton, as the reference's
 * run() does (jit/jitmain.cpp:11-49): bounds start at
 * [0, min(upper_bound, UINT64_MAX)], each algorithm may tighten them, and
 * per-algorithm milliseconds are recorded.  `result->word` (if non-NULL)
 * receives a reset word of length mlsw_upper_bound when one was found and
 * verified (the reference's Exact returns no word; this one does). */
int sw_solve(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const sw_plan* plan,
             sw_result* result);

/* Same as sw_solve with the plan given as JSON text (evaluated for this n, k). */
int sw_solve_json(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, const char* plan_json,
                  sw_result* result);

/* Solve `count` automata with the same plan (evaluated per automaton's n, k).
 * deltas holds the automata back to back (n_i*k_i entries each); results[i]
 * gets instance i (set results[i].word / word_capacity beforehand to receive
 * words).  `workers` device streams (0 = min(count, 16)), each driven by its
 * own host thread, solve instances concurrently on the context's GPU.  The
 * reference solves the automata of a file one after another
 * (app/main.cpp:48-78); there is no batched counterpart.
 *
 * Automata of at most 256 states (n * k <= 4096) whose plan is a single
 * Exact run are solved on the device without host round trips:
 *   - those with n * log2(k) at most the context's batched_limit (default
 *     104: binary automata up to 104 states, ternary up to 65; k <= 4) by one
 *     persistent launch per set width, one GPU block per automaton at a time,
 *     lists in shared memory;
 *   - the others, and those the first launch cannot finish within its
 *     capacities, by one persistent launch per set width on thread-block
 *     clusters (cluster_size CTAs per automaton, lists in the cluster's
 *     L2-resident global region) when n * log2(k) is at most cluster_limit
 *     (and cluster_size is not -1).
 * What neither finishes within its capacities, and every other automaton,
 * runs on the worker streams.  workers = 0 uses the context's tuned count
 * (sw_autotune_batch / sw_set_batch_tuning), else min(count, 16). */
int sw_solve_batch(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                   const char* plan_json, sw_result* results, uint32_t workers);

typedef struct {
  uint32_t workers;      /* worker streams when sw_solve_batch gets 0; 0 = min(count, 16) */
  double batched_limit;  /* n * log2(k) bound for the batched launch; < 0 disables it */
  int32_t cluster_size;  /* CTAs per automaton of the cluster launch (1..16); 0 = 8; -1 disables it */
  double cluster_limit;  /* n * log2(k) bound for the cluster launch, default 160 (above it: worker streams) */
} sw_batch_tuning;

/* What the last sw_solve_batch on this context did on the device (no
 * counterpart in the reference, which solves one automaton at a time). */
typedef struct {
  uint32_t small_solved;    /* automata finished by the shared-memory batched launch */
  uint32_t cluster_solved;  /* automata finished by the cluster launch */
  uint32_t streamed;        /* automata solved on the worker streams */
  uint32_t launches;        /* batched kernel launches */
  double device_ms;         /* CUDA-event time of the batched launches on the batch stream */
  uint64_t meet_pairs;      /* logical (F, B) pairs of the cluster launches' meet checks */
  uint64_t children;        /* children expanded by the cluster launches */
  uint64_t staged_bytes;    /* backward rows the cluster launches' meet checks staged (bit-sliced) on chip */
  uint64_t steps;           /* BFS levels of the cluster launches */
  uint32_t graph_replays;   /* device rounds replayed from a CUDA graph captured for an earlier batch of the same
                               shape (each round's launches are captured once per shape and buffer set) */
} sw_batch_profile;

int sw_batch_last_profile(sw_context* ctx, sw_batch_profile* out);

int sw_get_batch_tuning(sw_context* ctx, sw_batch_tuning* out);
int sw_set_batch_tuning(sw_context* ctx, const sw_batch_tuning* in);

/* Batch autotuner: times the batch (wall clock, best of `reps` runs, 0 = 1)
 * first at each candidate worker count with the current batched_limit, then
 * at each candidate batched_limit with the best worker count, and keeps the
 * fastest pair as the context's tuning (its cluster_size is kept).  NULL candidate lists use the
 * defaults (workers 8, 12, 16, 24 clipped to count; limits -1, 104, 1024).
 * ms (if not NULL) receives n_workers + n_limits times in that order (4 + 3
 * for the defaults); *best the chosen tuning.  results hold the last run. */
int sw_autotune_batch(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                      const char* plan_json, sw_result* results, const uint32_t* worker_candidates,
                      uint32_t n_workers, const double* limit_candidates, uint32_t n_limits, uint32_t reps,
                      double* ms, sw_batch_tuning* best);

/* Cluster-launch autotuner: times the batch (wall clock, best of `reps`)
 * first at each candidate cluster_size (CTAs per automaton, 1..16) with the
 * current cluster_limit, then at each candidate cluster_limit (n * log2(k)
 * bound of the automata the cluster launch takes; -1 = none) with the best
 * size, and keeps the fastest pair in the context's tuning (workers and
 * batched_limit unchanged).  NULL candidate lists use the defaults (sizes
 * 2, 4, 8, 16; limits -1, 128, 160, 200).  ms (if not NULL) receives
 * n_sizes + n_limits times; *best the chosen tuning.  No counterpart in the
 * reference. */
int sw_autotune_cluster(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                        const char* plan_json, sw_result* results, const int32_t* size_candidates, uint32_t n_sizes,
                        const double* limit_candidates, uint32_t n_limits, uint32_t reps, double* ms,
                        sw_batch_tuning* best);

/* ---- subset-check launch shape and its autotuner -----------------------
 * No counterpart in the reference (its trie walk has no launch shape).  The
 * subset check (sw_subsets_check and every check inside the searches) cuts
 * the sorted list S into tiles of tile_rows rows with an AND mask per tile and
 * per super-tile of tiles_per_super tiles; a block of `warps` warps tests 32
 * queries per warp against the tiles of one chunk of S, and S is chunked so
 * that the grid holds about grid_factor blocks per SM.  A context keeps one
 * shape per row width (words = ceil(n / 64), 1..8) and list size class; the
 * shape changes speed only, never results. */
typedef struct {
  int32_t tile_rows;        /* rows of S per tile staged in shared memory: 32, 64 or 128 (default 64) */
  int32_t warps;            /* warps of 32 queries per block: 4, 8 or 16 (default 8) */
  int32_t tiles_per_super;  /* tiles per super-tile AND mask: 4, 8, 16 or 32 (default 16) */
  int32_t grid_factor;      /* target blocks per SM of the grid, 1..64 (default 16) */
} sw_scan_shape;

#define SW_SCAN_SIZE_CLASSES 2    /* class 0: lists S of fewer than SW_SCAN_LARGE_ROWS rows; 1: larger */
#define SW_SCAN_LARGE_ROWS 32768u

int sw_get_scan_shape(sw_context* ctx, uint32_t words, uint32_t size_class, sw_scan_shape* out);
/* SW_OK when `shape` is a valid launch shape for rows of `words` words (the
 * rule sw_set_scan_shape applies), else SW_ERR_INVALID_ARGUMENT with the
 * reason in sw_last_error().  Host-only: needs no device. */
int sw_scan_shape_check(uint32_t words, const sw_scan_shape* shape);
/* SW_ERR_INVALID_ARGUMENT for a value outside the lists above, or when two
 * tiles per warp (8 * words * tile_rows * 2 * warps bytes) exceed 200 KiB. */
int sw_set_scan_shape(sw_context* ctx, uint32_t words, uint32_t size_class, const sw_scan_shape* in);

typedef struct {
  uint32_t words;       /* row width of the key */
  uint32_t size_class;  /* list size class of the key */
  uint64_t checks;      /* subset checks of this key in one pass over the automata */
  double ms_start;      /* their CUDA-event milliseconds (mask build + scan) with the starting shape */
  double ms_best;       /* with the chosen shape */
  sw_scan_shape shape;  /* the chosen shape, kept on the context */
} sw_scan_tuned;

/* Subset-check autotuner: solves the automata one after another on the
 * context's stream (plan_json; NULL = plain Exact) with every subset check
 * timed by CUDA events per (words, size class) key, then, knob by knob
 * (tile_rows 32/64/128, warps 4/8/16, tiles_per_super 4/8/16/32, grid_factor
 * 4/8/16/32/64), reruns them once per candidate value with that value set for
 * every key, and each key keeps its fastest value (coordinate descent; a value
 * must beat the key's best by 2%; best of `reps` passes, 0 = 1).  out (up to
 * out_cap entries) receives one entry per key the automata used, *out_count
 * their number.  The chosen shapes stay on the context. */
int sw_autotune_scan(sw_context* ctx, uint32_t count, const uint32_t* deltas, const uint32_t* ns, const uint32_t* ks,
                     const char* plan_json, uint32_t reps, sw_scan_tuned* out, uint32_t out_cap,
                     uint32_t* out_count);

/* ---- measurement --------------------------------------------------------
 * No counterpart in the reference (its timers are host RAII timers,
 * synchrolib/utils/timer.hpp:9-41).  Between sw_profile_begin and
 * sw_profile_end every kernel launch of the context is bracketed by CUDA
 * events on the context's stream; sw_profile_end synchronises and reports, per
 * kernel class, the launches, summed device milliseconds and the algorithmic
 * bytes those launches had to move.  Classes: 0 subset-query tree walks,
 * 1 layer expansion, 2 radix sorts, 3 everything else. */
typedef struct {
  uint64_t launches;
  double ms;
  double bytes;
} sw_kernel_profile;

#define SW_PROFILE_CLASSES 4
int sw_profile_begin(sw_context* ctx);
int sw_profile_end(sw_context* ctx, sw_kernel_profile out[SW_PROFILE_CLASSES]);
/* The cudaStream_t (as void*) every kernel of `ctx` is launched on. */
void* sw_context_stream(sw_context* ctx);

/* ---- kernel-level entry points (host buffers, reference bitset layout) ---
 * These are the device operations the reference offloads, exposed for parity
 * tests and for callers that drive their own search. */

/* Image (inverse = 0) or preimage-union (inverse = 1) of `count` sets under
 * one letter.  Replaces preprocessed_transition_kernel
 * (synchrolib/data_structures/cuda/preprocessed_transition_kernel.cu:54-88)
 * and PreprocessedTransition::apply (preprocessed_transitions.cpp:56-93). */
int sw_apply_transition(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, uint32_t letter,
                        int32_t inverse, const uint64_t* from, uint64_t* to, uint64_t count);

/* results[i] = 1 if some sets[j] ⊆ checks[i] (sets[j] ⊊ checks[i] when
 * proper), else 0.  Replaces SubsetsImplicitTrieKernel::run /
 * subsets_trie_kernel_impl_v2 and the proper variant
 * (synchrolib/data_structures/cuda/subsets_implicit_trie_kernel.cu:13-92,
 * 183-223) and SubsetsImplicitTrie::check_contains_subset
 * (synchrolib/data_structures/subsets_implicit_trie.hpp:29-44). */
int sw_subsets_check(sw_context* ctx, uint32_t n, const uint64_t* sets, uint64_t set_count, const uint64_t* checks,
                     uint64_t check_count, int32_t proper, uint8_t* results);

/* Sort (in the reference's order, subset.hpp:71-77) and deduplicate `count`
 * sets in place; *out_count receives the number kept.  Replaces
 * sort_keep_unique (synchrolib/utils/vector.hpp:13-27). */
int sw_sort_unique(sw_context* ctx, uint32_t n, uint64_t* sets, uint64_t count, uint64_t* out_count);

/* ---- learned distance model (no reference counterpart) -------------------
 * A set S is scored by y = w3 · relu(W2 relu(W1 x + b1) + b2) + b3 with
 * x = sum over q in S of relu(feat(q) · Phi + c): per-state BF16 embeddings
 * from fixed per-state features (so one model fits automata of any size),
 * dense layers 64 -> 128 -> 128 on the tensor cores with FP32 accumulation.
 * Parameters are SW_MLP_PARAMS floats: Phi[16][64], c[64], W1[64][128],
 * b1[128], W2[128][128], b2[128], w3[128], b3.  Sets passed to these calls
 * use 8 words per set in the reference bit layout (state q = bit q % 64 of
 * word q / 64). */
#define SW_MLP_PARAMS 26049
#define SW_STATE_FEATURES 16

/* The model a context's LearnedBeam uses (copied; replaces the previous one). */
int sw_context_set_model(sw_context* ctx, const float* params, uint32_t count);
int sw_context_get_model(sw_context* ctx, float* params, uint32_t count);

/* Per-state feature rows of an automaton: out[n * SW_STATE_FEATURES]. */
int sw_state_features(const uint32_t* delta, uint32_t n, uint32_t k, float* out);

/* Training pairs: sets of the dominance-pruned forward BFS layers of the
 * automaton (at most `per_layer` per layer, evenly spread), each labelled
 * with its exact shortest merge length, found by subset queries against the
 * inverse BFS layers from the singletons (labels above the inverse depth
 * reached are censored to that depth + 1); depths[i] = the forward layer of
 * set i (may be NULL).  *length = the reset length. */
int sw_distance_pairs(sw_context* ctx, const uint32_t* delta, uint32_t n, uint32_t k, uint32_t per_layer,
                      uint64_t max_inverse_sets, uint64_t* sets, float* labels, uint32_t* depths, uint64_t capacity,
                      uint64_t* count, uint32_t* length);

/* Model output for `count` sets of one automaton (loads `params` into ctx). */
int sw_mlp_forward(sw_context* ctx, const float* params, const uint32_t* delta, uint32_t n, uint32_t k,
                   const uint64_t* sets, uint64_t count, float* out);

/* Gradient of the mean squared error over the batch (loads `params`). */
int sw_mlp_gradient(sw_context* ctx, const float* params, const uint32_t* delta, uint32_t n, uint32_t k,
                    const uint64_t* sets, const float* labels, uint64_t count, float* grad, float* loss);

/* Adam training over labelled sets of many automata; pairs of automaton i
 * are [offsets[i], offsets[i+1]).  `params` in: start, out: trained (also
 * loaded into ctx).  *loss = mean batch loss of the last epoch. */
int sw_mlp_train(sw_context* ctx, float* params, uint32_t automata, const uint32_t* deltas, const uint32_t* ns,
                 const uint32_t* ks, const uint64_t* offsets, const uint64_t* sets, const float* labels,
                 uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* loss);

/* sw_mlp_train with a ranking term: groups[j] is a group id per pair (its
 * BFS layer); the loss adds rank_weight / batch times, over the pairs (a, b)
 * of one group in a batch with labels[a] < labels[b], log(1 + exp(y_a - y_b)),
 * so that within a layer a set nearer to a singleton scores lower — the order
 * a beam keeps.  rank_weight = 0 is plain sw_mlp_train. */
int sw_mlp_train_ranked(sw_context* ctx, float* params, uint32_t automata, const uint32_t* deltas,
                        const uint32_t* ns, const uint32_t* ks, const uint64_t* offsets, const uint64_t* sets,
                        const float* labels, const uint32_t* groups, float rank_weight, uint32_t epochs,
                        uint32_t batch, float lr, uint64_t seed, float* loss);

/* ---- allocation-free variant --------------------------------------------
 * No counterpart in the reference (its GPU helpers cudaMalloc and cudaFree
 * on every call, preprocessed_transition_kernel.cu:65-87).
 *
 * For callers that must not have the library allocate device memory — an
 * application whose own pool allocator owns the device budget, or a service
 * that forbids allocation while it serves requests.  Same check as
 * sw_subsets_check, but on device buffers the caller owns and with no
 * cudaMalloc / cudaFree / allocating library call: the scratch it needs (the
 * AND masks of the set list's row tiles) is a static device array of the
 * library, sized for SW_NOALLOC_MAX_SETS sets (about 1 MB; every GPU that
 * loads the library keeps it until the process exits).  Larger set lists are
 * rejected with SW_ERR_CAPACITY.
 *
 * Rows use the device layout: W = ceil(n / 64) uint64 words (1 to 8); state
 * q is bit (63 - q % 64) of word q / 64; unused bits are 0.  d_sets must be
 * 16-byte aligned (its row tiles move as 16-byte loads), d_checks 8-byte and
 * d_results 4-byte aligned; other pointers are rejected with
 * SW_ERR_INVALID_ARGUMENT before any work is queued.
 * d_results[i] (uint32) becomes 1 if some d_sets row ⊆ d_checks row i
 * (⊊ when proper), else 0.  The work is queued on `stream` (NULL = default
 * stream); the call returns without waiting for it.  The first call on a
 * device looks up the scratch array's device address with that device
 * current; make that first call before any stream capture.  All calls share
 * the one scratch array and each overwrites it: calls that can run at the
 * same time on the GPU race and must be ordered by the caller.  Errors are
 * reported like every other entry point (status code + sw_last_error()). */
#define SW_NOALLOC_MAX_SETS (1u << 20)
int sw_subsets_check_device_noalloc(uint32_t n, const uint64_t* d_sets, uint64_t set_count, const uint64_t* d_checks,
                                    uint64_t check_count, int32_t proper, uint32_t* d_results, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SYNCHROWORDS_H */
