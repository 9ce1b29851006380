/* ORACLE — test infrastructure, not product.
 *
 * C interface of the CPU restatement of SynchroLib's Exact and Beam
 * algorithms (oracle/oracle.cpp).  Only tests, the smoke check and bench.py's
 * CPU-baseline leg load it.  Parameters are the evaluated values of the
 * reference's per-algorithm defines (algorithm/exact/config.hpp:24-46,
 * algorithm/beam/config.hpp:23-44, app/jit.hpp:112-141).
 */
#ifndef SYNCHRO_ORACLE_H
#define SYNCHRO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* AlgoResult bounds (algorithm.hpp:19-42), in/out. */
typedef struct {
  int32_t non_synchro;
  uint64_t lower;
  uint64_t upper;
} oracle_bounds;

typedef struct {
  int32_t dfs;                 /* DFS */
  int32_t dfs_shortcut;        /* DFS_SHORTCUT */
  int32_t strict_memory_limit; /* STRICT_MEMORY_LIMIT */
  uint64_t max_memory_mb;      /* MAX_MEMORY */
  uint64_t dfs_min_list_size;  /* DFS_MIN_LIST_SIZE */
  uint64_t bfs_small_list_size;/* BFS_SMALL_LIST_SIZE */
  uint32_t threads;            /* THREADS */
} oracle_exact_params;

typedef struct {
  uint64_t beam_size;     /* BEAM_SIZE */
  int32_t dynamic;        /* DYNAMIC */
  uint64_t min_beam_size; /* MIN_BEAM_SIZE */
  uint64_t max_beam_size; /* MAX_BEAM_SIZE */
  double beam_exact_ratio;/* BEAM_EXACT_RATIO */
  int64_t max_iter;       /* MAX_ITER */
  int32_t presort_indeg;  /* PRESORT_INDEG */
} oracle_beam_params;

/* One meet-in-the-middle step as the reference logs it at VERBOSE level
 * (meet_in_the_middle.cpp:121-126, 157-162): phase 0 = BFS, 1 = IBFS,
 * 2 = entering DFS (list_bfs = trie sets, list_invbfs = initial list),
 * 3 = DFS found a word of length `len`. */
typedef struct {
  int32_t phase;
  int32_t novisited;
  uint64_t len;
  uint64_t list_bfs;
  uint64_t list_invbfs;
} oracle_trace_step;

typedef struct {
  oracle_trace_step* steps;
  uint64_t capacity;
  uint64_t count;
} oracle_trace;

int oracle_exact(const uint32_t* delta, uint32_t n, uint32_t k, const oracle_exact_params* p,
                 oracle_bounds* r, oracle_trace* trace);
int oracle_beam(const uint32_t* delta, uint32_t n, uint32_t k, const oracle_beam_params* p,
                oracle_bounds* r);
int oracle_brute(const uint32_t* delta, uint32_t n, uint32_t k, int64_t* out);
/* Eppstein greedy bound (eppstein.hpp:82-114); `r` in/out, word optional. */
int oracle_eppstein(const uint32_t* delta, uint32_t n, uint32_t k, oracle_bounds* r, uint32_t* word,
                    uint64_t word_cap, uint64_t* word_len);

#ifdef __cplusplus
}
#endif
#endif
