// Device parts of the reference's small algorithms: the Eppstein greedy upper
// bound (pairs.cu) and the power-set BFS `Brute` (brute.cu).  Launchers are
// asynchronous on the given stream; scratch comes from the caller.
#pragma once
#include "common.cuh"
#include "kernels.cuh"

namespace sw {

// ---- Eppstein (synchrolib/algorithm/eppstein/eppstein.hpp:82-114 over the
// pairs tree of synchrolib/data_structures/pairs_tree.hpp:25-62) ----------

// Result words written by launch_eppstein into `out` (u32[8]).
enum EppsteinStatus : u32 {
  kEppFound = 0,       // out[1..2] = length (lo, hi), out[3] = letters written
  kEppOverBound = 1,   // the greedy word grew past `upper` (eppstein.hpp:104-106)
  kEppNonSynchro = 2,  // some pair never reaches the diagonal (pairs_tree.hpp:95-100)
  kEppWordCapacity = 3,
};

size_t eppstein_scratch_bytes(int n);

// One block: breadth-first pair tree (per pair {p, q} the length of the
// shortest word merging it and that word's first letter, the same first
// letter the reference's queue order records), then the greedy walk that
// repeatedly merges the closest pair of the current image.  Letters go to
// `word` (capacity `word_cap`).
void launch_eppstein(const TransTables& t, u64 upper, void* scratch, u32* out, uint8_t* word, u64 word_cap,
                     cudaStream_t s);

// ---- Brute (synchrolib/algorithm/brute/brute.hpp:88-122), n <= 32 --------

// Bitmap of visited subsets: 2^n bits.
size_t brute_visited_bytes(int n);

// One BFS level: every image of every frontier mask under every letter that
// was not visited yet is marked and appended to `next` (next_count[0] counts,
// capped at next_cap: the excess is counted but not stored).  found[0] = 1 and
// found[1] = the mask when a singleton is produced.
void launch_brute_level(const uint16_t* delta, int n, int k, const u32* frontier, u32 count, u32* visited,
                        u32* next, u32 next_cap, u32* next_count, u32* found, cudaStream_t s);

// Word back-tracking: best[0] = min over (i, a) with image(level[i], a) ==
// target of i * k + a (caller initialises best[0] to ~0).
void launch_brute_parent(const uint16_t* delta, int n, int k, const u32* level, u32 count, u32 target, u64* best,
                         cudaStream_t s);

// ---- Batched exact search for small automata (batch_small.cu) -----------

// One automaton of a batch: n <= 64 W states, k <= 4 letters; delta[q*k + a]
// (u8) at delta_off of the delta pool, its backward seeds (ascending) at
// seed_off of the seed pool; lengths 1..max_len are searched.
struct SmallInstance {
  u32 n, k, delta_off, seed_off, seed_count, max_len;
};
// status 0: found, length and word_len letters at words + i * word_stride;
// 1: lists outgrew the shared-memory capacities (solve it another way);
// 2: no meeting pair within max_len.
// status: 0 solved, 1 over a capacity, 2 no meeting within max_len.
// why (status 1): bits 0-7 the capacity (1 children, 2 layer, 3 visited,
// 4 depth, 5 word buffer), bits 8+ the layers searched when it stopped.
struct SmallResult {
  u32 status, length, word_len, why;
};

int small_batch_blocks();
// Raises the shared-memory limits of the batched kernels on the current
// device (done before a launch is captured into a CUDA graph).
void small_batch_prepare();
size_t small_batch_origin_words(int W, u32 blocks);
size_t small_batch_visited_words(int W, u32 blocks);
// One persistent launch of `blocks` blocks over `count` automata of set width
// W (1 to 4 words, n <= 64 W); origins, visited and counter are scratch.
void launch_small_batch(int W, const SmallInstance* inst, u32 count, const uint8_t* delta_pool,
                        const uint8_t* seed_pool, SmallResult* results, uint8_t* words, u32 word_stride, u32* origins,
                        u64* visited, u32 blocks, u32* counter, cudaStream_t s);

// Device-resident search on thread-block clusters (batch_cluster.cu): one
// cluster of `cs` CTAs per automaton (n <= 256, n * k <= 4096), lists in a
// per-cluster global region.  Same instances and results as the small batch;
// status 1 may also report why 6 (a hash-table probe ran out).
struct ClusterCaps {
  u32 vis = 0;        // visited rows per side (every layer of the side, in order)
  u32 ch = 0;         // children of one step
  u32 vtab_bits = 0;  // log2 slots of a side's visited table (>= 2 * vis)
  u32 ltab_bits = 0;  // log2 slots of the step's child table (>= 2 * ch)
};
ClusterCaps cluster_default_caps();
// Bytes of scratch for `clusters` clusters.  It must be zero-filled before its
// first launch, and again before the tags the launches take from its counter
// (cluster_tags_per_launch) could wrap around 2^32.
size_t cluster_scratch_bytes(u32 clusters, const ClusterCaps& c);
u32 cluster_max_clusters_supported();
// Clusters of `cs` CTAs that fit on the current device at once.
u32 cluster_batch_max_clusters(int W, int cs);
// Tags a launch of `count` automata can take: one per search, one per step.
constexpr u64 cluster_tags_per_launch(u32 count) { return (u64)count * (2 + 2 * 1024); }
void launch_cluster_batch(int W, int cs, u32 clusters, const SmallInstance* inst, u32 count,
                          const uint8_t* delta_pool, const uint8_t* seed_pool, SmallResult* results, uint8_t* words,
                          u32 word_stride, void* scratch, const ClusterCaps& caps, u32* counter, u64* stats,
                          cudaStream_t s);

}  // namespace sw
