// Launchers for the device kernels of the exact search (kernels.cu).
//
// Every launcher is asynchronous on the given stream; scratch buffers come
// from the caller (no allocation inside).  Kernel roles and the reference
// functions they replace:
//   expand        PreprocessedTransition::apply
//                 (synchrolib/data_structures/preprocessed_transitions.cpp:56-93,
//                  cuda/preprocessed_transition_kernel.cu:19-88)
//   radix sort +  sort_keep_unique (synchrolib/utils/vector.hpp:13-27)
//   unique
//   subset check  SubsetsImplicitTrie::check_contains_subset / reduce
//   (subset_      (synchrolib/data_structures/subsets_implicit_trie.hpp:29-266,
//   check.cu)      cuda/subsets_implicit_trie_kernel.cu:13-92) and
//                 SubsetsTrie::contains_subset_of (subsets_trie.hpp:78-90)
#pragma once
#include "common.cuh"

namespace sw {

// Per-letter transition tables as staged into shared memory by `expand`.
// Layout (all u16): delta[a*n + q]; inv_beg[a*(n+1) + t] ..inv_beg[..+1] index
// inv_src[a*n + e] (CSR of preimages).
struct TransTables {
  const uint16_t* delta = nullptr;   // k*n
  const uint16_t* inv_beg = nullptr; // k*(n+1)
  const uint16_t* inv_src = nullptr; // k*n
  int n = 0, k = 0;
};

// Sort key of a side: the 64 states whose pattern leads the key (identity =
// states 0..63, i.e. word 0 of the row).
struct KeyMap {
  uint16_t q[64];
  int identity = 1;
};

// out[(a*m + i)] = image (kImage) or preimage of in[i] under letter a.  With
// keys (and vals) given, each child o = a*m + i also gets its layer key
// keys[2o..2o+1] (as launch_layer_keys with `map`) and vals[o] = o.
void launch_expand(int W, bool image, const u64* in, u32 m, const TransTables& t, u64* out, cudaStream_t s,
                   u64* keys = nullptr, u32* vals = nullptr, const KeyMap& map = KeyMap{});

// Scratch sizing for the sort / scan helpers.
size_t scan_temp_bytes(u32 n);
size_t sort_temp_bytes(int R, u32 m);

// Exclusive prefix sum of in[0..n) into out; *total_dev receives the sum.
void launch_scan(const u32* in, u32* out, u32 n, u32* total_dev, void* temp, cudaStream_t s);

// Stable sort of m rows of R words (word 0 most significant) with a u32
// payload.  Result lands in (keys, vals); (keys_alt, vals_alt) are scratch of
// the same size.  Up to 2^20 rows: 2048-row chunks sorted in shared memory,
// then pairwise merges; beyond: LSD radix passes over 8-bit digits, digits
// constant over all rows skipped.  Returns the number of kernels launched;
// *data_passes (optional) = full read+write passes over the rows.
int radix_sort_rows(int R, u64* keys, u32* vals, u64* keys_alt, u32* vals_alt, u32 m, void* temp,
                     cudaStream_t s, int* data_passes = nullptr);

// flags[i] = 1 if row i differs from row i-1 (rows sorted).
void launch_unique_flags(int W, const u64* rows, u32 m, u32* flags, cudaStream_t s);

// Stream compaction of rows (+ optional payload) by flags; pos = exclusive scan of flags.
void launch_compact(int W, const u64* rows, const u32* vals, const u32* flags, const u32* pos, u32 m, u64* out_rows,
                    u32* out_vals, cudaStream_t s);

enum QueryMode : int {
  kQuerySubset = 0,        // hit(c) = exists s in S, s ⊆ c
  kQueryProperSubset = 1,  // hit(c) = exists s in S, s ⊊ c
  kQueryDisjoint = 2,      // hit(c) = exists s in S, s ∩ c = ∅  (s ⊆ ~c)
};

// Tiled subset check (subset_check.cu): for each query row c, flags[c] |=
// hit(c) (or, with `stop`, record one witness pair and let all warps exit
// early: witness[0] = found flag, witness[1] = query index, witness[2] = set
// index).  S is cut into tiles of sh.tile_rows rows; tile_and[t] (W words) =
// AND of the tile's rows, then one mask per super-tile of
// sh.tiles_per_super tiles, from launch_tile_and with the same shape.  `flags` must start zeroed (non-stop
// mode).  `bytes_ctr` (optional) accumulates the bytes of S tiles staged on
// chip.  S must start 16-byte aligned (its tiles move by bulk copies).  *err
// is set to 1 when a wait for a tile copy runs out (its bounded poll limit);
// the results of that launch are then incomplete.
// Launch shape of the subset check: rows of S per staged tile (32, 64, 128),
// warps of 32 queries per block (4, 8, 16), tiles per super-tile mask (4, 8,
// 16, 32) and the grid's target blocks per SM (1..64), which sets how finely
// S is chunked over blockIdx.y.  Results do not depend on it.
struct ScanShape {
  int tile_rows = 64;
  int warps = 8;
  int tiles_per_super = 16;
  int grid_factor = 16;
};
// Shapes per row width W (1..8) and list size class: class 0 for lists S of
// fewer than kScanLargeRows rows, class 1 for larger ones.
constexpr int kScanSizeClasses = 2;
constexpr u32 kScanLargeRows = 1u << 15;
constexpr size_t kMaxScanSmem = 200 * 1024;
struct ScanShapes {
  ScanShape s[8][kScanSizeClasses];
  const ScanShape& pick(int W, u32 m) const { return s[W - 1][m >= kScanLargeRows ? 1 : 0]; }
};
bool scan_shape_valid(int W, const ScanShape& sh);
size_t scan_smem_bytes(int W, const ScanShape& sh);
size_t subset_check_temp_bytes(int W, u32 m, const ScanShape& sh);
void launch_tile_and(int W, const u64* S, u32 m, u64* tile_and, const ScanShape& sh, cudaStream_t s);
void launch_subset_check(int W, int mode, const u64* S, u32 m, const u64* tile_and, const u64* Q, u32 q, int n,
                         u32* flags, u32* witness, bool stop, const ScanShape& sh, cudaStream_t s, u64* bytes_ctr,
                         u32* err);

// out = sorted merge of two sorted, mutually disjoint row arrays.
void launch_merge(int W, const u64* A, u32 na, const u64* B, u32 nb, u64* out, cudaStream_t s);

// rows[i] = complement of rows[i] within n states.
void launch_complement(int W, u64* rows, u32 m, int n, cudaStream_t s);

// out[i] = popcount of row i.
void launch_popcount(int W, const u64* rows, u32 m, u32* out, cudaStream_t s);

// flags[i] = AND/OR combine: out[i] = (a[i] == 0 && b[i] == 0).
void launch_keep_flags(const u32* a, const u32* b, u32 m, u32* out, cudaStream_t s);

// Layer keys keys[2i..2i+1] = (the map's 64 states of row i packed MSB-first,
// 32-bit mix of the row in the high half): sort order of a layer and of the
// visited list of one side.
void launch_layer_keys(int W, const u64* rows, u32 m, u64* keys, cudaStream_t s, const KeyMap& map = KeyMap{});
// Merge of two row arrays sorted by the same layer key.
void launch_merge_key(int W, const u64* A, u32 na, const u64* B, u32 nb, u64* out, cudaStream_t s,
                      const KeyMap& map = KeyMap{});
// flags[i] = 1 if row i of C equals a row of V (flags untouched otherwise);
// V and C sorted by the same layer key.
// Duplicate removal of a key-sorted layer and compaction in one launch
// (decoupled look-back over tiles): child vals[i] of C is kept when it
// differs from child vals[i-1] and equals no row of the key-sorted visited
// list V (keys = the children's sorted layer keys); out_rows / out_vals
// receive the kept children in sort order, *total their count.  `status`
// holds dedup_compact_status_words(m) words (zero-filled when first
// allocated), `ctr` one word that is zero before the first launch (each
// launch leaves it zero); `epoch` is 1..2^30-1 and must differ from the
// previous launch's on the same status array.  *err is set to 2 if a bounded
// wait ran out.
size_t dedup_compact_status_words(u32 m);
void launch_dedup_compact(int W, const u64* C, const u32* vals, const u64* keys, u32 m, const u64* V, u32 nv,
                          const KeyMap& map, u64* out_rows, u32* out_vals, u32* total, u64* status, u32* ctr,
                          u32 epoch, u32* err, cudaStream_t s);
void launch_member_key(int W, const u64* V, u32 nv, const u64* C, u32 nc, u32* flags, cudaStream_t s,
                       const KeyMap& map = KeyMap{});
// flags[i] = 0 where flags[i] = 1 and row i of C equals a row of V (same
// layer-key order as launch_member_key).
void launch_clear_members(int W, const u64* V, u32 nv, const u64* C, u32 nc, u32* flags, cudaStream_t s,
                          const KeyMap& map = KeyMap{});
// counts[q] += rows containing state q (counts: 64*W entries, caller-zeroed).
void launch_state_counts(int W, const u64* rows, u32 m, u32* counts, cudaStream_t s);

// p[i] = i.
void launch_iota(u32* p, u32 m, cudaStream_t s);

// dst[i] = src[idx[i]] (rows of W words).
void launch_gather_rows(int W, const u64* src, const u32* idx, u32 m, u64* dst, cudaStream_t s);

// Beam sort keys: keys[i] = [n - |row i|, bit-reversed words of row i] (R words).
void launch_beam_keys(int W, const u64* rows, u32 m, int n, int R, u64* keys, cudaStream_t s);

// dst[i] = src[idx[i]] (u32 payloads).
void launch_gather_u32(const u32* src, const u32* idx, u32 m, u32* dst, cudaStream_t s);

// Ascending sort keys of beam candidates: keys[i] = primary << 32 | i with
// primary = the order-preserving bits of score[i] (counts null), counts[i]
// (score null), or counts[i] << 16 | leading 16 bits of score[i] (both).
void launch_score_keys(const float* score, const u32* counts, u32 m, u64* keys, cudaStream_t s);

// Fill u32 array with a value.
void launch_fill_u32(u32* p, u32 value, u32 m, cudaStream_t s);

}  // namespace sw
