/**
 *  @file launchers.h
 *  @brief Host-side launch entry points of the engine's kernels, one translation unit per kernel family so the
 *         template instantiations compile in parallel.
 */
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

cudaError_t launch_plan(plan_args_t const &args, plan_bins_t *bins, pair_task_t *tasks, std::int64_t *results,
                        int sm_count, cudaStream_t stream);
/** Marks the bytes of both tapes and assigns dense codes (`alphabet->code`, `symbols`, `bits`, `present`), on the
 *  device. With `sample_bytes` > 0 only the first `sample_bytes` of each tape's data are marked: a guess of the
 *  alphabet that the kernels reading it must verify. The alphabet's mark words must be zero on entry (they start
 *  zeroed and the code pass clears them again). */
cudaError_t launch_alphabet(tape_t const &queries, tape_t const &candidates, bool has_candidates,
                            batch_alphabet_t *alphabet, int sm_count, cudaStream_t stream,
                            std::uint64_t sample_bytes = 0);
/** Unit-cost Levenshtein over a cross product (`args.mode == mode_cross_k`) straight into `out` (row stride in
 *  elements), one thread per cell; sets `*flag` to 1 if a string has more than 64 bytes (its cells are then not
 *  written). */
cudaError_t launch_myers_direct(plan_args_t const &args, std::int64_t *out, std::uint64_t stride,
                                std::uint32_t *flag, int sm_count, cudaStream_t stream);
cudaError_t launch_scatter_output(plan_args_t const &args, std::int64_t const *results, std::int64_t *out,
                                  std::uint64_t stride, int sm_count, cudaStream_t stream);

/** One Min-Hash dimension: modulus m (2^42 < m < 2^43), multiplier a (< 640), D = -a^w mod m, the quotient
 *  estimate's constant mu = floor(2^74 / m) (< 2^32), window width w. */
struct fingerprint_dim_t {
    std::uint64_t modulo, discard;
    std::uint32_t multiplier, mu, width, reserved;
};
/** The reference's parameters of dimension @p dim for a window of @p width bytes and a reproducibility @p seed. */
fingerprint_dim_t fingerprint_dimension(std::uint64_t dim, std::uint64_t width, std::uint64_t seed);
/** Min-Hash fingerprints of every text: rows `hashes_stride` / `counts_stride` bytes apart, `dimensions` columns. */
cudaError_t launch_fingerprints(tape_t const &texts, fingerprint_dim_t const *params, std::uint32_t dimensions,
                                std::uint32_t *hashes, std::uint64_t hashes_stride, std::uint32_t *counts,
                                std::uint64_t counts_stride, int sm_count, cudaStream_t stream);

/** The set of a batch's code points (UTF-8 Levenshtein) as a bitmap over every value the decoder can produce (lead
 *  bytes give at most 21 bits), and the rank of each bitmap word: a code point's code is the number of distinct code
 *  points below it. */
constexpr int rune_bits_k = 21;
constexpr std::uint32_t rune_words_k = (1u << rune_bits_k) / 32; // 65,536 words of 32 code points
struct rune_set_t {
    std::uint32_t present[rune_words_k]; // bit (r & 31) of word r >> 5: code point r occurs in the batch
    std::uint32_t rank[rune_words_k];    // distinct code points below word w's first
    std::uint32_t symbols;               // distinct code points
    std::uint32_t overflow;              // always 0: every decodable value has its bit
};
/** Counts each string's code points into `counts[i]` and marks them in `set` (both zeroed by the caller);
 *  `end` is the tape's last offset: a sequence cut off there reads zeros beyond it. */
cudaError_t launch_utf8_count(tape_t const &tape, std::uint64_t end, std::uint64_t *counts, rune_set_t *set,
                              int sm_count, cudaStream_t stream);
/** Ranks the set's bitmap words and counts the distinct code points (one CTA). */
cudaError_t launch_utf8_codes(rune_set_t *set, cudaStream_t stream);
/** Device scratch the exclusive scan of `count + 1` counts needs. */
std::size_t utf8_scan_scratch_bytes(std::uint64_t count);
/** `offsets[0..count]` = exclusive scan of `counts[0..count]` (counts[count] must be 0). */
cudaError_t launch_utf8_scan(std::uint64_t const *counts, std::uint64_t *offsets, std::uint64_t count, void *scratch,
                             std::size_t scratch_bytes, cudaStream_t stream);
/** Writes each string's codes at `out + offsets[i]` (in codes): one byte each, or 16 bits each when `wide`. */
cudaError_t launch_utf8_write(tape_t const &tape, std::uint64_t end, std::uint64_t const *offsets,
                              rune_set_t const *set, void *out, bool wide, int sm_count, cudaStream_t stream);

/** Shape of a wavefront-DP launch for one engine configuration. */
struct dp_launch_shape_t {
    int threads_per_cta;
    int warps_per_cta;
    int shared_bytes;
    int ctas_per_sm; // from the occupancy calculator
    int rows_per_lane;
    int group_ctas_per_sm = 0; // band kernels: the same for the grouped (several CTAs per pair) kernel
};

/** Launch shape of the wavefront kernel for (kind, affine, cell bits, classes); ctas_per_sm = 0 if unsupported.
 *  `direct`: the direct-table instance (costs from a dense 256 x 256 table in shared memory). */
dp_launch_shape_t dp_shape(int kind, bool affine, int cell_bits, int classes, bool direct = false, bool wide = false);

/** Runs the wavefront kernel over bins [key_begin, key_end). `scratch` holds `ctas * warps_per_cta` rows of
 *  `scratch_cells_per_warp` cells of `cell_bits` bits. Costs with a `direct_table` run the direct-table instance;
 *  `wide`: strings of 16-bit codes (Levenshtein). */
cudaError_t launch_dp(int kind, bool affine, int cell_bits, int key_begin, int key_end, pair_task_t const *tasks,
                      plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                      std::size_t scratch_cells_per_warp, int ctas, cudaStream_t stream, bool wide = false);

/** Launch shape of the 16x2 packed wavefront kernel with `rows` (4, 8, 12, 16) rows per lane and `warps` (1..8)
 *  warps per CTA; ctas_per_sm = 0 if unsupported. `compare` (a `compare_mode_t`, dp_packed.cuh): the Levenshtein
 *  instances that compare codes instead of reading a profile (batches over more than 32 byte values). */
dp_launch_shape_t dp16_shape(int kind, bool affine, int rows, int classes, int warps, int compare = 0,
                             bool wide = false);

/** Runs the 16x2 packed wavefront kernel over bins [key_begin, key_end): two scheduled pairs per warp. `scratch`
 *  holds `ctas * warps_per_cta` rows of `scratch_cells_per_warp` 32-bit words. */
cudaError_t launch_dp16(int kind, bool affine, int rows, int key_begin, int key_end, pair_task_t const *tasks,
                        plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                        std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream,
                        int compare = 0, bool wide = false);

/** The compare-mode halves of `dp16_shape` and `launch_dp16` (Levenshtein only; `wide`: strings of 16-bit codes),
 *  built in their own translation unit. */
dp_launch_shape_t dp16_compare_shape(bool affine, int rows, int classes, int warps, int compare, bool wide);
cudaError_t launch_dp16_compare(bool affine, int rows, int key_begin, int key_end, pair_task_t const *tasks,
                                plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                                std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream,
                                int compare, bool wide);

/** Launch shape of the band kernel (one CTA of several warps per long pair, 32-bit cells); `direct`: the
 *  direct-table instance; `rows_per_lane` 8 (strips of 256 rows) or 4 (128 rows: for groups of CTAs per pair). */
dp_launch_shape_t band_shape(int kind, bool affine, int classes, bool direct = false, bool wide = false,
                             int rows_per_lane = 8);
/** Warps per band CTA (ring slots per CTA). */
int band_warps_per_cta();

/** Runs the band kernel over bins [key_begin, key_end). `scratch` holds `ctas * band_warps_per_cta()` ring slots of
 *  `ring_cells_per_slot` 32-bit cells. Bounded waits that give up set bit 0 of `bins->error_flags`. With
 *  `group_states` (one zeroed `band_group_state_bytes()` record per group) the grouped kernel runs instead: a
 *  cooperative launch of `ctas` CTAs in groups of `group_ctas`, each group sharing one pair at a time. */
cudaError_t launch_band(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                        score_costs_t const &costs, std::int64_t *results, void *scratch,
                        std::size_t ring_cells_per_slot, int ctas, cudaStream_t stream, void *group_states = nullptr,
                        int group_ctas = 1, bool wide = false, // costs with a `direct_table` run the direct-table
                        int rows_per_lane = 8);                // instance; `wide`: 16-bit codes
/** Bytes of one group's state record, and the most CTAs a group may have. */
std::size_t band_group_state_bytes();
int band_group_max_ctas();

/** Launch shape of the 16-bit band kernel (one CTA per long pair, two row strips per warp in 16x2 cells);
 *  `compare` (a `compare_mode_t`): the Levenshtein instances that compare codes instead of reading a profile;
 *  `rows_per_lane` 8 (512-row super-strips) or 4 (256 rows: for groups of CTAs per pair). */
dp_launch_shape_t band16_shape(int kind, bool affine, int classes, int compare = 0, bool wide = false,
                               int rows_per_lane = 8);

/** Runs the 16-bit band kernel over bins [key_begin, key_end). `scratch` holds `ctas * band_warps_per_cta()` ring
 *  slots of `ring_words_per_slot` 32-bit words (twice that for local scores, which may rescore a pair on 32-bit
 *  cells). Bounded waits that give up set bit 0 of `bins->error_flags`. */
cudaError_t launch_band16(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks,
                          plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                          std::size_t ring_words_per_slot, int ctas, cudaStream_t stream, void *group_states = nullptr,
                          int group_ctas = 1, int compare = 0, bool wide = false, int rows_per_lane = 8);

/** Short pairs (shorter side at most 128) on the segmented 16x2 kernel: `shape` 0-6 for shorter sides up to 16, 32,
 *  64, 128, 24, 48, 96 (`short_segment_rows`); shapes 4-6 have 12 rows per lane, shapes 0-3 16 when compare mode or
 *  at most 8 classes, else 8 (`short_rows_for`); `compare` as for the 16x2 wavefront (Levenshtein only). */
int short_rows_for(int classes, int compare, int shape);
int short_segment_rows(int shape);
dp_launch_shape_t short_shape(int kind, bool affine, int shape, int classes, int warps, int compare = 0);
cudaError_t launch_short(int kind, bool affine, int shape, int key_begin, int key_end, pair_task_t const *tasks,
                         plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, int ctas, int warps,
                         cudaStream_t stream, int compare = 0);

/** Very long unit-cost pairs on chains of warps (myers_chain.cuh): one cooperative launch scores pairs
 *  [first, first + pairs) of bin `key` with `words` (1, 2, 4) words per lane and `planes` code planes, each pair on
 *  `strips_per_pair` warps (1,024 x words rows each) and its share of `scratch`
 *  (`myers_chain_scratch_bytes(strips_per_pair, link_stride, pairs)` bytes in all; `link_stride` at least the
 *  longest text). 8 warps per CTA; the launch clears the state it needs. */
std::uint64_t myers_chain_scratch_bytes(std::uint32_t strips_per_pair, std::uint64_t link_stride, std::uint32_t pairs);
int myers_chain_ctas_per_sm(int words, int planes);
cudaError_t launch_myers_chain(int words, int planes, pair_task_t const *tasks, plan_bins_t *bins, int key,
                               std::uint32_t first, std::uint32_t pairs, std::uint32_t strips_per_pair,
                               batch_alphabet_t const *alphabet, std::int64_t *results, void *scratch,
                               std::uint64_t link_stride, std::uint32_t wait_polls, cudaStream_t stream);

/** Bit-parallel kernels over strings of 16-bit codes (UTF-8 calls over more than 256 code points, 16 code planes):
 *  thread per pair over the bins of `words` words (1..8), and warp per pair over the warp bins (1..8 words per
 *  lane). */
cudaError_t launch_myers_wide(int words, bool exact, pair_task_t const *tasks, plan_bins_t const *bins, int key_begin,
                              int key_end, std::int64_t *results, int ctas, cudaStream_t stream);
cudaError_t launch_myers_warp_wide(int words, pair_task_t const *tasks, plan_bins_t *bins, int key_begin, int key_end,
                                   std::int64_t *results, int ctas, cudaStream_t stream);

/** Runs the bit-parallel kernel over bins [key_begin, key_end) with `words` words (1..16) and `planes` code planes
 *  (2, 3, 5 or 8). `exact` = every pair in the bins needs exactly `words` words (the binned schedule); otherwise
 *  pairs may be shorter (the plain schedule puts every bit-parallel pair in one bin and launches the word count of
 *  the batch's longest pattern). */
cudaError_t launch_myers(int words, int planes, bool exact, pair_task_t const *tasks, plan_bins_t const *bins,
                         int key_begin, int key_end, batch_alphabet_t const *alphabet, std::int64_t *results, int ctas,
                         cudaStream_t stream);
int myers_threads_per_cta();
/** The shared-table bit-parallel kernel for batches over at most four symbol codes: bins [key_begin, key_end),
 *  patterns of at most 32 x `words` rows (1..16). A pair holding a byte outside `alphabet->present` sets bit 1 of
 *  `bins->error_flags` (its score is then not valid). */
cudaError_t launch_myers_table(int words, int key_begin, int key_end, pair_task_t const *tasks,
                               plan_bins_t *bins, batch_alphabet_t const *alphabet, std::int64_t *results,
                               int ctas, cudaStream_t stream);
/** Planes actually instantiated for a requested minimum. */
int myers_planes_for(int bits_needed);

} // namespace szs_gb300
