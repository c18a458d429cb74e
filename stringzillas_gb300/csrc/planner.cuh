/**
 *  @file planner.cuh
 *  @brief Device-side planning of one batch: enumerate the pairs of a call, answer the trivial ones, choose a
 *         route and a length bin for the rest, and counting-sort them into bins.
 *
 *  The reference does this with a materialisation kernel, a min/max probe, a histogram, a scan and a scatter,
 *  syncing the host between stages (include/stringzillas/similarities/cuda.cuh:1583-1747, :1859-1914). Here the
 *  whole plan stays on the device: three kernels, no host round trip until the launch list is read back, and
 *  bins are ordered so persistent kernels meet the longest pairs first (longest-processing-time order).
 *
 *  Bin keys:
 *    [0, 272)    Myers: key = words * 16 + text-length class (words 1..16)
 *    [272, 304)  32-bit wavefront DP: key = 272 + (31 - size class), size class ~ log2(n * m)
 *    [304, 336)  64-bit wavefront DP: same layout
 *    [336, 1360) 16x2 packed wavefront DP: key = 336 + 256 * rows-per-lane index + 8 * (31 - n class)
 *                + (7 - ratio class), n class = 4 log2(n) - 12 (quarter octaves of the shorter side), ratio class
 *                = 2 log2(m / n); rows per lane R in {4, 8, 12, 16}, chosen per pair. A warp scores two consecutive
 *                pairs of a bin at once and pays for the larger of each dimension, so bins are narrow in both.
 *    [1360, 1392) band (one CTA per pair, 32-bit cells): key = 1360 + (31 - size class), size class ~ log2(n * m)
 *    [1392, 1424) 16-bit band (one CTA per pair, 16x2 cells): same layout from 1392
 *    [1424, 1488) warp-per-pair Myers (unit Levenshtein, shorter side 513..8,192): key = 1424 + 8 * (8 - W)
 *                 + (7 - text class), W = words per lane = ceil(n / 1024), text class ~ log2(m) - 9
 *    [1488, 1824) short pairs on 16x2 cells (shorter side <= 128): key = 1488 + 48 * shape + (47 - m class),
 *                 shape 0/4/1/5/2/6/3 for n <= 16/24/32/48/64/96/128, m class = m / 16 below 512, then
 *                 32 + log2(m) - 9
 *    1824         unit-cost Levenshtein beyond the warp kernel (shorter side 8,193 .. 2^20): a chain of warps per pair
 */
#pragma once
#include "engine_types.cuh"

namespace szs_gb300 {

constexpr int bin_keys_k = 2048;
constexpr int bin_myers_begin_k = 0;
constexpr int bin_dp32_begin_k = 272;
constexpr int bin_dp64_begin_k = 304;
constexpr int bin_dp16_begin_k = 336;
constexpr int bin_dp_classes_k = 32;
constexpr int bin_dp16_classes_k = 1024;
constexpr int dp16_row_choices_k = 4;       // rows per lane 4, 8, 12, 16
constexpr int dp16_classes_per_rows_k = 256; // shape classes within one rows-per-lane choice (32 n x 8 ratio)
constexpr int bin_band_begin_k = bin_dp16_begin_k + bin_dp16_classes_k; // 1360
constexpr int bin_band16_begin_k = bin_band_begin_k + bin_dp_classes_k;  // 1392
static_assert(bin_band16_begin_k + bin_dp_classes_k <= bin_keys_k, "bin layout exceeds the key space");
static_assert(bin_keys_k % 2 == 0 && bin_keys_k / 2 <= 1024, "the scan kernel uses one CTA of bin_keys_k / 2 threads");
constexpr int band_min_rows_k = 1024;        // default: 32-bit pairs whose shorter side exceeds this take a whole CTA
/** Built-in relative costs of one lane step of the 16x2 route with 4, 8, 12, 16 rows per lane, measured on GB300
 *  (affine protein alignment, shorter sides 128-1,023). */
constexpr int packed_step_cost_k[4] = {100, 165, 245, 330};
constexpr int band_min_rows_packed_k = 2048; // default for pairs that fit 16-bit cells (the 16-bit band above it)
constexpr int band_min_rows_few_k = 1024;    // default for calls with fewer pairs than one 16x2 wave (32 per SM)
constexpr int band_min_rows_compare_k = 2048; // default for compare-mode Levenshtein pairs on 16-bit cells
constexpr int myers_max_words_k = 16;
constexpr int myers_wide_max_words_k = 8; // 16-bit codes take 16 code planes: the thread route stops at 8 words
// Words per lane of the warp kernel: patterns up to 32 * 32 * 8 = 8,192 rows. Longer ones take the bands: a pair of
// 8-16k characters keeps one warp busy for milliseconds, and a call rarely has enough of them to fill the GPU.
constexpr int myers_warp_max_words_k = 8;
constexpr int myers_warp_classes_k = 8;    // text-length classes per words count (longest first)
constexpr int bin_myers_warp_begin_k = bin_band16_begin_k + bin_dp_classes_k; // 1424
static_assert(bin_myers_warp_begin_k + myers_warp_max_words_k * myers_warp_classes_k <= bin_keys_k,
              "bin layout exceeds the key space");
constexpr int bin_short_begin_k = bin_myers_warp_begin_k + myers_warp_max_words_k * myers_warp_classes_k; // 1488
constexpr int short_shapes_k = 7;      // segments holding 16, 32, 64, 128, then 24, 48 and 96 rows
constexpr int short_m_classes_k = 48;  // text-length classes per shape
constexpr int short_max_rows_k = 128;  // default: shorter sides up to this take the short route
static_assert(bin_short_begin_k + short_shapes_k * short_m_classes_k <= bin_keys_k, "bin layout exceeds the key space");
constexpr int bin_myers_chain_k = bin_short_begin_k + short_shapes_k * short_m_classes_k; // 1824
static_assert(bin_myers_chain_k < bin_keys_k, "bin layout exceeds the key space");
constexpr std::uint32_t myers_chain_max_rows_k = 1u << 20; // longest pattern a chain of warps takes

/** Which pairs a call scores. */
enum pair_mode_t : int {
    mode_pairwise_k = 0,  // (i, i)
    mode_cross_k = 1,     // (q, c) for all q, c
    mode_symmetric_k = 2, // (q, c) for c <= q, mirrored on output
};

/** A tape as the kernels see it: `base + offsets[i]` is the start of string i. */
struct tape_t {
    std::uint8_t const *base;
    void const *offsets;
    std::uint64_t count;
    int offset_bits; // 32 or 64
};

/** Everything the planning kernels need. */
struct plan_args_t {
    tape_t queries, candidates;
    int mode;
    std::uint64_t pairs;
    std::uint64_t candidates_count; // columns of the cross product
    int kind, affine;
    int open, extend, match, mismatch;
    int unit_levenshtein;   // 0/1/1/1 Levenshtein: bit-parallel route
    int magnitude;          // max |cost| over substitution and gap costs, at least 1
    int local_gain;         // local scores with non-positive gaps: max(0, largest substitution cost); else -1
    int steps_beyond_span;  // 1 linear, 3 affine (serial.hpp:126-140)
    int force_route;        // -1: normal planning; otherwise one bin per route, input order (the plain form)
    int wide;               // UTF-8 calls over more than 256 code points: the tapes hold 16-bit codes, offsets in codes
    int packed_allowed;     // 1 if the 16x2 route may hold the substitution costs in int8 profiles
    int dense;              // dense-table engine: its profile holds the batch's bytes, at most 32 of them
    batch_alphabet_t const *alphabet; // Levenshtein: the batch alphabet, read on the device (may be null)
    // Tuning by length class k = floor(log2(shorter side)), 15 for everything longer.
    std::uint8_t packed_rows[16];     // 0: per-pair step-cost model; else rows per lane 4, 8, 12, 16
    std::uint8_t cell_bits[16];       // 0: narrowest safe; 32: never 16-bit cells; 64: 64-bit cells
    std::uint32_t band_min_rows;      // shorter sides above this take the band (pairs on 32-bit cells)
    std::uint32_t band_min_rows_packed; // the same for pairs that fit 16-bit cells
    std::uint16_t packed_step_cost[4];  // relative cost of one lane step with 4, 8, 12, 16 rows per lane
    std::uint32_t band_min_rows_compare; // the same for compare-mode Levenshtein pairs (no profile)
    std::uint32_t short_max_rows;        // 16x2 pairs whose shorter side is at most this take the short route
};

/** Per-bin counters the planner fills. */
struct plan_bins_t {
    std::uint32_t count[bin_keys_k];
    std::uint32_t begin[bin_keys_k];
    std::uint32_t fill[bin_keys_k];
    std::uint32_t cursor[bin_keys_k];
    std::uint32_t max_cols;
    std::uint32_t error_flags;
    std::uint64_t cells;
    std::uint64_t scheduled;
    std::uint32_t max_myers_rows;      // longest pattern on the thread-per-pair bit-parallel route
    std::uint32_t max_myers_warp_rows; // longest pattern on the warp-per-pair bit-parallel route
    std::uint32_t max_chain_rows;      // longest pattern on the chained bit-parallel route
    std::uint32_t reserved;
};

} // namespace szs_gb300
