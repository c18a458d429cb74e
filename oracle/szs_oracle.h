/**
 *  @file oracle/szs_oracle.h
 *  @brief CPU restatement of StringZillas' byte-level scoring path (Levenshtein, Needleman-Wunsch,
 *         Smith-Waterman; linear or affine gaps; 32-class substitution tables).
 *
 *  TEST INFRASTRUCTURE ONLY. This is the parity oracle and the CPU baseline. The product library never calls it;
 *  only tests, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 *  Every function returns the exact integer optimum of the recurrence the reference evaluates in
 *  `include/stringzillas/similarities/serial.hpp` (cited per function in `szs_oracle.c`), computed in 64-bit
 *  arithmetic, so no overflow can occur for any input the reference accepts.
 */
#ifndef SZS_ORACLE_H_
#define SZS_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/** Scoring kinds, numbered like the product engine's kinds. */
enum oracle_kind_t {
    oracle_levenshtein_k = 0,      /**< minimize, uniform match/mismatch costs */
    oracle_needleman_wunsch_k = 1, /**< maximize, global, class table */
    oracle_smith_waterman_k = 2,   /**< maximize, local, class table */
};

/** Costs for one engine, mirroring the reference's `szs_*_init` arguments. */
typedef struct oracle_costs_t {
    int kind;                       /**< `oracle_kind_t` */
    int8_t match, mismatch;         /**< Levenshtein only */
    int8_t open, extend;            /**< gap costs; `open == extend` means linear gaps */
    uint8_t byte_to_class[256];     /**< NW / SW only */
    int8_t class_costs[32 * 32];    /**< NW / SW only, row-major [first class][second class] */
    int8_t const *dense_costs;      /**< NW / SW, optional: [first byte][second byte] 256 x 256, replaces the
                                         class fold when set (the engine's dense-table extension; no reference
                                         counterpart) */
    int utf8;                       /**< Levenshtein over UTF-8 code points instead of bytes (the batch drivers) */
} oracle_costs_t;

/** Scores one pair. Levenshtein results are non-negative for non-negative costs. */
int64_t oracle_score_pair(oracle_costs_t const *costs, char const *first, size_t first_length, char const *second,
                          size_t second_length);

/** Unit-cost Levenshtein distance by the bit-parallel method (Myers 1999 blocks, Hyyrö's formulation). */
uint64_t oracle_levenshtein_bitparallel(char const *first, size_t first_length, char const *second,
                                        size_t second_length);

/**
 *  Pairwise batch over two Arrow-like tapes (offsets have count + 1 entries): `results[i] = score(first_i, second_i)`.
 *  Runs on @p threads host threads (0 = all online cores) with dynamic work distribution. Returns 0 on success.
 */
int oracle_score_pairs_u64tape(oracle_costs_t const *costs, char const *first_data, uint64_t const *first_offsets,
                               char const *second_data, uint64_t const *second_offsets, size_t count,
                               int64_t *results, size_t threads);

/**
 *  Cross-product over two tapes, or the symmetric self-similarity when @p candidates_data is NULL:
 *  `results[q * stride + c] = score(queries_q, candidates_c)`; the symmetric case scores `c <= q` and mirrors,
 *  as `serial.hpp:2540-2580` does.
 */
int oracle_score_cross_u64tape(oracle_costs_t const *costs, char const *queries_data, uint64_t const *queries_offsets,
                               size_t queries_count, char const *candidates_data, uint64_t const *candidates_offsets,
                               size_t candidates_count, int64_t *results, size_t results_stride, size_t threads);

/**
 *  Min-Hash fingerprints (include/stringzillas/fingerprints/serial.hpp): for each of @p dimensions rolling hashes,
 *  the minimum hash over all windows of the dimension's width and how often it occurs. Dimension d rolls a
 *  Rabin-Karp hash `(state * multiplier + byte + 1) mod modulo` with parameters from `splitmix64` streams of
 *  `seed + d` (:33-41, :426-432, :326-333), in exact integer arithmetic (the reference's double-precision Barrett
 *  steps are exact on these magnitudes). Widths follow the engine's layout (c/stringzillas/fingerprints.cuh:34-140):
 *  64-dimension slices per width when every width gets a whole number of slices, else widths interleaved per
 *  dimension. Rows of @p min_hashes / @p min_counts are @p hashes_stride / @p counts_stride bytes apart.
 */
int oracle_fingerprints_u64tape(size_t dimensions, size_t const *window_widths, size_t window_widths_count,
                                uint64_t seed, char const *data, uint64_t const *offsets, size_t count,
                                uint32_t *min_hashes, size_t hashes_stride, uint32_t *min_counts,
                                size_t counts_stride);

#ifdef __cplusplus
}
#endif

#endif
