/**
 *  @file engine_types.cuh
 *  @brief Types shared by the host orchestration and the device kernels of the GB300 scoring engine.
 *
 *  Terminology: a "pair" is one (first, second) string pair whose score lands in one output cell. Inside the DP
 *  kernels the pair is laid out as a matrix of `rows` (the shorter string, held in registers, 32 lanes x R rows per
 *  "strip") by `cols` (the longer string, streamed column by column). `transposed` records that rows came from the
 *  second string, so class-table lookups swap their operands back and scores stay `cost(first[i], second[j])`,
 *  as the reference's walkers guarantee (include/stringzillas/similarities/serial.hpp:1179, :721-722).
 */
#pragma once
#include <cstdint>

namespace szs_gb300 {

enum score_kind_t : int {
    kind_levenshtein_k = 0,      // minimise, uniform match / mismatch
    kind_needleman_wunsch_k = 1, // maximise, global, class table
    kind_smith_waterman_k = 2,   // maximise, local, class table
};

/** How a pair is scored; chosen per pair by the planner. */
enum pair_route_t : int {
    route_trivial_k = 0, // an empty side: answered by the closed form, no kernel
    route_myers_k = 1,   // unit-cost Levenshtein, bit-parallel, thread per pair
    route_dp32_k = 2,    // wavefront DP, 32-bit cells, warp per pair
    route_dp64_k = 3,    // wavefront DP, 64-bit cells, warp per pair (only when 32-bit could overflow)
};

/** Compare modes of the 16x2 kernels: Levenshtein over more than 32 byte values keeps both pairs' row codes instead
 *  of a profile, and a cell's substitution cost follows from comparing them with the column's codes. */
enum compare_mode_t : int {
    compare_none_k = 0,     // costs from the int8 profiles
    compare_multiply_k = 1, // costs by one multiply-add: exact when match and mismatch, as shifted, have one sign
    compare_select_k = 2,   // costs by a half mask and one logic operation
};

/** The compare mode for Levenshtein costs `match` and `mismatch` as the 16x2 kernels hold them (minus `open` for
 *  affine tracks). */
inline int compare_mode_for(int match, int mismatch) {
    return (match < 0) == (mismatch < 0) ? compare_multiply_k : compare_select_k;
}

/** One scheduled pair. 32 bytes; the planner writes these in scheduled order. */
struct pair_task_t {
    std::uint8_t const *rows;  // the string laid along DP rows (the shorter one)
    std::uint8_t const *cols;  // the string laid along DP columns
    std::uint32_t rows_length; // n >= 1 for DP routes
    std::uint32_t cols_length; // m >= 1 for DP routes
    std::uint32_t slot;        // index into the dense per-pair results array
    std::uint32_t transposed;  // 1 if rows came from the second string
};

/** Costs as the kernels see them. Copied into shared memory by every CTA that needs the tables. */
struct score_costs_t {
    int kind;                       // score_kind_t
    int affine;                     // 0: linear gaps (open == extend), 1: affine
    int open, extend;               // gap costs; a gap of length k costs open + (k-1)*extend
    int match, mismatch;            // Levenshtein substitution costs
    int classes;                    // number of compact column classes (NW / SW), <= 32
    int local_limit16;              // local scores on 16-bit cells are exact while every cell stays below this
                                    // (32767 - largest substitution gain); 0 when gaps may be positive
    std::uint32_t wait_polls;       // band kernels: polls before a ring wait gives up and fails the call
    std::uint32_t barrier_polls;    // grouped band kernels: polls before a group barrier gives up
    std::int8_t const *direct_table; // dense-table calls over more than 32 bytes: the 256 x 256 [first byte]
                                     // [second byte] table in device memory, read by the direct-table kernels
    std::uint8_t byte_to_compact[256];  // byte -> compact class, indexing `profile_table` rows
    std::int8_t profile_table[32 * 32]; // [compact column class][row class] cost, already oriented for rows=first
    std::int8_t profile_table_t[32 * 32]; // same for rows=second (transposed lookups)
    std::uint8_t byte_to_class[256];      // byte -> full class of the reference's 32x32 table
};

/** Bounds of the band kernels' waits (each poll sleeps about 100 ns in a ring wait, 200 ns at a barrier): about
 *  0.4 s and 3 s. A tuning may lower them, never raise them. */
constexpr std::uint32_t band_wait_polls_default_k = 1u << 22;
constexpr std::uint32_t band_barrier_polls_default_k = 1u << 24;

/** Alphabet of a batch: byte -> dense code, and the number of code bits the bit-parallel kernel needs. */
struct batch_alphabet_t {
    std::uint8_t code[256];
    std::uint32_t symbols;
    std::uint32_t bits;
    std::uint32_t mask_scratch[8]; // bytes seen, accumulated by the mark pass and cleared by the code pass
    std::uint32_t present[8];      // the bytes of the batch (bit b of word b / 32); absent bytes also have code 0
};

} // namespace szs_gb300
