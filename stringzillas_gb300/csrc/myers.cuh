/**
 *  @file myers.cuh
 *  @brief Unit-cost Levenshtein distance by the bit-parallel method, one thread per pair.
 *
 *  Algorithm: G. Myers, "A fast bit-vector algorithm for approximate string matching based on dynamic
 *  programming" (JACM 1999), in H. Hyyrö's edit-distance form: the top row grows by one per column, so a 1 is
 *  shifted into the horizontal-positive vector at row 0. The pattern (the shorter string, n <= 32*W) spans W
 *  32-bit words held in registers and the vertical deltas are updated for all n rows per text character with
 *  a multi-word add whose carries, and the shifted-out horizontal deltas, ripple from word to word.
 *
 *  Match masks: instead of a 256-entry table per pattern, the pattern is stored as B bit-planes of its characters'
 *  codes in a batch-wide alphabet of at most 2^B symbols (DNA: B = 2). The mask for a text character of code c is
 *  `AND_b (bit_b(c) ? plane_b : ~plane_b)`, one LOP3 per plane and word, with the per-character selectors read from
 *  a shared table. The multi-word add chains through the carry flag (one add per word), and the text is consumed in
 *  aligned 8-byte chunks whose 8 characters are unrolled, so a warp's threads do not diverge per character.
 *
 *  Replaces the reference's Myers tiers (include/stringzillas/similarities/cuda.cuh:2072-2634), which read a
 *  256 x words mask table from shared memory. The serial oracle answers unit-cost Levenshtein the same way
 *  (serial.hpp:1656-1865, :2135-2138), so the distance is exact.
 */
#pragma once
#include "dp_cells.cuh"
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

/**
 *  Per-byte match-mask selectors for B planes: `select[byte][b]` is all-ones where bit b of the byte's code is 0, so
 *  the match mask of a word is `AND_b (plane_b ^ select_b)`. Kept in shared memory: one table lookup per text
 *  character replaces the per-plane bit extraction.
 */
template <int bits_>
struct plane_selectors_t {
    std::uint32_t select[256][bits_];
};

/** Bit-parallel state of one pattern (all rows) and the step over one text character. */
template <int words_, int bits_, bool exact_>
struct myers_state_t {
    static constexpr int W = words_, B = bits_;
    std::uint32_t planes[B][W];
    std::uint32_t pv[W], mv[W];
    std::int32_t score;
    std::uint32_t last_bit;
    int last_word;

    __device__ __forceinline__ void step(std::uint32_t const (&select)[B]) {
        std::uint32_t eq[W], xv[W], sum[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t e = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < B; ++b) e &= planes[b][w] ^ select[b];
            eq[w] = e;
            xv[w] = e | mv[w];
            sum[w] = e & pv[w];
        }
        // Multi-word (Eq & Pv) + Pv: one add per word, the carry rippling upwards through the carry flag.
        asm volatile("add.cc.u32 %0, %0, %1;" : "+r"(sum[0]) : "r"(pv[0]));
#pragma unroll
        for (int w = 1; w < W; ++w) asm volatile("addc.cc.u32 %0, %0, %1;" : "+r"(sum[w]) : "r"(pv[w]));
        std::uint32_t ph_prev = 1u << 31, mh_prev = 0u; // shifting these in brings +1 into row 0, 0 into mh
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t const xh = (sum[w] ^ pv[w]) | eq[w];
            std::uint32_t const ph = mv[w] | ~(xh | pv[w]);
            std::uint32_t const mh = pv[w] & xh;
            if (exact_ ? w == W - 1 : w == last_word)
                score += (std::int32_t)((ph >> last_bit) & 1u) - (std::int32_t)((mh >> last_bit) & 1u);
            std::uint32_t const ph_shifted = __funnelshift_l(ph_prev, ph, 1);
            std::uint32_t const mh_shifted = __funnelshift_l(mh_prev, mh, 1);
            pv[w] = mh_shifted | ~(xv[w] | ph_shifted);
            mv[w] = ph_shifted & xv[w];
            ph_prev = ph, mh_prev = mh;
        }
    }

    template <typename selectors_type_>
    __device__ __forceinline__ void step_byte(selectors_type_ const &table, std::uint32_t byte) {
        std::uint32_t select[B];
#pragma unroll
        for (int b = 0; b < B; ++b) select[b] = table.select[byte][b];
        step(select);
    }
};

template <int words_, int bits_, bool exact_>
__device__ __forceinline__ std::uint32_t myers_distance(std::uint8_t const *pattern, std::uint32_t n,
                                                        std::uint8_t const *text, std::uint32_t m,
                                                        std::uint8_t const *code,
                                                        plane_selectors_t<bits_> const &selectors) {
    constexpr int W = words_, B = bits_;
    myers_state_t<W, B, exact_> state;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        std::uint32_t acc[B];
#pragma unroll
        for (int b = 0; b < B; ++b) acc[b] = 0;
        std::uint32_t const base = w * 32u;
        std::uint32_t const valid = n > base ? min(32u, n - base) : 0u;
        for (std::uint32_t k = 0; k < valid; ++k) {
            std::uint32_t const c = code[pattern[base + k]];
#pragma unroll
            for (int b = 0; b < B; ++b) acc[b] |= ((c >> b) & 1u) << k;
        }
#pragma unroll
        for (int b = 0; b < B; ++b) state.planes[b][w] = acc[b];
    }
#pragma unroll
    for (int w = 0; w < W; ++w) state.pv[w] = 0xFFFFFFFFu, state.mv[w] = 0u;
    state.last_bit = (n - 1) & 31u;
    state.last_word = exact_ ? W - 1 : int((n - 1) / 32u); // the word holding row n
    state.score = (std::int32_t)n;

    // Text: a ragged head up to 8-byte alignment, whole aligned 8-byte chunks with the 8 columns unrolled (no
    // per-character branches, so the lanes of a warp stay converged), and a ragged tail.
    std::uintptr_t const address = reinterpret_cast<std::uintptr_t>(text);
    std::uint32_t head = (std::uint32_t)((8 - (address & 7)) & 7);
    if (head > m) head = m;
    for (std::uint32_t j = 0; j < head; ++j) state.step_byte(selectors, text[j]);
    std::uint64_t const *chunks = reinterpret_cast<std::uint64_t const *>(text + head);
    std::uint32_t const full = (m - head) / 8;
    for (std::uint32_t c = 0; c < full; ++c) {
        std::uint64_t const word = __ldg(chunks + c);
        std::uint32_t const lo = (std::uint32_t)word, hi = (std::uint32_t)(word >> 32);
#pragma unroll
        for (int k = 0; k < 4; ++k) state.step_byte(selectors, (lo >> (8 * k)) & 0xFFu);
#pragma unroll
        for (int k = 0; k < 4; ++k) state.step_byte(selectors, (hi >> (8 * k)) & 0xFFu);
    }
    for (std::uint32_t j = head + full * 8; j < m; ++j) state.step_byte(selectors, text[j]);
    return (std::uint32_t)state.score;
}

/** Thread-per-pair kernel over bins [key_begin, key_end), patterns of at most 32 x `words_` rows (exactly that many
 *  words when `exact_`). */
template <int words_, int bits_, bool exact_>
__global__ void __launch_bounds__(128) myers_kernel(pair_task_t const *__restrict__ tasks,
                                                    plan_bins_t const *__restrict__ bins, int key_begin, int key_end,
                                                    batch_alphabet_t const *__restrict__ alphabet,
                                                    std::int64_t *__restrict__ results) {
    __shared__ std::uint8_t code_s[256];
    __shared__ plane_selectors_t<bits_> selectors_s;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        std::uint32_t const c = alphabet->code[i];
        code_s[i] = (std::uint8_t)c;
#pragma unroll
        for (int b = 0; b < bits_; ++b) selectors_s.select[i][b] = ((c >> b) & 1u) ? 0u : 0xFFFFFFFFu;
    }
    __syncthreads();
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    for (std::uint32_t index = blockIdx.x * blockDim.x + threadIdx.x; index < count;
         index += gridDim.x * blockDim.x) {
        pair_task_t const task = tasks[begin + index];
        results[task.slot] =
            myers_distance<words_, bits_, exact_>(task.rows, task.rows_length, task.cols, task.cols_length, code_s,
                                                  selectors_s);
    }
}

/** Planes a 16-bit code needs: UTF-8 calls over more than 256 code points score with all 16. */
constexpr int myers_wide_planes_k = 16;

/** Selectors of a 16-bit code, from its bits (a 65,536-entry shared table would not fit): all-ones where the bit
 *  is 0, as in `plane_selectors_t`. */
template <int bits_>
__device__ __forceinline__ void code_selectors(std::uint32_t code, std::uint32_t (&select)[bits_]) {
#pragma unroll
    for (int b = 0; b < bits_; ++b) select[b] = ((code >> b) & 1u) - 1u;
}

/** Thread-per-pair kernel over strings of 16-bit codes (UTF-8 calls over more than 256 code points). */
template <int words_, bool exact_>
__global__ void __launch_bounds__(128) myers_wide_kernel(pair_task_t const *__restrict__ tasks,
                                                         plan_bins_t const *__restrict__ bins, int key_begin,
                                                         int key_end, std::int64_t *__restrict__ results) {
    constexpr int W = words_, B = myers_wide_planes_k;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    for (std::uint32_t index = blockIdx.x * blockDim.x + threadIdx.x; index < count;
         index += gridDim.x * blockDim.x) {
        pair_task_t const task = tasks[begin + index];
        auto const *pattern = reinterpret_cast<std::uint16_t const *>(task.rows);
        std::uint32_t const n = task.rows_length, m = task.cols_length;
        myers_state_t<W, B, exact_> state;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t acc[B];
#pragma unroll
            for (int b = 0; b < B; ++b) acc[b] = 0;
            std::uint32_t const base = w * 32u;
            std::uint32_t const valid = n > base ? min(32u, n - base) : 0u;
            for (std::uint32_t k = 0; k < valid; ++k) {
                std::uint32_t const c = pattern[base + k];
#pragma unroll
                for (int b = 0; b < B; ++b) acc[b] |= ((c >> b) & 1u) << k;
            }
#pragma unroll
            for (int b = 0; b < B; ++b) state.planes[b][w] = acc[b];
        }
#pragma unroll
        for (int w = 0; w < W; ++w) state.pv[w] = 0xFFFFFFFFu, state.mv[w] = 0u;
        state.last_bit = (n - 1) & 31u;
        state.last_word = exact_ ? W - 1 : int((n - 1) / 32u);
        state.score = (std::int32_t)n;
        code16_stream_t text;
        text.open_at(task.cols);
        for (std::uint32_t j = 0; j < m; ++j) {
            std::uint32_t select[B];
            code_selectors<B>(text.next(), select);
            state.step(select);
        }
        results[task.slot] = (std::uint32_t)state.score;
    }
}

} // namespace szs_gb300