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
 *  `AND_b (bit_b(c) ? plane_b : ~plane_b)`, one LOP3 per plane and word.
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

template <int words_, int bits_, bool exact_>
__device__ __forceinline__ std::uint32_t myers_distance(std::uint8_t const *pattern, std::uint32_t n,
                                                        std::uint8_t const *text, std::uint32_t m,
                                                        std::uint8_t const *code) {
    constexpr int W = words_, B = bits_;
    std::uint32_t planes[B][W];
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
        for (int b = 0; b < B; ++b) planes[b][w] = acc[b];
    }

    std::uint32_t pv[W], mv[W];
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] = 0xFFFFFFFFu, mv[w] = 0u;
    std::uint32_t const last_bit = (n - 1) & 31u;
    int const last_word = exact_ ? W - 1 : int((n - 1) / 32u); // the word holding row n
    std::int32_t score = (std::int32_t)n;

    byte_stream_t stream;
    stream.open_at(text);
    for (std::uint32_t j = 0; j < m; ++j) {
        std::uint32_t const c = code[stream.next()];
        std::uint32_t flip[B];
#pragma unroll
        for (int b = 0; b < B; ++b) flip[b] = ((c >> b) & 1u) ? 0u : 0xFFFFFFFFu;
        std::uint32_t eq[W], xv[W], xh[W];
        std::uint32_t carry = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t e = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < B; ++b) e &= planes[b][w] ^ flip[b];
            eq[w] = e;
            xv[w] = e | mv[w];
            // Multi-word (Eq & Pv) + Pv with the carry rippling upwards.
            std::uint64_t const sum = (std::uint64_t)(e & pv[w]) + pv[w] + carry;
            carry = (std::uint32_t)(sum >> 32);
            xh[w] = ((std::uint32_t)sum ^ pv[w]) | e;
        }
        std::uint32_t ph_prev = 1u << 31, mh_prev = 0u; // shifting these in brings +1 into row 0, 0 into mh
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t const ph = mv[w] | ~(xh[w] | pv[w]);
            std::uint32_t const mh = pv[w] & xh[w];
            if (w == last_word)
                score += (std::int32_t)((ph >> last_bit) & 1u) - (std::int32_t)((mh >> last_bit) & 1u);
            std::uint32_t const ph_shifted = __funnelshift_l(ph_prev, ph, 1);
            std::uint32_t const mh_shifted = __funnelshift_l(mh_prev, mh, 1);
            pv[w] = mh_shifted | ~(xv[w] | ph_shifted);
            mv[w] = ph_shifted & xv[w];
            ph_prev = ph, mh_prev = mh;
        }
    }
    return (std::uint32_t)score;
}

/** Thread-per-pair kernel over the Myers bin of one word count. */
template <int words_, int bits_, bool exact_>
__global__ void __launch_bounds__(128) myers_kernel(pair_task_t const *__restrict__ tasks,
                                                    plan_bins_t const *__restrict__ bins,
                                                    batch_alphabet_t const *__restrict__ alphabet,
                                                    std::int64_t *__restrict__ results) {
    __shared__ std::uint8_t code_s[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) code_s[i] = alphabet->code[i];
    __syncthreads();
    int const key_begin = bin_myers_begin_k + words_ * 16, key_end = key_begin + 16;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    for (std::uint32_t index = blockIdx.x * blockDim.x + threadIdx.x; index < count;
         index += gridDim.x * blockDim.x) {
        pair_task_t const task = tasks[begin + index];
        results[task.slot] =
            myers_distance<words_, bits_, exact_>(task.rows, task.rows_length, task.cols, task.cols_length, code_s);
    }
}

} // namespace szs_gb300
