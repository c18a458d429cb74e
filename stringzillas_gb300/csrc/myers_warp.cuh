/**
 *  @file myers_warp.cuh
 *  @brief Unit-cost Levenshtein by the bit-parallel method for patterns of 513 to 8,192 characters: one warp per
 *         pair, the pattern's words spread over the lanes, the text swept through the lanes as a pipeline.
 *
 *  The thread-per-pair kernel (myers.cuh) keeps a whole pattern of up to 16 words in one thread's registers. A longer
 *  pattern is cut into 32 slices of W words (W = ceil(n / 1,024) <= 8): lane L holds rows [32 W L, 32 W (L + 1)).
 *  One column of the bit-parallel step needs, for lane L's lowest word, three bits of lane L - 1's highest word in
 *  the same column: the carry out of the multi-word add and the top bits of the horizontal deltas Ph and Mh that are
 *  shifted in. So at step t lane L scores text column t - L, and lane L + 1 takes the carry, the two delta bits and
 *  the column's character from lane L one step later, all packed into one 32-bit shuffle. Lane 0 shifts +1 into row 0
 *  (the top row grows by one per column) and nothing into the carry; it takes the text from a 32-byte chunk the warp
 *  loads together every 32 steps. The lane holding row n - 1 keeps the score, as the thread kernel does.
 *
 *  The reference reaches patterns of 2,048 characters with its Myers tiers (include/stringzillas/similarities/
 *  cuda.cuh:2072-2634); its serial engine (serial.hpp:1656-1865) answers unit-cost Levenshtein exactly the same way.
 */
#pragma once
#include "myers.cuh"

namespace szs_gb300 {

/** The distance of one pair, computed by the whole warp; every lane returns it. `wide_`: strings of 16-bit codes
 *  (their own codes, selectors from the code's bits), else bytes mapped through the batch alphabet. */
template <int words_, int bits_, bool wide_ = false>
__device__ __forceinline__ std::uint32_t myers_warp_distance(pair_task_t const &task, std::uint8_t const *code,
                                                             plane_selectors_t<bits_> const *selectors) {
    constexpr int W = words_, B = bits_;
    int const lane = threadIdx.x & 31;
    std::uint32_t const n = task.rows_length, m = task.cols_length;
    int const lanes_used = int((n + 32u * W - 1) / (32u * W));

    // This lane's slice of the pattern as B bit planes of its characters' codes.
    std::uint32_t planes[B][W];
    std::uint32_t const lane_base = (std::uint32_t)lane * 32u * W;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        std::uint32_t acc[B];
#pragma unroll
        for (int b = 0; b < B; ++b) acc[b] = 0;
        std::uint32_t const base = lane_base + 32u * w;
        std::uint32_t const valid = n > base ? min(32u, n - base) : 0u;
        for (std::uint32_t k = 0; k < valid; ++k) {
            std::uint32_t const c = wide_ ? symbol_at<true>(task.rows, base + k) : code[task.rows[base + k]];
#pragma unroll
            for (int b = 0; b < B; ++b) acc[b] |= ((c >> b) & 1u) << k;
        }
#pragma unroll
        for (int b = 0; b < B; ++b) planes[b][w] = acc[b];
    }
    std::uint32_t pv[W], mv[W];
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] = 0xFFFFFFFFu, mv[w] = 0u;

    std::uint32_t const last_row = n - 1;
    int const score_lane = int(last_row / (32u * W));
    int const score_word = int((last_row / 32u) % W);
    std::uint32_t const score_bit = last_row & 31u;
    std::int32_t score = (std::int32_t)n;

    std::uint32_t out = 0;   // to lane + 1: symbol | carry << 16 | top Ph bit << 17 | top Mh bit << 18
    std::uint32_t chunk = 0; // the text symbol of column (t & ~31) + lane
    std::uint32_t const steps = m + (std::uint32_t)lanes_used - 1;
    for (std::uint32_t t = 0; t < steps; ++t) {
        if ((t & 31u) == 0) chunk = t + lane < m ? symbol_at<wide_>(task.cols, t + lane) : 0u;
        std::uint32_t const staged = __shfl_sync(0xFFFFFFFFu, chunk, int(t & 31u));
        std::uint32_t in = __shfl_up_sync(0xFFFFFFFFu, out, 1);
        if (lane == 0) in = staged | (1u << 17); // no carry into row 0; +1 shifted into its horizontal delta
        int const j = (int)t - lane;
        if (lane < lanes_used && j >= 0 && j < (int)m) {
            std::uint32_t const byte = in & 0xFFFFu;
            std::uint32_t select[B];
            if constexpr (wide_) code_selectors<B>(byte, select);
            else {
#pragma unroll
                for (int b = 0; b < B; ++b) select[b] = selectors->select[byte][b];
            }
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
            // Multi-word (Eq & Pv) + Pv with the carry from the lane below: the carry flag starts as that bit.
            std::uint32_t const carry_in = (in >> 16) & 1u;
            std::uint32_t carry_out, scratch;
            asm volatile("add.cc.u32 %0, %1, 0xFFFFFFFF;" : "=r"(scratch) : "r"(carry_in));
#pragma unroll
            for (int w = 0; w < W; ++w) asm volatile("addc.cc.u32 %0, %0, %1;" : "+r"(sum[w]) : "r"(pv[w]));
            asm volatile("addc.u32 %0, 0, 0;" : "=r"(carry_out));
            std::uint32_t ph_prev = ((in >> 17) & 1u) << 31, mh_prev = ((in >> 18) & 1u) << 31;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                std::uint32_t const xh = (sum[w] ^ pv[w]) | eq[w];
                std::uint32_t const ph = mv[w] | ~(xh | pv[w]);
                std::uint32_t const mh = pv[w] & xh;
                if (lane == score_lane && w == score_word)
                    score += (std::int32_t)((ph >> score_bit) & 1u) - (std::int32_t)((mh >> score_bit) & 1u);
                std::uint32_t const ph_shifted = __funnelshift_l(ph_prev, ph, 1);
                std::uint32_t const mh_shifted = __funnelshift_l(mh_prev, mh, 1);
                pv[w] = mh_shifted | ~(xv[w] | ph_shifted);
                mv[w] = ph_shifted & xv[w];
                ph_prev = ph, mh_prev = mh;
            }
            out = byte | carry_out << 16 | (ph_prev >> 31) << 17 | (mh_prev >> 31) << 18;
        }
    }
    return (std::uint32_t)__shfl_sync(0xFFFFFFFFu, score, score_lane);
}

/** Warp-per-pair kernel over bins [key_begin, key_end) with at most `words_` words per lane; warps pull pairs from
 *  the first bin's cursor. */
template <int words_, int bits_>
__global__ void __launch_bounds__(256) myers_warp_kernel(pair_task_t const *__restrict__ tasks,
                                                         plan_bins_t *__restrict__ bins, int key_begin, int key_end,
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
    int const lane = threadIdx.x & 31;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    while (true) {
        std::uint32_t index = 0;
        if (lane == 0) index = atomicAdd(&bins->cursor[key_begin], 1u);
        index = __shfl_sync(0xFFFFFFFFu, index, 0);
        if (index >= count) break;
        pair_task_t const task = tasks[begin + index];
        std::uint32_t const distance = myers_warp_distance<words_, bits_>(task, code_s, &selectors_s);
        if (lane == 0) results[task.slot] = distance;
    }
}

/** The same over strings of 16-bit codes (UTF-8 calls over more than 256 code points): 16 planes, no tables. */
template <int words_>
__global__ void __launch_bounds__(256) myers_warp_wide_kernel(pair_task_t const *__restrict__ tasks,
                                                              plan_bins_t *__restrict__ bins, int key_begin,
                                                              int key_end, std::int64_t *__restrict__ results) {
    int const lane = threadIdx.x & 31;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    while (true) {
        std::uint32_t index = 0;
        if (lane == 0) index = atomicAdd(&bins->cursor[key_begin], 1u);
        index = __shfl_sync(0xFFFFFFFFu, index, 0);
        if (index >= count) break;
        pair_task_t const task = tasks[begin + index];
        std::uint32_t const distance = myers_warp_distance<words_, myers_wide_planes_k, true>(
            task, nullptr, static_cast<plane_selectors_t<myers_wide_planes_k> const *>(nullptr));
        if (lane == 0) results[task.slot] = distance;
    }
}

} // namespace szs_gb300