/**
 *  @file myers_table.cuh
 *  @brief Unit-cost Levenshtein distance by the bit-parallel method, one thread per pair, for batches over at most
 *         four distinct symbols (DNA): match masks read from a per-thread table in shared memory.
 *
 *  Same algorithm as myers.cuh (G. Myers, JACM 1999, in H. Hyyrö's edit-distance form; the pattern is the shorter
 *  string, n <= 32 * W rows in W 32-bit words of registers, the multi-word add chained through the carry flag), with
 *  three changes that take work off the integer ALU pipe, which bounds the kernel:
 *
 *  - **Match masks from shared memory.** Each thread writes, once per pair, the W-word match mask of every symbol
 *    code (4 x W words) into its own column of a shared table, laid out `[word / 4][code][thread]` in 16-byte groups
 *    so that a warp's reads of one group are contiguous per code. A text character then costs one code lookup and
 *    ceil(W / 4) 16-byte shared loads instead of two logic operations per word on the code planes.
 *  - **No per-column score tracking.** The distance is read once, after the last column: the vertical deltas of the
 *    last column give `D[n][m] = D[0][m] + sum(Pv[i] - Mv[i], i = 1..n) = m + popc(Pv) - popc(Mv)` over the rows
 *    1..n, where the top row D[0][j] = j is the boundary of the global distance.
 *  - **Loads ahead of use.** The text's first words (during the pattern's setup) and each next aligned 8-byte word of
 *    the text (while the current one is scored) are in flight before they are needed; the pattern is read in aligned
 *    8-byte words too, not byte by byte.
 *
 *  The alphabet may be a guess from a sample of the batch (`alphabet->present`): a byte outside it gets a marker code
 *  and a table offset that still lands inside the table, every pair ORs its codes and offsets together, and a pair
 *  that met a marker sets bit 1 of the plan's error word, on which the host scores the call again with the exact
 *  alphabet. Known codes (0..3) and offsets (multiples of 2,048) never carry the marker bit.
 *
 *  Per text character and pattern word the step is ten ALU operations (Xv, Eq & Pv, the carried add, Xh, Ph, Mh,
 *  two funnel shifts, Pv, Mv). The kernel takes its bins as a key range, so the plain form can run every pair with
 *  the word count of the batch's longest pattern (rows past a pattern's end are masked out of the final count).
 *
 *  Replaces, for DNA-like alphabets, the reference's Myers tiers (include/stringzillas/similarities/cuda.cuh:
 *  2072-2634); the serial oracle answers unit-cost Levenshtein the same way (serial.hpp:1656-1865, :2135-2138).
 */
#pragma once
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

constexpr int myers_table_threads_k = 128;
constexpr int myers_table_symbols_k = 4;
constexpr std::uint32_t myers_table_unknown_k = 16; // code and offset marker of a byte outside the alphabet

/** Bytes of the shared match-mask table of one CTA for patterns of `words` words. */
__host__ __device__ constexpr int myers_table_shared_bytes(int words) {
    return myers_table_symbols_k * ((words + 3) / 4) * myers_table_threads_k * 16;
}

template <int words_>
struct myers_table_state_t {
    static constexpr int W = words_, Q = (words_ + 3) / 4;
    std::uint32_t pv[W], mv[W];

    /** One text column: `masks` is this thread's row of the table for the column's symbol code. */
    __device__ __forceinline__ void step(unsigned char const *masks) {
        std::uint32_t eq[4 * Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            uint4 const v = *reinterpret_cast<uint4 const *>(
                masks + q * myers_table_symbols_k * myers_table_threads_k * 16);
            eq[4 * q + 0] = v.x, eq[4 * q + 1] = v.y, eq[4 * q + 2] = v.z, eq[4 * q + 3] = v.w;
        }
        std::uint32_t xv[W], sum[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            xv[w] = eq[w] | mv[w];
            sum[w] = eq[w] & pv[w];
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
            std::uint32_t const ph_shifted = __funnelshift_l(ph_prev, ph, 1);
            std::uint32_t const mh_shifted = __funnelshift_l(mh_prev, mh, 1);
            pv[w] = mh_shifted | ~(xv[w] | ph_shifted);
            mv[w] = ph_shifted & xv[w];
            ph_prev = ph, mh_prev = mh;
        }
    }
};

/**
 *  Thread-per-pair kernel over bins [key_begin, key_end) with patterns of at most 32 x `words_` rows, for batches
 *  whose alphabet has at most four codes.
 */
/** CTAs per SM the register budget is set for: 48 registers up to 4 words, 56 up to 8, 64 at 9 and 72 beyond (the
 *  shared table allows 8 CTAs from 9 words on and 7 from 13). */
__host__ __device__ constexpr int myers_table_min_ctas(int words) {
    return words <= 4 ? 10 : (words <= 8 ? 9 : (words <= 9 ? 8 : 7));
}

template <int words_>
__global__ void __launch_bounds__(myers_table_threads_k, myers_table_min_ctas(words_))
    myers_table_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key_begin,
                       int key_end, batch_alphabet_t const *__restrict__ alphabet,
                       std::int64_t *__restrict__ results) {
    constexpr int W = words_, Q = (words_ + 3) / 4;
    constexpr unsigned code_stride = myers_table_threads_k * 16;                         // bytes between codes
    constexpr unsigned group_stride = myers_table_symbols_k * myers_table_threads_k * 16; // between word groups
    extern __shared__ __align__(16) unsigned char table_s[];
    __shared__ std::uint32_t offset_s[256]; // byte -> code * code_stride
    __shared__ std::uint8_t code_s[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        std::uint32_t const c = alphabet->code[i] & (myers_table_symbols_k - 1);
        bool const known = (alphabet->present[i >> 5] >> (i & 31)) & 1u;
        code_s[i] = known ? (std::uint8_t)c : (std::uint8_t)myers_table_unknown_k;
        offset_s[i] = known ? c * code_stride : myers_table_unknown_k; // 16 bytes on: still inside the table
    }
    __syncthreads();
    unsigned char *const mine = table_s + threadIdx.x * 16u;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    for (std::uint32_t index = blockIdx.x * blockDim.x + threadIdx.x; index < count;
         index += gridDim.x * blockDim.x) {
        pair_task_t const task = tasks[begin + index];
        std::uint8_t const *pattern = task.rows;
        std::uint32_t const n = task.rows_length, m = task.cols_length;

        // Text, read as aligned 8-byte words, never past the one holding its last byte: a ragged head from the
        // first word, whole words (each loaded one word ahead of its use) and a ragged tail. The first two words are
        // requested before the pattern's setup, so their latency overlaps it.
        std::uintptr_t const text_address = reinterpret_cast<std::uintptr_t>(task.cols);
        std::uint64_t const *text_words = reinterpret_cast<std::uint64_t const *>(text_address & ~std::uintptr_t(7));
        std::uint32_t const text_skew = (std::uint32_t)(text_address & 7);
        std::uint32_t const text_last = (text_skew + m - 1) >> 3; // the aligned word holding the last byte
        std::uint64_t const first_word = __ldg(text_words);
        std::uint32_t const head = text_skew ? min(8u - text_skew, m) : 0u;
        std::uint32_t const start_word = text_skew ? 1u : 0u; // the first whole word
        std::uint32_t const full = (m - head) / 8, tail = m - head - 8 * full;
        std::uint64_t next = start_word == 0 ? first_word : (text_last >= 1 ? __ldg(text_words + 1) : 0ull);

        // Code planes of the pattern. Its bytes are read as aligned 8-byte words, never past the aligned word that
        // holds its last byte (so never outside the page of a valid byte), and realigned with byte permutes. The
        // 2-bit codes of 16 rows are accumulated base 4 (one multiply-add per row), and an unshuffle of the even and
        // odd bits separates the two planes. Rows past the pattern's end hold garbage: they lie below row n, which
        // they cannot influence, and the final count masks them out.
        std::uintptr_t const pattern_address = reinterpret_cast<std::uintptr_t>(pattern);
        uint2 const *aligned = reinterpret_cast<uint2 const *>(pattern_address & ~std::uintptr_t(7));
        std::uint32_t const skew = (std::uint32_t)(pattern_address & 7); // bytes before row 0 in its aligned word
        std::uint32_t const last_word = (skew + n - 1) >> 3;              // the aligned word holding row n - 1
        std::uint32_t const select = 0x3210u + 0x1111u * (skew & 3u);
        bool const upper = skew >= 4;
        std::uint32_t seen = 0; // OR of every code and table offset of the pair: the marker bit flags a guess missed
        std::uint32_t first_bytes = 0; // the pattern's first byte, four times
        std::uint32_t plane0[W], plane1[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t a0 = 0, a1 = 0;
            if (32u * w < n) {
                std::uint32_t const valid = min(32u, n - 32u * w); // rows of this word inside the pattern
                std::uint32_t halves[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    // Rows 32 w + 16 h .. + 15 from three aligned 8-byte words (clamped to the last one).
                    std::uint32_t v[6];
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        uint2 const two = __ldg(aligned + min(4u * w + 2u * h + i, last_word));
                        v[2 * i] = two.x, v[2 * i + 1] = two.y;
                    }
                    std::uint32_t r[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        r[j] = __byte_perm(upper ? v[j + 1] : v[j], upper ? v[j + 2] : v[j + 1], select);
                    if (w == 0 && h == 0) first_bytes = __byte_perm(r[0], 0u, 0u);
                    // Rows past the pattern's end may hold other strings' bytes or bytes past the tape: they take
                    // the pattern's first byte instead, so they never raise the marker on their own.
                    if (valid < 32u) {
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            int const keep = (int)valid - 16 * h - 4 * j; // bytes of r[j] inside the pattern
                            std::uint32_t const mask =
                                keep >= 4 ? 0xFFFFFFFFu : (keep <= 0 ? 0u : 0xFFFFFFFFu >> (32 - 8 * keep));
                            r[j] = (r[j] & mask) | (first_bytes & ~mask);
                        }
                    }
                    std::uint32_t x = 0; // row 16 h + k's code at bits 2k (plane 0) and 2k + 1 (plane 1)
#pragma unroll
                    for (int k = 15; k >= 0; --k) {
                        std::uint32_t const code = code_s[__byte_perm(r[k / 4], 0u, 0x4440u + (k & 3))];
                        x = x * 4u + code;
                        seen |= code;
                    }
                    // Unshuffle: even bits to the low half, odd bits to the high half.
                    std::uint32_t t;
                    t = (x ^ (x >> 1)) & 0x22222222u, x ^= t ^ (t << 1);
                    t = (x ^ (x >> 2)) & 0x0C0C0C0Cu, x ^= t ^ (t << 2);
                    t = (x ^ (x >> 4)) & 0x00F000F0u, x ^= t ^ (t << 4);
                    t = (x ^ (x >> 8)) & 0x0000FF00u, x ^= t ^ (t << 8);
                    halves[h] = x;
                }
                a0 = __byte_perm(halves[0], halves[1], 0x5410u);
                a1 = __byte_perm(halves[0], halves[1], 0x7632u);
            }
            plane0[w] = a0, plane1[w] = a1;
        }
        // The four codes' match masks into this thread's column of the table.
#pragma unroll
        for (int c = 0; c < myers_table_symbols_k; ++c) {
            std::uint32_t const s0 = (c & 1) ? 0u : ~0u, s1 = (c & 2) ? 0u : ~0u;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                std::uint32_t v[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    int const w = 4 * q + r;
                    v[r] = w < W ? ((plane0[w] ^ s0) & (plane1[w] ^ s1)) : 0u;
                }
                *reinterpret_cast<uint4 *>(mine + c * code_stride + q * group_stride) =
                    make_uint4(v[0], v[1], v[2], v[3]);
            }
        }

        myers_table_state_t<W> state;
#pragma unroll
        for (int w = 0; w < W; ++w) state.pv[w] = 0xFFFFFFFFu, state.mv[w] = 0u;

        auto column = [&](std::uint32_t byte) {
            std::uint32_t const offset = offset_s[byte];
            seen |= offset;
            state.step(mine + offset);
        };
        for (std::uint32_t j = 0; j < head; ++j) column((std::uint32_t)(first_word >> (8 * (text_skew + j))) & 0xFFu);
        for (std::uint32_t c = 0; c < full; ++c) {
            std::uint64_t const word = next;
            std::uint32_t const upcoming_word = start_word + c + 1;
            if (upcoming_word <= text_last) next = __ldg(text_words + upcoming_word);
            std::uint32_t const lo = (std::uint32_t)word, hi = (std::uint32_t)(word >> 32);
#pragma unroll
            for (int k = 0; k < 4; ++k) column(__byte_perm(lo, 0u, 0x4440u + k));
#pragma unroll
            for (int k = 0; k < 4; ++k) column(__byte_perm(hi, 0u, 0x4440u + k));
        }
        for (std::uint32_t j = 0; j < tail; ++j) column((std::uint32_t)(next >> (8 * j)) & 0xFFu); // the last word

        // D[n][m] = m + (rows 1..n of the last column's +1 deltas) - (its -1 deltas).
        std::int32_t score = (std::int32_t)m;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t const base = w * 32u;
            std::uint32_t const mask = n >= base + 32u ? 0xFFFFFFFFu : (n > base ? (1u << (n - base)) - 1u : 0u);
            score += __popc(state.pv[w] & mask) - __popc(state.mv[w] & mask);
        }
        results[task.slot] = score;
        if (seen & myers_table_unknown_k) atomicOr(&bins->error_flags, 2u);
    }
}

} // namespace szs_gb300
