/**
 *  @file direct.cu
 *  @brief Cross products of short tokens under unit-cost Levenshtein: one thread per output cell, no planning.
 *
 *  A cross-product call over strings of at most 64 bytes spends most of its time in planning when it
 *  takes the general path: the pair enumeration, binning and task scatter touch every pair, and a host round trip
 *  separates planning from scoring. When every string of both tapes has at most 64 bytes, each output cell is one
 *  bit-parallel distance over a pattern of at most two 32-bit words, cheap enough to compute where it lands. So one
 *  kernel takes one cell per thread (a query per grid row, candidates across the row, so no division per cell): it
 *  reads the two strings through the tapes' offsets, lays the shorter one's bytes out as 8 bit planes of one or two
 *  words, runs the Myers / Hyyrö step over the longer one's bytes (match masks from the planes, one logic operation
 *  per plane and word), and writes the distance into the caller's matrix. A string longer than 64 bytes raises a
 *  flag instead; the host then runs the general path for the whole call, which writes every cell again.
 *
 *  Counterpart of the reference's single-word direct path for tiny-token cross products
 *  (include/stringzillas/similarities/cuda.cuh:3892-3936); the distances are those of the serial engine
 *  (serial.hpp:1656-1865).
 */
#include "launchers.h"
#include "planner.cuh"

#include <cuda_runtime.h>

#include <algorithm>

namespace szs_gb300 {

namespace {

__device__ __forceinline__ void direct_string(tape_t const &tape, std::uint64_t index, std::uint8_t const *&start,
                                              std::uint64_t &length) {
    std::uint64_t begin, end;
    if (tape.offset_bits == 32) {
        auto const *offsets = static_cast<std::uint32_t const *>(tape.offsets);
        begin = offsets[index], end = offsets[index + 1];
    }
    else {
        auto const *offsets = static_cast<std::uint64_t const *>(tape.offsets);
        begin = offsets[index], end = offsets[index + 1];
    }
    start = tape.base + begin;
    length = end - begin;
}

/** Unit-cost edit distance of a pattern of 1..32 x `words_` bytes against a text of 1..64 bytes. */
template <int words_>
__device__ __forceinline__ std::uint32_t direct_distance(std::uint8_t const *pattern, std::uint32_t n,
                                                        std::uint8_t const *text, std::uint32_t m) {
    constexpr int W = words_;
    std::uint32_t planes[8][W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
#pragma unroll
        for (int b = 0; b < 8; ++b) planes[b][w] = 0u;
        std::uint32_t const rows = n > 32u * w ? min(32u, n - 32u * w) : 0u;
        for (std::uint32_t k = 0; k < rows; ++k) {
            std::uint32_t const byte = pattern[32u * w + k];
#pragma unroll
            for (int b = 0; b < 8; ++b) planes[b][w] |= ((byte >> b) & 1u) << k;
        }
    }
    std::uint32_t pv[W], mv[W];
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] = 0xFFFFFFFFu, mv[w] = 0u;
    for (std::uint32_t j = 0; j < m; ++j) {
        std::uint32_t const byte = text[j];
        std::uint32_t eq[W], xv[W], sum[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            eq[w] = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < 8; ++b) eq[w] &= planes[b][w] ^ (((byte >> b) & 1u) - 1u);
            xv[w] = eq[w] | mv[w];
            sum[w] = eq[w] & pv[w];
        }
        if constexpr (W == 1) sum[0] += pv[0];
        else asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(sum[0]), "+r"(sum[1]) : "r"(pv[0]), "r"(pv[1]));
        std::uint32_t ph_prev = 1u << 31, mh_prev = 0u; // +1 shifted into row 0
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
    // D[n][m] = m + (rows 1..n of the last column's +1 deltas) - (its -1 deltas).
    std::uint32_t distance = m;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        std::uint32_t const base = 32u * w;
        std::uint32_t const mask = n >= base + 32u ? 0xFFFFFFFFu : (n > base ? (1u << (n - base)) - 1u : 0u);
        distance += __popc(pv[w] & mask) - __popc(mv[w] & mask);
    }
    return distance;
}

/** One output cell per thread: queries along the grid's y dimension, candidates along x (no division per cell). */
__global__ void __launch_bounds__(256) myers_direct_kernel(plan_args_t const args, std::int64_t *__restrict__ out,
                                                           std::uint64_t stride, std::uint32_t *__restrict__ flag) {
    std::uint64_t const queries = args.queries.count, candidates = args.candidates_count;
    for (std::uint64_t q = blockIdx.y; q < queries; q += gridDim.y) {
        std::uint8_t const *first;
        std::uint64_t n;
        direct_string(args.queries, q, first, n);
        for (std::uint64_t c = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < candidates;
             c += (std::uint64_t)gridDim.x * blockDim.x) {
            std::uint8_t const *second;
            std::uint64_t m;
            direct_string(args.candidates, c, second, m);
            if (n > 64u || m > 64u) {
                atomicOr(flag, 1u);
                continue;
            }
            std::uint32_t distance;
            bool const swap = m < n;
            std::uint8_t const *pattern = swap ? second : first, *text = swap ? first : second;
            std::uint32_t const rows = (std::uint32_t)(swap ? m : n), cols = (std::uint32_t)(swap ? n : m);
            if (rows == 0) distance = cols;
            else if (rows <= 32u) distance = direct_distance<1>(pattern, rows, text, cols);
            else distance = direct_distance<2>(pattern, rows, text, cols);
            out[q * stride + c] = distance;
        }
    }
}

} // namespace

cudaError_t launch_myers_direct(plan_args_t const &args, std::int64_t *out, std::uint64_t stride,
                                std::uint32_t *flag, int sm_count, cudaStream_t stream) {
    if (args.mode != mode_cross_k) return cudaErrorInvalidValue;
    std::uint64_t const columns = (args.candidates_count + 255) / 256;
    unsigned const grid_x = (unsigned)(columns < 64 ? (columns ? columns : 1) : 64);
    std::uint64_t const rows_wanted = ((std::uint64_t)sm_count * 16 + grid_x - 1) / grid_x;
    unsigned const grid_y = (unsigned)std::min<std::uint64_t>(std::min<std::uint64_t>(args.queries.count, rows_wanted),
                                                              65535);
    myers_direct_kernel<<<dim3(grid_x, grid_y ? grid_y : 1), 256, 0, stream>>>(args, out, stride, flag);
    return cudaGetLastError();
}

} // namespace szs_gb300
