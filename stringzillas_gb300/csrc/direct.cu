/**
 *  @file direct.cu
 *  @brief Cross products of short tokens under unit-cost Levenshtein: one thread per output cell, no planning.
 *
 *  A cross-product (or symmetric) call over strings of at most 64 bytes spends most of its time in planning when it
 *  takes the general path: the pair enumeration, binning and task scatter touch every pair, and a host round trip
 *  separates planning from scoring. When every string of both tapes has at most 64 bytes, each output cell is one
 *  bit-parallel distance over a pattern of at most two 32-bit words, cheap enough to compute where it lands. So one
 *  kernel takes one cell per thread: it reads the two strings through the tapes' offsets, lays the shorter one's
 *  bytes out as 8 bit planes of two words, runs the Myers / Hyyrö step over the longer one's bytes (match masks from
 *  the planes, one logic operation per plane and word), and writes the distance into the caller's matrix (both
 *  mirrored cells for the symmetric form). A string longer than 64 bytes raises a flag instead; the host then runs
 *  the general path for the whole call, which writes every cell again.
 *
 *  Counterpart of the reference's single-word direct path for tiny-token cross products
 *  (include/stringzillas/similarities/cuda.cuh:3892-3936); the distances are those of the serial engine
 *  (serial.hpp:1656-1865).
 */
#include "launchers.h"
#include "planner.cuh"

#include <cuda_runtime.h>

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

/** Unit-cost edit distance of a pattern of 1..64 bytes against a text of 1..64 bytes. */
__device__ __forceinline__ std::uint32_t direct_distance(std::uint8_t const *pattern, std::uint32_t n,
                                                        std::uint8_t const *text, std::uint32_t m) {
    std::uint32_t planes[8][2];
#pragma unroll
    for (int b = 0; b < 8; ++b) planes[b][0] = planes[b][1] = 0u;
    for (std::uint32_t i = 0; i < n; ++i) {
        std::uint32_t const byte = pattern[i];
        std::uint32_t const bit = 1u << (i & 31u);
        bool const high = i >= 32u;
#pragma unroll
        for (int b = 0; b < 8; ++b)
            if ((byte >> b) & 1u) {
                if (high) planes[b][1] |= bit;
                else planes[b][0] |= bit;
            }
    }
    std::uint32_t pv[2] = {0xFFFFFFFFu, 0xFFFFFFFFu}, mv[2] = {0u, 0u};
    for (std::uint32_t j = 0; j < m; ++j) {
        std::uint32_t const byte = text[j];
        std::uint32_t eq[2] = {0xFFFFFFFFu, 0xFFFFFFFFu};
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            std::uint32_t const select = ((byte >> b) & 1u) - 1u; // all-ones where the text bit is 0
            eq[0] &= planes[b][0] ^ select;
            eq[1] &= planes[b][1] ^ select;
        }
        std::uint32_t const xv0 = eq[0] | mv[0], xv1 = eq[1] | mv[1];
        std::uint32_t sum0 = eq[0] & pv[0], sum1 = eq[1] & pv[1];
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(sum0), "+r"(sum1) : "r"(pv[0]), "r"(pv[1]));
        std::uint32_t const xh0 = (sum0 ^ pv[0]) | eq[0], xh1 = (sum1 ^ pv[1]) | eq[1];
        std::uint32_t const ph0 = mv[0] | ~(xh0 | pv[0]), ph1 = mv[1] | ~(xh1 | pv[1]);
        std::uint32_t const mh0 = pv[0] & xh0, mh1 = pv[1] & xh1;
        std::uint32_t const ph_shift0 = (ph0 << 1) | 1u, ph_shift1 = __funnelshift_l(ph0, ph1, 1);
        std::uint32_t const mh_shift0 = mh0 << 1, mh_shift1 = __funnelshift_l(mh0, mh1, 1);
        pv[0] = mh_shift0 | ~(xv0 | ph_shift0), pv[1] = mh_shift1 | ~(xv1 | ph_shift1);
        mv[0] = ph_shift0 & xv0, mv[1] = ph_shift1 & xv1;
    }
    // D[n][m] = m + (rows 1..n of the last column's +1 deltas) - (its -1 deltas).
    std::uint32_t const mask0 = n >= 32u ? 0xFFFFFFFFu : (1u << n) - 1u;
    std::uint32_t const mask1 = n >= 64u ? 0xFFFFFFFFu : (n > 32u ? (1u << (n - 32u)) - 1u : 0u);
    return m + __popc(pv[0] & mask0) + __popc(pv[1] & mask1) - __popc(mv[0] & mask0) - __popc(mv[1] & mask1);
}

__global__ void __launch_bounds__(256) myers_direct_kernel(plan_args_t const args, std::int64_t *__restrict__ out,
                                                           std::uint64_t stride, std::uint32_t *__restrict__ flag) {
    for (std::uint64_t p = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < args.pairs;
         p += (std::uint64_t)gridDim.x * blockDim.x) {
        std::uint64_t q, c;
        if (args.mode == mode_cross_k) q = p / args.candidates_count, c = p % args.candidates_count;
        else {
            std::uint64_t row = (std::uint64_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) / 2.0);
            while (row * (row + 1) / 2 > p) --row;
            while ((row + 1) * (row + 2) / 2 <= p) ++row;
            q = row, c = p - row * (row + 1) / 2;
        }
        std::uint8_t const *first, *second;
        std::uint64_t n, m;
        direct_string(args.queries, q, first, n);
        direct_string(args.mode == mode_symmetric_k ? args.queries : args.candidates, c, second, m);
        if (n > 64u || m > 64u) {
            atomicOr(flag, 1u);
            continue;
        }
        std::uint32_t distance;
        if (n == 0 || m == 0) distance = (std::uint32_t)(n > m ? n : m);
        else if (n <= m) distance = direct_distance(first, (std::uint32_t)n, second, (std::uint32_t)m);
        else distance = direct_distance(second, (std::uint32_t)m, first, (std::uint32_t)n);
        out[q * stride + c] = distance;
        if (args.mode == mode_symmetric_k && q != c) out[c * stride + q] = distance;
    }
}

} // namespace

cudaError_t launch_myers_direct(plan_args_t const &args, std::int64_t *out, std::uint64_t stride,
                                std::uint32_t *flag, int sm_count, cudaStream_t stream) {
    std::uint64_t const needed = (args.pairs + 255) / 256;
    std::uint64_t const cap = (std::uint64_t)sm_count * 8;
    int const grid = (int)(needed < cap ? (needed ? needed : 1) : cap);
    myers_direct_kernel<<<grid, 256, 0, stream>>>(args, out, stride, flag);
    return cudaGetLastError();
}

} // namespace szs_gb300
