/**
 *  @file myers_chain.cuh
 *  @brief Unit-cost Levenshtein of very long pairs (more than 8,192 characters on the shorter side) by the
 *         bit-parallel method, one pair spread over a chain of warps across the whole GPU.
 *
 *  The warp-per-pair kernel (myers_warp.cuh) cuts a pattern into 32 lane slices of W words and pipelines the text
 *  through the lanes: lane L scores column t - L at step t and hands lane L + 1 three bits per column - the carry out
 *  of its multi-word add and the top bits of its horizontal deltas Ph and Mh - together with the column's character.
 *  The same hand-over works between warps: here warp k owns rows [1024 W k, 1024 W (k + 1)) of the pattern, its
 *  lane 0 takes the three bits of every column from warp k - 1's lane 31 (through a byte per column in global
 *  memory, L2-resident) instead of the row-0 boundary, and its lane 31 publishes them for warp k + 1. A pattern of
 *  100,000 rows becomes a pipeline of 98 warps (W = 1) that all advance along the text at once, each a few columns
 *  behind the warp above, where the general route gave the pair a band of CTAs over 32-bit cells.
 *
 *  Progress is a column count per warp, published by lane 31 with a GPU-scope release store every 32 columns and
 *  at the end; the next warp's acquire loads wait (bounded: `wait_polls` polls) until the 32 columns it stages next
 *  are published. Each warp stages the column codes a chunk ahead in a shared ring, so a step's match masks do not
 *  wait on the lane above: only the three bits travel between lanes. Steps come in chunks of 32 unrolled steps with
 *  no range checks wherever every lane is on a real column. The grid is one cooperative launch, so every warp of the chain is resident while the next one waits
 *  on it; a wait that gives up sets bit 0 of the plan's error word and the warp abandons the pair. No per-column
 *  score is tracked: after the last column, `D[n][m] = m + popc(Pv) - popc(Mv)` over rows 1..n, so each warp adds its
 *  rows' count into one 64-bit sum and the warp that finishes last writes the result.
 *
 *  Same recurrence as the reference's Myers tiers (include/stringzillas/similarities/cuda.cuh:2072-2634) and serial
 *  engine (serial.hpp:1656-1865); the reference scores such pairs with its tiled DP tier (cuda.cuh:616-1096).
 */
#pragma once
#include "myers.cuh"

namespace szs_gb300 {

constexpr int myers_chain_threads_k = 256;

/** Per-pair state of a chain in global memory, cleared before each launch: the warps' published column counts,
 *  the count of warps done and the sum of their rows' vertical deltas. Links (one byte per column per warp
 *  boundary) follow it. */
struct myers_chain_state_t {
    std::uint32_t done;
    std::uint32_t reserved;
    long long delta_sum;
};

/** Bytes of one pair's chain scratch: its state, `strips` progress words, then `strips - 1` links. */
__host__ __device__ inline std::uint64_t myers_chain_pair_bytes(std::uint32_t strips, std::uint64_t link_stride) {
    return 256 + ((std::uint64_t)strips * 4 + 255) / 256 * 256 + (std::uint64_t)strips * link_stride;
}

/**
 *  One wave of chains: pairs [first, first + pairs) of bin `key`, each given `strips` consecutive warps (its own
 *  chain needs ceil(n / (1,024 W)) of them; the rest exit) and `myers_chain_pair_bytes(strips, link_stride)` bytes of
 *  `scratch`, whose head (state and progress) the launcher clears.
 */
template <int words_, int bits_>
__global__ void __launch_bounds__(myers_chain_threads_k)
    myers_chain_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key,
                       std::uint32_t first, std::uint32_t pairs, std::uint32_t strips_per_pair,
                       batch_alphabet_t const *__restrict__ alphabet, std::int64_t *__restrict__ results,
                       unsigned char *__restrict__ scratch, std::uint64_t link_stride, std::uint32_t wait_polls) {
    constexpr int W = words_, B = bits_;
    __shared__ std::uint8_t code_s[256];
    __shared__ std::uint8_t ring_s[myers_chain_threads_k / 32][128];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) code_s[i] = alphabet->code[i];
    __syncthreads();
    std::uint32_t const global_warp = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    std::uint32_t const pair_in_wave = global_warp / strips_per_pair, warp = global_warp % strips_per_pair;
    if (pair_in_wave >= pairs) return; // whole warps past the wave
    pair_task_t const task = tasks[bins->begin[key] + first + pair_in_wave];
    std::uint32_t const n = task.rows_length, m = task.cols_length;
    constexpr std::uint32_t rows_per_warp = 32u * 32u * W;
    std::uint32_t const strips = (n + rows_per_warp - 1) / rows_per_warp;
    if (warp >= strips) return; // a whole warp: nobody waits on chain links past the pair's last strip
    unsigned char *const pair_scratch = scratch + (std::uint64_t)pair_in_wave * myers_chain_pair_bytes(strips_per_pair, link_stride);
    auto *state = reinterpret_cast<myers_chain_state_t *>(pair_scratch);
    auto *progress = reinterpret_cast<std::uint32_t *>(pair_scratch + 256);
    std::uint8_t *links = pair_scratch + 256 + ((std::uint64_t)strips_per_pair * 4 + 255) / 256 * 256;
    int const lane = threadIdx.x & 31;
    bool const first_strip = warp == 0, last_strip = warp + 1 == strips;

    // This lane's W words of the pattern as B code planes.
    std::uint32_t planes[B][W];
    std::uint32_t const lane_base = warp * rows_per_warp + (std::uint32_t)lane * 32u * W;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        std::uint32_t acc[B];
#pragma unroll
        for (int b = 0; b < B; ++b) acc[b] = 0;
        std::uint32_t const base = lane_base + 32u * w;
        std::uint32_t const valid = n > base ? min(32u, n - base) : 0u;
        for (std::uint32_t k = 0; k < valid; ++k) {
            std::uint32_t const c = code_s[task.rows[base + k]];
#pragma unroll
            for (int b = 0; b < B; ++b) acc[b] |= ((c >> b) & 1u) << k;
        }
#pragma unroll
        for (int b = 0; b < B; ++b) planes[b][w] = acc[b];
    }
    std::uint32_t pv[W], mv[W];
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] = 0xFFFFFFFFu, mv[w] = 0u;

    std::uint8_t const *upstream = first_strip ? nullptr : links + (std::uint64_t)(warp - 1) * link_stride;
    std::uint8_t *downstream = last_strip ? nullptr : links + (std::uint64_t)warp * link_stride;
    int const warp_in_cta = threadIdx.x / 32;
    std::uint8_t *ring = ring_s[warp_in_cta]; // column codes, by column mod 128, staged a chunk ahead
    bool healthy = true;
    std::uint32_t out = 0;   // to lane + 1: carry | top Ph bit << 1 | top Mh bit << 2
    std::uint32_t chunk = 0; // lane L: the three bits entering row 0 of this strip at column (t & ~31) + L

    // Stages chunk `c` (columns 32c..32c+31): bits from above into `chunk`, and the codes of the next chunk into the
    // ring (the ring holds columns t - 31 .. t + 63 at step t). Returns false if the wait for the warp above gave up.
    auto stage = [&](std::uint32_t t) -> bool {
        std::uint32_t const column = t + (std::uint32_t)lane;
        if (column + 32u < m) ring[(column + 32u) & 127u] = code_s[task.cols[column + 32u]];
        if (first_strip) chunk = 2u; // +1 shifted into row 0's horizontal delta, no carry
        else if (t < m) {
            std::uint32_t const needed = min(m, t + 32u);
            int ok = 1;
            if (lane == 0) {
                std::uint32_t polls = 0;
                while (true) {
                    std::uint32_t seen;
                    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(seen) : "l"(&progress[warp - 1]));
                    if (seen >= needed) break;
                    if (*reinterpret_cast<volatile std::uint32_t *>(&bins->error_flags) & 1u) {
                        ok = 0;
                        break;
                    }
                    if (++polls > wait_polls) {
                        atomicOr(&bins->error_flags, 1u);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            if (!__shfl_sync(0xFFFFFFFFu, ok, 0)) return false;
            __syncwarp();
            chunk = column < m ? (std::uint32_t)__ldcg(upstream + column) : 0u;
        }
        __syncwarp();
        return true;
    };
    // One step: lane L scores column t - L. The column's code comes from the ring (off the chain of dependencies);
    // only the three bits travel between lanes.
    auto step = [&](std::uint32_t t, auto checked_tag) {
        constexpr bool checked = decltype(checked_tag)::value;
        int const j = (int)t - lane;
        std::uint32_t const code = ring[(std::uint32_t)j & 127u];
        std::uint32_t const staged = __shfl_sync(0xFFFFFFFFu, chunk, int(t & 31u));
        std::uint32_t in = __shfl_up_sync(0xFFFFFFFFu, out, 1);
        if (lane == 0) in = staged;
        if (checked && !(j >= 0 && j < (int)m)) return;
        std::uint32_t eq[W], xv[W], sum[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            std::uint32_t e = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < B; ++b) e &= planes[b][w] ^ (((code >> b) & 1u) - 1u);
            eq[w] = e;
            xv[w] = e | mv[w];
            sum[w] = e & pv[w];
        }
        // Multi-word (Eq & Pv) + Pv with the carry from the rows above: the carry flag starts as that bit.
        std::uint32_t carry_out, scratch;
        asm volatile("add.cc.u32 %0, %1, 0xFFFFFFFF;" : "=r"(scratch) : "r"(in & 1u));
#pragma unroll
        for (int w = 0; w < W; ++w) asm volatile("addc.cc.u32 %0, %0, %1;" : "+r"(sum[w]) : "r"(pv[w]));
        asm volatile("addc.u32 %0, 0, 0;" : "=r"(carry_out));
        std::uint32_t ph_prev = in << 30, mh_prev = in << 29; // bit 31: the Ph / Mh bit shifted in from above
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
        out = carry_out | ((ph_prev >> 31) << 1) | ((mh_prev >> 31) << 2);
        if (lane == 31 && downstream) {
            downstream[j] = (std::uint8_t)out;
            if (((std::uint32_t)j & 31u) == 31u || j + 1 == (int)m) // release: the bytes before the count
                asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(&progress[warp]), "r"((std::uint32_t)j + 1)
                             : "memory");
        }
    };

    if (lane < (int)m) ring[lane] = code_s[task.cols[lane]];
    std::uint32_t const steps = m + 31u;
    // Steady chunks: every lane on a real column for all 32 steps (31 <= t and t + 31 < m): no range checks.
    std::uint32_t const steady_first = 32u, steady_end = m >= 32u ? (m / 32u) * 32u : 0u;
    std::uint32_t t = 0;
    for (; t < steps && healthy; ++t) {
        if (t >= steady_first && t < steady_end) break;
        if ((t & 31u) == 0 && !stage(t)) healthy = false;
        else step(t, std::true_type {});
    }
    for (; t < steady_end && healthy; t += 32u) {
        if (!stage(t)) {
            healthy = false;
            break;
        }
#pragma unroll
        for (std::uint32_t k = 0; k < 32u; ++k) step(t + k, std::false_type {});
    }
    for (; t < steps && healthy; ++t) {
        if ((t & 31u) == 0 && !stage(t)) {
            healthy = false;
            break;
        }
        step(t, std::true_type {});
    }
    if (!healthy) return;
    // D[n][m] = m + sum over rows 1..n of the last column's +1 deltas minus its -1 deltas.
    long long delta = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        std::uint32_t const base = lane_base + 32u * w;
        std::uint32_t const mask = n >= base + 32u ? 0xFFFFFFFFu : (n > base ? (1u << (n - base)) - 1u : 0u);
        delta += __popc(pv[w] & mask) - __popc(mv[w] & mask);
    }
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) delta += __shfl_xor_sync(0xFFFFFFFFu, delta, offset);
    if (lane == 0) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&state->delta_sum), (unsigned long long)delta);
        __threadfence();
        if (atomicAdd(&state->done, 1u) + 1u == strips) {
            __threadfence();
            long long const total = *reinterpret_cast<volatile long long *>(&state->delta_sum);
            results[task.slot] = (std::int64_t)m + total;
        }
    }
}

} // namespace szs_gb300
