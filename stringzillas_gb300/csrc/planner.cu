/**
 *  @file planner.cu
 *  @brief Planning kernels: pair enumeration, routing, binning, the batch alphabet, and the output scatter.
 */
#include "launchers.h"
#include "planner.cuh"

#include <cuda_runtime.h>

#include <algorithm>

namespace szs_gb300 {

__device__ __forceinline__ void tape_string(tape_t const &tape, std::uint64_t index, std::uint8_t const *&start,
                                            std::uint64_t &length, int wide) {
    std::uint64_t begin, end;
    if (tape.offset_bits == 32) {
        auto const *offsets = static_cast<std::uint32_t const *>(tape.offsets);
        begin = offsets[index], end = offsets[index + 1];
    }
    else {
        auto const *offsets = static_cast<std::uint64_t const *>(tape.offsets);
        begin = offsets[index], end = offsets[index + 1];
    }
    start = tape.base + (wide ? 2 * begin : begin); // 16-bit codes: lengths stay in codes
    length = end - begin;
}

/** Maps a flat pair index onto (query, candidate); the symmetric form walks the lower triangle row by row, the
 *  order `cross_sequentially_` uses (serial.hpp:2565-2576). */
__device__ __forceinline__ void pair_indices(plan_args_t const &args, std::uint64_t p, std::uint64_t &q,
                                             std::uint64_t &c) {
    if (args.mode == mode_pairwise_k) q = c = p;
    else if (args.mode == mode_cross_k) q = p / args.candidates_count, c = p % args.candidates_count;
    else {
        std::uint64_t row = (std::uint64_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) / 2.0);
        while (row * (row + 1) / 2 > p) --row;
        while ((row + 1) * (row + 2) / 2 <= p) ++row;
        q = row, c = p - row * (row + 1) / 2;
    }
}

/** Closed form of a pair with an empty side (serial.hpp:142-151, :2493-2496). */
__device__ __forceinline__ std::int64_t trivial_score(plan_args_t const &args, std::uint64_t n, std::uint64_t m) {
    if (args.kind == kind_smith_waterman_k) return 0;
    std::uint64_t const length = n > m ? n : m;
    if (!args.affine) return (std::int64_t)args.open * (std::int64_t)length;
    return length == 0 ? 0 : (std::int64_t)args.open + (std::int64_t)args.extend * (std::int64_t)(length - 1);
}

__device__ __forceinline__ int floor_log2_u64(std::uint64_t x) { return x ? 63 - __clzll((long long)x) : 0; }

struct pair_route_info_t {
    int key; // -1 for trivial
    std::uint8_t const *rows, *cols;
    std::uint32_t n, m;
    std::uint32_t transposed;
};

/** Routing decision for one pair. The 32-bit bound mirrors the reference's `worst_case_reach` (serial.hpp:117-140)
 *  with one extra step of headroom for the E/F intermediates. */
__device__ __forceinline__ pair_route_info_t route_pair(plan_args_t const &args, std::uint8_t const *first,
                                                        std::uint64_t first_length, std::uint8_t const *second,
                                                        std::uint64_t second_length) {
    pair_route_info_t info;
    info.key = -1;
    // Rows take the shorter string; equal lengths keep the first string on rows.
    bool const swap = second_length < first_length;
    info.rows = swap ? second : first;
    info.cols = swap ? first : second;
    info.n = (std::uint32_t)(swap ? second_length : first_length);
    info.m = (std::uint32_t)(swap ? first_length : second_length);
    info.transposed = swap ? 1u : 0u;
    if (first_length == 0 || second_length == 0) return info;
    std::uint64_t const n = info.n, m = info.m;
    int const thread_words = args.wide ? myers_wide_max_words_k : myers_max_words_k;
    if (args.unit_levenshtein && n <= 32u * thread_words) {
        if (args.force_route >= 0) {
            info.key = bin_myers_begin_k + thread_words * 16; // plain form: one bin, one kernel shape
            return info;
        }
        // A warp's threads take as long as its longest text: classes of 16 columns over the shortest text a pattern
        // of this word count can face (no text is shorter than its pattern), then four octaves; longest first.
        int const words = int((n + 31) / 32);
        std::uint64_t const over = m - 32u * (words - 1) - 1;
        int const text_class = over < 12 * 16 ? int(over / 16) : min(15, 12 + floor_log2_u64(over / (12 * 16)));
        info.key = bin_myers_begin_k + words * 16 + (15 - text_class);
        return info;
    }
    if (args.unit_levenshtein && !args.wide && n > 32u * 32u * myers_warp_max_words_k && n <= myers_chain_max_rows_k) {
        info.key = bin_myers_chain_k; // one bin in both forms: a chain of warps per pair, one launch each
        return info;
    }
    if (args.unit_levenshtein && n <= 32u * 32u * myers_warp_max_words_k) {
        // Longer patterns: one warp per pair, W words per lane.
        if (args.force_route >= 0) {
            info.key = bin_myers_warp_begin_k; // plain form: one bin (16 words per lane), input order
            return info;
        }
        int const words = int((n + 1023) / 1024);
        int text_class = floor_log2_u64(m) - 9;
        text_class = text_class < 0 ? 0 : (text_class > myers_warp_classes_k - 1 ? myers_warp_classes_k - 1 : text_class);
        info.key = bin_myers_warp_begin_k + (myers_warp_max_words_k - words) * myers_warp_classes_k +
                   (myers_warp_classes_k - 1 - text_class);
        return info;
    }
    bool const maximize = args.kind != kind_levenshtein_k;
    std::uint64_t const span = maximize ? n + m : (n > m ? n : m);
    std::uint64_t const reach = (span + (std::uint64_t)args.steps_beyond_span + 1) * (std::uint64_t)args.magnitude;
    bool const fits32_early = reach < (1ull << 31) - 1;
    int const length_class = min(15, floor_log2_u64(n));
    // Local scores with non-positive gaps stay in [0, gain * min(n, m)] (a local path gains at most one substitution
    // per diagonal step) and their gap tracks never fall below open + 2 extend: a tighter bound than the reach.
    std::uint64_t const reach16 =
        args.local_gain >= 0 ? (std::uint64_t)args.local_gain * (n < m ? n : m) + 1 : reach;
    // The 16x2 routes hold costs in a 32-class profile: dense-table calls over more bytes than that stay on the
    // 32-bit routes. Levenshtein calls over more bytes, or over 16-bit codes, take them in compare mode (codes
    // compared, no profile).
    bool const profile_fits = (args.kind != kind_levenshtein_k && !args.dense) ||
                              (args.alphabet && args.alphabet->symbols <= 32);
    bool const compare_fits = args.kind == kind_levenshtein_k && (args.alphabet != nullptr || args.wide);
    // A tuned cell width: 32 keeps the class off 16-bit cells, 64 puts it on the 64-bit wavefront (the route the
    // reach bound takes for spans near 2^31 / magnitude, reachable on any pair this way).
    bool const force64 = args.cell_bits[length_class] == 64;
    bool const packed = args.packed_allowed && (profile_fits || compare_fits) && reach16 < 32767 &&
                        args.cell_bits[length_class] == 0;
    std::uint64_t const band_rows = !packed        ? args.band_min_rows
                                    : profile_fits ? args.band_min_rows_packed
                                                   : args.band_min_rows_compare;
    // Local scores with non-positive gaps take the 16-bit band even beyond their proven bound: the kernel checks the
    // running maximum against the 16-bit limit and scores a pair that reached it again on 32-bit cells.
    bool const local_band16 =
        args.local_gain >= 0 && args.packed_allowed && profile_fits && args.cell_bits[length_class] == 0;
    // Short pairs: a few lanes per pair instead of a warp (dp_short.cuh).
    if (packed && !args.wide && n <= args.short_max_rows) {
        if (args.force_route >= 0) {
            info.key = bin_short_begin_k + 3 * short_m_classes_k; // plain form: one bin (128-row segments), input order
            return info;
        }
        int const shape = n <= 16   ? 0
                          : n <= 24 ? 4
                          : n <= 32 ? 1
                          : n <= 48 ? 5
                          : n <= 64 ? 2
                          : n <= 96 ? 6
                                    : 3;
        int m_class = m < 512 ? int(m / 16) : 32 + floor_log2_u64(m) - 9;
        m_class = m_class > short_m_classes_k - 1 ? short_m_classes_k - 1 : m_class;
        info.key = bin_short_begin_k + shape * short_m_classes_k + (short_m_classes_k - 1 - m_class);
        return info;
    }
    if (n > band_rows && fits32_early && !force64) {
        // Long pairs take a band in both forms (16-bit cells when they fit); the plain form keeps them in one bin,
        // in input order.
        int const band_begin = (packed || local_band16) ? bin_band16_begin_k : bin_band_begin_k;
        if (args.force_route >= 0) {
            info.key = band_begin;
            return info;
        }
        int size_class = floor_log2_u64(n * m) - 10;
        size_class = size_class < 0 ? 0 : (size_class > bin_dp_classes_k - 1 ? bin_dp_classes_k - 1 : size_class);
        info.key = band_begin + (bin_dp_classes_k - 1 - size_class);
        return info;
    }
    if (packed) {
        if (args.force_route >= 0) {
            info.key = bin_dp16_begin_k + dp16_classes_per_rows_k; // plain form: one bin (8 rows per lane), input order
            return info;
        }
        // Rows per lane: a tuned choice for the length class, else the least strips(R) x (m + 31) steps x the
        // measured cost of one step with R rows per lane (a strip holds 32 R rows, so the last strip's padding
        // rows count as work).
        int best_choice = 0;
        if (args.packed_rows[length_class]) best_choice = args.packed_rows[length_class] / 4 - 1; // tuned
        else {
            float best_cost = 3.4e38f;
            for (int choice = 0; choice < dp16_row_choices_k; ++choice) {
                std::uint64_t const rows = 4u * (choice + 1);
                std::uint64_t const strips = (n + 32 * rows - 1) / (32 * rows);
                float const cost = (float)strips * (float)(m + 31) * (float)args.packed_step_cost[choice];
                if (cost < best_cost) best_cost = cost, best_choice = choice;
            }
        }
        // Quarter octaves of the shorter side, half octaves of the aspect ratio: the two pairs a warp scores at
        // once come from one bin, so they have nearly the same strips and the same number of steps.
        int n_class = (int)(4.0f * __log2f((float)n)) - 12;
        n_class = n_class < 0 ? 0 : (n_class > 31 ? 31 : n_class);
        int ratio_class = (int)(2.0f * __log2f((float)m / (float)n));
        ratio_class = ratio_class < 0 ? 0 : (ratio_class > 7 ? 7 : ratio_class);
        info.key = bin_dp16_begin_k + best_choice * dp16_classes_per_rows_k + 8 * (31 - n_class) + (7 - ratio_class);
        return info;
    }
    bool const fits32 = reach < (1ull << 31) - 1 && !force64;
    int const base = fits32 ? bin_dp32_begin_k : bin_dp64_begin_k;
    if (args.force_route >= 0) {
        info.key = base; // one bin, input order is kept by the caller's launch
        return info;
    }
    int size_class = floor_log2_u64(n * m) - 10;
    size_class = size_class < 0 ? 0 : (size_class > bin_dp_classes_k - 1 ? bin_dp_classes_k - 1 : size_class);
    info.key = base + (bin_dp_classes_k - 1 - size_class);
    return info;
}

__device__ __forceinline__ pair_route_info_t route_of_pair(plan_args_t const &args, std::uint64_t p) {
    std::uint64_t q, c;
    pair_indices(args, p, q, c);
    std::uint8_t const *first, *second;
    std::uint64_t first_length, second_length;
    tape_string(args.queries, q, first, first_length, args.wide);
    tape_string(args.mode == mode_symmetric_k ? args.queries : args.candidates, c, second, second_length, args.wide);
    return route_pair(args, first, first_length, second, second_length);
}

/** Pass 1: answer trivial pairs, count pairs per bin, track the longest column string and total cells. */
__global__ void plan_count_kernel(plan_args_t const args, plan_bins_t *__restrict__ bins,
                                  std::int64_t *__restrict__ results) {
    __shared__ std::uint32_t histogram[bin_keys_k];
    __shared__ unsigned long long block_cells;
    __shared__ std::uint32_t block_max_cols, block_max_myers, block_max_myers_warp, block_max_chain;
    for (int i = threadIdx.x; i < bin_keys_k; i += blockDim.x) histogram[i] = 0;
    if (threadIdx.x == 0)
        block_cells = 0, block_max_cols = 0, block_max_myers = 0, block_max_myers_warp = 0, block_max_chain = 0;
    __syncthreads();
    std::uint64_t thread_cells = 0;
    std::uint32_t thread_max_cols = 0, thread_max_myers = 0, thread_max_myers_warp = 0, thread_max_chain = 0;
    int const lane = threadIdx.x & 31;
    // Warp-wide rounds, so that the lanes of a warp that share a bin (most of them, in a batch of similar pairs)
    // count with one shared-memory atomic instead of contending for the same counter.
    std::uint64_t const stride = (std::uint64_t)gridDim.x * blockDim.x;
    for (std::uint64_t base = (std::uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < args.pairs;
         base += stride) {
        std::uint64_t const p = base + lane;
        pair_route_info_t info;
        info.key = -1, info.n = info.m = 0;
        if (p < args.pairs) info = route_of_pair(args, p);
        unsigned const key = info.key < 0 ? 0xFFFFFFFFu : (unsigned)info.key;
        unsigned const peers = __match_any_sync(0xFFFFFFFFu, key);
        if (key != 0xFFFFFFFFu && lane == __ffs(peers) - 1) atomicAdd(&histogram[key], (unsigned)__popc(peers));
        if (p >= args.pairs) continue;
        thread_cells += (std::uint64_t)info.n * info.m;
        if (info.key < 0) {
            results[p] = trivial_score(args, info.n, info.m);
            continue;
        }
        if (info.key >= bin_dp32_begin_k) thread_max_cols = max(thread_max_cols, info.m);
        if (info.key >= bin_myers_warp_begin_k && info.key < bin_short_begin_k)
            thread_max_myers_warp = max(thread_max_myers_warp, info.n);
        else if (info.key == bin_myers_chain_k) thread_max_chain = max(thread_max_chain, info.n);
        else if (info.key < bin_myers_begin_k + (myers_max_words_k + 1) * 16)
            thread_max_myers = max(thread_max_myers, info.n);
    }
    // Reduce over the warp first: 32 lanes' atomics on one shared word would serialise.
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1)
        thread_cells += __shfl_xor_sync(0xFFFFFFFFu, thread_cells, offset);
    thread_max_cols = __reduce_max_sync(0xFFFFFFFFu, thread_max_cols);
    thread_max_myers = __reduce_max_sync(0xFFFFFFFFu, thread_max_myers);
    thread_max_myers_warp = __reduce_max_sync(0xFFFFFFFFu, thread_max_myers_warp);
    thread_max_chain = __reduce_max_sync(0xFFFFFFFFu, thread_max_chain);
    if (lane == 0) {
        atomicAdd(&block_cells, (unsigned long long)thread_cells);
        atomicMax(&block_max_cols, thread_max_cols);
        atomicMax(&block_max_myers, thread_max_myers);
        atomicMax(&block_max_myers_warp, thread_max_myers_warp);
        atomicMax(&block_max_chain, thread_max_chain);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < bin_keys_k; i += blockDim.x)
        if (histogram[i]) atomicAdd(&bins->count[i], histogram[i]);
    if (threadIdx.x == 0) {
        atomicAdd((unsigned long long *)&bins->cells, block_cells);
        atomicMax(&bins->max_cols, block_max_cols);
        atomicMax(&bins->max_myers_rows, block_max_myers);
        atomicMax(&bins->max_myers_warp_rows, block_max_myers_warp);
        atomicMax(&bins->max_chain_rows, block_max_chain);
    }
}

/** Pass 2: exclusive scan of bin counts (one CTA of `bin_keys_k / 2` threads, two adjacent keys each). */
__global__ void plan_scan_kernel(plan_bins_t *__restrict__ bins) {
    constexpr int threads = bin_keys_k / 2;
    __shared__ std::uint32_t scan[threads];
    int const i = threadIdx.x;
    std::uint32_t const first = bins->count[2 * i], second = bins->count[2 * i + 1];
    std::uint32_t const own = first + second;
    scan[i] = own;
    __syncthreads();
    for (int offset = 1; offset < threads; offset <<= 1) {
        std::uint32_t const add = i >= offset ? scan[i - offset] : 0u;
        __syncthreads();
        scan[i] += add;
        __syncthreads();
    }
    std::uint32_t const before = scan[i] - own;
    bins->begin[2 * i] = before;
    bins->begin[2 * i + 1] = before + first;
    bins->fill[2 * i] = bins->fill[2 * i + 1] = 0;
    bins->cursor[2 * i] = bins->cursor[2 * i + 1] = 0;
    if (i == threads - 1) bins->scheduled = scan[i];
}

/**
 *  Pass 3: write each routed pair into its bin. A CTA takes one contiguous range of pairs: it counts the range's
 *  pairs per bin in shared memory, reserves each bin's slots with one global atomic, then routes the range again and
 *  places every pair at its reserved base plus a shared-memory rank. Lanes of a warp that share a bin take their
 *  ranks with one atomic in both passes.
 */
__global__ void plan_scatter_kernel(plan_args_t const args, plan_bins_t *__restrict__ bins,
                                    pair_task_t *__restrict__ tasks) {
    __shared__ std::uint32_t counts[bin_keys_k];
    __shared__ std::uint32_t bases[bin_keys_k];
    int const lane = threadIdx.x & 31;
    std::uint64_t const per_block = (args.pairs + gridDim.x - 1) / gridDim.x;
    std::uint64_t const begin = min(args.pairs, (std::uint64_t)blockIdx.x * per_block);
    std::uint64_t const end = min(args.pairs, begin + per_block);
    for (int i = threadIdx.x; i < bin_keys_k; i += blockDim.x) counts[i] = 0;
    __syncthreads();
    // A warp's lanes that share a bin: one shared-memory atomic for all of them; returns this lane's rank.
    auto claim = [&](unsigned key) -> std::uint32_t {
        unsigned const peers = __match_any_sync(0xFFFFFFFFu, key);
        int const leader = __ffs(peers) - 1;
        std::uint32_t first = 0;
        if (lane == leader && key != 0xFFFFFFFFu) first = atomicAdd(&counts[key], (unsigned)__popc(peers));
        first = __shfl_sync(0xFFFFFFFFu, first, leader);
        return first + __popc(peers & ((1u << lane) - 1u));
    };
    // The range is walked in warp-wide rounds so every lane of a warp takes part in each `claim`.
    std::uint64_t const rounds_begin = begin + (threadIdx.x & ~31u);
    for (std::uint64_t base = rounds_begin; base < end; base += blockDim.x) {
        std::uint64_t const p = base + lane;
        pair_route_info_t info;
        info.key = -1;
        if (p < end) info = route_of_pair(args, p);
        claim(info.key < 0 ? 0xFFFFFFFFu : (unsigned)info.key);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < bin_keys_k; i += blockDim.x) {
        std::uint32_t const here = counts[i];
        bases[i] = here ? bins->begin[i] + atomicAdd(&bins->fill[i], here) : 0u;
        counts[i] = 0;
    }
    __syncthreads();
    for (std::uint64_t base = rounds_begin; base < end; base += blockDim.x) {
        std::uint64_t const p = base + lane;
        pair_route_info_t info;
        info.key = -1;
        if (p < end) info = route_of_pair(args, p);
        unsigned const key = info.key < 0 ? 0xFFFFFFFFu : (unsigned)info.key;
        std::uint32_t const rank = claim(key);
        if (key != 0xFFFFFFFFu) {
            pair_task_t task;
            task.rows = info.rows, task.cols = info.cols;
            task.rows_length = info.n, task.cols_length = info.m;
            task.slot = (std::uint32_t)p;
            task.transposed = info.transposed;
            tasks[bases[key] + rank] = task;
        }
    }
}

/** Marks every byte value present in a tape's data range [offsets[0], offsets[count]), read on the device; 16 bytes
 *  per load where aligned. Grid-stride over the CTAs given to the tape: the first `tape_ctas` CTAs take `first`, the
 *  others `second` (both passes run in one launch, so their loads overlap). */
__global__ void alphabet_mark_kernel(tape_t const first_tape, tape_t const second_tape, unsigned tape_ctas,
                                     std::uint64_t sample_bytes, std::uint32_t *__restrict__ symbol_mask) {
    bool const on_second = blockIdx.x >= tape_ctas;
    tape_t const &tape = on_second ? second_tape : first_tape;
    unsigned const block = on_second ? blockIdx.x - tape_ctas : blockIdx.x;
    unsigned const blocks = on_second ? gridDim.x - tape_ctas : tape_ctas;
    // One flag byte per symbol, set with plain stores (every writer stores 1), folded into the mask at the end.
    __shared__ __align__(16) std::uint8_t seen[256];
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x) seen[i] = 0;
    __syncthreads();
    std::uint64_t first, last;
    if (tape.offset_bits == 32) {
        auto const *offsets = static_cast<std::uint32_t const *>(tape.offsets);
        first = offsets[0], last = offsets[tape.count];
    }
    else {
        auto const *offsets = static_cast<std::uint64_t const *>(tape.offsets);
        first = offsets[0], last = offsets[tape.count];
    }
    std::uint8_t const *data = tape.base + first;
    std::uint64_t const length = sample_bytes && last - first > sample_bytes ? sample_bytes : last - first;
    std::uintptr_t const address = reinterpret_cast<std::uintptr_t>(data);
    std::uint64_t head = (16 - (address & 15)) & 15;
    if (head > length) head = length;
    std::uint64_t const thread = (std::uint64_t)block * blockDim.x + threadIdx.x;
    std::uint64_t const threads = (std::uint64_t)blocks * blockDim.x;
    if (thread < head) seen[data[thread]] = 1;
    std::uint64_t const body = (length - head) / 16;
    uint4 const *vectors = reinterpret_cast<uint4 const *>(data + head);
    // Four 16-byte loads in flight per thread before their flags are stored (the pass is bound by HBM).
    constexpr int unroll = 4;
    for (std::uint64_t v0 = thread; v0 < body; v0 += threads * unroll) {
        uint4 x[unroll];
#pragma unroll
        for (int u = 0; u < unroll; ++u) {
            std::uint64_t const v = v0 + u * threads;
            // Past the end: repeat the first byte, which is in the data (body > 0 implies length >= 16).
            std::uint32_t const filler = std::uint32_t(data[head]) * 0x01010101u;
            x[u] = v < body ? __ldcs(vectors + v) : make_uint4(filler, filler, filler, filler);
        }
#pragma unroll
        for (int u = 0; u < unroll; ++u) {
            std::uint32_t const words[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int s = 0; s < 32; s += 8) seen[(words[k] >> s) & 0xFF] = 1;
        }
    }
    std::uint64_t const tail_begin = head + body * 16;
    if (thread < length - tail_begin) seen[data[tail_begin + thread]] = 1;
    __syncthreads();
    if (threadIdx.x < 8) {
        std::uint32_t word = 0;
        for (int b = 0; b < 32; ++b) word |= std::uint32_t(seen[threadIdx.x * 32 + b] != 0) << b;
        if (word) atomicOr(&symbol_mask[threadIdx.x], word);
    }
}

/** Dense codes for the marked bytes; `bits` = planes the Myers kernel needs (1..8). Clears the mask afterwards so
 *  the next call starts from zero. */
__global__ void alphabet_codes_kernel(std::uint32_t *__restrict__ symbol_mask,
                                      batch_alphabet_t *__restrict__ alphabet) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    std::uint32_t next = 0;
    for (int b = 0; b < 256; ++b) {
        bool const present = (symbol_mask[b >> 5] >> (b & 31)) & 1u;
        alphabet->code[b] = present ? (std::uint8_t)next : 0;
        next += present;
    }
    std::uint32_t bits = 1;
    while ((1u << bits) < next) ++bits;
    alphabet->symbols = next;
    alphabet->bits = bits;
    for (int k = 0; k < 8; ++k) alphabet->present[k] = symbol_mask[k], symbol_mask[k] = 0;
}

/** Dense per-pair results into the caller's matrix (device-resident output). */
__global__ void scatter_output_kernel(plan_args_t const args, std::int64_t const *__restrict__ results,
                                      std::int64_t *__restrict__ out, std::uint64_t stride) {
    for (std::uint64_t p = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < args.pairs;
         p += (std::uint64_t)gridDim.x * blockDim.x) {
        std::int64_t const value = results[p];
        if (args.mode == mode_pairwise_k) {
            out[p] = value;
            continue;
        }
        std::uint64_t q, c;
        pair_indices(args, p, q, c);
        out[q * stride + c] = value;
        if (args.mode == mode_symmetric_k && q != c) out[c * stride + q] = value;
    }
}

/** Launches @p kernel with its stream's priority as an explicit launch attribute, so that a graph captured from a
 *  high-priority stream keeps the priority in its kernel nodes (the planning of pipelined chunks runs ahead of
 *  queued scoring). */
template <typename... params_, typename... args_>
static cudaError_t launch_prioritised(void (*kernel)(params_...), unsigned grid, unsigned block, cudaStream_t stream,
                                      args_ const &...args) {
    int priority = 0;
    cudaError_t const queried = cudaStreamGetPriority(stream, &priority);
    if (queried != cudaSuccess) return queried;
    cudaLaunchConfig_t config = {};
    config.gridDim = dim3(grid);
    config.blockDim = dim3(block);
    config.stream = stream;
    cudaLaunchAttribute attribute;
    attribute.id = cudaLaunchAttributePriority;
    attribute.val.priority = priority;
    config.attrs = &attribute;
    config.numAttrs = 1;
    return cudaLaunchKernelEx(&config, kernel, args...);
}

static int grid_for(std::uint64_t items, int block, int sm_count, int per_sm = 8) {
    std::uint64_t const needed = (items + block - 1) / block;
    std::uint64_t const cap = (std::uint64_t)sm_count * per_sm;
    return (int)(needed < cap ? (needed ? needed : 1) : cap);
}

cudaError_t launch_plan(plan_args_t const &args, plan_bins_t *bins, pair_task_t *tasks, std::int64_t *results,
                        int sm_count, cudaStream_t stream) {
    cudaError_t status = cudaMemsetAsync(bins, 0, sizeof(plan_bins_t), stream);
    if (status != cudaSuccess) return status;
    if (args.pairs == 0) return cudaSuccess;
    status = launch_prioritised(plan_count_kernel, grid_for(args.pairs, 256, sm_count), 256, stream, args, bins, results);
    if (status != cudaSuccess) return status;
    status = launch_prioritised(plan_scan_kernel, 1, bin_keys_k / 2, stream, bins);
    if (status != cudaSuccess) return status;
    return launch_prioritised(plan_scatter_kernel, grid_for(args.pairs, 256, sm_count), 256, stream, args, bins, tasks);
}

cudaError_t launch_alphabet(tape_t const &queries, tape_t const &candidates, bool has_candidates,
                            batch_alphabet_t *alphabet, int sm_count, cudaStream_t stream, std::uint64_t sample_bytes) {
    std::uint32_t *mask = alphabet->mask_scratch;
    // A sample needs few CTAs: 16 bytes per thread and load.
    unsigned const per_tape = sample_bytes ? (unsigned)std::min<std::uint64_t>((std::uint64_t)sm_count * 8,
                                                                                sample_bytes / (256 * 16 * 4) + 1)
                                           : (unsigned)sm_count * 8;
    cudaError_t const status = launch_prioritised(alphabet_mark_kernel, has_candidates ? 2 * per_tape : per_tape, 256,
                                                  stream, queries, has_candidates ? candidates : queries, per_tape,
                                                  sample_bytes, mask);
    if (status != cudaSuccess) return status;
    return launch_prioritised(alphabet_codes_kernel, 1, 32, stream, mask, alphabet);
}

cudaError_t launch_scatter_output(plan_args_t const &args, std::int64_t const *results, std::int64_t *out,
                                  std::uint64_t stride, int sm_count, cudaStream_t stream) {
    if (args.pairs == 0) return cudaSuccess;
    scatter_output_kernel<<<grid_for(args.pairs, 256, sm_count), 256, 0, stream>>>(args, results, out, stride);
    return cudaGetLastError();
}

} // namespace szs_gb300
