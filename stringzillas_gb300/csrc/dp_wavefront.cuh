/**
 *  @file dp_wavefront.cuh
 *  @brief Warp-per-pair anti-diagonal wavefront for Levenshtein / Needleman-Wunsch / Smith-Waterman scores.
 *
 *  Layout of one pair inside a warp:
 *  - The rows string (length n) is cut into strips of `32 * R` rows. In a strip, lane `L` owns rows
 *    `L*R .. L*R+R-1` and keeps, in registers, their H (and affine E) values of the previous column.
 *  - The columns string (length m) is streamed: at step `t`, lane `L` updates column `j = t + 1 - L`, so the warp
 *    sweeps an anti-diagonal of 32 register tiles. The bottom H (and F) of lane `L`'s tile reach lane `L+1`
 *    through `__shfl_up_sync` one step later, together with the column's character class: no shared-memory round
 *    trip and no barrier inside a strip.
 *  - Lane 0 takes its "up" values from the strip's top boundary: the closed-form row 0 for the first strip, or the
 *    previous strip's bottom row, which lane 31 wrote to the warp's scratch row in global memory (L2-resident).
 *  - Substitution costs of a class table come from a per-warp shared-memory profile `profile[column class][row]`
 *    (int8), so each lane fetches its R costs with one 8-byte load per column; uniform (Levenshtein) costs compare
 *    bytes held in registers.
 *
 *  This replaces the reference's warp tier (include/stringzillas/similarities/cuda.cuh:1123-1452 with the Hopper
 *  `tile_scorer`s of hopper.cuh:38-539), which keeps three (seven) anti-diagonals in shared memory and
 *  synchronises the warp once per diagonal. Results equal the serial recurrences
 *  (include/stringzillas/similarities/serial.hpp:663-1079) bit for bit.
 */
#pragma once
#include <type_traits>
#include "dp_cells.cuh"
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

constexpr int warp_size_k = 32;

/** Compile-time description of one wavefront kernel instance. */
template <int kind_, bool affine_, typename cell_type_, int rows_per_lane_>
struct dp_policy_t {
    static constexpr int kind_k = kind_;
    static constexpr bool affine_k = affine_;
    static constexpr bool maximize_k = kind_ != kind_levenshtein_k;
    static constexpr bool local_k = kind_ == kind_smith_waterman_k;
    static constexpr bool uniform_k = kind_ == kind_levenshtein_k; // byte equality instead of a class table
    static constexpr int rows_per_lane_k = rows_per_lane_;
    static constexpr int strip_rows_k = warp_size_k * rows_per_lane_;
    static constexpr bool direct_k = false; // substitution costs from per-warp class profiles
    static constexpr bool wide_k = false;   // strings of bytes (16-bit codes: `wide_policy_t<>`)
    using cell_t = cell_type_;
    using ops_t = cell_ops_t<cell_t, maximize_k>;
};

/** The same kernel reading substitution costs straight from a dense 256 x 256 table that each CTA stages in shared
 *  memory (dense-table calls over more than 32 distinct bytes, which no 32-class profile can hold). */
template <typename policy_>
struct direct_policy_t : policy_ {
    static constexpr bool direct_k = true;
};

/** The same kernel over strings of 16-bit codes (UTF-8 Levenshtein over more than 256 code points); uniform costs. */
template <typename policy_>
struct wide_policy_t : policy_ {
    static_assert(policy_::uniform_k, "16-bit codes are compared, not looked up in a table");
    static constexpr bool wide_k = true;
};

constexpr int direct_table_bytes_k = 256 * 256;

/** Shared-memory bytes one warp needs for its substitution profile over @p classes column classes. */
template <typename policy_>
__host__ __device__ constexpr int dp_profile_bytes_per_warp(int classes) {
    return (policy_::uniform_k || policy_::direct_k) ? 0 : classes * policy_::strip_rows_k;
}

/** Shared-memory bytes of one CTA: the staged costs plus one profile per warp (or the direct table). */
template <typename policy_>
__host__ __device__ constexpr int dp_shared_bytes(int warps_per_cta, int classes) {
    return int((sizeof(score_costs_t) + 15) / 16 * 16) + warps_per_cta * dp_profile_bytes_per_warp<policy_>(classes) +
           (policy_::direct_k ? direct_table_bytes_k : 0);
}

/** Copies the dense table into the CTA's shared memory (16 bytes per load); the caller synchronises. */
__device__ __forceinline__ void stage_direct_table(std::int8_t const *table, std::int8_t *table_s) {
    auto const *src = reinterpret_cast<uint4 const *>(table);
    auto *dst = reinterpret_cast<uint4 *>(table_s);
    for (unsigned i = threadIdx.x; i < direct_table_bytes_k / 16; i += blockDim.x) dst[i] = src[i];
}

/**
 *  Scores one pair with one warp. All 32 lanes must call it with the same task.
 *  @param scratch  this warp's scratch row: (m + 1) x 2 cells, used only when n spans several strips.
 *  @param profile  this warp's shared-memory profile area (class-table engines only).
 *  @param costs    the engine costs, in shared memory.
 */
template <typename policy_>
__device__ __forceinline__ std::int64_t dp_score_pair_warp(pair_task_t const &task, score_costs_t const &costs,
                                                           typename policy_::cell_t *scratch, std::int8_t *profile,
                                                           std::int8_t const *table_s = nullptr) {
    using cell_t = typename policy_::cell_t;
    using ops = typename policy_::ops_t;
    constexpr int R = policy_::rows_per_lane_k;
    constexpr int S = policy_::strip_rows_k;
    constexpr bool affine = policy_::affine_k;
    constexpr bool local = policy_::local_k;

    int const lane = threadIdx.x & 31;
    std::uint32_t const n = task.rows_length, m = task.cols_length;
    cell_t const open = (cell_t)costs.open, extend = (cell_t)costs.extend;
    cell_t const gap = open; // linear gap cost
    boundary_t<cell_t> const edge {open, extend, affine, local};
    std::int8_t const *table = task.transposed ? costs.profile_table_t : costs.profile_table;

    cell_t result = 0;
    cell_t lane_best = 0; // local scores: running maximum over valid cells, starts at 0 like the reference

    for (std::uint32_t strip_base = 0; strip_base < n; strip_base += S) {
        std::uint32_t const rows_here = min((std::uint32_t)S, n - strip_base);
        bool const last_strip = strip_base + S >= n;
        int const last_lane = int((rows_here - 1) / R);
        // First row (1-based) owned by this lane.
        std::int64_t const row0 = (std::int64_t)strip_base + lane * R + 1;

        // Row characters: uniform costs compare bytes, class tables go through the per-warp profile.
        std::uint32_t row_bytes[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::int64_t const i = row0 + r;
            row_bytes[r] = i <= (std::int64_t)n ? symbol_at<policy_::wide_k>(task.rows, i - 1) : 0u;
        }
        // Dense tables: each row's part of the table index, oriented once per strip (the column's part is one shift
        // per step), so a cell's gather address is one OR.
        if constexpr (policy_::direct_k) {
#pragma unroll
            for (int r = 0; r < R; ++r) row_bytes[r] = task.transposed ? row_bytes[r] : row_bytes[r] << 8;
        }
        if constexpr (!policy_::uniform_k && !policy_::direct_k) {
            // profile[cc * S + row_in_strip] = cost(row class, column class cc), oriented by `transposed`.
            __syncwarp();
            int const classes = costs.classes;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                int const row_class = costs.byte_to_class[row_bytes[r]];
                for (int cc = 0; cc < classes; ++cc)
                    profile[cc * S + lane * R + r] = table[cc * 32 + row_class];
            }
            __syncwarp();
        }

        // Left boundary (column 0) of this lane's rows.
        cell_t h_col[R], e_col[R], best_row[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            h_col[r] = edge.score(row0 + r);
            e_col[r] = affine ? edge.gap(row0 + r) : 0;
            best_row[r] = 0;
        }
        // Diagonal seed: H of the row above this lane's first row, at column 0.
        cell_t diag_up = edge.score(row0 - 1);

        // Lane 0's top-boundary source.
        std::conditional_t<policy_::wide_k, code16_stream_t, byte_stream_t> column_stream;
        column_stream.open_at(task.cols);
        cell_t const *top = scratch;
        auto top_h = [&](std::uint32_t j) -> cell_t {
            return strip_base == 0 ? edge.score(j) : top[2 * j + 0];
        };
        auto top_f = [&](std::uint32_t j) -> cell_t {
            return strip_base == 0 ? edge.gap(j) : top[2 * j + 1];
        };
        auto column_code = [&](std::uint32_t byte) -> int {
            if constexpr (policy_::uniform_k || policy_::direct_k) return int(byte);
            else return costs.byte_to_compact[byte];
        };
        // Prefetched inputs of lane 0 for its next column.
        cell_t next_h = 0, next_f = 0;
        int next_code = 0;
        if (lane == 0) {
            next_h = top_h(1);
            next_f = affine ? top_f(1) : 0;
            next_code = column_code(column_stream.next());
        }

        cell_t out_h = 0, out_f = 0;
        int out_code = 0;
        std::uint32_t const steps = m + (std::uint32_t)last_lane;
        bool const write_bottom = !last_strip;
        // One step of the sweep. `steady` steps are those where all 32 lanes hold rows of a full strip and real
        // columns (31 <= t < m): no range predicates.
        auto step = [&](std::uint32_t t, auto steady_tag) {
            constexpr bool steady = decltype(steady_tag)::value;
            cell_t up_h = __shfl_up_sync(0xFFFFFFFFu, out_h, 1);
            cell_t up_f = affine ? __shfl_up_sync(0xFFFFFFFFu, out_f, 1) : 0;
            int code = __shfl_up_sync(0xFFFFFFFFu, out_code, 1);
            if (lane == 0) {
                up_h = next_h, up_f = next_f, code = next_code;
                std::uint32_t const j_next = t + 2;
                if (j_next <= m) {
                    next_h = top_h(j_next);
                    if (affine) next_f = top_f(j_next);
                    next_code = column_code(column_stream.next());
                }
            }
            std::int64_t const j = (std::int64_t)t + 1 - lane;
            if (steady || (j >= 1 && j <= (std::int64_t)m && lane <= last_lane)) {
                cell_t diag = diag_up;
                diag_up = up_h;
                cell_t h_up = up_h, f_up = up_f;
                // Substitution costs of this lane's rows against the column character.
                cell_t subs[R];
                if constexpr (policy_::uniform_k) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        subs[r] = (row_bytes[r] == (std::uint32_t)code) ? (cell_t)costs.match : (cell_t)costs.mismatch;
                }
                else if constexpr (policy_::direct_k) {
                    // table[first byte][second byte]: rows are the first string unless the pair was transposed.
                    std::uint32_t const column_key = task.transposed ? (std::uint32_t)code << 8 : (std::uint32_t)code;
#pragma unroll
                    for (int r = 0; r < R; ++r) subs[r] = (cell_t)table_s[row_bytes[r] | column_key];
                }
                else {
                    static_assert(R % 8 == 0, "profile loads are 8 bytes wide");
#pragma unroll
                    for (int r8 = 0; r8 < R; r8 += 8) {
                        uint2 const packed = *reinterpret_cast<uint2 const *>(profile + code * S + lane * R + r8);
                        // One byte permute per cost (the byte, its sign bit copied above it).
                        subs[r8 + 0] = (cell_t)signed_byte<0>(packed.x), subs[r8 + 1] = (cell_t)signed_byte<1>(packed.x);
                        subs[r8 + 2] = (cell_t)signed_byte<2>(packed.x), subs[r8 + 3] = (cell_t)signed_byte<3>(packed.x);
                        subs[r8 + 4] = (cell_t)signed_byte<0>(packed.y), subs[r8 + 5] = (cell_t)signed_byte<1>(packed.y);
                        subs[r8 + 6] = (cell_t)signed_byte<2>(packed.y), subs[r8 + 7] = (cell_t)signed_byte<3>(packed.y);
                    }
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    cell_t h;
                    if constexpr (affine) {
                        cell_t const e = ops::add_opt(e_col[r], extend, h_col[r] + open);
                        cell_t const f = ops::add_opt(f_up, extend, h_up + open);
                        if constexpr (local) h = ops::opt3_relu(diag + subs[r], e, f);
                        else h = ops::opt3(diag + subs[r], e, f);
                        e_col[r] = e;
                        f_up = f;
                    }
                    else {
                        if constexpr (local) h = ops::add_opt_relu(ops::opt2(h_up, h_col[r]), gap, diag + subs[r]);
                        else h = ops::add_opt(ops::opt2(h_up, h_col[r]), gap, diag + subs[r]);
                    }
                    diag = h_col[r];
                    h_col[r] = h;
                    h_up = h;
                    if constexpr (local) best_row[r] = max(best_row[r], h);
                }
                out_h = h_up, out_f = f_up, out_code = code;
                if (write_bottom && lane == 31) {
                    scratch[2 * j + 0] = out_h;
                    if (affine) scratch[2 * j + 1] = out_f;
                }
            }
        };
        std::uint32_t const fill_end = min(steps, 31u);
        std::uint32_t const steady_end = (last_lane == 31 && m >= 32u) ? max(fill_end, min(steps, m)) : fill_end;
        std::uint32_t t = 0;
        for (; t < fill_end; ++t) step(t, std::false_type {});
        // Two steps per iteration: the row state alternates between two register sets instead of being copied back.
#pragma unroll 2
        for (; t < steady_end; ++t) step(t, std::true_type {});
        for (; t < steps; ++t) step(t, std::false_type {});
        // Fold this strip's contribution.
        if constexpr (local) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (row0 + r <= (std::int64_t)n) lane_best = max(lane_best, best_row[r]);
        }
        else if (last_strip) {
            int const bottom_row = int((rows_here - 1) % R);
            cell_t h_last = h_col[0];
#pragma unroll
            for (int r = 1; r < R; ++r)
                if (r == bottom_row) h_last = h_col[r];
            result = __shfl_sync(0xFFFFFFFFu, h_last, last_lane);
        }
        __syncwarp();
    }
    if constexpr (local) {
#pragma unroll
        for (int offset = 16; offset > 0; offset >>= 1)
            lane_best = max(lane_best, __shfl_xor_sync(0xFFFFFFFFu, lane_best, offset));
        result = lane_best;
    }
    return (std::int64_t)result;
}

/**
 *  Persistent wavefront kernel over the scheduled range of one route. Warps pull pairs from a shared cursor, so a
 *  few long pairs cannot stall a CTA while the others idle.
 */
template <typename policy_>
__global__ void __launch_bounds__(256) dp_wavefront_kernel(pair_task_t const *__restrict__ tasks,
                                                           plan_bins_t *__restrict__ bins, int key_begin, int key_end,
                                                           score_costs_t const costs, std::int64_t *__restrict__ results,
                                                           typename policy_::cell_t *__restrict__ scratch,
                                                           std::size_t scratch_cells_per_warp) {
    using cell_t = typename policy_::cell_t;
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + ((sizeof(score_costs_t) + 15) / 16) * 16);

    // Stage the cost tables in shared memory once per CTA.
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    if constexpr (policy_::direct_k) stage_direct_table(costs.direct_table, profiles);
    __syncthreads();

    int const lane = threadIdx.x & 31;
    int const warp_in_cta = threadIdx.x >> 5;
    std::size_t const global_warp = (std::size_t)blockIdx.x * (blockDim.x >> 5) + warp_in_cta;
    cell_t *warp_scratch = scratch + global_warp * scratch_cells_per_warp;
    std::int8_t *warp_profile = profiles + warp_in_cta * dp_profile_bytes_per_warp<policy_>(costs.classes);

    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    while (true) {
        std::uint32_t index = 0;
        if (lane == 0) index = atomicAdd(&bins->cursor[key_begin], 1u);
        index = __shfl_sync(0xFFFFFFFFu, index, 0);
        if (index >= count) break;
        pair_task_t const task = tasks[begin + index];
        std::int64_t const score = dp_score_pair_warp<policy_>(task, costs_s, warp_scratch, warp_profile, profiles);
        if (lane == 0) results[task.slot] = score;
    }
}

} // namespace szs_gb300
