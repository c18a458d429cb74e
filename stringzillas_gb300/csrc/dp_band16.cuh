/**
 *  @file dp_band16.cuh
 *  @brief Long pairs on 16x2 packed cells: one CTA per pair, each warp scoring two row strips of it at once.
 *
 *  The band kernel (dp_band.cuh) gives a long pair a CTA whose warps form a ring of row strips. Here the cells are
 *  16-bit and every warp carries two consecutive strips of the same pair: strip 2s in the low halves and strip
 *  2s + 1 in the high halves of its registers (a "super-strip" of 64 R rows). The high halves run the same sweep
 *  32 columns behind the low halves: lane 0's high half takes its "up" values from lane 31's low half of the previous
 *  step (a rotating shuffle instead of `__shfl_up_sync`), so the boundary between the two strips never leaves the
 *  registers. Both halves read their substitution costs from two per-warp profiles interleaved by one byte permute,
 *  and the cell update is that of the 16x2 warp route (dp_packed.cuh): five DPX operations per two cells for affine
 *  gaps. Global scores come here only when the reference's worst-case reach proves every value fits int16. Local
 *  scores with non-positive gaps come here whatever their length: while every cell stays below 32767 minus the
 *  largest substitution gain, no 16-bit value can have wrapped (each cell is exact given exact neighbours below the
 *  limit, and the first cell to reach the limit is itself exact and lands in the running maximum), so a pair whose
 *  maximum stays below the limit is exact, and one that reaches it is scored again on 32-bit cells by the same CTA.
 *
 *  Super-strips form the ring of the band kernel: super-strip k writes its bottom row (packed H + open and F per
 *  column) into slot k mod W, super-strip k + 1 reads it as its top; progress words and bounded waits are those of
 *  dp_band.cuh. Replaces, like the band kernel, the reference's device tier (include/stringzillas/similarities/
 *  cuda.cuh:616-1096).
 */
#pragma once
#include <type_traits>

#include "dp_band.cuh"
#include "dp_packed.cuh"

namespace szs_gb300 {

/** `compare_`: Levenshtein over more than 32 byte values, costs from comparing codes (`compare_mode_t`); `wide_`
 *  (compare modes only): strings of 16-bit codes. */
template <int kind_, bool affine_, int rows_per_lane_, int compare_ = compare_none_k, bool wide_ = false,
          int columns_per_step_ = 1>
struct band16_policy_t {
    static constexpr int kind_k = kind_;
    static constexpr bool affine_k = affine_;
    static constexpr bool maximize_k = kind_ != kind_levenshtein_k;
    static constexpr bool local_k = kind_ == kind_smith_waterman_k;
    static constexpr int rows_per_lane_k = rows_per_lane_;
    static constexpr int strip_rows_k = warp_size_k * rows_per_lane_; // rows of one half
    static constexpr int super_rows_k = 2 * strip_rows_k;             // rows of one warp's super-strip
    static constexpr bool compare_k = compare_ != compare_none_k;
    static constexpr bool multiply_k = compare_ == compare_multiply_k;
    static constexpr bool wide_k = wide_;
    static constexpr int columns_k = columns_per_step_; // columns each half of a lane scores per step: 1 or 2
    static_assert(!compare_k || kind_ == kind_levenshtein_k, "only Levenshtein costs are a function of equality");
    static_assert(!wide_ || compare_k, "16-bit codes have no profile");
};

constexpr int band16_chunk_k = 64; // lane 0's top values and codes are staged, waited for and published 64 at a time

/** Per-warp staging of lane 0's inputs: packed (H + open, F) of the top row, low-half column codes. */
struct band16_chunk_t {
    std::uint32_t top[band16_chunk_k];
    std::uint32_t code[band16_chunk_k];
};

template <typename policy_>
__host__ __device__ constexpr int band16_profile_bytes_per_warp(int classes) {
    return policy_::compare_k ? 0 : 2 * classes * policy_::strip_rows_k;
}

template <typename policy_>
__host__ __device__ constexpr int band16_shared_bytes(int classes) {
    return int((sizeof(score_costs_t) + 15) / 16 * 16) + int((sizeof(band_shared_t) + 15) / 16 * 16) +
           band_warps_k * (band16_profile_bytes_per_warp<policy_>(classes) + int(sizeof(band16_chunk_t)));
}

/**
 *  Scores super-strips w, w + W, ... of one pair with warp w. Returns the warp's contribution: the running maximum of
 *  its valid cells for local scores, the corner cell for the warp owning row n of global scores (else 0).
 */
template <typename policy_>
__device__ __forceinline__ std::int32_t band16_score_warp(pair_task_t const &task, score_costs_t const &costs,
                                                          band_ring_t const &sync, std::uint32_t *ring,
                                                          std::size_t ring_words_per_slot, std::int8_t *profile,
                                                          band16_chunk_t &chunk) {
    using ops = packed_ops_t<policy_::maximize_k>;
    constexpr int R = policy_::rows_per_lane_k;
    constexpr int S = policy_::strip_rows_k;
    constexpr int SS = policy_::super_rows_k;
    constexpr bool affine = policy_::affine_k;
    constexpr bool local = policy_::local_k;
    std::uint32_t const W = (std::uint32_t)sync.members;
    int const warp = sync.member;
    constexpr bool compare = policy_::compare_k;
    static_assert(R % 4 == 0, "profile rows are read in 4-byte words");
    constexpr int words = compare ? 1 : R / 4; // profile words per half (unused in compare mode)

    int const lane = threadIdx.x & 31;
    int const from_lane = (lane + 31) & 31; // the lane whose previous outputs feed this lane
    std::uint32_t const n = task.rows_length, m = task.cols_length;
    std::int32_t const open = costs.open, extend = costs.extend;
    std::uint32_t const open2 = pack16(open, open), extend2 = pack16(extend, extend);
    boundary_t<std::int32_t> const edge {open, extend, affine, local};
    int const classes = costs.classes;
    std::int8_t const *table = task.transposed ? costs.profile_table_t : costs.profile_table;
    std::int8_t *profile_lo = profile;
    std::int8_t *profile_hi = profile + classes * S;
    std::int32_t const h_shift = affine ? open : 0; // affine tracks carry H + open (see dp_packed.cuh)
    auto gap_seed = [&](std::int64_t i) -> std::int32_t {
        return local ? open + extend : open + extend + edge.score(i);
    };
    // The code of column j; in compare mode negated within 16 bits (see compare_costs_t).
    auto column_code = [&](std::uint32_t j) -> std::uint32_t {
        std::uint32_t const c =
            policy_::wide_k ? symbol_at<true>(task.cols, j - 1) : (std::uint32_t)costs.byte_to_compact[task.cols[j - 1]];
        return compare ? (0u - c) & 0xFFFFu : c;
    };
    // Compare mode: costs of equal and different codes, shifted like the profile for affine tracks.
    compare_costs_t const compared(costs.match - h_shift, costs.mismatch - h_shift);

    std::uint32_t const super_strips = (n + SS - 1) / SS;
    std::int32_t result = 0;
    std::uint32_t lane_best = 0;
    int const lane_rows = lane * R;

    for (std::uint32_t k = (std::uint32_t)warp; k < super_strips; k += W) {
        std::uint32_t const base = k * SS;
        std::uint32_t const rows_here = min((std::uint32_t)SS, n - base);
        bool const last_strip = k + 1 == super_strips;
        int const last_vlane = int((rows_here - 1) / R); // 0..63: lanes 32.. are the high halves
        std::int64_t const row0_lo = (std::int64_t)base + lane_rows + 1, row0_hi = row0_lo + S;
        int const slot_in = int((k + W - 1) % W), slot_out = int(k % W);
        std::uint32_t const *top = ring + (std::size_t)slot_in * ring_words_per_slot;
        std::uint32_t *bottom = ring + (std::size_t)slot_out * ring_words_per_slot;

        std::uint32_t row_codes[compare ? R : 1]; // compare mode: both halves' row codes instead of profiles
        __syncwarp();
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::int64_t const i_lo = row0_lo + r, i_hi = row0_hi + r;
            if constexpr (policy_::wide_k) {
                std::uint32_t const code_lo = i_lo <= (std::int64_t)n ? symbol_at<true>(task.rows, i_lo - 1) : 0u;
                std::uint32_t const code_hi = i_hi <= (std::int64_t)n ? symbol_at<true>(task.rows, i_hi - 1) : 0u;
                row_codes[r] = code_lo | (code_hi << 16);
                continue;
            }
            int const class_lo = costs.byte_to_class[i_lo <= (std::int64_t)n ? task.rows[i_lo - 1] : 0u];
            int const class_hi = costs.byte_to_class[i_hi <= (std::int64_t)n ? task.rows[i_hi - 1] : 0u];
            if constexpr (compare) row_codes[r] = std::uint32_t(class_lo) | (std::uint32_t(class_hi) << 16);
            else
                for (int cc = 0; cc < classes; ++cc) {
                    profile_lo[cc * S + lane_rows + r] = std::int8_t(table[cc * 32 + class_lo] - h_shift);
                    profile_hi[cc * S + lane_rows + r] = std::int8_t(table[cc * 32 + class_hi] - h_shift);
                }
        }
        std::uint32_t h_col[R], e_col[R], best_row[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            h_col[r] = pack16(edge.score(row0_lo + r) + h_shift, edge.score(row0_hi + r) + h_shift);
            e_col[r] = pack16(gap_seed(row0_lo + r), gap_seed(row0_hi + r));
            best_row[r] = 0;
        }
        std::uint32_t diag_up = pack16(edge.score(row0_lo - 1) + h_shift, edge.score(row0_hi - 1) + h_shift);

        // The lane, half and row holding row n (global scores, last super-strip only).
        int const v_n = int((n - 1 - base) / R), r_n = int((n - 1 - base) % R);
        int const capture_lane = last_strip ? (v_n & 31) : -1;
        bool const capture_hi = v_n >= 32;

        bool const bottom_writer = !last_strip && lane == 31;
        bool healthy = true;
        if constexpr (policy_::columns_k == 1) {
            std::uint32_t const steps = m + (std::uint32_t)last_vlane;
            std::uint32_t out_h = 0, out_f = 0;
            std::uint32_t code_now = lane == 0 ? column_code(1) : 0u;
            __syncwarp();
            [[maybe_unused]] std::uint32_t p_lo[words], p_hi[words]; // profile words (unused in compare mode)
            if constexpr (!compare) {
                load_profile_words<R>(profile_lo + (code_now & 0xFF) * S + lane_rows, p_lo);
                load_profile_words<R>(profile_hi + ((code_now >> 8) & 0xFF) * S + lane_rows, p_hi);
            }

            // `steady`: every lane's two columns are real and below m (63 <= t < m - 1): no masks, no capture.
            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (band16_chunk_k - 1);
                if (e == 0) {
                    // The strip above must have published the columns staged now; this strip publishes its own.
                    std::uint32_t const need = min(m, t + band16_chunk_k);
                    if (k > 0 && t + 1 <= m) healthy = band_wait(sync, slot_in, ((unsigned long long)k << 32) | need);
                    if (bottom_writer && t > 63)
                        band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | min(m, t - 63));
                    __syncwarp();
#pragma unroll
                    for (int c = lane; c < band16_chunk_k; c += 32) {
                        std::uint32_t const j = t + 1 + c;
                        std::uint32_t word = 0;
                        if (j <= m) {
                            if (k == 0) word = pack16(edge.score(j) + h_shift, gap_seed(j));
                            else word = __ldcg(top + j);
                        }
                        chunk.top[c] = word;
                        chunk.code[c] = j + 1 <= m ? column_code(j + 1) : 0u;
                    }
                    __syncwarp();
                }
                std::uint32_t const staged_top = chunk.top[e], staged_code = chunk.code[e];
                std::uint32_t up_h = __shfl_sync(0xFFFFFFFFu, out_h, from_lane);
                std::uint32_t up_f = affine ? __shfl_sync(0xFFFFFFFFu, out_f, from_lane) : 0u;
                std::uint32_t code_next = __shfl_sync(0xFFFFFFFFu, code_now, from_lane);
                if (lane == 0) {
                    // Low half: the strip's top row; high half: lane 31's low half (the row just above).
                    up_h = __byte_perm(staged_top, up_h, 0x5410);
                    up_f = __byte_perm(staged_top, up_f, 0x5432);
                    // Codes: the low half's in byte 0 and the high half's in byte 1 (profiles; the staged codes are
                    // below 256, so their byte 1 is a zero byte), or in bits 0-15 and 16-31 (compare mode).
                    code_next = __byte_perm(staged_code, code_next, compare ? 0x5410 : 0x1140);
                }
                [[maybe_unused]] std::uint32_t q_lo[words], q_hi[words];
                if constexpr (!compare) {
                    load_profile_words<R>(profile_lo + (code_next & 0xFF) * S + lane_rows, q_lo);
                    load_profile_words<R>(profile_hi + ((code_next >> 8) & 0xFF) * S + lane_rows, q_hi);
                }

                int const j_lo = (int)t + 1 - lane, j_hi = j_lo - 32;
                // Low half past m, high half not yet started: a lane with neither real column skips the update.
                bool const active = steady || (j_lo >= 1 && j_hi <= (int)m);
                if (active) {
                    // A high half that has not reached column 1 keeps its column-0 state (blended back below).
                    std::uint32_t const keep = (steady || j_hi >= 1) ? 0u : 0xFFFF0000u;
                    std::uint32_t diag = diag_up;
                    diag_up = steady ? up_h : ((up_h & ~keep) | (diag_up & keep));
                    std::uint32_t h_up = up_h, f_up = up_f;
                    std::uint32_t subs[R], cell_h[R];
                    if constexpr (compare) compared.rows<policy_::multiply_k>(row_codes, code_now, subs);
                    else {
#pragma unroll
                        for (int w = 0; w < words; ++w) {
                            subs[4 * w + 0] = interleave_signed_bytes<0>(p_lo[w], p_hi[w]);
                            subs[4 * w + 1] = interleave_signed_bytes<1>(p_lo[w], p_hi[w]);
                            subs[4 * w + 2] = interleave_signed_bytes<2>(p_lo[w], p_hi[w]);
                            subs[4 * w + 3] = interleave_signed_bytes<3>(p_lo[w], p_hi[w]);
                        }
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::uint32_t h, kept;
                        [[maybe_unused]] std::uint32_t e_new = 0; // affine tracks only
                        if constexpr (affine) {
                            e_new = ops::add_opt(e_col[r], extend2, h_col[r]);
                            std::uint32_t const x = ops::add_opt(diag, subs[r], e_new);
                            f_up = ops::add_opt(f_up, extend2, h_up);
                            h = local ? ops::opt2_relu(x, f_up) : ops::opt2(x, f_up);
                            kept = ops::add(h, open2);
                        }
                        else {
                            std::uint32_t const substitution = ops::add(diag, subs[r]);
                            std::uint32_t const x = ops::add_opt(h_col[r], open2, substitution);
                            if constexpr (local) h = ops::add_opt_relu(h_up, open2, x);
                            else h = ops::add_opt(h_up, open2, x);
                            kept = h;
                        }
                        cell_h[r] = h;
                        diag = h_col[r];
                        if constexpr (steady) {
                            h_col[r] = kept;
                            if constexpr (affine) e_col[r] = e_new;
                        }
                        else {
                            h_col[r] = (kept & ~keep) | (h_col[r] & keep);
                            if constexpr (affine) e_col[r] = (e_new & ~keep) | (e_col[r] & keep);
                        }
                        h_up = kept;
                    }
                    if constexpr (local) {
                        if constexpr (steady) {
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_h[r], 0u);
                        }
                        else {
                            std::uint32_t const mask = ((j_lo >= 1 && j_lo <= (int)m) ? 0x0000FFFFu : 0u) |
                                                       ((j_hi >= 1 && j_hi <= (int)m) ? 0xFFFF0000u : 0u);
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_h[r] & mask, 0u);
                        }
                    }
                    else if constexpr (!steady) {
                        if (lane == capture_lane && (capture_hi ? j_hi : j_lo) == (int)m) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == r_n) result = capture_hi ? high16(cell_h[r]) : low16(cell_h[r]);
                        }
                    }
                    out_h = h_up, out_f = f_up;
                    if (bottom_writer && (steady || (j_hi >= 1 && j_hi <= (int)m)))
                        __stcg(bottom + j_hi, __byte_perm(out_h, out_f, 0x7632));
                }
                code_now = code_next;
                if constexpr (!compare) {
#pragma unroll
                    for (int w = 0; w < words; ++w) p_lo[w] = q_lo[w], p_hi[w] = q_hi[w];
                }
            };

            std::uint32_t const fill_end = min(steps, 63u);
            std::uint32_t const steady_end = m >= 64u ? max(fill_end, min(steps, m - 1u)) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end && healthy; ++t) step(t, std::false_type {});
            // Two steps per iteration: the row state alternates between two register sets instead of being copied
            // back.
#pragma unroll 2
            for (; t < steady_end && healthy; ++t) step(t, std::true_type {});
            for (; t < steps && healthy; ++t) step(t, std::false_type {});
        }
        else {
            // Two columns per step: at step t the low half of lane l scores columns 2(t - l) + 1 and 2(t - l) + 2, its
            // high half the pair 32 steps (64 columns) behind; as in the 32-bit band, a round of shuffles and the
            // step's fixed work serve twice the cells and the second column's cells run beside the first column's
            // next row. A sweep takes ceil(m / 2) + 63 steps; staging stays 64 columns (32 steps) at a time.
            constexpr std::uint32_t steps_per_chunk = band16_chunk_k / 2;
            std::uint32_t const column_pairs = (m + 1) / 2;
            std::uint32_t const steps = column_pairs + (std::uint32_t)last_vlane;
            std::uint32_t out_ha = 0, out_hb = 0, out_fa = 0, out_fb = 0;
            // Each column's codes as in the one-column sweep (low half in byte 0 or bits 0-15, high half above).
            std::uint32_t code_a = lane == 0 ? column_code(1) : 0u;
            std::uint32_t code_b = lane == 0 && m >= 2 ? column_code(2) : 0u;
            __syncwarp();
            [[maybe_unused]] std::uint32_t pa_lo[words], pa_hi[words], pb_lo[words], pb_hi[words];
            if constexpr (!compare) {
                load_profile_words<R>(profile_lo + (code_a & 0xFF) * S + lane_rows, pa_lo);
                load_profile_words<R>(profile_hi + ((code_a >> 8) & 0xFF) * S + lane_rows, pa_hi);
                load_profile_words<R>(profile_lo + (code_b & 0xFF) * S + lane_rows, pb_lo);
                load_profile_words<R>(profile_hi + ((code_b >> 8) & 0xFF) * S + lane_rows, pb_hi);
            }
            auto substitutions = [&](std::uint32_t code, std::uint32_t const (&p_lo)[words],
                                     std::uint32_t const (&p_hi)[words], std::uint32_t (&subs)[R]) {
                if constexpr (compare) compared.rows<policy_::multiply_k>(row_codes, code, subs);
                else {
#pragma unroll
                    for (int w = 0; w < words; ++w) {
                        subs[4 * w + 0] = interleave_signed_bytes<0>(p_lo[w], p_hi[w]);
                        subs[4 * w + 1] = interleave_signed_bytes<1>(p_lo[w], p_hi[w]);
                        subs[4 * w + 2] = interleave_signed_bytes<2>(p_lo[w], p_hi[w]);
                        subs[4 * w + 3] = interleave_signed_bytes<3>(p_lo[w], p_hi[w]);
                    }
                }
            };
            // One packed cell pair: returns H and sets `kept` (H + open for affine tracks, else H), updating E
            // (from its left) and F (for the cell below) as the one-column sweep does.
            auto cell = [&](std::uint32_t diag, std::uint32_t left_kept, std::uint32_t &e, std::uint32_t up_kept,
                            std::uint32_t &f_up, std::uint32_t substitution, std::uint32_t &kept) -> std::uint32_t {
                std::uint32_t h;
                if constexpr (affine) {
                    e = ops::add_opt(e, extend2, left_kept);
                    std::uint32_t const x = ops::add_opt(diag, substitution, e);
                    f_up = ops::add_opt(f_up, extend2, up_kept);
                    h = local ? ops::opt2_relu(x, f_up) : ops::opt2(x, f_up);
                    kept = ops::add(h, open2);
                }
                else {
                    std::uint32_t const x = ops::add_opt(left_kept, open2, ops::add(diag, substitution));
                    if constexpr (local) h = ops::add_opt_relu(up_kept, open2, x);
                    else h = ops::add_opt(up_kept, open2, x);
                    kept = h;
                }
                return h;
            };

            // `steady`: every lane's four columns are real and below m (63 <= t, 2t + 2 < m): no masks, no capture.
            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (steps_per_chunk - 1);
                if (e == 0) {
                    // The strip above must have published the columns staged now; this strip publishes its own
                    // (before step t its last lane's high half has finished columns up to 2(t - 63)).
                    std::uint32_t const first_column = 2 * t + 1;
                    std::uint32_t const need = min(m, 2 * t + band16_chunk_k);
                    if (k > 0 && first_column <= m)
                        healthy = band_wait(sync, slot_in, ((unsigned long long)k << 32) | need);
                    if (bottom_writer && t > 63)
                        band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | min(m, 2 * (t - 63)));
                    __syncwarp();
#pragma unroll
                    for (int c = lane; c < band16_chunk_k; c += 32) {
                        std::uint32_t const j = first_column + c;
                        std::uint32_t word = 0;
                        if (j <= m) {
                            if (k == 0) word = pack16(edge.score(j) + h_shift, gap_seed(j));
                            else word = __ldcg(top + j);
                        }
                        chunk.top[c] = word;
                        chunk.code[c] = j + 2 <= m ? column_code(j + 2) : 0u; // lane 0's codes one step ahead
                    }
                    __syncwarp();
                }
                std::uint32_t const staged_top_a = chunk.top[2 * e], staged_top_b = chunk.top[2 * e + 1];
                std::uint32_t const staged_code_a = chunk.code[2 * e], staged_code_b = chunk.code[2 * e + 1];
                std::uint32_t up_ha = __shfl_sync(0xFFFFFFFFu, out_ha, from_lane);
                std::uint32_t up_hb = __shfl_sync(0xFFFFFFFFu, out_hb, from_lane);
                std::uint32_t up_fa = affine ? __shfl_sync(0xFFFFFFFFu, out_fa, from_lane) : 0u;
                std::uint32_t up_fb = affine ? __shfl_sync(0xFFFFFFFFu, out_fb, from_lane) : 0u;
                std::uint32_t next_a = __shfl_sync(0xFFFFFFFFu, code_a, from_lane);
                std::uint32_t next_b = __shfl_sync(0xFFFFFFFFu, code_b, from_lane);
                if (lane == 0) {
                    // Low half: the strip's top row; high half: lane 31's low half (the row just above).
                    up_ha = __byte_perm(staged_top_a, up_ha, 0x5410);
                    up_hb = __byte_perm(staged_top_b, up_hb, 0x5410);
                    up_fa = __byte_perm(staged_top_a, up_fa, 0x5432);
                    up_fb = __byte_perm(staged_top_b, up_fb, 0x5432);
                    next_a = __byte_perm(staged_code_a, next_a, compare ? 0x5410 : 0x1140);
                    next_b = __byte_perm(staged_code_b, next_b, compare ? 0x5410 : 0x1140);
                }
                [[maybe_unused]] std::uint32_t qa_lo[words], qa_hi[words], qb_lo[words], qb_hi[words];
                if constexpr (!compare) {
                    load_profile_words<R>(profile_lo + (next_a & 0xFF) * S + lane_rows, qa_lo);
                    load_profile_words<R>(profile_hi + ((next_a >> 8) & 0xFF) * S + lane_rows, qa_hi);
                    load_profile_words<R>(profile_lo + (next_b & 0xFF) * S + lane_rows, qb_lo);
                    load_profile_words<R>(profile_hi + ((next_b >> 8) & 0xFF) * S + lane_rows, qb_hi);
                }

                int const ja_lo = 2 * ((int)t - lane) + 1, ja_hi = ja_lo - 64;
                // Low half past m, high half not yet started: a lane with neither real column skips the update.
                bool const active = steady || (ja_lo >= 1 && ja_hi <= (int)m);
                if (active) {
                    // A high half that has not reached column 1 keeps its column-0 state (blended back below).
                    std::uint32_t const keep = (steady || ja_hi >= 1) ? 0u : 0xFFFF0000u;
                    std::uint32_t diag_a = diag_up, diag_b = up_ha;
                    diag_up = steady ? up_hb : ((up_hb & ~keep) | (diag_up & keep));
                    std::uint32_t h_up_a = up_ha, h_up_b = up_hb, f_up_a = up_fa, f_up_b = up_fb;
                    std::uint32_t subs_a[R], subs_b[R], cell_a[R], cell_b[R];
                    substitutions(code_a, pa_lo, pa_hi, subs_a);
                    substitutions(code_b, pb_lo, pb_hi, subs_b);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::uint32_t e_left = e_col[r], kept_a, kept_b;
                        cell_a[r] = cell(diag_a, h_col[r], e_left, h_up_a, f_up_a, subs_a[r], kept_a);
                        cell_b[r] = cell(diag_b, kept_a, e_left, h_up_b, f_up_b, subs_b[r], kept_b);
                        diag_a = h_col[r];
                        diag_b = kept_a;
                        if constexpr (steady) {
                            h_col[r] = kept_b;
                            if constexpr (affine) e_col[r] = e_left;
                        }
                        else {
                            h_col[r] = (kept_b & ~keep) | (h_col[r] & keep);
                            if constexpr (affine) e_col[r] = (e_left & ~keep) | (e_col[r] & keep);
                        }
                        h_up_a = kept_a;
                        h_up_b = kept_b;
                    }
                    if constexpr (local) {
                        if constexpr (steady) {
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_a[r], cell_b[r]);
                        }
                        else {
                            auto half_mask = [&](int j_lo, int j_hi) {
                                return ((j_lo >= 1 && j_lo <= (int)m) ? 0x0000FFFFu : 0u) |
                                       ((j_hi >= 1 && j_hi <= (int)m) ? 0xFFFF0000u : 0u);
                            };
                            std::uint32_t const mask_a = half_mask(ja_lo, ja_hi);
                            std::uint32_t const mask_b = half_mask(ja_lo + 1, ja_hi + 1);
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                best_row[r] = __vimax3_s16x2(best_row[r], cell_a[r] & mask_a, cell_b[r] & mask_b);
                        }
                    }
                    else if constexpr (!steady) {
                        int const ja = capture_hi ? ja_hi : ja_lo;
                        if (lane == capture_lane && (ja == (int)m || ja + 1 == (int)m)) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == r_n) {
                                    std::uint32_t const cell_m = ja == (int)m ? cell_a[r] : cell_b[r];
                                    result = capture_hi ? high16(cell_m) : low16(cell_m);
                                }
                        }
                    }
                    out_ha = h_up_a, out_hb = h_up_b, out_fa = f_up_a, out_fb = f_up_b;
                    if (bottom_writer && (steady || (ja_hi >= 1 && ja_hi <= (int)m))) {
                        __stcg(bottom + ja_hi, __byte_perm(out_ha, out_fa, 0x7632));
                        if (steady || ja_hi + 1 <= (int)m)
                            __stcg(bottom + ja_hi + 1, __byte_perm(out_hb, out_fb, 0x7632));
                    }
                }
                code_a = next_a, code_b = next_b;
                if constexpr (!compare) {
#pragma unroll
                    for (int w = 0; w < words; ++w)
                        pa_lo[w] = qa_lo[w], pa_hi[w] = qa_hi[w], pb_lo[w] = qb_lo[w], pb_hi[w] = qb_hi[w];
                }
            };

            std::uint32_t const fill_end = min(steps, 63u);
            std::uint32_t const steady_end = m / 2 > 64u ? max(fill_end, min(steps, m / 2 - 1u)) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end && healthy; ++t) step(t, std::false_type {});
#pragma unroll 2
            for (; t < steady_end && healthy; ++t) step(t, std::true_type {});
            for (; t < steps && healthy; ++t) step(t, std::false_type {});
        }
        __syncwarp();
        if (bottom_writer) band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | m);
        if constexpr (local) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                std::uint32_t const keep_rows = ((row0_lo + r <= (std::int64_t)n) ? 0x0000FFFFu : 0u) |
                                                ((row0_hi + r <= (std::int64_t)n) ? 0xFFFF0000u : 0u);
                lane_best = __vimax3_s16x2(lane_best, best_row[r] & keep_rows, 0u);
            }
        }
        if (!healthy) break;
    }
    if constexpr (local) {
        std::int32_t best = max(low16(lane_best), high16(lane_best));
#pragma unroll
        for (int offset = 16; offset > 0; offset >>= 1) best = max(best, __shfl_xor_sync(0xFFFFFFFFu, best, offset));
        return best;
    }
    else {
        std::uint32_t const last = super_strips - 1;
        int const owner_lane = int(((n - 1 - last * SS) / R) & 31);
        return __shfl_sync(0xFFFFFFFFu, result, owner_lane);
    }
}

/** Persistent 16-bit band kernel: one pair per CTA at a time, pulled from a cursor over bins [key_begin, key_end). */
template <typename policy_>
__global__ void __launch_bounds__(band_warps_k * 32)
    band16_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key_begin, int key_end,
                  score_costs_t const costs, std::int64_t *__restrict__ results, std::uint32_t *__restrict__ scratch,
                  std::size_t ring_words_per_slot) {
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::size_t const costs_bytes = (sizeof(score_costs_t) + 15) / 16 * 16;
    band_shared_t &shared = *reinterpret_cast<band_shared_t *>(shared_bytes + costs_bytes);
    std::size_t const shared_state_bytes = (sizeof(band_shared_t) + 15) / 16 * 16;
    std::size_t const profile_bytes = (std::size_t)band16_profile_bytes_per_warp<policy_>(costs.classes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + costs_bytes + shared_state_bytes);
    auto *chunks = reinterpret_cast<band16_chunk_t *>(profiles + band_warps_k * profile_bytes);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Local kernels keep room for a 32-bit ring (two words per column) in case a pair has to be scored again.
    constexpr std::size_t ring_scale = policy_::local_k ? 2 : 1;
    std::uint32_t *ring = scratch + (std::size_t)blockIdx.x * band_warps_k * ring_words_per_slot * ring_scale;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) shared.pair_index = atomicAdd(&bins->cursor[key_begin], 1u);
        if (threadIdx.x < band_warps_k) shared.progress[threadIdx.x] = 0ull;
        if (threadIdx.x == 0) shared.failed = 0u;
        __syncthreads();
        std::uint32_t const index = shared.pair_index;
        if (index >= count) break;
        pair_task_t const task = tasks[begin + index];
        std::int32_t const value = band16_score_warp<policy_>(task, costs_s, band_cta_ring(shared, warp, costs_s.wait_polls), ring,
                                                              ring_words_per_slot, profiles + warp * profile_bytes,
                                                              chunks[warp]);
        if (lane == 0) shared.warp_result[warp] = value;
        __syncthreads();
        if constexpr (policy_::local_k) {
            // Every cell below the limit means no 16-bit value wrapped (each is exact given exact neighbours below
            // it); a maximum at the limit means some may have, so the pair is scored again on 32-bit cells with the
            // band kernel's own code, in this CTA's shared memory and ring.
            if (threadIdx.x == 0) {
                std::int32_t best = 0;
                for (int w = 0; w < band_warps_k; ++w) best = max(best, shared.warp_result[w]);
                shared.redo = (!shared.failed && best >= costs_s.local_limit16) ? 1u : 0u;
                if (shared.redo) shared.failed = 0u;
            }
            if (threadIdx.x < band_warps_k) shared.progress[threadIdx.x] = 0ull;
            __syncthreads();
            if (shared.redo) {
                using wide_t = band_policy_t<policy_::kind_k, policy_::affine_k, policy_::rows_per_lane_k>;
                static_assert(band_profile_bytes_per_warp<wide_t>(32) <= band16_profile_bytes_per_warp<policy_>(32),
                              "the 32-bit profile must fit the 16-bit one's space");
                static_assert(sizeof(band_chunk_t) <= sizeof(band16_chunk_t), "chunk staging must fit");
                std::size_t const wide_profile = (std::size_t)band_profile_bytes_per_warp<wide_t>(costs.classes);
                std::int32_t const wide = band_score_warp<wide_t>(
                    task, costs_s, band_cta_ring(shared, warp, costs_s.wait_polls), reinterpret_cast<std::int32_t *>(ring),
                    2 * ring_words_per_slot, profiles + warp * wide_profile,
                    *reinterpret_cast<band_chunk_t *>(&chunks[warp]));
                if (lane == 0) shared.warp_result[warp] = wide;
                __syncthreads();
            }
        }
        if (threadIdx.x == 0) {
            std::int64_t score;
            if (policy_::local_k) {
                std::int32_t best = 0;
                for (int w = 0; w < band_warps_k; ++w) best = max(best, shared.warp_result[w]);
                score = best;
            }
            else {
                std::uint32_t const super_strips = (task.rows_length + policy_::super_rows_k - 1) / policy_::super_rows_k;
                score = shared.warp_result[(super_strips - 1) % band_warps_k];
            }
            if (shared.failed) atomicOr(&bins->error_flags, 1u);
            results[task.slot] = score;
        }
    }
}

/**
 *  Grouped 16-bit band kernel: G co-resident CTAs (one cooperative launch) share each pair, their G x W warps forming
 *  one ring of super-strips (see `band_group_kernel`). A local pair whose group maximum reached the 16-bit limit is
 *  scored again by the same group on 32-bit cells, with the second pass's ring words.
 */
template <typename policy_>
__global__ void __launch_bounds__(band_warps_k * 32)
    band16_group_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key_begin,
                        int key_end, score_costs_t const costs, std::int64_t *__restrict__ results,
                        std::uint32_t *__restrict__ scratch, std::size_t ring_words_per_slot,
                        band_group_state_t *__restrict__ group_states, int group_ctas) {
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::size_t const costs_bytes = (sizeof(score_costs_t) + 15) / 16 * 16;
    band_shared_t &shared = *reinterpret_cast<band_shared_t *>(shared_bytes + costs_bytes);
    std::size_t const shared_state_bytes = (sizeof(band_shared_t) + 15) / 16 * 16;
    std::size_t const profile_bytes = (std::size_t)band16_profile_bytes_per_warp<policy_>(costs.classes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + costs_bytes + shared_state_bytes);
    auto *chunks = reinterpret_cast<band16_chunk_t *>(profiles + band_warps_k * profile_bytes);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    int const warp = threadIdx.x >> 5;
    int const group = (int)blockIdx.x / group_ctas, rank = (int)blockIdx.x % group_ctas;
    int const groups = (int)gridDim.x / group_ctas;
    int const members = group_ctas * band_warps_k;
    band_group_state_t *state = group_states + group;
    constexpr std::size_t ring_scale = policy_::local_k ? 2 : 1;
    std::uint32_t *ring = scratch + (std::size_t)group * members * ring_words_per_slot * ring_scale;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    std::uint32_t barriers = 0, iteration = 0;
    for (std::uint32_t index = (std::uint32_t)group; index < count; index += (std::uint32_t)groups, ++iteration) {
        int const parity = int(iteration & 1u);
        if (!band_group_barrier(state, group_ctas, ++barriers, shared.gate, costs_s.barrier_polls)) break;
        if (rank == 0) band_group_reset(state, parity ^ 1, members);
        pair_task_t const task = tasks[begin + index];
        int const member = rank * band_warps_k + warp;
        band_pass_state_t *pass = &state->pass[parity][0];
        {
            band_ring_t const sync {pass->progress, &state->failed, members, member, true, costs_s.wait_polls};
            std::int32_t const value = band16_score_warp<policy_>(task, costs_s, sync, ring, ring_words_per_slot,
                                                                  profiles + warp * profile_bytes, chunks[warp]);
            std::uint32_t const super_strips =
                (task.rows_length + policy_::super_rows_k - 1) / policy_::super_rows_k;
            band_group_contribute<policy_::local_k>(*pass, value,
                                                    (int)((super_strips - 1) % (std::uint32_t)members) == member);
        }
        if (!band_group_barrier(state, group_ctas, ++barriers, shared.gate, costs_s.barrier_polls)) break;
        if constexpr (policy_::local_k) {
            // The group's maximum decides, identically in every CTA, whether 16-bit values may have wrapped.
            if (*reinterpret_cast<volatile std::int32_t *>(&pass->best) >= costs_s.local_limit16) {
                using wide_t = band_policy_t<policy_::kind_k, policy_::affine_k, policy_::rows_per_lane_k>;
                std::size_t const wide_profile = (std::size_t)band_profile_bytes_per_warp<wide_t>(costs.classes);
                pass = &state->pass[parity][1];
                band_ring_t const sync {pass->progress, &state->failed, members, member, true, costs_s.wait_polls};
                std::int32_t const wide = band_score_warp<wide_t>(
                    task, costs_s, sync, reinterpret_cast<std::int32_t *>(ring), 2 * ring_words_per_slot,
                    profiles + warp * wide_profile, *reinterpret_cast<band_chunk_t *>(&chunks[warp]));
                band_group_contribute<true>(*pass, wide, false);
                if (!band_group_barrier(state, group_ctas, ++barriers, shared.gate, costs_s.barrier_polls)) break;
            }
        }
        if (rank == 0 && threadIdx.x == 0)
            results[task.slot] = *reinterpret_cast<volatile std::int32_t *>(&pass->best);
    }
    __syncthreads();
    if (rank == 0 && threadIdx.x == 0 && *reinterpret_cast<volatile std::uint32_t *>(&state->failed))
        atomicOr(&bins->error_flags, 1u);
}

} // namespace szs_gb300
