/**
 *  @file dp_packed.cuh
 *  @brief Wavefront DP with 16x2 packed cells: one warp scores two pairs at once, pair A in the low halves and pair
 *         B in the high halves of every register, with DPX 16x2 instructions.
 *
 *  Taken only when the length bound proves every value of both pairs fits int16 (the planner checks
 *  `(span + steps + 1) * magnitude < 32767` per pair). Cells of rows or columns beyond a pair's own length are
 *  computed but never flow into that pair's real cells (information only moves down and right), and the two halves
 *  never interact (16x2 instructions have no carries between halves), so such filler cannot change a result even
 *  when it wraps.
 *
 *  Affine tracks keep `Ĥ = H + open` instead of H (both gap tracks extend from H + open) and take the substitution
 *  profile as `s - open`, so that every cell is five fused DPX operations:
 *
 *      E = max(E_left + extend, Ĥ_left)
 *      X = max(Ĥ_diag + (s - open), E)            (= max(H_diag + s, E))
 *      F = max(F_up + extend, Ĥ_up)
 *      H = max(X, F)                              (local: also max(., 0))
 *      Ĥ = H + open
 *
 *  (min for Levenshtein). The planner routes an affine pair here only when every `s - open` of its table fits a
 *  byte. Substitution costs come from two per-warp int8 profiles, one per pair, and one byte-permute with sign
 *  replication builds the packed cost of both pairs for a row.
 *
 *  The layout of a pair inside the warp is the one of dp_wavefront.cuh: strips of 32 x R rows, lane L owns rows
 *  L*R..L*R+R-1, column j = t + 1 - L at step t, bottom values passed down with `__shfl_up_sync`, lane 0 fed by the
 *  closed-form row 0 or by the previous strip's bottom row in the warp's scratch row.
 */
#pragma once
#include <type_traits>

#include "dp_cells.cuh"
#include "dp_wavefront.cuh"
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

/** `compare_`: a `compare_mode_t` (engine_types.cuh); other than `compare_none_k`, Levenshtein over more than 32 byte
 *  values with costs from comparing codes instead of profiles. `wide_` (compare modes only): strings of 16-bit codes
 *  (UTF-8 calls over more than 256 code points), compared as they are. */
template <int kind_, bool affine_, int rows_per_lane_, int compare_ = compare_none_k, bool wide_ = false,
          int columns_per_step_ = 1>
struct dp16_policy_t {
    static constexpr int kind_k = kind_;
    static constexpr bool affine_k = affine_;
    static constexpr bool maximize_k = kind_ != kind_levenshtein_k;
    static constexpr bool local_k = kind_ == kind_smith_waterman_k;
    static constexpr int rows_per_lane_k = rows_per_lane_;
    static constexpr int strip_rows_k = warp_size_k * rows_per_lane_;
    static constexpr bool compare_k = compare_ != compare_none_k;
    static constexpr bool multiply_k = compare_ == compare_multiply_k;
    static constexpr bool wide_k = wide_;
    static constexpr int columns_k = columns_per_step_; // columns a lane scores per step: 1 or 2
    static_assert(!compare_k || kind_ == kind_levenshtein_k, "only Levenshtein costs are a function of equality");
    static_assert(!wide_ || compare_k, "16-bit codes have no profile");
};

/** Per-warp shared profile bytes: two pairs x classes x strip rows (none in compare mode). */
template <typename policy_>
__host__ __device__ constexpr int dp16_profile_bytes_per_warp(int classes) {
    return policy_::compare_k ? 0 : 2 * classes * policy_::strip_rows_k;
}

constexpr int dp16_chunk_bytes_k = 3 * 64 * 4;

template <typename policy_>
__host__ __device__ constexpr int dp16_shared_bytes(int warps_per_cta, int classes) {
    return int((sizeof(score_costs_t) + 15) / 16 * 16) +
           warps_per_cta * (dp16_profile_bytes_per_warp<policy_>(classes) + dp16_chunk_bytes_k);
}

constexpr std::uint32_t packed_floor_k = 0x80008000u; // -32768 in both halves: max(x + y, floor) == x + y

__device__ __forceinline__ std::uint32_t pack16(std::int32_t lo, std::int32_t hi) {
    return (std::uint32_t(lo) & 0xFFFFu) | (std::uint32_t(hi) << 16);
}
__device__ __forceinline__ std::int32_t low16(std::uint32_t x) { return std::int32_t(std::int16_t(x & 0xFFFFu)); }
__device__ __forceinline__ std::int32_t high16(std::uint32_t x) { return std::int32_t(std::int16_t(x >> 16)); }

/** Byte `b` of `x` and byte `b` of `y`, each sign-extended to 16 bits: {lo: x.b, hi: y.b}. */
template <int b_>
__device__ __forceinline__ std::uint32_t interleave_signed_bytes(std::uint32_t x, std::uint32_t y) {
    constexpr std::uint32_t selector = std::uint32_t(b_) | (std::uint32_t(8 + b_) << 4) | (std::uint32_t(4 + b_) << 8) |
                                       (std::uint32_t(12 + b_) << 12);
    std::uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(y), "r"(selector));
    return r;
}

template <bool maximize_>
struct packed_ops_t {
    __device__ __forceinline__ static std::uint32_t add(std::uint32_t a, std::uint32_t b) {
        return maximize_ ? __viaddmax_s16x2(a, b, packed_floor_k) : __viaddmin_s16x2(a, b, 0x7FFF7FFFu);
    }
    __device__ __forceinline__ static std::uint32_t opt2(std::uint32_t a, std::uint32_t b) {
        return maximize_ ? __vimax3_s16x2(a, b, b) : __vimin3_s16x2(a, b, b);
    }
    __device__ __forceinline__ static std::uint32_t add_opt(std::uint32_t a, std::uint32_t b, std::uint32_t c) {
        return maximize_ ? __viaddmax_s16x2(a, b, c) : __viaddmin_s16x2(a, b, c);
    }
    __device__ __forceinline__ static std::uint32_t add_opt_relu(std::uint32_t a, std::uint32_t b, std::uint32_t c) {
        return __viaddmax_s16x2_relu(a, b, c);
    }
    __device__ __forceinline__ static std::uint32_t opt2_relu(std::uint32_t a, std::uint32_t b) {
        return __vimax_s16x2_relu(a, b);
    }
};

constexpr int chunk_columns_k = 64; // lane 0's boundary values and column codes are staged 64 columns at a time

/** Reads a lane's R profile bytes (R a multiple of 4) with the widest loads their alignment allows. */
template <int rows_>
__device__ __forceinline__ void load_profile_words(std::int8_t const *source, std::uint32_t (&out)[rows_ / 4]) {
    if constexpr (rows_ % 16 == 0) {
#pragma unroll
        for (int v = 0; v < rows_ / 16; ++v) {
            uint4 const x = reinterpret_cast<uint4 const *>(source)[v];
            out[4 * v + 0] = x.x, out[4 * v + 1] = x.y, out[4 * v + 2] = x.z, out[4 * v + 3] = x.w;
        }
    }
    else if constexpr (rows_ % 8 == 0) {
#pragma unroll
        for (int v = 0; v < rows_ / 8; ++v) {
            uint2 const x = reinterpret_cast<uint2 const *>(source)[v];
            out[2 * v + 0] = x.x, out[2 * v + 1] = x.y;
        }
    }
    else {
#pragma unroll
        for (int v = 0; v < rows_ / 4; ++v) out[v] = reinterpret_cast<std::uint32_t const *>(source)[v];
    }
}

/**
 *  Packed substitution costs in compare mode. Row codes hold pair A's code in the low half and pair B's in the high
 *  half (byte codes, or 16-bit codes); column codes travel negated per half (`-c mod 2^16`), so one DPX add-min,
 *  `min(row + column, 1)` per unsigned half with the add wrapping inside the half, is 0 exactly where the codes are
 *  equal and 1 where they differ. Then either
 *
 *  - `multiply`: one integer multiply-add, `differs * (mismatch - match) + match2`, on the multiply-add pipe. Exact
 *    when `match` and `mismatch` (as shifted for the call) have the same sign: the low half's value and `match` then
 *    borrow from the high half alike (both negative) or not at all (both non-negative);
 *  - or a half mask `differs * 0xFFFF` and one logic operation selecting `mismatch` or `match`.
 */
struct compare_costs_t {
    std::uint32_t match2, mismatch2; // both halves
    std::uint32_t delta;             // mismatch - match, two's complement

    __device__ __forceinline__ compare_costs_t(std::int32_t match, std::int32_t mismatch)
        : match2(pack16(match, match)), mismatch2(pack16(mismatch, mismatch)), delta(std::uint32_t(mismatch - match)) {}

    /** Column codes `ca`, `cb` as they travel: negated per half. */
    __device__ __forceinline__ static std::uint32_t column_codes(std::uint32_t ca, std::uint32_t cb) {
        return ((0u - ca) & 0xFFFFu) | ((0u - cb) << 16);
    }
    /** Costs of R rows against one column. */
    template <bool multiply_, int rows_>
    __device__ __forceinline__ void rows(std::uint32_t const (&row_codes)[rows_], std::uint32_t negated_column_codes,
                                         std::uint32_t (&out)[rows_]) const {
        if constexpr (multiply_) {
#pragma unroll
            for (int r = 0; r < rows_; ++r)
                out[r] = __viaddmin_u16x2(row_codes[r], negated_column_codes, 0x00010001u) * delta + match2;
        }
        else {
#pragma unroll
            for (int r = 0; r < rows_; ++r) {
                std::uint32_t const mask = __viaddmin_u16x2(row_codes[r], negated_column_codes, 0x00010001u) * 0xFFFFu;
                out[r] = (mask & mismatch2) | (~mask & match2);
            }
        }
    }
};

/** Per-warp staging area for lane 0: top-boundary H (Ĥ for affine tracks) and F, and packed column codes, of the
 *  next 64 columns. */
struct column_chunk_t {
    std::uint32_t top_h[chunk_columns_k];
    std::uint32_t top_f[chunk_columns_k];
    std::uint32_t code[chunk_columns_k];
};

/**
 *  Scores tasks @p a and @p b (b may be absent: `b_present == false`) with one warp. All lanes call it together.
 *
 *  Per step t, lane L updates column j = t + 1 - L for both pairs. The dependency chain a step waits on is the
 *  shuffle of the upper lane's bottom values plus, per row, F, H and Ĥ (affine) or H alone (linear, with
 *  X = max(H_left + gap, diag + s) computed off the chain). Column codes travel one step ahead of
 *  the values (a lane forwards its current code, which is the code of the next lane's next column), so every
 *  profile load is issued a step before it is used.
 *
 *  @param scratch  this warp's scratch row, (longest column + 1) x 2 packed words
 *  @param profile  this warp's shared profile area, dp16_profile_bytes_per_warp bytes
 *  @param chunk    this warp's staging area
 */
template <typename policy_>
__device__ __forceinline__ void dp16_score_couple(pair_task_t const &a, pair_task_t const &b, bool b_present,
                                                  score_costs_t const &costs, std::uint32_t *scratch,
                                                  std::int8_t *profile, column_chunk_t &chunk, std::int64_t &score_a,
                                                  std::int64_t &score_b) {
    using ops = packed_ops_t<policy_::maximize_k>;
    constexpr int R = policy_::rows_per_lane_k;
    constexpr int S = policy_::strip_rows_k;
    constexpr bool affine = policy_::affine_k;
    constexpr bool local = policy_::local_k;
    constexpr bool compare = policy_::compare_k;
    static_assert(R % 4 == 0, "profile rows are read in 4-byte words");
    constexpr int words = compare ? 1 : R / 4; // profile words per pair (unused in compare mode)

    int const lane = threadIdx.x & 31;
    std::uint32_t const n_a = a.rows_length, m_a = a.cols_length;
    std::uint32_t const n_b = b_present ? b.rows_length : 0u, m_b = b_present ? b.cols_length : 0u;
    std::uint32_t const n_max = max(n_a, n_b), m_max = max(m_a, m_b), m_min = min(m_a, m_b);
    std::int32_t const open = costs.open, extend = costs.extend;
    std::uint32_t const open2 = pack16(open, open), extend2 = pack16(extend, extend);
    std::uint32_t const extend_open2 = pack16(extend + open, extend + open);
    boundary_t<std::int32_t> const edge {open, extend, affine, local};
    int const classes = costs.classes;
    std::int8_t const *table_a = a.transposed ? costs.profile_table_t : costs.profile_table;
    std::int8_t const *table_b = b.transposed ? costs.profile_table_t : costs.profile_table;
    std::int8_t *profile_a = profile;
    std::int8_t *profile_b = profile + classes * S;
    std::uint8_t const *cols_b = b_present ? b.cols : a.cols;

    // Affine tracks: Ĥ = H + open (the one value both gap tracks extend from), E and F as they are; the profile holds
    // s - open so that Ĥ_diag + (s - open) = H_diag + s. The host routes a pair here only when s - open fits a byte.
    // Linear tracks: H as it is.
    std::int32_t const h_shift = affine ? open : 0;
    // Gap-track seeds: global `open + extend + M[i][0]`, local `open + extend` (unused by linear tracks).
    auto gap_seed = [&](std::int64_t i) -> std::int32_t {
        return local ? open + extend : open + extend + edge.score(i);
    };
    // Packed codes of column j (1-based) of both pairs: 8-bit halves for profile lookups, negated 16-bit halves in
    // compare mode (16-bit strings: their own codes).
    auto column_code = [&](std::uint32_t j) -> std::uint32_t {
        if constexpr (policy_::wide_k) {
            std::uint32_t const ca = j <= m_a ? symbol_at<true>(a.cols, j - 1) : 0u;
            std::uint32_t const cb = j <= m_b ? symbol_at<true>(cols_b, j - 1) : 0u;
            return compare_costs_t::column_codes(ca, cb);
        }
        else {
            std::uint32_t const ca = j <= m_a ? costs.byte_to_compact[a.cols[j - 1]] : 0u;
            std::uint32_t const cb = j <= m_b ? costs.byte_to_compact[cols_b[j - 1]] : 0u;
            return compare ? compare_costs_t::column_codes(ca, cb) : ca | (cb << 8);
        }
    };
    // Compare mode: costs of equal and different codes (shifted like the profile for affine tracks).
    compare_costs_t const compared(costs.match - (affine ? open : 0), costs.mismatch - (affine ? open : 0));

    std::int32_t result_a = 0, result_b = 0;
    std::uint32_t lane_best = 0; // packed running maxima of valid cells (local scores), starts at 0 like the reference

    for (std::uint32_t strip_base = 0; strip_base < n_max; strip_base += S) {
        std::uint32_t const rows_here = min((std::uint32_t)S, n_max - strip_base);
        bool const last_strip = strip_base + S >= n_max;
        int const last_lane = int((rows_here - 1) / R);
        std::int64_t const row0 = (std::int64_t)strip_base + lane * R + 1;

        // Profiles of both pairs for this strip: profile[cc * S + row] = cost(row class, column class cc); in compare
        // mode, the rows' packed codes instead.
        std::uint32_t row_codes[compare ? R : 1];
        __syncwarp();
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::int64_t const i = row0 + r;
            if constexpr (policy_::wide_k) {
                std::uint32_t const code_a = i <= (std::int64_t)n_a ? symbol_at<true>(a.rows, i - 1) : 0u;
                std::uint32_t const code_b = i <= (std::int64_t)n_b ? symbol_at<true>(b.rows, i - 1) : 0u;
                row_codes[r] = code_a | (code_b << 16);
                continue;
            }
            int const class_a = costs.byte_to_class[i <= (std::int64_t)n_a ? a.rows[i - 1] : 0u];
            int const class_b = costs.byte_to_class[i <= (std::int64_t)n_b ? b.rows[i - 1] : 0u];
            if constexpr (compare) row_codes[r] = std::uint32_t(class_a) | (std::uint32_t(class_b) << 16);
            else
                for (int cc = 0; cc < classes; ++cc) {
                    profile_a[cc * S + lane * R + r] = std::int8_t(table_a[cc * 32 + class_a] - h_shift);
                    profile_b[cc * S + lane * R + r] = std::int8_t(table_b[cc * 32 + class_b] - h_shift);
                }
        }

        std::uint32_t h_col[R], e_col[R], best_row[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::int32_t const h = edge.score(row0 + r) + h_shift;
            h_col[r] = pack16(h, h);
            std::int32_t const e = gap_seed(row0 + r);
            e_col[r] = pack16(e, e);
            best_row[r] = 0;
        }
        std::int32_t const diag_seed = edge.score(row0 - 1) + h_shift;
        std::uint32_t diag_up = pack16(diag_seed, diag_seed);

        // Lanes holding each pair's last row in this strip, and the row inside the lane.
        bool const a_ends_here = strip_base < n_a && strip_base + S >= n_a;
        bool const b_ends_here = b_present && strip_base < n_b && strip_base + S >= n_b;
        int const a_lane = a_ends_here ? int((n_a - 1 - strip_base) / R) : -1;
        int const b_lane = b_ends_here ? int((n_b - 1 - strip_base) / R) : -1;
        int const a_row = int((n_a - 1 - strip_base) % R), b_row = int((n_b - 1 - strip_base) % R);

        bool const write_bottom = !last_strip;
        bool const bottom_writer = write_bottom && lane == 31;
        int const lane_rows = lane * R;
        if constexpr (policy_::columns_k == 1) {
            std::uint32_t const steps = m_max + (std::uint32_t)last_lane;
            std::uint32_t out_h = 0, out_f = 0;
            std::uint32_t code_now = lane == 0 ? column_code(1) : 0u;
            __syncwarp();
            [[maybe_unused]] std::uint32_t pa_now[words], pb_now[words]; // profile words (unused in compare mode)
            if constexpr (!compare) {
                load_profile_words<R>(profile_a + (code_now & 0xFF) * S + lane * R, pa_now);
                load_profile_words<R>(profile_b + (code_now >> 8) * S + lane * R, pb_now);
            }

            // One step of the sweep. `steady` steps are those where every lane is on a real column below both pairs'
            // ends (31 <= t < m_min - 1): no range predicates, no masks, no result capture.
            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (chunk_columns_k - 1);
                if (e == 0) {
                    // Stage lane 0's next 64 top-boundary values (columns t+1..) and codes (columns t+2..).
                    __syncwarp();
#pragma unroll
                    for (int k = lane; k < chunk_columns_k; k += 32) {
                        std::uint32_t const j = t + 1 + k;
                        std::uint32_t h = 0, f = 0;
                        if (j <= m_max) {
                            if (strip_base == 0) {
                                std::int32_t const v = edge.score(j) + h_shift, g = gap_seed(j);
                                h = pack16(v, v), f = pack16(g, g);
                            }
                            else {
                                uint2 const stored = *reinterpret_cast<uint2 const *>(scratch + 2 * j);
                                h = stored.x, f = stored.y;
                            }
                        }
                        chunk.top_h[k] = h;
                        chunk.top_f[k] = f;
                        chunk.code[k] = j + 1 <= m_max ? column_code(j + 1) : 0u;
                    }
                    __syncwarp();
                }
                std::uint32_t const staged_h = chunk.top_h[e], staged_f = chunk.top_f[e], staged_code = chunk.code[e];
                std::uint32_t up_h = __shfl_up_sync(0xFFFFFFFFu, out_h, 1);
                std::uint32_t up_f = affine ? __shfl_up_sync(0xFFFFFFFFu, out_f, 1) : 0u;
                std::uint32_t code_next = __shfl_up_sync(0xFFFFFFFFu, code_now, 1);
                if (lane == 0) up_h = staged_h, up_f = staged_f, code_next = staged_code;
                [[maybe_unused]] std::uint32_t pa_next[words], pb_next[words];
                if constexpr (!compare) {
                    load_profile_words<R>(profile_a + (code_next & 0xFF) * S + lane_rows, pa_next);
                    load_profile_words<R>(profile_b + (code_next >> 8) * S + lane_rows, pb_next);
                }

                int const j = (int)t + 1 - lane;
                bool const active = steady || (j >= 1 && j <= (int)m_max && lane <= last_lane);
                if (active) {
                    std::uint32_t diag = diag_up;
                    diag_up = up_h;
                    std::uint32_t h_up = up_h, f_up = up_f;
                    std::uint32_t subs[R], cell_h[R];
                    if constexpr (compare) compared.rows<policy_::multiply_k>(row_codes, code_now, subs);
                    else {
#pragma unroll
                        for (int w = 0; w < words; ++w) {
                            subs[4 * w + 0] = interleave_signed_bytes<0>(pa_now[w], pb_now[w]);
                            subs[4 * w + 1] = interleave_signed_bytes<1>(pa_now[w], pb_now[w]);
                            subs[4 * w + 2] = interleave_signed_bytes<2>(pa_now[w], pb_now[w]);
                            subs[4 * w + 3] = interleave_signed_bytes<3>(pa_now[w], pb_now[w]);
                        }
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::uint32_t h, kept;
                        if constexpr (affine) {
                            // h_col, h_up and diag hold Ĥ = H + open; e_col and f_up hold E and F.
                            // E = max(E + ext, H + open); x = max(H_diag + s, E); F = max(F + ext, H + open).
                            std::uint32_t const e_new = ops::add_opt(e_col[r], extend2, h_col[r]);
                            std::uint32_t const x = ops::add_opt(diag, subs[r], e_new);
                            f_up = ops::add_opt(f_up, extend2, h_up);
                            h = local ? ops::opt2_relu(x, f_up) : ops::opt2(x, f_up);
                            kept = ops::add(h, open2);
                            e_col[r] = e_new;
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
                        h_col[r] = kept;
                        h_up = kept;
                    }
                    if constexpr (local) {
                        if constexpr (steady) {
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_h[r], 0u);
                        }
                        else {
                            // Columns past one pair's end carry filler in that half: mask it out of the maxima
                            // (H >= 0).
                            std::uint32_t const mask = j <= (int)m_min ? 0xFFFFFFFFu
                                                                       : ((j <= (int)m_a ? 0x0000FFFFu : 0u) |
                                                                          (j <= (int)m_b ? 0xFFFF0000u : 0u));
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_h[r] & mask, 0u);
                        }
                    }
                    else if constexpr (!steady) {
                        if (lane == a_lane && j == (int)m_a) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == a_row) result_a = low16(cell_h[r]);
                        }
                        if (lane == b_lane && j == (int)m_b) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == b_row) result_b = high16(cell_h[r]);
                        }
                    }
                    out_h = h_up, out_f = f_up;
                    if (bottom_writer) *reinterpret_cast<uint2 *>(scratch + 2 * j) = make_uint2(out_h, out_f);
                }
                code_now = code_next;
                if constexpr (!compare) {
#pragma unroll
                    for (int w = 0; w < words; ++w) pa_now[w] = pa_next[w], pb_now[w] = pb_next[w];
                }
            };

            std::uint32_t const fill_end = min(steps, 31u);
            std::uint32_t const steady_end = m_min >= 1u + 31u ? max(fill_end, m_min - 1u) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end; ++t) step(t, std::false_type {});
#pragma unroll 2
            for (; t < steady_end; ++t) step(t, std::true_type {});
            for (; t < steps; ++t) step(t, std::false_type {});
        }
        else {
            // Two columns per step: at step t lane l scores columns 2(t - l) + 1 and 2(t - l) + 2 of both pairs, so a
            // round of shuffles, the code words, the profile lookups and the step's fixed work serve twice the
            // cells, and the second column's cells run beside the first column's next row. A strip takes
            // ceil(m_max / 2) + last lane steps; staging stays 64 columns (32 steps) at a time.
            constexpr std::uint32_t steps_per_chunk = chunk_columns_k / 2;
            std::uint32_t const steps = (m_max + 1) / 2 + (std::uint32_t)last_lane;
            std::uint32_t out_ha = 0, out_hb = 0, out_fa = 0, out_fb = 0;
            std::uint32_t code_a = lane == 0 ? column_code(1) : 0u; // both pairs' codes of the lane's two columns
            std::uint32_t code_b = lane == 0 && m_max >= 2 ? column_code(2) : 0u;
            __syncwarp();
            [[maybe_unused]] std::uint32_t pa_a[words], pb_a[words], pa_b[words], pb_b[words]; // pair, column
            if constexpr (!compare) {
                load_profile_words<R>(profile_a + (code_a & 0xFF) * S + lane_rows, pa_a);
                load_profile_words<R>(profile_b + (code_a >> 8) * S + lane_rows, pb_a);
                load_profile_words<R>(profile_a + (code_b & 0xFF) * S + lane_rows, pa_b);
                load_profile_words<R>(profile_b + (code_b >> 8) * S + lane_rows, pb_b);
            }
            auto substitutions = [&](std::uint32_t code, std::uint32_t const (&p_a)[words],
                                     std::uint32_t const (&p_b)[words], std::uint32_t (&subs)[R]) {
                if constexpr (compare) compared.rows<policy_::multiply_k>(row_codes, code, subs);
                else {
#pragma unroll
                    for (int w = 0; w < words; ++w) {
                        subs[4 * w + 0] = interleave_signed_bytes<0>(p_a[w], p_b[w]);
                        subs[4 * w + 1] = interleave_signed_bytes<1>(p_a[w], p_b[w]);
                        subs[4 * w + 2] = interleave_signed_bytes<2>(p_a[w], p_b[w]);
                        subs[4 * w + 3] = interleave_signed_bytes<3>(p_a[w], p_b[w]);
                    }
                }
            };
            // One packed cell pair as in the one-column sweep: returns H, sets `kept` (Ĥ for affine tracks, else H)
            // and updates E (from the left) and F (for the cell below).
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

            // `steady`: every lane's two columns are real and below both pairs' ends (31 <= t, 2t + 2 < m_min).
            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (steps_per_chunk - 1);
                if (e == 0) {
                    // Stage lane 0's next 64 top-boundary values (columns 2t + 1..) and codes (columns 2t + 3..).
                    __syncwarp();
#pragma unroll
                    for (int k = lane; k < chunk_columns_k; k += 32) {
                        std::uint32_t const j = 2 * t + 1 + k;
                        std::uint32_t h = 0, f = 0;
                        if (j <= m_max) {
                            if (strip_base == 0) {
                                std::int32_t const v = edge.score(j) + h_shift, g = gap_seed(j);
                                h = pack16(v, v), f = pack16(g, g);
                            }
                            else {
                                uint2 const stored = *reinterpret_cast<uint2 const *>(scratch + 2 * j);
                                h = stored.x, f = stored.y;
                            }
                        }
                        chunk.top_h[k] = h;
                        chunk.top_f[k] = f;
                        chunk.code[k] = j + 2 <= m_max ? column_code(j + 2) : 0u;
                    }
                    __syncwarp();
                }
                std::uint32_t up_ha = __shfl_up_sync(0xFFFFFFFFu, out_ha, 1);
                std::uint32_t up_hb = __shfl_up_sync(0xFFFFFFFFu, out_hb, 1);
                std::uint32_t up_fa = affine ? __shfl_up_sync(0xFFFFFFFFu, out_fa, 1) : 0u;
                std::uint32_t up_fb = affine ? __shfl_up_sync(0xFFFFFFFFu, out_fb, 1) : 0u;
                std::uint32_t next_a = __shfl_up_sync(0xFFFFFFFFu, code_a, 1);
                std::uint32_t next_b = __shfl_up_sync(0xFFFFFFFFu, code_b, 1);
                if (lane == 0) {
                    up_ha = chunk.top_h[2 * e], up_hb = chunk.top_h[2 * e + 1];
                    up_fa = chunk.top_f[2 * e], up_fb = chunk.top_f[2 * e + 1];
                    next_a = chunk.code[2 * e], next_b = chunk.code[2 * e + 1];
                }
                [[maybe_unused]] std::uint32_t qa_a[words], qb_a[words], qa_b[words], qb_b[words];
                if constexpr (!compare) {
                    load_profile_words<R>(profile_a + (next_a & 0xFF) * S + lane_rows, qa_a);
                    load_profile_words<R>(profile_b + (next_a >> 8) * S + lane_rows, qb_a);
                    load_profile_words<R>(profile_a + (next_b & 0xFF) * S + lane_rows, qa_b);
                    load_profile_words<R>(profile_b + (next_b >> 8) * S + lane_rows, qb_b);
                }

                int const ja = 2 * ((int)t - lane) + 1;
                bool const active = steady || (ja >= 1 && ja <= (int)m_max && lane <= last_lane);
                if (active) {
                    std::uint32_t diag_a = diag_up, diag_b = up_ha;
                    diag_up = up_hb;
                    std::uint32_t h_up_a = up_ha, h_up_b = up_hb, f_up_a = up_fa, f_up_b = up_fb;
                    std::uint32_t subs_a[R], subs_b[R], cell_a[R], cell_b[R];
                    substitutions(code_a, pa_a, pb_a, subs_a);
                    substitutions(code_b, pa_b, pb_b, subs_b);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::uint32_t e_left = e_col[r], kept_a, kept_b;
                        cell_a[r] = cell(diag_a, h_col[r], e_left, h_up_a, f_up_a, subs_a[r], kept_a);
                        cell_b[r] = cell(diag_b, kept_a, e_left, h_up_b, f_up_b, subs_b[r], kept_b);
                        diag_a = h_col[r];
                        diag_b = kept_a;
                        h_col[r] = kept_b;
                        if constexpr (affine) e_col[r] = e_left;
                        h_up_a = kept_a;
                        h_up_b = kept_b;
                    }
                    if constexpr (local) {
                        if constexpr (steady) {
#pragma unroll
                            for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_a[r], cell_b[r]);
                        }
                        else {
                            // Columns past one pair's end carry filler in that half: masked out of the maxima.
                            auto half_mask = [&](int j) {
                                return j <= (int)m_min ? 0xFFFFFFFFu
                                                       : ((j <= (int)m_a ? 0x0000FFFFu : 0u) |
                                                          (j <= (int)m_b ? 0xFFFF0000u : 0u));
                            };
                            std::uint32_t const mask_a = half_mask(ja), mask_b = half_mask(ja + 1);
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                best_row[r] = __vimax3_s16x2(best_row[r], cell_a[r] & mask_a, cell_b[r] & mask_b);
                        }
                    }
                    else if constexpr (!steady) {
                        if (lane == a_lane && (ja == (int)m_a || ja + 1 == (int)m_a)) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == a_row) result_a = low16(ja == (int)m_a ? cell_a[r] : cell_b[r]);
                        }
                        if (lane == b_lane && (ja == (int)m_b || ja + 1 == (int)m_b)) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == b_row) result_b = high16(ja == (int)m_b ? cell_a[r] : cell_b[r]);
                        }
                    }
                    out_ha = h_up_a, out_hb = h_up_b, out_fa = f_up_a, out_fb = f_up_b;
                    if (bottom_writer) {
                        *reinterpret_cast<uint2 *>(scratch + 2 * ja) = make_uint2(out_ha, out_fa);
                        if (steady || ja + 1 <= (int)m_max)
                            *reinterpret_cast<uint2 *>(scratch + 2 * (ja + 1)) = make_uint2(out_hb, out_fb);
                    }
                }
                code_a = next_a, code_b = next_b;
                if constexpr (!compare) {
#pragma unroll
                    for (int w = 0; w < words; ++w)
                        pa_a[w] = qa_a[w], pb_a[w] = qb_a[w], pa_b[w] = qa_b[w], pb_b[w] = qb_b[w];
                }
            };

            std::uint32_t const fill_end = min(steps, 31u);
            std::uint32_t const steady_end =
                m_min >= 1u && (m_min - 1u) / 2u > 31u ? max(fill_end, (m_min - 1u) / 2u) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end; ++t) step(t, std::false_type {});
#pragma unroll 2
            for (; t < steady_end; ++t) step(t, std::true_type {});
            for (; t < steps; ++t) step(t, std::false_type {});
        }
        if constexpr (local) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                std::uint32_t const keep = ((row0 + r <= (std::int64_t)n_a) ? 0x0000FFFFu : 0u) |
                                           ((row0 + r <= (std::int64_t)n_b) ? 0xFFFF0000u : 0u);
                lane_best = __vimax3_s16x2(lane_best, best_row[r] & keep, 0u);
            }
        }
        __syncwarp();
    }
    if constexpr (local) {
#pragma unroll
        for (int offset = 16; offset > 0; offset >>= 1)
            lane_best = __vimax3_s16x2(lane_best, __shfl_xor_sync(0xFFFFFFFFu, lane_best, offset), 0u);
        result_a = low16(lane_best), result_b = high16(lane_best);
    }
    else {
        // The capturing lanes hold the results; broadcast them.
        int const a_owner = (int)((n_a - 1) % S) / R;
        int const b_owner = b_present ? (int)((n_b - 1) % S) / R : 0;
        result_a = __shfl_sync(0xFFFFFFFFu, result_a, a_owner);
        result_b = __shfl_sync(0xFFFFFFFFu, result_b, b_owner);
    }
    score_a = result_a;
    score_b = result_b;
}

/** Persistent kernel over the 16x2 bins: warps take two consecutive scheduled pairs at a time. */
template <typename policy_>
__global__ void __launch_bounds__(256) dp16_wavefront_kernel(pair_task_t const *__restrict__ tasks,
                                                             plan_bins_t *__restrict__ bins, int key_begin,
                                                             int key_end, score_costs_t const costs,
                                                             std::int64_t *__restrict__ results,
                                                             std::uint32_t *__restrict__ scratch,
                                                             std::size_t scratch_cells_per_warp) {
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + ((sizeof(score_costs_t) + 15) / 16) * 16);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    int const lane = threadIdx.x & 31;
    int const warp_in_cta = threadIdx.x >> 5;
    std::size_t const global_warp = (std::size_t)blockIdx.x * (blockDim.x >> 5) + warp_in_cta;
    std::uint32_t *warp_scratch = scratch + global_warp * scratch_cells_per_warp;
    std::size_t const profile_bytes = (std::size_t)dp16_profile_bytes_per_warp<policy_>(costs.classes);
    auto *chunks = reinterpret_cast<column_chunk_t *>(profiles + (blockDim.x >> 5) * profile_bytes);
    std::int8_t *warp_profile = profiles + warp_in_cta * profile_bytes;
    column_chunk_t &warp_chunk = chunks[warp_in_cta];
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    while (true) {
        std::uint32_t index = 0;
        if (lane == 0) index = atomicAdd(&bins->cursor[key_begin], 2u);
        index = __shfl_sync(0xFFFFFFFFu, index, 0);
        if (index >= count) break;
        pair_task_t const first = tasks[begin + index];
        bool const has_second = index + 1 < count;
        pair_task_t const second = has_second ? tasks[begin + index + 1] : first;
        std::int64_t score_a = 0, score_b = 0;
        dp16_score_couple<policy_>(first, second, has_second, costs_s, warp_scratch, warp_profile, warp_chunk, score_a,
                                   score_b);
        if (lane == 0) {
            results[first.slot] = score_a;
            if (has_second) results[second.slot] = score_b;
        }
    }
}

} // namespace szs_gb300
