/**
 *  @file dp_short.cuh
 *  @brief Short pairs (shorter side at most 128): a warp cut into segments of 1 to 16 lanes, each segment scoring
 *         two pairs at once on 16x2 packed cells, so a warp holds up to 64 pairs.
 *
 *  The 16x2 wavefront (dp_packed.cuh) gives a pair a whole warp: lane L owns rows L*R..L*R+R-1 of a strip of
 *  32 x R rows. A pair of 40 rows on R = 4 keeps 10 of the 32 lanes busy and pays 31 fill steps per strip. Here a
 *  warp is cut into 32 / L segments of L lanes (`__shfl_up_sync` with width L keeps each segment's neighbour exchange
 *  inside it), every segment holds one strip of L x R rows of two pairs (pair A in the low halves, pair B in the high
 *  halves), and a pair's whole column fits that strip, so there are no boundary rows in global memory and no fill
 *  steps beyond L - 1. The cell update is the one of dp_packed.cuh (affine tracks keep Ĥ = H + open; five DPX
 *  operations per packed register):
 *
 *      E = max(E_left + extend, Ĥ_left)
 *      X = max(Ĥ_diag + (s - open), E)
 *      F = max(F_up + extend, Ĥ_up)
 *      H = max(X, F)                              (local: also max(., 0))
 *      Ĥ = H + open
 *
 *  (min for Levenshtein). Substitution costs come from per-pair int8 profiles in shared memory (one strip per pair),
 *  or, for Levenshtein over more than 32 byte values, from comparing codes (`compare_costs_t`). A profile is written
 *  from a row-class-major copy of the table with 16-byte loads and 4 x 4 byte transposes, one 4-byte store per
 *  class and 4 rows. Each segment's lane 0 takes the top boundary from its closed form (advanced one column per step)
 *  and the column codes from a register the segment's lanes load L columns at a time. A segment runs
 *  max(m_A, m_B) + L - 1 steps; the warp runs its slowest segment's steps, so the planner bins these pairs by the
 *  length of their longer side.
 *
 *  Counterpart of the reference's register tier for short pairs (include/stringzillas/similarities/cuda.cuh:
 *  4837-5031, one thread per pair with 16-bit rows), and the same recurrences as its serial walkers
 *  (serial.hpp:723-725, :924-930, local clamps :817-818, :1045-1046).
 */
#pragma once
#include <type_traits>

#include "dp_cells.cuh"
#include "dp_packed.cuh"
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

template <int kind_, bool affine_, int lanes_, int rows_per_lane_, int compare_ = compare_none_k>
struct short_policy_t {
    static constexpr int kind_k = kind_;
    static constexpr bool affine_k = affine_;
    static constexpr bool maximize_k = kind_ != kind_levenshtein_k;
    static constexpr bool local_k = kind_ == kind_smith_waterman_k;
    static constexpr int lanes_k = lanes_;
    static constexpr int rows_per_lane_k = rows_per_lane_;
    static constexpr int segment_rows_k = lanes_ * rows_per_lane_;
    static constexpr int segments_k = warp_size_k / lanes_;
    static constexpr bool compare_k = compare_ != compare_none_k;
    static constexpr bool multiply_k = compare_ == compare_multiply_k;
    static_assert(lanes_ == 1 || lanes_ == 2 || lanes_ == 4 || lanes_ == 8 || lanes_ == 16, "segments of 1 to 16 lanes");
    static_assert(rows_per_lane_ % 4 == 0, "profile rows are read in 4-byte words");
    static_assert(!compare_k || kind_ == kind_levenshtein_k, "only Levenshtein costs are a function of equality");
};

/** Per-warp shared profile bytes: segments x two pairs x classes x segment rows (none in compare mode). */
template <typename policy_>
__host__ __device__ constexpr int short_profile_bytes_per_warp(int classes) {
    return policy_::compare_k ? 0 : policy_::segments_k * 2 * classes * policy_::segment_rows_k;
}

/** Costs, both orientations of the row-class-major table (`row_costs`), then the warps' profiles. */
template <typename policy_>
__host__ __device__ constexpr int short_shared_bytes(int warps_per_cta, int classes) {
    return int((sizeof(score_costs_t) + 15) / 16 * 16) + 2 * 32 * 32 +
           warps_per_cta * short_profile_bytes_per_warp<policy_>(classes);
}

/** 4 x 4 byte transpose: out[c] holds byte c of in[0], in[1], in[2], in[3]. */
__device__ __forceinline__ void transpose_bytes_4x4(std::uint32_t const (&in)[4], std::uint32_t (&out)[4]) {
    std::uint32_t const t0 = __byte_perm(in[0], in[1], 0x5140u), t1 = __byte_perm(in[0], in[1], 0x7362u);
    std::uint32_t const t2 = __byte_perm(in[2], in[3], 0x5140u), t3 = __byte_perm(in[2], in[3], 0x7362u);
    out[0] = __byte_perm(t0, t2, 0x5410u), out[1] = __byte_perm(t0, t2, 0x7632u);
    out[2] = __byte_perm(t1, t3, 0x5410u), out[3] = __byte_perm(t1, t3, 0x7632u);
}

/**
 *  Writes one pair's profile for this lane's R rows: profile[cc * S + lane row] = row_costs[row class][cc] for every
 *  column class cc. Each row's 32 costs come in two 16-byte loads of the row-class-major table, and 4 x 4 byte
 *  transposes turn them into one 4-byte word per class and 4 rows.
 */
template <int rows_, int segment_rows_>
__device__ __forceinline__ void short_write_profile(std::uint8_t const *row_costs,
                                                    std::uint32_t const (&row_class)[rows_], int classes,
                                                    std::int8_t *profile, int lane_row0) {
#pragma unroll
    for (int g = 0; g < rows_ / 4; ++g) {
        std::uint32_t costs[4][8]; // rows 4g..4g+3, classes 0..31 (four per word)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint4 const lo = *reinterpret_cast<uint4 const *>(row_costs + row_class[4 * g + k] * 32);
            uint4 const hi = *reinterpret_cast<uint4 const *>(row_costs + row_class[4 * g + k] * 32 + 16);
            costs[k][0] = lo.x, costs[k][1] = lo.y, costs[k][2] = lo.z, costs[k][3] = lo.w;
            costs[k][4] = hi.x, costs[k][5] = hi.y, costs[k][6] = hi.z, costs[k][7] = hi.w;
        }
#pragma unroll
        for (int cg = 0; cg < 8; ++cg) {
            if (4 * cg >= classes) break;
            std::uint32_t const in[4] = {costs[0][cg], costs[1][cg], costs[2][cg], costs[3][cg]};
            std::uint32_t out[4];
            transpose_bytes_4x4(in, out);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (4 * cg + c < classes)
                    *reinterpret_cast<std::uint32_t *>(profile + (4 * cg + c) * segment_rows_ + lane_row0 + 4 * g) =
                        out[c];
        }
    }
}

/**
 *  Scores this segment's pairs @p a and @p b (either may be absent) with the segment's L lanes; all 32 lanes of the
 *  warp call it together. Results land in every lane of the segment.
 */
template <typename policy_>
__device__ __forceinline__ void short_score_segment(pair_task_t const &a, bool a_present, pair_task_t const &b,
                                                    bool b_present, score_costs_t const &costs,
                                                    std::uint8_t const *row_costs, std::int8_t *profile,
                                                    std::int64_t &score_a, std::int64_t &score_b) {
    using ops = packed_ops_t<policy_::maximize_k>;
    constexpr int L = policy_::lanes_k;
    constexpr int R = policy_::rows_per_lane_k;
    constexpr int S = policy_::segment_rows_k;
    constexpr bool affine = policy_::affine_k;
    constexpr bool local = policy_::local_k;
    constexpr bool compare = policy_::compare_k;
    constexpr int words = compare ? 1 : R / 4;

    int const lane = threadIdx.x & 31;
    int const segment_lane = lane & (L - 1);
    int const segment_base = lane & ~(L - 1);
    std::uint32_t const n_a = a_present ? a.rows_length : 0u, m_a = a_present ? a.cols_length : 0u;
    std::uint32_t const n_b = b_present ? b.rows_length : 0u, m_b = b_present ? b.cols_length : 0u;
    std::uint32_t const n_max = max(n_a, n_b), m_max = max(m_a, m_b), m_min = min(m_a, m_b);
    std::int32_t const open = costs.open, extend = costs.extend;
    std::uint32_t const open2 = pack16(open, open), extend2 = pack16(extend, extend);
    boundary_t<std::int32_t> const edge {open, extend, affine, local};
    int const classes = costs.classes;
    std::int8_t *profile_a = profile;
    std::int8_t *profile_b = profile + classes * S;
    std::int32_t const h_shift = affine ? open : 0;
    auto gap_seed = [&](std::int64_t i) -> std::int32_t {
        return local ? open + extend : open + extend + edge.score(i);
    };
    auto column_code = [&](std::uint32_t j) -> std::uint32_t {
        std::uint32_t const ca = j >= 1 && j <= m_a ? costs.byte_to_compact[a.cols[j - 1]] : 0u;
        std::uint32_t const cb = j >= 1 && j <= m_b ? costs.byte_to_compact[b.cols[j - 1]] : 0u;
        return compare ? compare_costs_t::column_codes(ca, cb) : ca | (cb << 8);
    };
    compare_costs_t const compared(costs.match - (affine ? open : 0), costs.mismatch - (affine ? open : 0));

    // The segment's rows: lane l owns rows l*R + 1 .. l*R + R of both pairs.
    std::int64_t const row0 = (std::int64_t)segment_lane * R + 1;
    std::uint32_t row_codes[compare ? R : 1];
    std::uint32_t class_a[R], class_b[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        std::int64_t const i = row0 + r;
        // Profile classes index a 32 x 32 table; compare mode keeps whole byte codes.
        std::uint32_t const class_mask = compare ? 0xFFu : 31u;
        class_a[r] = costs.byte_to_class[i <= (std::int64_t)n_a ? a.rows[i - 1] : 0u] & class_mask;
        class_b[r] = costs.byte_to_class[i <= (std::int64_t)n_b ? b.rows[i - 1] : 0u] & class_mask;
        if constexpr (compare) row_codes[r] = class_a[r] | (class_b[r] << 16);
    }
    if constexpr (!compare) {
        short_write_profile<R, S>(row_costs + (a.transposed ? 1024 : 0), class_a, classes, profile_a, segment_lane * R);
        short_write_profile<R, S>(row_costs + (b.transposed ? 1024 : 0), class_b, classes, profile_b, segment_lane * R);
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

    int const last_lane = n_max ? int((n_max - 1) / R) : -1;
    int const a_lane = n_a ? int((n_a - 1) / R) : -1, a_row = n_a ? int((n_a - 1) % R) : 0;
    int const b_lane = n_b ? int((n_b - 1) / R) : -1, b_row = n_b ? int((n_b - 1) % R) : 0;
    // Steps of this segment, then of the warp (its slowest segment); the steady steps are those where every lane of
    // every segment is on a column inside both of its pairs (lanes below a segment's last row compute filler that
    // nothing reads), so they need no range checks, masks or result captures.
    std::uint32_t warp_steps = m_max && n_max ? m_max + (std::uint32_t)last_lane : 0u;
    std::uint32_t steady_end = m_min;
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) {
        warp_steps = max(warp_steps, __shfl_xor_sync(0xFFFFFFFFu, warp_steps, offset));
        steady_end = min(steady_end, __shfl_xor_sync(0xFFFFFFFFu, steady_end, offset));
    }
    std::uint32_t const fill_end = min(warp_steps, (std::uint32_t)(L - 1));
    steady_end = steady_end >= 1u ? max(fill_end, min(warp_steps, steady_end - 1u)) : fill_end;

    std::uint32_t out_h = 0, out_f = 0;
    std::uint32_t code_now = segment_lane == 0 ? column_code(1) : 0u;
    std::uint32_t staged_code = 0; // lane l of the segment: the code of column (block start) + 2 + l
    // Row 0 of the next column, for the segment's lane 0: its closed form, advanced by one column per step.
    std::int32_t const top_first = edge.score(1) + h_shift, top_step = affine ? extend : open;
    std::uint32_t top_h = pack16(top_first, top_first);
    std::uint32_t top_f = pack16(gap_seed(1), gap_seed(1));
    std::uint32_t const top_delta = local ? 0u : pack16(top_step, top_step);
    __syncwarp();
    [[maybe_unused]] std::uint32_t pa_now[words], pb_now[words];
    if constexpr (!compare) {
        load_profile_words<R>(profile_a + (code_now & 0xFF) * S + segment_lane * R, pa_now);
        load_profile_words<R>(profile_b + (code_now >> 8) * S + segment_lane * R, pb_now);
    }
    std::int32_t result_a = 0, result_b = 0;

    auto step = [&](std::uint32_t t, auto steady_tag) {
        constexpr bool steady = decltype(steady_tag)::value;
        std::uint32_t code_next;
        std::uint32_t up_h, up_f;
        if constexpr (L == 1) {
            // One lane per segment: every lane is a segment's first, and reads its own next code.
            code_next = column_code(t + 2);
            up_h = top_h, up_f = top_f;
        }
        else {
            std::uint32_t const e = t & (L - 1);
            if (e == 0) staged_code = column_code(t + 2 + segment_lane);
            std::uint32_t const fetched = __shfl_sync(0xFFFFFFFFu, staged_code, segment_base + (int)e);
            up_h = __shfl_up_sync(0xFFFFFFFFu, out_h, 1, L);
            up_f = affine ? __shfl_up_sync(0xFFFFFFFFu, out_f, 1, L) : 0u;
            code_next = __shfl_up_sync(0xFFFFFFFFu, code_now, 1, L);
            if (segment_lane == 0) up_h = top_h, up_f = top_f, code_next = fetched;
        }
        top_h = __vadd2(top_h, top_delta), top_f = __vadd2(top_f, top_delta);
        [[maybe_unused]] std::uint32_t pa_next[words], pb_next[words];
        if constexpr (!compare) {
            load_profile_words<R>(profile_a + (code_next & 0xFF) * S + segment_lane * R, pa_next);
            load_profile_words<R>(profile_b + (code_next >> 8) * S + segment_lane * R, pb_next);
        }
        int const j = (int)t + 1 - segment_lane;
        if (steady || (j >= 1 && j <= (int)m_max && segment_lane <= last_lane)) {
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
                    // Columns past one pair's end carry filler in that half: masked out of the maxima (H >= 0).
                    std::uint32_t const mask = j <= (int)m_min ? 0xFFFFFFFFu
                                                               : ((j <= (int)m_a ? 0x0000FFFFu : 0u) |
                                                                  (j <= (int)m_b ? 0xFFFF0000u : 0u));
#pragma unroll
                    for (int r = 0; r < R; ++r) best_row[r] = __vimax3_s16x2(best_row[r], cell_h[r] & mask, 0u);
                }
            }
            else if constexpr (!steady) {
                if (segment_lane == a_lane && j == (int)m_a) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if (r == a_row) result_a = low16(cell_h[r]);
                }
                if (segment_lane == b_lane && j == (int)m_b) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if (r == b_row) result_b = high16(cell_h[r]);
                }
            }
            out_h = h_up, out_f = f_up;
        }
        code_now = code_next;
        if constexpr (!compare) {
#pragma unroll
            for (int w = 0; w < words; ++w) pa_now[w] = pa_next[w], pb_now[w] = pb_next[w];
        }
    };
    std::uint32_t t = 0;
    for (; t < fill_end; ++t) step(t, std::false_type {});
    for (; t < steady_end; ++t) step(t, std::true_type {});
    for (; t < warp_steps; ++t) step(t, std::false_type {});

    if constexpr (local) {
        std::uint32_t lane_best = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::uint32_t const keep = ((row0 + r <= (std::int64_t)n_a) ? 0x0000FFFFu : 0u) |
                                       ((row0 + r <= (std::int64_t)n_b) ? 0xFFFF0000u : 0u);
            lane_best = __vimax3_s16x2(lane_best, best_row[r] & keep, 0u);
        }
#pragma unroll
        for (int offset = L / 2; offset > 0; offset >>= 1)
            lane_best = __vimax3_s16x2(lane_best, __shfl_xor_sync(0xFFFFFFFFu, lane_best, offset), 0u);
        result_a = low16(lane_best), result_b = high16(lane_best);
    }
    else {
        result_a = __shfl_sync(0xFFFFFFFFu, result_a, segment_base + (a_lane < 0 ? 0 : a_lane));
        result_b = __shfl_sync(0xFFFFFFFFu, result_b, segment_base + (b_lane < 0 ? 0 : b_lane));
    }
    score_a = result_a;
    score_b = result_b;
}

/** Persistent kernel over the short bins [key_begin, key_end): each warp takes 2 x (32 / L) consecutive scheduled
 *  pairs at a time, two per segment. */
template <typename policy_>
__global__ void __launch_bounds__(256) dp16_short_kernel(pair_task_t const *__restrict__ tasks,
                                                         plan_bins_t *__restrict__ bins, int key_begin, int key_end,
                                                         score_costs_t const costs,
                                                         std::int64_t *__restrict__ results) {
    constexpr int L = policy_::lanes_k;
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::uint8_t *row_costs = shared_bytes + ((sizeof(score_costs_t) + 15) / 16) * 16;
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(row_costs + 2 * 32 * 32);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
        // Row-class-major copies of both orientations: row_costs[o][row class][column class] = table - shift (the
        // affine tracks' s - open, which the planner checked fits a byte).
        std::int32_t const shift = policy_::affine_k ? costs.open : 0;
        for (unsigned i = threadIdx.x; i < 2 * 32 * 32; i += blockDim.x) {
            unsigned const o = i >> 10, row = (i >> 5) & 31u, column = i & 31u;
            std::int8_t const *table = o ? costs.profile_table_t : costs.profile_table;
            row_costs[i] = (std::uint8_t)(std::int8_t)(table[column * 32 + row] - shift);
        }
    }
    __syncthreads();
    int const lane = threadIdx.x & 31;
    int const warp_in_cta = threadIdx.x >> 5;
    int const segment = lane / L;
    std::size_t const warp_profile_bytes = (std::size_t)short_profile_bytes_per_warp<policy_>(costs.classes);
    std::int8_t *segment_profile = profiles + warp_in_cta * warp_profile_bytes +
                                   (std::size_t)segment * 2 * costs.classes * policy_::segment_rows_k;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    constexpr std::uint32_t per_warp = 2 * policy_::segments_k;
    while (true) {
        std::uint32_t index = 0;
        if (lane == 0) index = atomicAdd(&bins->cursor[key_begin], per_warp);
        index = __shfl_sync(0xFFFFFFFFu, index, 0);
        if (index >= count) break;
        std::uint32_t const index_a = index + 2u * (std::uint32_t)segment, index_b = index_a + 1u;
        bool const a_present = index_a < count, b_present = index_b < count;
        pair_task_t const a = tasks[begin + (a_present ? index_a : index)];
        pair_task_t const b = b_present ? tasks[begin + index_b] : a;
        std::int64_t score_a = 0, score_b = 0;
        short_score_segment<policy_>(a, a_present, b, b_present, costs_s, row_costs, segment_profile, score_a,
                                     score_b);
        if ((lane & (L - 1)) == 0) {
            if (a_present) results[a.slot] = score_a;
            if (b_present) results[b.slot] = score_b;
        }
    }
}

} // namespace szs_gb300
