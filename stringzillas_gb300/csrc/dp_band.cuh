/**
 *  @file dp_band.cuh
 *  @brief Long pairs: one CTA per pair, its warps working on consecutive row strips at once.
 *
 *  A single warp sweeps a pair strip by strip, so one pair of 30,000 x 30,000 cells keeps one warp busy for
 *  seconds while the rest of the GPU idles. Here the W warps of a CTA form a ring: warp w scores strips
 *  w, w + W, w + 2W, ... of the same pair. Strip k's bottom row (H and F̂ per column) goes to ring slot k mod W of the
 *  CTA's scratch rows; strip k + 1 reads it as its top boundary while strip k is still advancing, so all W strips
 *  run at the same time, each a few chunks of columns behind the one above. Replaces the reference's tiled device
 *  tier (include/stringzillas/similarities/cuda.cuh:616-1096), which spins without a bound on per-tile progress
 *  flags in global memory.
 *
 *  Progress: ring slot s holds one 64-bit word in shared memory, `(strip + 1) << 32 | columns written`. Slots are
 *  reused every W strips, so the word only grows; a consumer of strip k - 1's row waits until the word reaches
 *  `k << 32 | columns needed`. Only warps of the same CTA wait on each other (co-resident by construction), and every
 *  wait is bounded: after `costs.wait_polls` polls (at most `band_wait_polls_default_k`) the warp raises the CTA's error flag, which also releases the
 *  other warps' waits, the pair is abandoned and the host reports an error for the call.
 *
 *  Groups: when a call has fewer long pairs than the GPU holds CTAs, G co-resident CTAs (one cooperative launch)
 *  share a pair and the ring spans all their G x W warps; its progress words, failure flag and a barrier counter
 *  then live in global memory (`band_group_state_t`), published with GPU-scope fences. Between pairs the CTAs of a
 *  group meet at a bounded barrier; the per-pair words are double-buffered by the pair's parity, so a CTA still
 *  reading one pair's result never sees the next pair's reset.
 *
 *  Inside a strip, lanes, steps, chunk staging and the shortened dependency chain are those of dp_packed.cuh, on
 *  32-bit cells with DPX `__viaddmax_s32` / `__viaddmin_s32`.
 */
#pragma once
#include "dp_cells.cuh"
#include "dp_packed.cuh"
#include "dp_wavefront.cuh"
#include "engine_types.cuh"
#include "planner.cuh"

namespace szs_gb300 {

constexpr int band_warps_k = 8;
constexpr int band_chunk_k = 32;                      // columns staged and published at a time

template <int kind_, bool affine_, int rows_per_lane_, int columns_per_step_ = 1>
struct band_policy_t {
    static constexpr int kind_k = kind_;
    static constexpr bool affine_k = affine_;
    static constexpr bool maximize_k = kind_ != kind_levenshtein_k;
    static constexpr bool local_k = kind_ == kind_smith_waterman_k;
    static constexpr bool uniform_k = kind_ == kind_levenshtein_k;
    static constexpr int rows_per_lane_k = rows_per_lane_;
    static constexpr int columns_k = columns_per_step_; // columns a lane scores per step of the sweep: 1 or 2
    static constexpr int strip_rows_k = warp_size_k * rows_per_lane_;
    static constexpr bool direct_k = false; // `direct_policy_t<>` reads costs from a dense table in shared memory
    static constexpr bool wide_k = false;   // `wide_policy_t<>`: strings of 16-bit codes
    using ops_t = cell_ops_t<std::int32_t, maximize_k>;
};

/** Per-warp staging of lane 0's inputs for the next `band_chunk_k` columns. */
struct band_chunk_t {
    std::int32_t top_h[band_chunk_k];
    std::int32_t top_f[band_chunk_k];
    std::uint32_t code[band_chunk_k];
};

/** Shared state of one CTA. */
struct band_shared_t {
    unsigned long long progress[band_warps_k];
    std::int32_t warp_result[band_warps_k];
    std::uint32_t pair_index;
    std::uint32_t failed;
    std::uint32_t redo; // 16-bit band: the pair reached the 16-bit limit and is scored again on 32-bit cells
    std::uint32_t gate; // grouped kernels: the outcome of the last group barrier
};

template <typename policy_>
__host__ __device__ constexpr int band_profile_bytes_per_warp(int classes) {
    return (policy_::uniform_k || policy_::direct_k) ? 0 : classes * policy_::strip_rows_k;
}

/** Costs, CTA state, per-warp profiles and chunk staging, then (direct-table instances) the dense table. */
template <typename policy_>
__host__ __device__ constexpr int band_shared_bytes(int classes) {
    return int((sizeof(score_costs_t) + 15) / 16 * 16) + int((sizeof(band_shared_t) + 15) / 16 * 16) +
           band_warps_k * (band_profile_bytes_per_warp<policy_>(classes) + int(sizeof(band_chunk_t))) +
           (policy_::direct_k ? direct_table_bytes_k : 0);
}

/** The ring a warp takes part in: its progress words and failure flag (the CTA's shared memory, or global memory
 *  for a group of CTAs), the number of warps in the ring and this warp's place in it. */
struct band_ring_t {
    unsigned long long *progress;
    std::uint32_t *failed;
    int members;
    int member;
    bool grid_scope; // progress and failure words are in global memory, shared with other CTAs
    std::uint32_t wait_polls; // polls before a wait gives up
};

__device__ __forceinline__ band_ring_t band_cta_ring(band_shared_t &shared, int warp, std::uint32_t wait_polls) {
    return {shared.progress, &shared.failed, band_warps_k, warp, false, wait_polls};
}

/** Lane 0 of a warp waits (bounded) until ring slot `slot` has reached `target`; the warp then proceeds together
 *  (the caller's `__syncwarp` orders the other lanes' ring reads after lane 0's wait). In a group's ring the
 *  progress word is read with GPU-scope acquire loads, which order the ring-row reads after it without a full fence,
 *  and the first polls do not sleep: a consumer running just behind its producer resumes within a poll. */
__device__ __forceinline__ bool band_wait(band_ring_t const &ring, int slot, unsigned long long target) {
    int const lane = threadIdx.x & 31;
    int ok = 1;
    if (lane == 0) {
        std::uint32_t polls = 0;
        while (true) {
            unsigned long long seen;
            if (ring.grid_scope)
                asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(seen) : "l"(&ring.progress[slot]) : "memory");
            else
                seen = *reinterpret_cast<volatile unsigned long long *>(&ring.progress[slot]);
            if (seen >= target) break;
            if (*reinterpret_cast<volatile std::uint32_t *>(ring.failed)) {
                ok = 0;
                break;
            }
            if (++polls > ring.wait_polls) {
                atomicExch(ring.failed, 1u);
                ok = 0;
                break;
            }
            if (!ring.grid_scope || polls > 16) __nanosleep(ring.grid_scope ? 64 : 100);
        }
        if (!ring.grid_scope) __threadfence_block();
    }
    ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
    return ok != 0;
}

/** Publishes `value` in ring slot `slot`. Called by the lane that wrote the published ring row, so a GPU-scope
 *  release store orders the row before the word in a group's ring. */
__device__ __forceinline__ void band_publish(band_ring_t const &ring, int slot, unsigned long long value) {
    if (ring.grid_scope) {
        asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(&ring.progress[slot]), "l"(value) : "memory");
    }
    else {
        __threadfence_block();
        *reinterpret_cast<volatile unsigned long long *>(&ring.progress[slot]) = value;
    }
}

/** Most CTAs one long pair can share (enough for every 128-row strip of a 250,000-row pair to have its own warp, so
 *  no warp sweeps a second strip after its first), and the ring words of a group. */
constexpr int band_group_max_ctas_k = 256;
constexpr int band_group_max_members_k = band_group_max_ctas_k * band_warps_k;

/** One pass over a pair (16-bit or 32-bit cells): ring progress and the combined result. */
struct band_pass_state_t {
    unsigned long long progress[band_group_max_members_k];
    std::int32_t best; // local scores: maximum over the group; global scores: the corner cell, from its owner
    std::uint32_t reserved;
};

/** A group's words in global memory: two pair parities x two passes, the failure flag and the barrier counter.
 *  Zeroed by the host before the launch. */
struct band_group_state_t {
    band_pass_state_t pass[2][2];
    std::uint32_t failed;
    std::uint32_t arrived;
};

/** Bounded barrier of the G CTAs of a group: the `number`-th meeting needs G * number arrivals. Returns false when the
 *  group failed or the wait ran out (then the group's failure flag is set). */
__device__ __forceinline__ bool band_group_barrier(band_group_state_t *group, int ctas, std::uint32_t number,
                                                   std::uint32_t &flag_in_shared, std::uint32_t barrier_polls) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&group->arrived, 1u);
        std::uint32_t const target = (std::uint32_t)ctas * number;
        std::uint32_t polls = 0;
        std::uint32_t ok = 1;
        while (*reinterpret_cast<volatile std::uint32_t *>(&group->arrived) < target) {
            if (*reinterpret_cast<volatile std::uint32_t *>(&group->failed)) {
                ok = 0;
                break;
            }
            if (++polls > barrier_polls) {
                atomicExch(&group->failed, 1u);
                ok = 0;
                break;
            }
            __nanosleep(200);
        }
        if (*reinterpret_cast<volatile std::uint32_t *>(&group->failed)) ok = 0;
        __threadfence();
        flag_in_shared = ok;
    }
    __syncthreads();
    return flag_in_shared != 0;
}

/**
 *  Scores strips w, w + W, ... of one pair with warp w. Returns this warp's contribution: the running maximum of its
 *  valid cells for local scores, the corner cell for the warp owning the last row of global scores (else 0).
 */
template <typename policy_>
__device__ __forceinline__ std::int32_t band_score_warp(pair_task_t const &task, score_costs_t const &costs,
                                                        band_ring_t const &sync, std::int32_t *ring,
                                                        std::size_t ring_cells_per_slot, std::int8_t *profile,
                                                        band_chunk_t &chunk, std::int8_t const *table_s = nullptr) {
    using ops = typename policy_::ops_t;
    constexpr int R = policy_::rows_per_lane_k;
    constexpr int S = policy_::strip_rows_k;
    constexpr bool affine = policy_::affine_k;
    constexpr bool local = policy_::local_k;
    std::uint32_t const W = (std::uint32_t)sync.members;
    int const warp = sync.member;
    static_assert(R % 4 == 0, "profile rows are read in 4-byte words");
    constexpr int words = R / 4;

    int const lane = threadIdx.x & 31;
    std::uint32_t const n = task.rows_length, m = task.cols_length;
    std::int32_t const open = costs.open, extend = costs.extend, extend_open = costs.open + costs.extend;
    boundary_t<std::int32_t> const edge {open, extend, affine, local};
    int const classes = costs.classes;
    std::int8_t const *table = task.transposed ? costs.profile_table_t : costs.profile_table;
    auto gap_seed = [&](std::int64_t i) -> std::int32_t { return local ? extend : extend + edge.score(i); };
    auto column_code = [&](std::uint32_t j) -> std::uint32_t {
        std::uint32_t const byte = symbol_at<policy_::wide_k>(task.cols, j - 1);
        if constexpr (policy_::uniform_k || policy_::direct_k) return byte;
        else return costs.byte_to_compact[byte];
    };

    std::uint32_t const strips = (n + S - 1) / S;
    std::int32_t result = 0;
    std::int32_t lane_best = 0;

    for (std::uint32_t k = (std::uint32_t)warp; k < strips; k += W) {
        std::uint32_t const strip_base = k * S;
        std::uint32_t const rows_here = min((std::uint32_t)S, n - strip_base);
        bool const last_strip = k + 1 == strips;
        int const last_lane = int((rows_here - 1) / R);
        std::int64_t const row0 = (std::int64_t)strip_base + lane * R + 1;
        int const slot_in = int((k + W - 1) % W), slot_out = int(k % W);
        std::int32_t const *top = ring + (std::size_t)slot_in * ring_cells_per_slot;
        std::int32_t *bottom = ring + (std::size_t)slot_out * ring_cells_per_slot;

        // Row characters / profile for this strip.
        std::uint32_t row_bytes[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            std::int64_t const i = row0 + r;
            row_bytes[r] = i <= (std::int64_t)n ? symbol_at<policy_::wide_k>(task.rows, i - 1) : 0u;
        }
        // Dense tables: each row's part of the table index, oriented once per strip.
        if constexpr (policy_::direct_k) {
#pragma unroll
            for (int r = 0; r < R; ++r) row_bytes[r] = task.transposed ? row_bytes[r] : row_bytes[r] << 8;
        }
        __syncwarp();
        if constexpr (!policy_::uniform_k && !policy_::direct_k) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                int const row_class = costs.byte_to_class[row_bytes[r]];
                for (int cc = 0; cc < classes; ++cc) profile[cc * S + lane * R + r] = table[cc * 32 + row_class];
            }
        }
        std::int32_t h_col[R], e_col[R], best_row[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            h_col[r] = edge.score(row0 + r);
            e_col[r] = affine ? gap_seed(row0 + r) : 0;
            best_row[r] = 0;
        }
        std::int32_t diag_up = edge.score(row0 - 1);
        int const result_lane = int((n - 1 - strip_base) / R), result_row = int((n - 1 - strip_base) % R);

        bool const write_bottom = !last_strip;
        bool healthy = true;
        if constexpr (policy_::columns_k == 1) {
            std::uint32_t const steps = m + (std::uint32_t)last_lane;
            std::int32_t out_h = 0, out_f = 0;
            std::uint32_t code_now = lane == 0 ? column_code(1) : 0u;
            __syncwarp();
            std::uint32_t p_now[words];
            if constexpr (!policy_::uniform_k && !policy_::direct_k)
                load_profile_words<R>(profile + (int)code_now * S + lane * R, p_now);

            // One step of the sweep. `steady` steps are those where every lane is on a real column of a full strip
            // (31 <= t < m, all 32 lanes hold rows): no range predicates and no corner capture.
            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (band_chunk_k - 1);
                if (e == 0) {
                    // Stage lane 0's next columns; strips below the first wait for the strip above to write them.
                    std::uint32_t const need = min(m, t + band_chunk_k);
                    if (k > 0 && t + 1 <= m) healthy = band_wait(sync, slot_in, ((unsigned long long)k << 32) | need);
                    __syncwarp();
                    for (int c = lane; c < band_chunk_k; c += 32) {
                        std::uint32_t const j = t + 1 + c;
                        std::int32_t h = 0, f = 0;
                        if (j <= m) {
                            if (k == 0) h = edge.score(j), f = gap_seed(j);
                            else h = __ldcg(top + 2 * j), f = __ldcg(top + 2 * j + 1);
                        }
                        chunk.top_h[c] = h;
                        chunk.top_f[c] = f;
                        chunk.code[c] = j + 1 <= m ? column_code(j + 1) : 0u;
                    }
                    __syncwarp();
                    // The writer of the bottom row publishes its finished columns (it wrote column j at step j + 30).
                    if (write_bottom && lane == 31 && t > 31) {
                        std::uint32_t const done = min(m, t - 31);
                        band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | done);
                    }
                }
                std::int32_t up_h = __shfl_up_sync(0xFFFFFFFFu, out_h, 1);
                std::int32_t up_f = affine ? __shfl_up_sync(0xFFFFFFFFu, out_f, 1) : 0;
                std::uint32_t code_next = __shfl_up_sync(0xFFFFFFFFu, code_now, 1);
                if (lane == 0) up_h = chunk.top_h[e], up_f = chunk.top_f[e], code_next = chunk.code[e];
                [[maybe_unused]] std::uint32_t p_next[words]; // profile words (unused by uniform and direct instances)
                if constexpr (!policy_::uniform_k && !policy_::direct_k)
                    load_profile_words<R>(profile + (int)code_next * S + lane * R, p_next);

                std::int64_t const j = (std::int64_t)t + 1 - lane;
                if (steady || (j >= 1 && j <= (std::int64_t)m && lane <= last_lane)) {
                    std::int32_t diag = diag_up;
                    diag_up = up_h;
                    std::int32_t h_up = up_h, f_up = up_f;
                    std::int32_t subs[R];
                    if constexpr (policy_::uniform_k) {
#pragma unroll
                        for (int r = 0; r < R; ++r) subs[r] = row_bytes[r] == code_now ? costs.match : costs.mismatch;
                    }
                    else if constexpr (policy_::direct_k) {
                        // table[first byte][second byte]: rows are the first string unless the pair was transposed.
                        std::uint32_t const column_key = task.transposed ? code_now << 8 : code_now;
#pragma unroll
                        for (int r = 0; r < R; ++r) subs[r] = table_s[row_bytes[r] | column_key];
                    }
                    else {
#pragma unroll
                        for (int w = 0; w < words; ++w) {
                            // One byte permute per cost (the byte, its sign bit copied above it).
                            subs[4 * w + 0] = signed_byte<0>(p_now[w]), subs[4 * w + 1] = signed_byte<1>(p_now[w]);
                            subs[4 * w + 2] = signed_byte<2>(p_now[w]), subs[4 * w + 3] = signed_byte<3>(p_now[w]);
                        }
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::int32_t const substitution = diag + subs[r];
                        std::int32_t h;
                        if constexpr (affine && R == 4) {
                            // Groups of CTAs per pair (4 rows per lane) are bound by each warp's step latency: the row
                            // chain here is two fused add-max deep, at five of them per cell.
                            std::int32_t const e_new = ops::add_opt(e_col[r], extend, h_col[r]);
                            std::int32_t const x = ops::add_opt(e_new, open, substitution);
                            std::int32_t const via_f = ops::add_opt(f_up, extend_open, x);
                            if constexpr (local) h = ops::add_opt_relu(h_up, open, via_f);
                            else h = ops::add_opt(h_up, open, via_f);
                            f_up = ops::add_opt(f_up, extend, h_up);
                            e_col[r] = e_new;
                        }
                        else if constexpr (affine) {
                            // CTAs per pair (8 rows per lane) fill the GPU and are bound by the integer ALU pipe: three
                            // fused operations per cell, the adds of the gap opening and the substitution left to the
                            // multiply-add pipe. e_col and f_up hold E and F minus the opening cost.
                            std::int32_t const e_new = ops::add_opt(e_col[r], extend, h_col[r]);
                            std::int32_t const f_new = ops::add_opt(f_up, extend, h_up);
                            if constexpr (local) h = ops::opt3_relu(substitution, e_new + open, f_new + open);
                            else h = ops::opt3(substitution, e_new + open, f_new + open);
                            f_up = f_new;
                            e_col[r] = e_new;
                        }
                        else {
                            std::int32_t const x = ops::add_opt(h_col[r], open, substitution);
                            if constexpr (local) h = ops::add_opt_relu(h_up, open, x);
                            else h = ops::add_opt(h_up, open, x);
                        }
                        diag = h_col[r];
                        h_col[r] = h;
                        h_up = h;
                        if constexpr (local) best_row[r] = max(best_row[r], h);
                    }
                    out_h = h_up, out_f = f_up;
                    if (write_bottom && lane == 31) {
                        __stcg(bottom + 2 * j, out_h);
                        __stcg(bottom + 2 * j + 1, out_f);
                    }
                    if constexpr (!local && !steady)
                        if (last_strip && lane == result_lane && j == (std::int64_t)m) {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r == result_row) result = h_col[r];
                        }
                }
                code_now = code_next;
                if constexpr (!policy_::uniform_k && !policy_::direct_k) {
#pragma unroll
                    for (int w = 0; w < words; ++w) p_now[w] = p_next[w];
                }
            };

            std::uint32_t const fill_end = min(steps, 31u);
            std::uint32_t const steady_end = (last_lane == 31 && m >= 32u) ? max(fill_end, min(steps, m)) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end && healthy; ++t) step(t, std::false_type {});
            // Two steps per iteration: the row state alternates between two register sets instead of being copied
            // back.
#pragma unroll 2
            for (; t < steady_end && healthy; ++t) step(t, std::true_type {});
            for (; t < steps && healthy; ++t) step(t, std::false_type {});
        }
        else {
            // Two columns per step: at step t lane l scores columns 2(t - l) + 1 and 2(t - l) + 2 of its R rows, so a
            // shuffle, a profile lookup and the step's fixed work serve 2R cells, and the second column's cells run
            // beside the first column's next row (the chain is R + 1 cells deep instead of 2R). A sweep takes
            // ceil(m / 2) + 31 steps, and the strip below may start 48 steps behind (32 columns staged at a time).
            constexpr std::uint32_t steps_per_chunk = band_chunk_k / 2;
            std::uint32_t const column_pairs = (m + 1) / 2;
            std::uint32_t const steps = column_pairs + (std::uint32_t)last_lane;
            std::int32_t out_ha = 0, out_hb = 0, out_fa = 0, out_fb = 0;
            // The codes of the lane's two current columns: column a in bits 0-15, column b in bits 16-31.
            std::uint32_t codes_now = lane == 0 ? column_code(1) | (m >= 2 ? column_code(2) << 16 : 0u) : 0u;
            __syncwarp();
            std::uint32_t pa_now[words], pb_now[words];
            if constexpr (!policy_::uniform_k && !policy_::direct_k) {
                load_profile_words<R>(profile + (int)(codes_now & 0xFFFFu) * S + lane * R, pa_now);
                load_profile_words<R>(profile + (int)(codes_now >> 16) * S + lane * R, pb_now);
            }
            auto substitutions = [&](std::uint32_t code, std::uint32_t const (&p)[words], std::int32_t (&subs)[R]) {
                if constexpr (policy_::uniform_k) {
#pragma unroll
                    for (int r = 0; r < R; ++r) subs[r] = row_bytes[r] == code ? costs.match : costs.mismatch;
                }
                else if constexpr (policy_::direct_k) {
                    std::uint32_t const column_key = task.transposed ? code << 8 : code;
#pragma unroll
                    for (int r = 0; r < R; ++r) subs[r] = table_s[row_bytes[r] | column_key];
                }
                else {
#pragma unroll
                    for (int w = 0; w < words; ++w) {
                        subs[4 * w + 0] = signed_byte<0>(p[w]), subs[4 * w + 1] = signed_byte<1>(p[w]);
                        subs[4 * w + 2] = signed_byte<2>(p[w]), subs[4 * w + 3] = signed_byte<3>(p[w]);
                    }
                }
            };
            // One cell from its left (H, and E as E - open), its upper H and F - open (updated for the cell below)
            // and its substitution score; the forms are those of the one-column sweep.
            auto cell = [&](std::int32_t left_h, std::int32_t &e, std::int32_t up_h, std::int32_t &f_up,
                            std::int32_t substitution) -> std::int32_t {
                std::int32_t h;
                if constexpr (affine && R == 4) {
                    std::int32_t const e_new = ops::add_opt(e, extend, left_h);
                    std::int32_t const x = ops::add_opt(e_new, open, substitution);
                    std::int32_t const via_f = ops::add_opt(f_up, extend_open, x);
                    if constexpr (local) h = ops::add_opt_relu(up_h, open, via_f);
                    else h = ops::add_opt(up_h, open, via_f);
                    f_up = ops::add_opt(f_up, extend, up_h);
                    e = e_new;
                }
                else if constexpr (affine) {
                    std::int32_t const e_new = ops::add_opt(e, extend, left_h);
                    std::int32_t const f_new = ops::add_opt(f_up, extend, up_h);
                    if constexpr (local) h = ops::opt3_relu(substitution, e_new + open, f_new + open);
                    else h = ops::opt3(substitution, e_new + open, f_new + open);
                    f_up = f_new;
                    e = e_new;
                }
                else {
                    std::int32_t const x = ops::add_opt(left_h, open, substitution);
                    if constexpr (local) h = ops::add_opt_relu(up_h, open, x);
                    else h = ops::add_opt(up_h, open, x);
                }
                return h;
            };

            auto step = [&](std::uint32_t t, auto steady_tag) {
                constexpr bool steady = decltype(steady_tag)::value;
                std::uint32_t const e = t & (steps_per_chunk - 1);
                if (e == 0) {
                    // Stage lane 0's next 32 columns; strips below the first wait for the strip above to write them.
                    std::uint32_t const first_column = 2 * t + 1;
                    std::uint32_t const need = min(m, 2 * t + band_chunk_k);
                    if (k > 0 && first_column <= m)
                        healthy = band_wait(sync, slot_in, ((unsigned long long)k << 32) | need);
                    __syncwarp();
                    for (int c = lane; c < band_chunk_k; c += 32) {
                        std::uint32_t const j = first_column + c;
                        std::int32_t h = 0, f = 0;
                        if (j <= m) {
                            if (k == 0) h = edge.score(j), f = gap_seed(j);
                            else {
                                int2 const cell_hf = __ldcg(reinterpret_cast<int2 const *>(top) + j);
                                h = cell_hf.x, f = cell_hf.y;
                            }
                        }
                        chunk.top_h[c] = h;
                        chunk.top_f[c] = f;
                        chunk.code[c] = j + 2 <= m ? column_code(j + 2) : 0u; // lane 0's codes one step ahead
                    }
                    __syncwarp();
                    // The writer of the bottom row publishes its finished columns (before step t: up to 2(t - 31)).
                    if (write_bottom && lane == 31 && t > 31) {
                        std::uint32_t const done = min(m, 2 * (t - 31));
                        band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | done);
                    }
                }
                std::int32_t up_ha = __shfl_up_sync(0xFFFFFFFFu, out_ha, 1);
                std::int32_t up_hb = __shfl_up_sync(0xFFFFFFFFu, out_hb, 1);
                std::int32_t up_fa = affine ? __shfl_up_sync(0xFFFFFFFFu, out_fa, 1) : 0;
                std::int32_t up_fb = affine ? __shfl_up_sync(0xFFFFFFFFu, out_fb, 1) : 0;
                std::uint32_t codes_next = __shfl_up_sync(0xFFFFFFFFu, codes_now, 1);
                if (lane == 0) {
                    up_ha = chunk.top_h[2 * e], up_hb = chunk.top_h[2 * e + 1];
                    up_fa = chunk.top_f[2 * e], up_fb = chunk.top_f[2 * e + 1];
                    codes_next = chunk.code[2 * e] | chunk.code[2 * e + 1] << 16;
                }
                [[maybe_unused]] std::uint32_t pa_next[words], pb_next[words];
                if constexpr (!policy_::uniform_k && !policy_::direct_k) {
                    load_profile_words<R>(profile + (int)(codes_next & 0xFFFFu) * S + lane * R, pa_next);
                    load_profile_words<R>(profile + (int)(codes_next >> 16) * S + lane * R, pb_next);
                }

                std::int64_t const ja = 2 * ((std::int64_t)t - lane) + 1;
                if (steady || (ja >= 1 && ja <= (std::int64_t)m && lane <= last_lane)) {
                    bool const valid_b = steady || ja + 1 <= (std::int64_t)m;
                    std::int32_t diag_a = diag_up, diag_b = up_ha;
                    diag_up = up_hb;
                    std::int32_t h_up_a = up_ha, h_up_b = up_hb, f_up_a = up_fa, f_up_b = up_fb;
                    std::int32_t subs_a[R], subs_b[R];
                    substitutions(codes_now & 0xFFFFu, pa_now, subs_a);
                    substitutions(codes_now >> 16, pb_now, subs_b);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        std::int32_t e_left = e_col[r];
                        std::int32_t const h_a = cell(h_col[r], e_left, h_up_a, f_up_a, diag_a + subs_a[r]);
                        std::int32_t const h_b = cell(h_a, e_left, h_up_b, f_up_b, diag_b + subs_b[r]);
                        diag_a = h_col[r];
                        diag_b = h_a;
                        h_col[r] = h_b;
                        e_col[r] = e_left;
                        h_up_a = h_a;
                        h_up_b = h_b;
                        if constexpr (local) {
                            best_row[r] = max(best_row[r], h_a);
                            if (valid_b) best_row[r] = max(best_row[r], h_b);
                        }
                        if constexpr (!local && !steady)
                            if (last_strip && lane == result_lane && r == result_row) {
                                if (ja == (std::int64_t)m) result = h_a;
                                if (ja + 1 == (std::int64_t)m) result = h_b;
                            }
                    }
                    out_ha = h_up_a, out_hb = h_up_b, out_fa = f_up_a, out_fb = f_up_b;
                    if (write_bottom && lane == 31) {
                        __stcg(reinterpret_cast<int2 *>(bottom) + ja, make_int2(out_ha, out_fa));
                        if (valid_b) __stcg(reinterpret_cast<int2 *>(bottom) + ja + 1, make_int2(out_hb, out_fb));
                    }
                }
                codes_now = codes_next;
                if constexpr (!policy_::uniform_k && !policy_::direct_k) {
#pragma unroll
                    for (int w = 0; w < words; ++w) pa_now[w] = pa_next[w], pb_now[w] = pb_next[w];
                }
            };

            // Steady steps: lane 31 on column pair >= 0 (t >= 31) and lane 0's second column within the pair
            // (2t + 2 <= m), all 32 lanes holding rows.
            std::uint32_t const fill_end = min(steps, 31u);
            std::uint32_t const steady_end =
                (last_lane == 31 && m / 2 > 31u) ? max(fill_end, min(steps, m / 2)) : fill_end;
            std::uint32_t t = 0;
            for (; t < fill_end && healthy; ++t) step(t, std::false_type {});
#pragma unroll 2
            for (; t < steady_end && healthy; ++t) step(t, std::true_type {});
            for (; t < steps && healthy; ++t) step(t, std::false_type {});
        }
        __syncwarp();
        if (write_bottom && lane == 31) band_publish(sync, slot_out, ((unsigned long long)(k + 1) << 32) | m);
        if constexpr (local) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (row0 + r <= (std::int64_t)n) lane_best = max(lane_best, best_row[r]);
        }
        if (!healthy) break;
    }
    if constexpr (local) {
#pragma unroll
        for (int offset = 16; offset > 0; offset >>= 1)
            lane_best = max(lane_best, __shfl_xor_sync(0xFFFFFFFFu, lane_best, offset));
        return lane_best;
    }
    else {
        // Only the lane holding row n of the last strip captured the corner; it is the warp's only non-zero value
        // for global scores when this warp owns the last strip.
        std::uint32_t const last_strip_index = strips - 1;
        int const owner_lane = int((n - 1 - last_strip_index * S) / R);
        return __shfl_sync(0xFFFFFFFFu, result, owner_lane);
    }
}

/** Persistent band kernel: one pair per CTA at a time, pulled from a cursor over bins [key_begin, key_end). */
template <typename policy_>
__global__ void __launch_bounds__(band_warps_k * 32)
    band_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key_begin, int key_end,
                score_costs_t const costs, std::int64_t *__restrict__ results, std::int32_t *__restrict__ scratch,
                std::size_t ring_cells_per_slot) {
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::size_t const costs_bytes = (sizeof(score_costs_t) + 15) / 16 * 16;
    band_shared_t &shared = *reinterpret_cast<band_shared_t *>(shared_bytes + costs_bytes);
    std::size_t const shared_state_bytes = (sizeof(band_shared_t) + 15) / 16 * 16;
    std::size_t const profile_bytes = (std::size_t)band_profile_bytes_per_warp<policy_>(costs.classes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + costs_bytes + shared_state_bytes);
    auto *chunks = reinterpret_cast<band_chunk_t *>(profiles + band_warps_k * profile_bytes);
    std::int8_t *table_s = reinterpret_cast<std::int8_t *>(chunks + band_warps_k);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    if constexpr (policy_::direct_k) stage_direct_table(costs.direct_table, table_s);
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    std::int32_t *ring = scratch + (std::size_t)blockIdx.x * band_warps_k * ring_cells_per_slot;
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
        std::int32_t const value = band_score_warp<policy_>(task, costs_s, band_cta_ring(shared, warp, costs_s.wait_polls), ring,
                                                            ring_cells_per_slot, profiles + warp * profile_bytes,
                                                            chunks[warp], table_s);
        if (lane == 0) shared.warp_result[warp] = value;
        __syncthreads();
        if (threadIdx.x == 0) {
            std::int64_t score;
            if (policy_::local_k) {
                std::int32_t best = 0;
                for (int w = 0; w < band_warps_k; ++w) best = max(best, shared.warp_result[w]);
                score = best;
            }
            else {
                std::uint32_t const strips = (task.rows_length + policy_::strip_rows_k - 1) / policy_::strip_rows_k;
                score = shared.warp_result[(strips - 1) % band_warps_k];
            }
            if (shared.failed) atomicOr(&bins->error_flags, 1u);
            results[task.slot] = score;
        }
    }
}

/** Clears the next pair's words of a group (both passes): called by the group's first CTA after the barrier that
 *  starts a pair, when every CTA has finished with the pair before it. */
__device__ __forceinline__ void band_group_reset(band_group_state_t *state, int parity, int members) {
    for (int i = threadIdx.x; i < members; i += blockDim.x) {
        state->pass[parity][0].progress[i] = 0ull;
        state->pass[parity][1].progress[i] = 0ull;
    }
    if (threadIdx.x == 0) state->pass[parity][0].best = 0, state->pass[parity][1].best = 0;
    __threadfence();
}

/** A warp's share of a pass: local scores take the group's maximum, global scores the corner from its owner warp. */
template <bool local_>
__device__ __forceinline__ void band_group_contribute(band_pass_state_t &pass, std::int32_t value, bool owner) {
    if ((threadIdx.x & 31) != 0) return;
    if constexpr (local_) atomicMax(&pass.best, value);
    else if (owner) {
        *reinterpret_cast<volatile std::int32_t *>(&pass.best) = value;
        __threadfence();
    }
}

/**
 *  Grouped band kernel: G co-resident CTAs (one cooperative launch, `group_ctas` = G) share each pair, their G x W
 *  warps forming one ring; group g scores pairs g, g + groups, ... of bins [key_begin, key_end).
 */
template <typename policy_>
__global__ void __launch_bounds__(band_warps_k * 32)
    band_group_kernel(pair_task_t const *__restrict__ tasks, plan_bins_t *__restrict__ bins, int key_begin,
                      int key_end, score_costs_t const costs, std::int64_t *__restrict__ results,
                      std::int32_t *__restrict__ scratch, std::size_t ring_cells_per_slot,
                      band_group_state_t *__restrict__ group_states, int group_ctas) {
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::size_t const costs_bytes = (sizeof(score_costs_t) + 15) / 16 * 16;
    band_shared_t &shared = *reinterpret_cast<band_shared_t *>(shared_bytes + costs_bytes);
    std::size_t const shared_state_bytes = (sizeof(band_shared_t) + 15) / 16 * 16;
    std::size_t const profile_bytes = (std::size_t)band_profile_bytes_per_warp<policy_>(costs.classes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + costs_bytes + shared_state_bytes);
    auto *chunks = reinterpret_cast<band_chunk_t *>(profiles + band_warps_k * profile_bytes);
    std::int8_t *table_s = reinterpret_cast<std::int8_t *>(chunks + band_warps_k);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    if constexpr (policy_::direct_k) stage_direct_table(costs.direct_table, table_s);
    int const warp = threadIdx.x >> 5;
    int const group = (int)blockIdx.x / group_ctas, rank = (int)blockIdx.x % group_ctas;
    int const groups = (int)gridDim.x / group_ctas;
    int const members = group_ctas * band_warps_k;
    band_group_state_t *state = group_states + group;
    std::int32_t *ring = scratch + (std::size_t)group * members * ring_cells_per_slot;
    std::uint32_t const begin = bins->begin[key_begin];
    std::uint32_t const count = bins->begin[key_end - 1] + bins->count[key_end - 1] - begin;
    std::uint32_t barriers = 0, iteration = 0;
    for (std::uint32_t index = (std::uint32_t)group; index < count; index += (std::uint32_t)groups, ++iteration) {
        int const parity = int(iteration & 1u);
        if (!band_group_barrier(state, group_ctas, ++barriers, shared.gate, costs_s.barrier_polls)) break;
        if (rank == 0) band_group_reset(state, parity ^ 1, members);
        pair_task_t const task = tasks[begin + index];
        band_pass_state_t &pass = state->pass[parity][0];
        band_ring_t const sync {pass.progress, &state->failed, members, rank * band_warps_k + warp, true,
                                costs_s.wait_polls};
        std::int32_t const value = band_score_warp<policy_>(task, costs_s, sync, ring, ring_cells_per_slot,
                                                            profiles + warp * profile_bytes, chunks[warp], table_s);
        std::uint32_t const strips = (task.rows_length + policy_::strip_rows_k - 1) / policy_::strip_rows_k;
        band_group_contribute<policy_::local_k>(pass, value, (int)((strips - 1) % (std::uint32_t)members) == sync.member);
        if (!band_group_barrier(state, group_ctas, ++barriers, shared.gate, costs_s.barrier_polls)) break;
        if (rank == 0 && threadIdx.x == 0)
            results[task.slot] = *reinterpret_cast<volatile std::int32_t *>(&pass.best);
    }
    __syncthreads();
    if (rank == 0 && threadIdx.x == 0 && *reinterpret_cast<volatile std::uint32_t *>(&state->failed))
        atomicOr(&bins->error_flags, 1u);
}

} // namespace szs_gb300
