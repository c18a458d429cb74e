/**
 *  @file kernels_short.cu
 *  @brief Instantiations and launcher of the segmented 16x2 kernel for short pairs (dp_short.cuh) for every cost
 *         family, profile and compare modes. Segment shapes 0-3 for shorter sides up to 16, 32, 64 and 128:
 *         either 2, 4, 8, 16 lanes x 8 rows (profiles over many classes: a warp's profiles stay at 32 x 8 rows per
 *         pair) or 1, 2, 4, 8 lanes x 16 rows (few classes or compare mode: fewer lanes and steps per pair); shapes
 *         4-6 for shorter sides up to 24, 48 and 96: 2, 4, 8 lanes x 12 rows, so that a pair pads its rows to at
 *         most 1.5x instead of 2x and the middle of each octave runs fewer fill steps.
 *
 *  Compiled three times, with `SZS_SHORT_ROWS` 8, 12 or 16, so the families build in parallel.
 */
#include "dp_short.cuh"
#include "launchers.h"

#ifndef SZS_SHORT_ROWS
#error "compile with -DSZS_SHORT_ROWS=<8|12|16>"
#endif

namespace szs_gb300 {

namespace {

template <int kind_, bool affine_, int lanes_, int rows_, int compare_>
dp_launch_shape_t short_shape_of(int classes, int warps) {
    using policy_t = short_policy_t<kind_, affine_, lanes_, rows_, compare_>;
    dp_launch_shape_t shape;
    shape.threads_per_cta = warps * 32;
    shape.warps_per_cta = warps;
    shape.rows_per_lane = rows_;
    shape.shared_bytes = short_shared_bytes<policy_t>(warps, classes);
    auto kernel = dp16_short_kernel<policy_t>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.ctas_per_sm = blocks;
    return shape;
}

template <int kind_, bool affine_, int lanes_, int rows_, int compare_>
cudaError_t short_launch_of(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                            score_costs_t const &costs, std::int64_t *results, int ctas, int warps,
                            cudaStream_t stream) {
    using policy_t = short_policy_t<kind_, affine_, lanes_, rows_, compare_>;
    int const shared = short_shared_bytes<policy_t>(warps, costs.classes);
    auto kernel = dp16_short_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, warps * 32, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results);
    return cudaGetLastError();
}

#if SZS_SHORT_ROWS == 12
// Segment shapes of this family: 4, 5, 6 for shorter sides up to 24, 48, 96 (2, 4, 8 lanes x 12 rows).
#define SZS_SHORT_SHAPES(call_, kind_, affine_, compare_, ...)                                                       \
    switch (shape) {                                                                                                 \
    case 4: return call_<kind_, affine_, 2, 12, compare_>(__VA_ARGS__);                                              \
    case 5: return call_<kind_, affine_, 4, 12, compare_>(__VA_ARGS__);                                              \
    case 6: return call_<kind_, affine_, 8, 12, compare_>(__VA_ARGS__);                                              \
    default: break;                                                                                                  \
    }
#else
// Segment shapes of this family: 0, 1, 2, 3 for shorter sides up to 16, 32, 64, 128 (lanes x rows).
#define SZS_SHORT_SHAPES(call_, kind_, affine_, compare_, ...)                                                       \
    switch (shape) {                                                                                                 \
    case 0: return call_<kind_, affine_, 16 / SZS_SHORT_ROWS, SZS_SHORT_ROWS, compare_>(__VA_ARGS__);                \
    case 1: return call_<kind_, affine_, 32 / SZS_SHORT_ROWS, SZS_SHORT_ROWS, compare_>(__VA_ARGS__);                \
    case 2: return call_<kind_, affine_, 64 / SZS_SHORT_ROWS, SZS_SHORT_ROWS, compare_>(__VA_ARGS__);                \
    case 3: return call_<kind_, affine_, 128 / SZS_SHORT_ROWS, SZS_SHORT_ROWS, compare_>(__VA_ARGS__);               \
    default: break;                                                                                                  \
    }
#endif

#define SZS_SHORT_DISPATCH(call_, ...)                                                                               \
    if (compare != compare_none_k) {                                                                                 \
        if (kind != kind_levenshtein_k) break;                                                                       \
        switch ((affine ? 2 : 0) + (compare == compare_multiply_k ? 1 : 0)) {                                        \
        case 0: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, false, compare_select_k, __VA_ARGS__) break;             \
        case 1: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, false, compare_multiply_k, __VA_ARGS__) break;           \
        case 2: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, true, compare_select_k, __VA_ARGS__) break;              \
        default: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, true, compare_multiply_k, __VA_ARGS__) break;           \
        }                                                                                                            \
        break;                                                                                                       \
    }                                                                                                                \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 0: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, false, compare_none_k, __VA_ARGS__) break;                   \
    case 1: SZS_SHORT_SHAPES(call_, kind_levenshtein_k, true, compare_none_k, __VA_ARGS__) break;                    \
    case 2: SZS_SHORT_SHAPES(call_, kind_needleman_wunsch_k, false, compare_none_k, __VA_ARGS__) break;              \
    case 3: SZS_SHORT_SHAPES(call_, kind_needleman_wunsch_k, true, compare_none_k, __VA_ARGS__) break;               \
    case 4: SZS_SHORT_SHAPES(call_, kind_smith_waterman_k, false, compare_none_k, __VA_ARGS__) break;                \
    case 5: SZS_SHORT_SHAPES(call_, kind_smith_waterman_k, true, compare_none_k, __VA_ARGS__) break;                 \
    default: break;                                                                                                  \
    }

} // namespace

#define SZS_CONCAT_(a, b) a##b
#define SZS_CONCAT(a, b) SZS_CONCAT_(a, b)

dp_launch_shape_t SZS_CONCAT(short_shape_rows, SZS_SHORT_ROWS)(int kind, bool affine, int shape, int classes,
                                                               int warps, int compare) {
    if (warps >= 1 && warps <= 8) do {
            SZS_SHORT_DISPATCH(short_shape_of, classes, warps)
        } while (false);
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t SZS_CONCAT(launch_short_rows, SZS_SHORT_ROWS)(int kind, bool affine, int shape, int key_begin,
                                                           int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                                                           score_costs_t const &costs, std::int64_t *results,
                                                           int ctas, int warps, cudaStream_t stream, int compare) {
    if (warps >= 1 && warps <= 8) do {
            SZS_SHORT_DISPATCH(short_launch_of, key_begin, key_end, tasks, bins, costs, results, ctas, warps, stream)
        } while (false);
    return cudaErrorInvalidValue;
}

#if SZS_SHORT_ROWS == 16

dp_launch_shape_t short_shape_rows8(int kind, bool affine, int shape, int classes, int warps, int compare);
cudaError_t launch_short_rows8(int kind, bool affine, int shape, int key_begin, int key_end, pair_task_t const *tasks,
                               plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, int ctas,
                               int warps, cudaStream_t stream, int compare);
dp_launch_shape_t short_shape_rows12(int kind, bool affine, int shape, int classes, int warps, int compare);
cudaError_t launch_short_rows12(int kind, bool affine, int shape, int key_begin, int key_end, pair_task_t const *tasks,
                                plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, int ctas,
                                int warps, cudaStream_t stream, int compare);

int short_rows_for(int classes, int compare, int shape) {
    if (shape >= 4) return 12;
    return compare != compare_none_k || classes <= 8 ? 16 : 8;
}

int short_segment_rows(int shape) {
    constexpr int rows[short_shapes_k] = {16, 32, 64, 128, 24, 48, 96};
    return shape >= 0 && shape < short_shapes_k ? rows[shape] : 0;
}

dp_launch_shape_t short_shape(int kind, bool affine, int shape, int classes, int warps, int compare) {
    switch (short_rows_for(classes, compare, shape)) {
    case 12: return short_shape_rows12(kind, affine, shape, classes, warps, compare);
    case 16: return short_shape_rows16(kind, affine, shape, classes, warps, compare);
    default: return short_shape_rows8(kind, affine, shape, classes, warps, compare);
    }
}

cudaError_t launch_short(int kind, bool affine, int shape, int key_begin, int key_end, pair_task_t const *tasks,
                         plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, int ctas, int warps,
                         cudaStream_t stream, int compare) {
    switch (short_rows_for(costs.classes, compare, shape)) {
    case 12:
        return launch_short_rows12(kind, affine, shape, key_begin, key_end, tasks, bins, costs, results, ctas, warps,
                                   stream, compare);
    case 16:
        return launch_short_rows16(kind, affine, shape, key_begin, key_end, tasks, bins, costs, results, ctas, warps,
                                   stream, compare);
    default:
        return launch_short_rows8(kind, affine, shape, key_begin, key_end, tasks, bins, costs, results, ctas, warps,
                                  stream, compare);
    }
}

#endif

} // namespace szs_gb300
