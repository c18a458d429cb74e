/**
 *  @file kernels_band16.cu
 *  @brief Instantiations and launcher of the 16-bit band kernel (dp_band16.cuh). Compiled twice, with
 *         `SZS_BAND16_ROWS` 8 (512-row super-strips) or 4 (256-row super-strips, for groups of CTAs per pair).
 */
#include "dp_band16.cuh"
#include "launchers.h"

namespace szs_gb300 {

namespace {

#ifndef SZS_BAND16_ROWS
#error "compile with -DSZS_BAND16_ROWS=<8|4>"
#endif
constexpr int band16_rows_per_lane_k = SZS_BAND16_ROWS;
#ifndef SZS_BAND16_COLUMNS
#define SZS_BAND16_COLUMNS 2
#endif
constexpr int band16_columns_k = SZS_BAND16_COLUMNS; // columns each half of a lane scores per step

template <int kind_, bool affine_, int compare_ = compare_none_k, bool wide_ = false>
using band16_instance_t =
    band16_policy_t<kind_, affine_, band16_rows_per_lane_k, compare_, wide_, band16_columns_k>;

template <int kind_, bool affine_, int compare_ = compare_none_k, bool wide_ = false>
dp_launch_shape_t band16_shape_of(int classes) {
    using policy_t = band16_instance_t<kind_, affine_, compare_, wide_>;
    dp_launch_shape_t shape;
    shape.threads_per_cta = band_warps_k * 32;
    shape.warps_per_cta = band_warps_k;
    shape.rows_per_lane = band16_rows_per_lane_k;
    shape.shared_bytes = band16_shared_bytes<policy_t>(classes);
    auto kernel = band16_kernel<policy_t>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.ctas_per_sm = blocks;
    auto grouped = band16_group_kernel<policy_t>;
    cudaFuncSetAttribute(grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, grouped, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.group_ctas_per_sm = blocks;
    return shape;
}

template <int kind_, bool affine_, int compare_ = compare_none_k, bool wide_ = false>
cudaError_t band16_launch_of(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                             score_costs_t const &costs, std::int64_t *results, void *scratch,
                             std::size_t ring_words_per_slot, int ctas, cudaStream_t stream, void *group_states,
                             int group_ctas) {
    using policy_t = band16_instance_t<kind_, affine_, compare_, wide_>;
    int const shared = band16_shared_bytes<policy_t>(costs.classes);
    if (group_states) {
        // The CTAs of a group wait on one another: a cooperative launch keeps the whole grid resident.
        auto grouped = band16_group_kernel<policy_t>;
        cudaError_t status = cudaFuncSetAttribute(grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
        if (status != cudaSuccess) return status;
        cudaLaunchConfig_t config {};
        config.gridDim = dim3((unsigned)ctas), config.blockDim = dim3(band_warps_k * 32);
        config.dynamicSmemBytes = (std::size_t)shared, config.stream = stream;
        cudaLaunchAttribute attribute {};
        attribute.id = cudaLaunchAttributeCooperative, attribute.val.cooperative = 1;
        config.attrs = &attribute, config.numAttrs = 1;
        return cudaLaunchKernelEx(&config, grouped, tasks, bins, key_begin, key_end, costs, results,
                                  static_cast<std::uint32_t *>(scratch), ring_words_per_slot,
                                  static_cast<band_group_state_t *>(group_states), group_ctas);
    }
    auto kernel = band16_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, band_warps_k * 32, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results,
                                                         static_cast<std::uint32_t *>(scratch), ring_words_per_slot);
    return cudaGetLastError();
}

} // namespace

#define SZS_CONCAT_(a, b) a##b
#define SZS_CONCAT(a, b) SZS_CONCAT_(a, b)

#define SZS_BAND16_DISPATCH(call_, ...)                                                                              \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 0: return call_<kind_levenshtein_k, false>(__VA_ARGS__);                                                    \
    case 1: return call_<kind_levenshtein_k, true>(__VA_ARGS__);                                                     \
    case 2: return call_<kind_needleman_wunsch_k, false>(__VA_ARGS__);                                               \
    case 3: return call_<kind_needleman_wunsch_k, true>(__VA_ARGS__);                                                \
    case 4: return call_<kind_smith_waterman_k, false>(__VA_ARGS__);                                                 \
    case 5: return call_<kind_smith_waterman_k, true>(__VA_ARGS__);                                                  \
    default: break;                                                                                                  \
    }

// Compare-mode instances: affine or not, multiply-add or select form, bytes or 16-bit codes.
#define SZS_BAND16_COMPARE_DISPATCH(call_, ...)                                                                      \
    switch ((affine ? 4 : 0) + (compare == compare_multiply_k ? 2 : 0) + (wide ? 1 : 0)) {                           \
    case 0: return call_<kind_levenshtein_k, false, compare_select_k, false>(__VA_ARGS__);                           \
    case 1: return call_<kind_levenshtein_k, false, compare_select_k, true>(__VA_ARGS__);                            \
    case 2: return call_<kind_levenshtein_k, false, compare_multiply_k, false>(__VA_ARGS__);                         \
    case 3: return call_<kind_levenshtein_k, false, compare_multiply_k, true>(__VA_ARGS__);                          \
    case 4: return call_<kind_levenshtein_k, true, compare_select_k, false>(__VA_ARGS__);                            \
    case 5: return call_<kind_levenshtein_k, true, compare_select_k, true>(__VA_ARGS__);                             \
    case 6: return call_<kind_levenshtein_k, true, compare_multiply_k, false>(__VA_ARGS__);                          \
    default: return call_<kind_levenshtein_k, true, compare_multiply_k, true>(__VA_ARGS__);                          \
    }

dp_launch_shape_t SZS_CONCAT(band16_shape_rows, SZS_BAND16_ROWS)(int kind, bool affine, int classes, int compare,
                                                                 bool wide) {
    if (compare != compare_none_k || wide) {
        if (kind != kind_levenshtein_k || compare == compare_none_k) return dp_launch_shape_t {0, 0, 0, 0, 0};
        SZS_BAND16_COMPARE_DISPATCH(band16_shape_of, classes)
    }
    SZS_BAND16_DISPATCH(band16_shape_of, classes)
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t SZS_CONCAT(launch_band16_rows, SZS_BAND16_ROWS)(int kind, bool affine, int key_begin, int key_end,
                                                          pair_task_t const *tasks, plan_bins_t *bins,
                                                          score_costs_t const &costs, std::int64_t *results,
                                                          void *scratch, std::size_t ring_words_per_slot, int ctas,
                                                          cudaStream_t stream, void *group_states, int group_ctas,
                                                          int compare, bool wide) {
    if (compare != compare_none_k || wide) {
        if (kind != kind_levenshtein_k || compare == compare_none_k) return cudaErrorInvalidValue;
        SZS_BAND16_COMPARE_DISPATCH(band16_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                                    ring_words_per_slot, ctas, stream, group_states, group_ctas)
    }
    SZS_BAND16_DISPATCH(band16_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                        ring_words_per_slot, ctas, stream, group_states, group_ctas)
    return cudaErrorInvalidValue;
}

#if SZS_BAND16_ROWS == 8

dp_launch_shape_t band16_shape_rows4(int kind, bool affine, int classes, int compare, bool wide);
cudaError_t launch_band16_rows4(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks,
                                plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                                std::size_t ring_words_per_slot, int ctas, cudaStream_t stream, void *group_states,
                                int group_ctas, int compare, bool wide);

dp_launch_shape_t band16_shape(int kind, bool affine, int classes, int compare, bool wide, int rows_per_lane) {
    return rows_per_lane == 4 ? band16_shape_rows4(kind, affine, classes, compare, wide)
                              : band16_shape_rows8(kind, affine, classes, compare, wide);
}

cudaError_t launch_band16(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks,
                          plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                          std::size_t ring_words_per_slot, int ctas, cudaStream_t stream, void *group_states,
                          int group_ctas, int compare, bool wide, int rows_per_lane) {
    if (rows_per_lane == 4)
        return launch_band16_rows4(kind, affine, key_begin, key_end, tasks, bins, costs, results, scratch,
                                   ring_words_per_slot, ctas, stream, group_states, group_ctas, compare, wide);
    return launch_band16_rows8(kind, affine, key_begin, key_end, tasks, bins, costs, results, scratch,
                               ring_words_per_slot, ctas, stream, group_states, group_ctas, compare, wide);
}

#endif

} // namespace szs_gb300
