/**
 *  @file kernels_band.cu
 *  @brief Instantiations and launcher of the band kernel (dp_band.cuh). Compiled twice, with `SZS_BAND_ROWS` 8 (one
 *         CTA per pair, and groups for a few long pairs) or 4 (groups of CTAs per pair: strips of 128 rows, so a
 *         single long pair spreads over twice the warps, each step half as long).
 */
#include "dp_band.cuh"
#include "launchers.h"

namespace szs_gb300 {

namespace {

#ifndef SZS_BAND_ROWS
#error "compile with -DSZS_BAND_ROWS=<8|4>"
#endif
constexpr int band_rows_per_lane_k = SZS_BAND_ROWS;

// Groups of CTAs per pair (the 4-row build) are bound by each warp's step latency: they take two columns per step.
template <int kind_, bool affine_>
using band_instance_t = band_policy_t<kind_, affine_, band_rows_per_lane_k, band_rows_per_lane_k == 4 ? 2 : 1>;

/** The instance for (direct table, 16-bit codes): at most one of the two. */
template <int kind_, bool affine_, bool direct_, bool wide_>
struct band_variant {
    using base_t = band_instance_t<kind_, affine_>;
    using type = std::conditional_t<direct_, direct_policy_t<base_t>,
                                    std::conditional_t<wide_, wide_policy_t<base_t>, base_t>>;
};

template <int kind_, bool affine_, bool direct_ = false, bool wide_ = false>
dp_launch_shape_t band_shape_of(int classes) {
    using policy_t = typename band_variant<kind_, affine_, direct_, wide_>::type;
    dp_launch_shape_t shape;
    shape.threads_per_cta = band_warps_k * 32;
    shape.warps_per_cta = band_warps_k;
    shape.rows_per_lane = band_rows_per_lane_k;
    shape.shared_bytes = band_shared_bytes<policy_t>(classes);
    auto kernel = band_kernel<policy_t>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.ctas_per_sm = blocks;
    auto grouped = band_group_kernel<policy_t>;
    cudaFuncSetAttribute(grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, grouped, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.group_ctas_per_sm = blocks;
    return shape;
}

template <int kind_, bool affine_, bool direct_ = false, bool wide_ = false>
cudaError_t band_launch_of(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                           score_costs_t const &costs, std::int64_t *results, void *scratch,
                           std::size_t ring_cells_per_slot, int ctas, cudaStream_t stream, void *group_states,
                           int group_ctas) {
    using policy_t = typename band_variant<kind_, affine_, direct_, wide_>::type;
    int const shared = band_shared_bytes<policy_t>(costs.classes);
    if (group_states) {
        // The CTAs of a group wait on one another: a cooperative launch keeps the whole grid resident.
        auto grouped = band_group_kernel<policy_t>;
        cudaError_t status = cudaFuncSetAttribute(grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
        if (status != cudaSuccess) return status;
        cudaLaunchConfig_t config {};
        config.gridDim = dim3((unsigned)ctas), config.blockDim = dim3(band_warps_k * 32);
        config.dynamicSmemBytes = (std::size_t)shared, config.stream = stream;
        cudaLaunchAttribute attribute {};
        attribute.id = cudaLaunchAttributeCooperative, attribute.val.cooperative = 1;
        config.attrs = &attribute, config.numAttrs = 1;
        return cudaLaunchKernelEx(&config, grouped, tasks, bins, key_begin, key_end, costs, results,
                                  static_cast<std::int32_t *>(scratch), ring_cells_per_slot,
                                  static_cast<band_group_state_t *>(group_states), group_ctas);
    }
    auto kernel = band_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, band_warps_k * 32, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results,
                                                         static_cast<std::int32_t *>(scratch), ring_cells_per_slot);
    return cudaGetLastError();
}

} // namespace

#define SZS_CONCAT_(a, b) a##b
#define SZS_CONCAT(a, b) SZS_CONCAT_(a, b)

#define SZS_BAND_DISPATCH(call_, ...)                                                                                \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 0: return call_<kind_levenshtein_k, false>(__VA_ARGS__);                                                    \
    case 1: return call_<kind_levenshtein_k, true>(__VA_ARGS__);                                                     \
    case 2: return call_<kind_needleman_wunsch_k, false>(__VA_ARGS__);                                               \
    case 3: return call_<kind_needleman_wunsch_k, true>(__VA_ARGS__);                                                \
    case 4: return call_<kind_smith_waterman_k, false>(__VA_ARGS__);                                                 \
    case 5: return call_<kind_smith_waterman_k, true>(__VA_ARGS__);                                                  \
    default: break;                                                                                                  \
    }

/** Direct-table instances (dense tables over more than 32 bytes) exist for the alignment kinds only. */
#define SZS_BAND_DIRECT_DISPATCH(call_, ...)                                                                         \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 2: return call_<kind_needleman_wunsch_k, false, true>(__VA_ARGS__);                                         \
    case 3: return call_<kind_needleman_wunsch_k, true, true>(__VA_ARGS__);                                          \
    case 4: return call_<kind_smith_waterman_k, false, true>(__VA_ARGS__);                                           \
    case 5: return call_<kind_smith_waterman_k, true, true>(__VA_ARGS__);                                            \
    default: break;                                                                                                  \
    }

/** 16-bit-code instances exist for Levenshtein only (UTF-8 calls). */
#define SZS_BAND_WIDE_DISPATCH(call_, ...)                                                                           \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 0: return call_<kind_levenshtein_k, false, false, true>(__VA_ARGS__);                                       \
    case 1: return call_<kind_levenshtein_k, true, false, true>(__VA_ARGS__);                                        \
    default: break;                                                                                                  \
    }

dp_launch_shape_t SZS_CONCAT(band_shape_rows, SZS_BAND_ROWS)(int kind, bool affine, int classes, bool direct, bool wide) {
    if (wide) {
        SZS_BAND_WIDE_DISPATCH(band_shape_of, classes)
    }
    else if (direct) {
        SZS_BAND_DIRECT_DISPATCH(band_shape_of, classes)
    }
    else {
        SZS_BAND_DISPATCH(band_shape_of, classes)
    }
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t SZS_CONCAT(launch_band_rows, SZS_BAND_ROWS)(int kind, bool affine, int key_begin, int key_end,
                                                      pair_task_t const *tasks, plan_bins_t *bins,
                                                      score_costs_t const &costs, std::int64_t *results, void *scratch,
                                                      std::size_t ring_cells_per_slot, int ctas, cudaStream_t stream,
                                                      void *group_states, int group_ctas, bool wide) {
    if (wide) {
        SZS_BAND_WIDE_DISPATCH(band_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                               ring_cells_per_slot, ctas, stream, group_states, group_ctas)
    }
    else if (costs.direct_table) {
        SZS_BAND_DIRECT_DISPATCH(band_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                                 ring_cells_per_slot, ctas, stream, group_states, group_ctas)
    }
    else {
        SZS_BAND_DISPATCH(band_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                          ring_cells_per_slot, ctas, stream, group_states, group_ctas)
    }
    return cudaErrorInvalidValue;
}

#if SZS_BAND_ROWS == 8

dp_launch_shape_t band_shape_rows4(int kind, bool affine, int classes, bool direct, bool wide);
cudaError_t launch_band_rows4(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks,
                              plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                              std::size_t ring_cells_per_slot, int ctas, cudaStream_t stream, void *group_states,
                              int group_ctas, bool wide);

int band_warps_per_cta() { return band_warps_k; }

dp_launch_shape_t band_shape(int kind, bool affine, int classes, bool direct, bool wide, int rows_per_lane) {
    return rows_per_lane == 4 ? band_shape_rows4(kind, affine, classes, direct, wide)
                              : band_shape_rows8(kind, affine, classes, direct, wide);
}

cudaError_t launch_band(int kind, bool affine, int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                        score_costs_t const &costs, std::int64_t *results, void *scratch,
                        std::size_t ring_cells_per_slot, int ctas, cudaStream_t stream, void *group_states,
                        int group_ctas, bool wide, int rows_per_lane) {
    if (rows_per_lane == 4)
        return launch_band_rows4(kind, affine, key_begin, key_end, tasks, bins, costs, results, scratch,
                                 ring_cells_per_slot, ctas, stream, group_states, group_ctas, wide);
    return launch_band_rows8(kind, affine, key_begin, key_end, tasks, bins, costs, results, scratch,
                             ring_cells_per_slot, ctas, stream, group_states, group_ctas, wide);
}

std::size_t band_group_state_bytes() { return sizeof(band_group_state_t); }
int band_group_max_ctas() { return band_group_max_ctas_k; }

#endif

} // namespace szs_gb300
