/**
 *  @file kernels_dp.cu
 *  @brief Instantiations and launcher of the wavefront DP kernel (dp_wavefront.cuh).
 */
#include "dp_wavefront.cuh"
#include "launchers.h"

namespace szs_gb300 {

namespace {

constexpr int dp_rows_per_lane_k = 8;
constexpr int dp_threads_k = 256;

template <int kind_, bool affine_, typename cell_t>
using dp_instance_t = dp_policy_t<kind_, affine_, cell_t, dp_rows_per_lane_k>;

/** The instance for (direct table, 16-bit codes): at most one of the two. */
template <int kind_, bool affine_, typename cell_t, bool direct_, bool wide_>
struct dp_variant {
    using base_t = dp_instance_t<kind_, affine_, cell_t>;
    using type = std::conditional_t<direct_, direct_policy_t<base_t>,
                                    std::conditional_t<wide_, wide_policy_t<base_t>, base_t>>;
};

template <int kind_, bool affine_, typename cell_t, bool direct_ = false, bool wide_ = false>
dp_launch_shape_t dp_shape_of(int classes) {
    using policy_t = typename dp_variant<kind_, affine_, cell_t, direct_, wide_>::type;
    dp_launch_shape_t shape;
    shape.threads_per_cta = dp_threads_k;
    shape.warps_per_cta = dp_threads_k / 32;
    shape.rows_per_lane = dp_rows_per_lane_k;
    shape.shared_bytes = dp_shared_bytes<policy_t>(shape.warps_per_cta, classes);
    auto kernel = dp_wavefront_kernel<policy_t>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.ctas_per_sm = blocks;
    return shape;
}

template <int kind_, bool affine_, typename cell_t, bool direct_ = false, bool wide_ = false>
cudaError_t dp_launch_of(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                         score_costs_t const &costs, std::int64_t *results, void *scratch,
                         std::size_t scratch_cells_per_warp, int ctas, cudaStream_t stream) {
    using policy_t = typename dp_variant<kind_, affine_, cell_t, direct_, wide_>::type;
    int const shared = dp_shared_bytes<policy_t>(dp_threads_k / 32, costs.classes);
    auto kernel = dp_wavefront_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, dp_threads_k, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results,
                                                   static_cast<cell_t *>(scratch), scratch_cells_per_warp);
    return cudaGetLastError();
}

} // namespace

#define SZS_DP_DISPATCH(call_, ...)                                                                                  \
    switch (kind * 4 + (affine ? 2 : 0) + (cell_bits == 64 ? 1 : 0)) {                                               \
    case 0: return call_<kind_levenshtein_k, false, std::int32_t>(__VA_ARGS__);                                      \
    case 1: return call_<kind_levenshtein_k, false, std::int64_t>(__VA_ARGS__);                                      \
    case 2: return call_<kind_levenshtein_k, true, std::int32_t>(__VA_ARGS__);                                       \
    case 3: return call_<kind_levenshtein_k, true, std::int64_t>(__VA_ARGS__);                                       \
    case 4: return call_<kind_needleman_wunsch_k, false, std::int32_t>(__VA_ARGS__);                                 \
    case 5: return call_<kind_needleman_wunsch_k, false, std::int64_t>(__VA_ARGS__);                                 \
    case 6: return call_<kind_needleman_wunsch_k, true, std::int32_t>(__VA_ARGS__);                                  \
    case 7: return call_<kind_needleman_wunsch_k, true, std::int64_t>(__VA_ARGS__);                                  \
    case 8: return call_<kind_smith_waterman_k, false, std::int32_t>(__VA_ARGS__);                                   \
    case 9: return call_<kind_smith_waterman_k, false, std::int64_t>(__VA_ARGS__);                                   \
    case 10: return call_<kind_smith_waterman_k, true, std::int32_t>(__VA_ARGS__);                                   \
    case 11: return call_<kind_smith_waterman_k, true, std::int64_t>(__VA_ARGS__);                                   \
    default: break;                                                                                                  \
    }

/** Direct-table instances exist for the alignment kinds only (dense tables are a Needleman-Wunsch / Smith-Waterman
 *  extension). */
#define SZS_DP_DIRECT_DISPATCH(call_, ...)                                                                           \
    switch (kind * 4 + (affine ? 2 : 0) + (cell_bits == 64 ? 1 : 0)) {                                               \
    case 4: return call_<kind_needleman_wunsch_k, false, std::int32_t, true>(__VA_ARGS__);                           \
    case 5: return call_<kind_needleman_wunsch_k, false, std::int64_t, true>(__VA_ARGS__);                           \
    case 6: return call_<kind_needleman_wunsch_k, true, std::int32_t, true>(__VA_ARGS__);                            \
    case 7: return call_<kind_needleman_wunsch_k, true, std::int64_t, true>(__VA_ARGS__);                            \
    case 8: return call_<kind_smith_waterman_k, false, std::int32_t, true>(__VA_ARGS__);                             \
    case 9: return call_<kind_smith_waterman_k, false, std::int64_t, true>(__VA_ARGS__);                             \
    case 10: return call_<kind_smith_waterman_k, true, std::int32_t, true>(__VA_ARGS__);                             \
    case 11: return call_<kind_smith_waterman_k, true, std::int64_t, true>(__VA_ARGS__);                             \
    default: break;                                                                                                  \
    }

/** 16-bit-code instances exist for Levenshtein only (UTF-8 calls). */
#define SZS_DP_WIDE_DISPATCH(call_, ...)                                                                             \
    switch (kind * 4 + (affine ? 2 : 0) + (cell_bits == 64 ? 1 : 0)) {                                               \
    case 0: return call_<kind_levenshtein_k, false, std::int32_t, false, true>(__VA_ARGS__);                         \
    case 1: return call_<kind_levenshtein_k, false, std::int64_t, false, true>(__VA_ARGS__);                         \
    case 2: return call_<kind_levenshtein_k, true, std::int32_t, false, true>(__VA_ARGS__);                          \
    case 3: return call_<kind_levenshtein_k, true, std::int64_t, false, true>(__VA_ARGS__);                          \
    default: break;                                                                                                  \
    }

dp_launch_shape_t dp_shape(int kind, bool affine, int cell_bits, int classes, bool direct, bool wide) {
    if (wide) {
        SZS_DP_WIDE_DISPATCH(dp_shape_of, classes)
    }
    else if (direct) {
        SZS_DP_DIRECT_DISPATCH(dp_shape_of, classes)
    }
    else {
        SZS_DP_DISPATCH(dp_shape_of, classes)
    }
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t launch_dp(int kind, bool affine, int cell_bits, int key_begin, int key_end, pair_task_t const *tasks,
                      plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                      std::size_t scratch_cells_per_warp, int ctas, cudaStream_t stream, bool wide) {
    if (wide) {
        SZS_DP_WIDE_DISPATCH(dp_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                             scratch_cells_per_warp, ctas, stream)
    }
    else if (costs.direct_table) {
        SZS_DP_DIRECT_DISPATCH(dp_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch,
                               scratch_cells_per_warp, ctas, stream)
    }
    else {
        SZS_DP_DISPATCH(dp_launch_of, key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp,
                        ctas, stream)
    }
    return cudaErrorInvalidValue;
}

} // namespace szs_gb300
