/**
 *  @file kernels_dp16.cu
 *  @brief Instantiations and launcher of the 16x2 packed wavefront kernel (dp_packed.cuh).
 */
#include "dp_packed.cuh"
#include "launchers.h"

namespace szs_gb300 {

namespace {

template <int kind_, bool affine_, int rows_, int compare_>
dp_launch_shape_t dp16_shape_rows(int classes, int warps) {
    using policy_t = dp16_policy_t<kind_, affine_, rows_, compare_>;
    dp_launch_shape_t shape;
    shape.threads_per_cta = warps * 32;
    shape.warps_per_cta = warps;
    shape.rows_per_lane = rows_;
    shape.shared_bytes = dp16_shared_bytes<policy_t>(shape.warps_per_cta, classes);
    auto kernel = dp16_wavefront_kernel<policy_t>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shape.shared_bytes);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, shape.threads_per_cta, shape.shared_bytes) !=
        cudaSuccess)
        blocks = 0;
    shape.ctas_per_sm = blocks;
    return shape;
}

template <int kind_, bool affine_, int compare_ = compare_none_k>
dp_launch_shape_t dp16_shape_of(int rows, int classes, int warps) {
    switch (rows) {
    case 4: return dp16_shape_rows<kind_, affine_, 4, compare_>(classes, warps);
    case 8: return dp16_shape_rows<kind_, affine_, 8, compare_>(classes, warps);
    case 12: return dp16_shape_rows<kind_, affine_, 12, compare_>(classes, warps);
    case 16: return dp16_shape_rows<kind_, affine_, 16, compare_>(classes, warps);
    default: return dp_launch_shape_t {0, 0, 0, 0, 0};
    }
}

template <int kind_, bool affine_, int rows_, int compare_>
cudaError_t dp16_launch_rows(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                             score_costs_t const &costs, std::int64_t *results, void *scratch,
                             std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream) {
    using policy_t = dp16_policy_t<kind_, affine_, rows_, compare_>;
    int const shared = dp16_shared_bytes<policy_t>(warps, costs.classes);
    auto kernel = dp16_wavefront_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, warps * 32, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results,
                                                     static_cast<std::uint32_t *>(scratch), scratch_cells_per_warp);
    return cudaGetLastError();
}

template <int kind_, bool affine_, int compare_ = compare_none_k>
cudaError_t dp16_launch_of(int rows, int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                           score_costs_t const &costs, std::int64_t *results, void *scratch,
                           std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream) {
    switch (rows) {
    case 4: return dp16_launch_rows<kind_, affine_, 4, compare_>(key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp, ctas, warps, stream);
    case 8: return dp16_launch_rows<kind_, affine_, 8, compare_>(key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp, ctas, warps, stream);
    case 12: return dp16_launch_rows<kind_, affine_, 12, compare_>(key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp, ctas, warps, stream);
    case 16: return dp16_launch_rows<kind_, affine_, 16, compare_>(key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp, ctas, warps, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace

#define SZS_DP16_DISPATCH(call_, ...)                                                                                \
    switch (kind * 2 + (affine ? 1 : 0)) {                                                                           \
    case 0: return call_<kind_levenshtein_k, false>(__VA_ARGS__);                                                    \
    case 1: return call_<kind_levenshtein_k, true>(__VA_ARGS__);                                                     \
    case 2: return call_<kind_needleman_wunsch_k, false>(__VA_ARGS__);                                               \
    case 3: return call_<kind_needleman_wunsch_k, true>(__VA_ARGS__);                                                \
    case 4: return call_<kind_smith_waterman_k, false>(__VA_ARGS__);                                                 \
    case 5: return call_<kind_smith_waterman_k, true>(__VA_ARGS__);                                                  \
    default: break;                                                                                                  \
    }

dp_launch_shape_t dp16_shape(int kind, bool affine, int rows, int classes, int warps, int compare) {
    if (warps < 1 || warps > 8) return dp_launch_shape_t {0, 0, 0, 0, 0};
    if (compare != compare_none_k) {
        if (kind != kind_levenshtein_k) return dp_launch_shape_t {0, 0, 0, 0, 0};
        switch ((affine ? 2 : 0) + (compare == compare_multiply_k ? 1 : 0)) {
        case 0: return dp16_shape_of<kind_levenshtein_k, false, compare_select_k>(rows, classes, warps);
        case 1: return dp16_shape_of<kind_levenshtein_k, false, compare_multiply_k>(rows, classes, warps);
        case 2: return dp16_shape_of<kind_levenshtein_k, true, compare_select_k>(rows, classes, warps);
        default: return dp16_shape_of<kind_levenshtein_k, true, compare_multiply_k>(rows, classes, warps);
        }
    }
    SZS_DP16_DISPATCH(dp16_shape_of, rows, classes, warps)
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t launch_dp16(int kind, bool affine, int rows, int key_begin, int key_end, pair_task_t const *tasks,
                        plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                        std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream, int compare) {
    if (warps < 1 || warps > 8) return cudaErrorInvalidValue;
    if (compare != compare_none_k) {
        if (kind != kind_levenshtein_k) return cudaErrorInvalidValue;
#define SZS_DP16_COMPARE(affine_, mode_)                                                                              \
    dp16_launch_of<kind_levenshtein_k, affine_, mode_>(rows, key_begin, key_end, tasks, bins, costs, results, scratch, \
                                                       scratch_cells_per_warp, ctas, warps, stream)
        switch ((affine ? 2 : 0) + (compare == compare_multiply_k ? 1 : 0)) {
        case 0: return SZS_DP16_COMPARE(false, compare_select_k);
        case 1: return SZS_DP16_COMPARE(false, compare_multiply_k);
        case 2: return SZS_DP16_COMPARE(true, compare_select_k);
        default: return SZS_DP16_COMPARE(true, compare_multiply_k);
        }
#undef SZS_DP16_COMPARE
    }
    SZS_DP16_DISPATCH(dp16_launch_of, rows, key_begin, key_end, tasks, bins, costs, results, scratch, scratch_cells_per_warp,
                      ctas, warps, stream)
    return cudaErrorInvalidValue;
}

} // namespace szs_gb300
