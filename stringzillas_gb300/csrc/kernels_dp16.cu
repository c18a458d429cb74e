/**
 *  @file kernels_dp16.cu
 *  @brief Instantiations and launcher of the 16x2 packed wavefront kernel (dp_packed.cuh).
 *
 *  Compiled twice: once for the profile instances and the public entry points, once with
 *  `SZS_DP16_COMPARE_UNIT` for the compare-mode instances (Levenshtein over more than 32 byte values, bytes or 16-bit
 *  codes), so the two halves of the instantiation work build in parallel.
 */
#include "dp_packed.cuh"
#include "launchers.h"

namespace szs_gb300 {

namespace {

// 8 rows per lane (the planner's choice for longer pairs) take two columns per step. 4 rows (short pairs) keep one:
// with two, the 31 steps by which lane 31 trails lane 0 would idle twice the columns of a short sweep (a cross
// product of 100-byte strings ran 6 % slower). 12 and 16 rows have no registers to spare.
template <int kind_, bool affine_, int rows_, int compare_, bool wide_>
using dp16_instance_t = dp16_policy_t<kind_, affine_, rows_, compare_, wide_, rows_ == 8 ? 2 : 1>;

template <int kind_, bool affine_, int rows_, int compare_, bool wide_>
dp_launch_shape_t dp16_shape_rows(int classes, int warps) {
    using policy_t = dp16_instance_t<kind_, affine_, rows_, compare_, wide_>;
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

template <int kind_, bool affine_, int compare_ = compare_none_k, bool wide_ = false>
dp_launch_shape_t dp16_shape_of(int rows, int classes, int warps) {
    switch (rows) {
    case 4: return dp16_shape_rows<kind_, affine_, 4, compare_, wide_>(classes, warps);
    case 8: return dp16_shape_rows<kind_, affine_, 8, compare_, wide_>(classes, warps);
    case 12: return dp16_shape_rows<kind_, affine_, 12, compare_, wide_>(classes, warps);
    case 16: return dp16_shape_rows<kind_, affine_, 16, compare_, wide_>(classes, warps);
    default: return dp_launch_shape_t {0, 0, 0, 0, 0};
    }
}

template <int kind_, bool affine_, int rows_, int compare_, bool wide_>
cudaError_t dp16_launch_rows(int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                             score_costs_t const &costs, std::int64_t *results, void *scratch,
                             std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream) {
    using policy_t = dp16_instance_t<kind_, affine_, rows_, compare_, wide_>;
    int const shared = dp16_shared_bytes<policy_t>(warps, costs.classes);
    auto kernel = dp16_wavefront_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, warps * 32, shared, stream>>>(tasks, bins, key_begin, key_end, costs, results,
                                                 static_cast<std::uint32_t *>(scratch), scratch_cells_per_warp);
    return cudaGetLastError();
}

template <int kind_, bool affine_, int compare_ = compare_none_k, bool wide_ = false>
cudaError_t dp16_launch_of(int rows, int key_begin, int key_end, pair_task_t const *tasks, plan_bins_t *bins,
                           score_costs_t const &costs, std::int64_t *results, void *scratch,
                           std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream) {
#define SZS_DP16_ROWS(rows_)                                                                                         \
    dp16_launch_rows<kind_, affine_, rows_, compare_, wide_>(key_begin, key_end, tasks, bins, costs, results, scratch, \
                                                             scratch_cells_per_warp, ctas, warps, stream)
    switch (rows) {
    case 4: return SZS_DP16_ROWS(4);
    case 8: return SZS_DP16_ROWS(8);
    case 12: return SZS_DP16_ROWS(12);
    case 16: return SZS_DP16_ROWS(16);
    default: return cudaErrorInvalidValue;
    }
#undef SZS_DP16_ROWS
}

} // namespace

#if defined(SZS_DP16_COMPARE_UNIT)

// Compare-mode instances: affine or not, multiply-add or select form, bytes or 16-bit codes.
#define SZS_DP16_COMPARE_DISPATCH(call_, ...)                                                                        \
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

dp_launch_shape_t dp16_compare_shape(bool affine, int rows, int classes, int warps, int compare, bool wide) {
    SZS_DP16_COMPARE_DISPATCH(dp16_shape_of, rows, classes, warps)
}

cudaError_t launch_dp16_compare(bool affine, int rows, int key_begin, int key_end, pair_task_t const *tasks,
                                plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                                std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream,
                                int compare, bool wide) {
    SZS_DP16_COMPARE_DISPATCH(dp16_launch_of, rows, key_begin, key_end, tasks, bins, costs, results, scratch,
                              scratch_cells_per_warp, ctas, warps, stream)
}

#else

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

dp_launch_shape_t dp16_shape(int kind, bool affine, int rows, int classes, int warps, int compare, bool wide) {
    if (warps < 1 || warps > 8) return dp_launch_shape_t {0, 0, 0, 0, 0};
    if (compare != compare_none_k || wide) {
        if (kind != kind_levenshtein_k || compare == compare_none_k) return dp_launch_shape_t {0, 0, 0, 0, 0};
        return dp16_compare_shape(affine, rows, classes, warps, compare, wide);
    }
    SZS_DP16_DISPATCH(dp16_shape_of, rows, classes, warps)
    return dp_launch_shape_t {0, 0, 0, 0, 0};
}

cudaError_t launch_dp16(int kind, bool affine, int rows, int key_begin, int key_end, pair_task_t const *tasks,
                        plan_bins_t *bins, score_costs_t const &costs, std::int64_t *results, void *scratch,
                        std::size_t scratch_cells_per_warp, int ctas, int warps, cudaStream_t stream, int compare,
                        bool wide) {
    if (warps < 1 || warps > 8) return cudaErrorInvalidValue;
    if (compare != compare_none_k || wide) {
        if (kind != kind_levenshtein_k || compare == compare_none_k) return cudaErrorInvalidValue;
        return launch_dp16_compare(affine, rows, key_begin, key_end, tasks, bins, costs, results, scratch,
                                   scratch_cells_per_warp, ctas, warps, stream, compare, wide);
    }
    SZS_DP16_DISPATCH(dp16_launch_of, rows, key_begin, key_end, tasks, bins, costs, results, scratch,
                      scratch_cells_per_warp, ctas, warps, stream)
    return cudaErrorInvalidValue;
}

#endif

} // namespace szs_gb300
