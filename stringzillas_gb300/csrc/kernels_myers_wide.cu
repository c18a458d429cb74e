/**
 *  @file kernels_myers_wide.cu
 *  @brief Instantiations of the bit-parallel kernels over strings of 16-bit codes (UTF-8 Levenshtein calls over more
 *         than 256 code points): thread per pair up to 8 words (16 code planes of 16 words would spill), warp per
 *         pair up to 8 words per lane.
 */
#include "launchers.h"
#include "myers.cuh"
#include "myers_warp.cuh"

namespace szs_gb300 {

namespace {

template <int words_>
cudaError_t thread_launch(bool exact, pair_task_t const *tasks, plan_bins_t const *bins, int key_begin, int key_end,
                          std::int64_t *results, int ctas, cudaStream_t stream) {
    if (exact) myers_wide_kernel<words_, true><<<ctas, 128, 0, stream>>>(tasks, bins, key_begin, key_end, results);
    else myers_wide_kernel<words_, false><<<ctas, 128, 0, stream>>>(tasks, bins, key_begin, key_end, results);
    return cudaGetLastError();
}

template <int words_>
cudaError_t warp_launch(pair_task_t const *tasks, plan_bins_t *bins, int key_begin, int key_end, std::int64_t *results,
                        int ctas, cudaStream_t stream) {
    myers_warp_wide_kernel<words_><<<ctas, 256, 0, stream>>>(tasks, bins, key_begin, key_end, results);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_myers_wide(int words, bool exact, pair_task_t const *tasks, plan_bins_t const *bins, int key_begin,
                              int key_end, std::int64_t *results, int ctas, cudaStream_t stream) {
    switch (words) {
    case 1: return thread_launch<1>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 2: return thread_launch<2>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 3: return thread_launch<3>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 4: return thread_launch<4>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 5: return thread_launch<5>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 6: return thread_launch<6>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 7: return thread_launch<7>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    case 8: return thread_launch<8>(exact, tasks, bins, key_begin, key_end, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_myers_warp_wide(int words, pair_task_t const *tasks, plan_bins_t *bins, int key_begin, int key_end,
                                   std::int64_t *results, int ctas, cudaStream_t stream) {
    switch (words) {
    case 1: return warp_launch<1>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 2: return warp_launch<2>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 3: return warp_launch<3>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 4: return warp_launch<4>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 5: return warp_launch<5>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 6: return warp_launch<6>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 7: return warp_launch<7>(tasks, bins, key_begin, key_end, results, ctas, stream);
    case 8: return warp_launch<8>(tasks, bins, key_begin, key_end, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace szs_gb300
