/**
 *  @file kernels_myers.cu
 *  @brief Instantiations of the bit-parallel kernel for one plane count, selected with -DSZS_MYERS_PLANES=<2|3|5|8>
 *         (the build compiles this file once per plane count, in parallel).
 */
#include "launchers.h"
#include "myers.cuh"
#include "myers_warp.cuh"

#ifndef SZS_MYERS_PLANES
#error "compile with -DSZS_MYERS_PLANES=<2|3|5|8>"
#endif

#define SZS_CONCAT_(a, b) a##b
#define SZS_CONCAT(a, b) SZS_CONCAT_(a, b)

namespace szs_gb300 {

constexpr int myers_threads_k = 128;

template <int words_>
static cudaError_t myers_launch_words(bool exact, pair_task_t const *tasks, plan_bins_t const *bins, int key_begin,
                                      int key_end, batch_alphabet_t const *alphabet, std::int64_t *results, int ctas,
                                      cudaStream_t stream) {
    if (exact)
        myers_kernel<words_, SZS_MYERS_PLANES, true>
            <<<ctas, myers_threads_k, 0, stream>>>(tasks, bins, key_begin, key_end, alphabet, results);
    else
        myers_kernel<words_, SZS_MYERS_PLANES, false>
            <<<ctas, myers_threads_k, 0, stream>>>(tasks, bins, key_begin, key_end, alphabet, results);
    return cudaGetLastError();
}

cudaError_t SZS_CONCAT(launch_myers_planes, SZS_MYERS_PLANES)(int words, bool exact, pair_task_t const *tasks,
                                                                plan_bins_t const *bins, int key_begin, int key_end,
                                                                batch_alphabet_t const *alphabet,
                                                                std::int64_t *results, int ctas, cudaStream_t stream) {
    switch (words) {
    case 1: return myers_launch_words<1>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 2: return myers_launch_words<2>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 3: return myers_launch_words<3>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 4: return myers_launch_words<4>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 5: return myers_launch_words<5>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 6: return myers_launch_words<6>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 7: return myers_launch_words<7>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 8: return myers_launch_words<8>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 9: return myers_launch_words<9>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 10: return myers_launch_words<10>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 11: return myers_launch_words<11>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 12: return myers_launch_words<12>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 13: return myers_launch_words<13>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 14: return myers_launch_words<14>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 15: return myers_launch_words<15>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 16: return myers_launch_words<16>(exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

template <int words_>
static cudaError_t myers_warp_launch_words(pair_task_t const *tasks, plan_bins_t *bins, int key_begin, int key_end,
                                           batch_alphabet_t const *alphabet, std::int64_t *results, int ctas,
                                           cudaStream_t stream) {
    myers_warp_kernel<words_, SZS_MYERS_PLANES>
        <<<ctas, 256, 0, stream>>>(tasks, bins, key_begin, key_end, alphabet, results);
    return cudaGetLastError();
}

cudaError_t SZS_CONCAT(launch_myers_warp_planes, SZS_MYERS_PLANES)(int words, pair_task_t const *tasks,
                                                                     plan_bins_t *bins, int key_begin, int key_end,
                                                                     batch_alphabet_t const *alphabet,
                                                                     std::int64_t *results, int ctas,
                                                                     cudaStream_t stream) {
    switch (words) {
    case 1: return myers_warp_launch_words<1>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 2: return myers_warp_launch_words<2>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 3: return myers_warp_launch_words<3>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 4: return myers_warp_launch_words<4>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 5: return myers_warp_launch_words<5>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 6: return myers_warp_launch_words<6>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 7: return myers_warp_launch_words<7>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 8: return myers_warp_launch_words<8>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace szs_gb300
