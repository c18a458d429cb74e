/**
 *  @file kernels_myers_table.cu
 *  @brief Instantiations of the shared-table bit-parallel kernel (batches over at most four symbol codes) for 1..16
 *         pattern words.
 */
#include "launchers.h"
#include "myers_table.cuh"

namespace szs_gb300 {

template <int words_>
static cudaError_t myers_table_launch_words(pair_task_t const *tasks, plan_bins_t *bins, int key_begin,
                                            int key_end, batch_alphabet_t const *alphabet, std::int64_t *results,
                                            int ctas, cudaStream_t stream) {
    int const shared = myers_table_shared_bytes(words_);
    auto kernel = myers_table_kernel<words_>;
    if (shared > 48 * 1024) {
        cudaError_t const status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
        if (status != cudaSuccess) return status;
    }
    kernel<<<ctas, myers_table_threads_k, shared, stream>>>(tasks, bins, key_begin, key_end, alphabet, results);
    return cudaGetLastError();
}

cudaError_t launch_myers_table(int words, int key_begin, int key_end, pair_task_t const *tasks,
                               plan_bins_t *bins, batch_alphabet_t const *alphabet, std::int64_t *results,
                               int ctas, cudaStream_t stream) {
    switch (words) {
    case 1: return myers_table_launch_words<1>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 2: return myers_table_launch_words<2>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 3: return myers_table_launch_words<3>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 4: return myers_table_launch_words<4>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 5: return myers_table_launch_words<5>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 6: return myers_table_launch_words<6>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 7: return myers_table_launch_words<7>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 8: return myers_table_launch_words<8>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 9: return myers_table_launch_words<9>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 10: return myers_table_launch_words<10>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 11: return myers_table_launch_words<11>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 12: return myers_table_launch_words<12>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 13: return myers_table_launch_words<13>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 14: return myers_table_launch_words<14>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 15: return myers_table_launch_words<15>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 16: return myers_table_launch_words<16>(tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace szs_gb300
