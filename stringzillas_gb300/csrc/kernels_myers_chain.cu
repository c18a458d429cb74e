/**
 *  @file kernels_myers_chain.cu
 *  @brief Instantiations and cooperative launcher of the chained bit-parallel kernel (myers_chain.cuh) for 1, 2 or
 *         4 words per lane and 2, 3, 5 or 8 code planes: one launch per wave of pairs that fits the GPU at once.
 */
#include "launchers.h"
#include "myers_chain.cuh"

namespace szs_gb300 {

namespace {

template <int words_, int bits_>
int chain_ctas_per_sm() {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, myers_chain_kernel<words_, bits_>,
                                                      myers_chain_threads_k, 0) != cudaSuccess)
        blocks = 0;
    return blocks;
}

template <int words_, int bits_>
cudaError_t chain_launch(pair_task_t const *tasks, plan_bins_t *bins, int key, std::uint32_t first, std::uint32_t pairs,
                         std::uint32_t strips_per_pair, batch_alphabet_t const *alphabet, std::int64_t *results,
                         void *scratch, std::uint64_t link_stride, std::uint32_t wait_polls, cudaStream_t stream) {
    // Clear every pair's state and progress words (the links are written before they are read).
    std::uint64_t const pair_bytes = myers_chain_pair_bytes(strips_per_pair, link_stride);
    std::uint64_t const head = 256 + ((std::uint64_t)strips_per_pair * 4 + 255) / 256 * 256;
    cudaError_t status = cudaMemset2DAsync(scratch, (std::size_t)pair_bytes, 0, (std::size_t)head, pairs, stream);
    if (status != cudaSuccess) return status;
    // The warps of a chain wait on one another: a cooperative launch keeps the whole grid resident.
    std::uint64_t const warps = (std::uint64_t)pairs * strips_per_pair;
    cudaLaunchConfig_t config {};
    config.gridDim = dim3((unsigned)((warps + 7) / 8)), config.blockDim = dim3(myers_chain_threads_k);
    config.dynamicSmemBytes = 0, config.stream = stream;
    cudaLaunchAttribute attribute {};
    attribute.id = cudaLaunchAttributeCooperative, attribute.val.cooperative = 1;
    config.attrs = &attribute, config.numAttrs = 1;
    return cudaLaunchKernelEx(&config, myers_chain_kernel<words_, bits_>, tasks, bins, key, first, pairs,
                              strips_per_pair, alphabet, results, static_cast<unsigned char *>(scratch), link_stride,
                              wait_polls);
}

#define SZS_CHAIN_DISPATCH(call_, ...)                                                                               \
    switch (words * 16 + planes) {                                                                                   \
    case 16 + 2: return call_<1, 2>(__VA_ARGS__);                                                                    \
    case 16 + 3: return call_<1, 3>(__VA_ARGS__);                                                                    \
    case 16 + 5: return call_<1, 5>(__VA_ARGS__);                                                                    \
    case 16 + 8: return call_<1, 8>(__VA_ARGS__);                                                                    \
    case 32 + 2: return call_<2, 2>(__VA_ARGS__);                                                                    \
    case 32 + 3: return call_<2, 3>(__VA_ARGS__);                                                                    \
    case 32 + 5: return call_<2, 5>(__VA_ARGS__);                                                                    \
    case 32 + 8: return call_<2, 8>(__VA_ARGS__);                                                                    \
    case 64 + 2: return call_<4, 2>(__VA_ARGS__);                                                                    \
    case 64 + 3: return call_<4, 3>(__VA_ARGS__);                                                                    \
    case 64 + 5: return call_<4, 5>(__VA_ARGS__);                                                                    \
    case 64 + 8: return call_<4, 8>(__VA_ARGS__);                                                                    \
    default: break;                                                                                                  \
    }

} // namespace

std::uint64_t myers_chain_scratch_bytes(std::uint32_t strips_per_pair, std::uint64_t link_stride, std::uint32_t pairs) {
    return myers_chain_pair_bytes(strips_per_pair, link_stride) * pairs;
}

int myers_chain_ctas_per_sm(int words, int planes) {
    SZS_CHAIN_DISPATCH(chain_ctas_per_sm)
    return 0;
}

cudaError_t launch_myers_chain(int words, int planes, pair_task_t const *tasks, plan_bins_t *bins, int key,
                               std::uint32_t first, std::uint32_t pairs, std::uint32_t strips_per_pair,
                               batch_alphabet_t const *alphabet, std::int64_t *results, void *scratch,
                               std::uint64_t link_stride, std::uint32_t wait_polls, cudaStream_t stream) {
    SZS_CHAIN_DISPATCH(chain_launch, tasks, bins, key, first, pairs, strips_per_pair, alphabet, results, scratch,
                       link_stride, wait_polls, stream)
    return cudaErrorInvalidValue;
}

} // namespace szs_gb300
