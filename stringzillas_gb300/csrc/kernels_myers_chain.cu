/**
 *  @file kernels_myers_chain.cu
 *  @brief Instantiations and cooperative launcher of the chained bit-parallel kernel (myers_chain.cuh) for 1, 2 or
 *         4 words per lane and 2, 3, 5 or 8 code planes.
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
cudaError_t chain_launch(pair_task_t const *tasks, plan_bins_t *bins, int key, int index,
                         batch_alphabet_t const *alphabet, std::int64_t *results, void *scratch,
                         std::uint64_t link_stride, std::uint32_t strips, int ctas, std::uint32_t wait_polls,
                         cudaStream_t stream) {
    auto *state = static_cast<myers_chain_state_t *>(scratch);
    auto *progress = reinterpret_cast<std::uint32_t *>(static_cast<unsigned char *>(scratch) + 256);
    auto *links = static_cast<std::uint8_t *>(scratch) + myers_chain_links_offset(strips);
    cudaError_t status = cudaMemsetAsync(scratch, 0, myers_chain_links_offset(strips), stream);
    if (status != cudaSuccess) return status;
    // The warps of a chain wait on one another: a cooperative launch keeps the whole grid resident.
    cudaLaunchConfig_t config {};
    config.gridDim = dim3((unsigned)ctas), config.blockDim = dim3(myers_chain_threads_k);
    config.dynamicSmemBytes = 0, config.stream = stream;
    cudaLaunchAttribute attribute {};
    attribute.id = cudaLaunchAttributeCooperative, attribute.val.cooperative = 1;
    config.attrs = &attribute, config.numAttrs = 1;
    return cudaLaunchKernelEx(&config, myers_chain_kernel<words_, bits_>, tasks, bins, key, index, alphabet, results,
                              state, progress, links, link_stride, wait_polls);
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

std::size_t myers_chain_links_offset(std::uint32_t strips) {
    return 256 + ((std::size_t)strips * 4 + 255) / 256 * 256;
}

int myers_chain_ctas_per_sm(int words, int planes) {
    SZS_CHAIN_DISPATCH(chain_ctas_per_sm)
    return 0;
}

cudaError_t launch_myers_chain(int words, int planes, pair_task_t const *tasks, plan_bins_t *bins, int key,
                               int index, batch_alphabet_t const *alphabet, std::int64_t *results, void *scratch,
                               std::uint64_t link_stride, std::uint32_t strips, int ctas, std::uint32_t wait_polls,
                               cudaStream_t stream) {
    SZS_CHAIN_DISPATCH(chain_launch, tasks, bins, key, index, alphabet, results, scratch, link_stride, strips, ctas,
                       wait_polls, stream)
    return cudaErrorInvalidValue;
}

} // namespace szs_gb300
