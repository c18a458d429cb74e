/**
 *  @file probe.cu
 *  @brief Measures the integer issue rates the scoring kernels are bound by, on the device at hand.
 *
 *  The wavefront and bit-parallel kernels are neither HBM- nor tensor-bound: their roof is the rate at which SMs
 *  retire 32-bit integer instructions (IADD3 / LOP3 / IMNMX) and the DPX fused add-min/max instructions
 *  (`__viaddmax_s32`, `__vimax3_s32`, `__viaddmax_s16x2`). Each probe kernel keeps 8 values per thread and, per round,
 *  computes 8 new ones, each from three values of the previous round (independent within a round, not foldable by the
 *  compiler), on every SM; it reports operations per second, where one operation is one intrinsic call (one cell
 *  update step for DPX, one 32-bit logic/add for the plain pipe).
 */
#include "stringzillas_gb300.h"

#include <cuda_runtime.h>

#include <cstdint>

namespace szs_gb300 {

constexpr int probe_chains_k = 8;
constexpr int probe_unroll_k = 16;

enum probe_kind_t : int {
    probe_lop3_k = 0,       // (x ^ y) | z : one LOP3
    probe_iadd3_k = 1,      // x + y + z : one IADD3
    probe_viaddmax_k = 2,   // max(x + y, z)
    probe_vimax3_k = 3,     // max(x, y, z)
    probe_viaddmax16_k = 4, // two 16-bit lanes of max(x + y, z)
    probe_count_k = 5,
};

template <int kind_>
__global__ void probe_kernel(std::uint32_t seed, int iterations, std::uint32_t *sink) {
    std::uint32_t a[probe_chains_k];
#pragma unroll
    for (int k = 0; k < probe_chains_k; ++k) a[k] = seed * (threadIdx.x + 3 * k + 1);
    a[0] ^= blockIdx.x;
    // Every round computes 8 new values, each from three values of the previous round, so the 8 operations of a
    // round are independent of each other and no chain can be folded algebraically by the compiler.
    for (int i = 0; i < iterations; ++i) {
#pragma unroll
        for (int u = 0; u < probe_unroll_k; ++u) {
            std::uint32_t next[probe_chains_k];
#pragma unroll
            for (int k = 0; k < probe_chains_k; ++k) {
                std::uint32_t const x = a[k], y = a[(k + 1) % probe_chains_k], z = a[(k + 3) % probe_chains_k];
                if constexpr (kind_ == probe_lop3_k) next[k] = (x ^ y) | z;
                else if constexpr (kind_ == probe_iadd3_k) next[k] = x + y + z;
                else if constexpr (kind_ == probe_viaddmax_k) next[k] = (std::uint32_t)__viaddmax_s32((int)x, (int)y, (int)z);
                else if constexpr (kind_ == probe_vimax3_k) next[k] = (std::uint32_t)__vimax3_s32((int)x, (int)y, (int)z);
                else next[k] = __viaddmax_s16x2(x, y, z);
            }
#pragma unroll
            for (int k = 0; k < probe_chains_k; ++k) a[k] = next[k];
        }
    }
    std::uint32_t folded = 0;
#pragma unroll
    for (int k = 0; k < probe_chains_k; ++k) folded ^= a[k];
    if (folded == 0x9E3779B9u) sink[threadIdx.x] = folded; // practically never; keeps the chains alive
}

template <int kind_>
static cudaError_t probe_one(int device, double &ops_per_second) {
    int sms = 0;
    cudaError_t status = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (status != cudaSuccess) return status;
    std::uint32_t *sink = nullptr;
    if ((status = cudaMalloc(&sink, 1024 * sizeof(std::uint32_t))) != cudaSuccess) return status;
    cudaEvent_t start, stop;
    cudaEventCreate(&start);
    cudaEventCreate(&stop);
    int const threads = 256, blocks = sms * 8, iterations = 2048;
    probe_kernel<kind_><<<blocks, threads>>>(12345u, 16, sink); // warm-up
    cudaEventRecord(start);
    probe_kernel<kind_><<<blocks, threads>>>(12345u, iterations, sink);
    cudaEventRecord(stop);
    status = cudaEventSynchronize(stop);
    float ms = 0;
    cudaEventElapsedTime(&ms, start, stop);
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    cudaFree(sink);
    if (status != cudaSuccess) return status;
    double const ops = (double)blocks * threads * iterations * probe_unroll_k * probe_chains_k;
    ops_per_second = ops / (ms * 1e-3);
    return cudaGetLastError();
}

} // namespace szs_gb300

extern "C" {

/**
 *  Measures, on @p gpu_device, the sustained rate (operations per second, whole GPU) of: [0] LOP3, [1] IADD3,
 *  [2] DPX `max(a + b, c)` on 32-bit lanes, [3] DPX `max(a, b, c)`, [4] DPX `max(a + b, c)` on 16x2 lanes (one op
 *  = one instruction covering two cells). No counterpart in the reference.
 */
SZS_GB300_API sz_status_t szs_gb300_measure_integer_peaks(sz_size_t gpu_device, double *ops_per_second,
                                                          sz_size_t count, char const **error_message) {
    using namespace szs_gb300;
    if (!ops_per_second || count < (sz_size_t)probe_count_k) {
        if (error_message) *error_message = "Need room for 5 rates";
        return sz_unexpected_dimensions_k;
    }
    int const device = (int)gpu_device;
    cudaError_t status = cudaSetDevice(device);
    if (status == cudaSuccess) status = probe_one<probe_lop3_k>(device, ops_per_second[0]);
    if (status == cudaSuccess) status = probe_one<probe_iadd3_k>(device, ops_per_second[1]);
    if (status == cudaSuccess) status = probe_one<probe_viaddmax_k>(device, ops_per_second[2]);
    if (status == cudaSuccess) status = probe_one<probe_vimax3_k>(device, ops_per_second[3]);
    if (status == cudaSuccess) status = probe_one<probe_viaddmax16_k>(device, ops_per_second[4]);
    if (status != cudaSuccess) {
        if (error_message) *error_message = cudaGetErrorName(status);
        return status == cudaErrorNoDevice || status == cudaErrorInvalidDevice ? sz_missing_gpu_k
                                                                                : sz_status_unknown_k;
    }
    if (error_message) *error_message = nullptr;
    return sz_success_k;
}

} // extern "C"
