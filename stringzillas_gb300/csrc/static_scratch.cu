/**
 *  @file static_scratch.cu
 *  @brief Pairwise scoring that allocates nothing: the wavefront kernel with its scratch rows in a fixed, file-scope
 *         device array instead of engine-owned `cudaMalloc` buffers.
 *
 *  Who needs it: callers that cannot call `cudaMalloc` / `cudaFree` - for example a host application whose own
 *  allocator already reserves the device memory, or a latency-bound loop where the implicit device-wide
 *  synchronisation of `cudaFree` would stall other streams. They pass device-resident inputs and a device-resident
 *  result array and get the same scores as `szs_*_pairwise_u64tape`.
 *
 *  How: one kernel launch, one warp per pair (grid-stride, input order), no planner and no task list. Pairs whose
 *  shorter side fits one strip (at most 256 bytes) need no scratch at all; longer ones use this warp's fixed row of
 *  `static_scratch_columns_k` (H, F) cells, so their longer side must be below that many bytes.
 *
 *  The array is shared by every call on a device and keeps the last call's contents: each call clears the control
 *  word it reads back, and two calls whose kernels overlap on the GPU (different streams, no ordering) race on it.
 */
#include "dp_wavefront.cuh"
#include "launchers.h"
#include "stringzillas_gb300.h"

#include <cuda_runtime.h>

#include <mutex>

namespace szs_gb300 {

constexpr int static_scratch_warps_k = 1024;
constexpr int static_scratch_threads_k = 256;
constexpr std::size_t static_scratch_columns_k = 2048;  // (H, F) pairs of 32-bit cells per warp row
constexpr std::size_t static_scratch_control_bytes_k = 256;
constexpr std::size_t static_scratch_row_bytes_k = static_scratch_columns_k * 2 * sizeof(std::int32_t);
constexpr std::size_t static_scratch_bytes_k =
    static_scratch_control_bytes_k + static_scratch_warps_k * static_scratch_row_bytes_k; // 16 MiB + 256 B

/** The scratch every call on a device shares; lives as long as the library stays loaded. */
static __device__ __align__(256) unsigned char static_scratch[static_scratch_bytes_k];

enum static_scratch_error_t : std::uint32_t {
    static_scratch_too_long_k = 1u,  // a multi-strip pair's longer side needs more columns than a row holds
    static_scratch_too_wide_k = 2u,  // a pair's scores could overflow 32-bit cells
};

struct static_scratch_control_t {
    std::uint32_t errors;
};

template <typename policy_>
__global__ void __launch_bounds__(static_scratch_threads_k)
    static_scratch_pairwise_kernel(tape_t const first, tape_t const second, std::uint64_t count,
                                   score_costs_t const costs, int steps_beyond_span, int magnitude,
                                   std::int64_t *__restrict__ results, unsigned char *__restrict__ scratch) {
    using cell_t = typename policy_::cell_t;
    extern __shared__ __align__(16) unsigned char shared_bytes[];
    score_costs_t &costs_s = *reinterpret_cast<score_costs_t *>(shared_bytes);
    std::int8_t *profiles = reinterpret_cast<std::int8_t *>(shared_bytes + ((sizeof(score_costs_t) + 15) / 16) * 16);
    {
        auto const *src = reinterpret_cast<std::uint32_t const *>(&costs);
        auto *dst = reinterpret_cast<std::uint32_t *>(&costs_s);
        for (unsigned i = threadIdx.x; i < sizeof(score_costs_t) / 4; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();

    auto *control = reinterpret_cast<static_scratch_control_t *>(scratch);
    int const lane = threadIdx.x & 31;
    int const warp_in_cta = threadIdx.x >> 5;
    std::uint64_t const warps = (std::uint64_t)gridDim.x * (blockDim.x >> 5);
    std::uint64_t const warp = (std::uint64_t)blockIdx.x * (blockDim.x >> 5) + warp_in_cta;
    cell_t *row = reinterpret_cast<cell_t *>(scratch + static_scratch_control_bytes_k +
                                             warp * static_scratch_row_bytes_k);
    std::int8_t *profile = profiles + warp_in_cta * dp_profile_bytes_per_warp<policy_>(costs.classes);

    for (std::uint64_t p = warp; p < count; p += warps) {
        auto const *first_offsets = static_cast<std::uint64_t const *>(first.offsets);
        auto const *second_offsets = static_cast<std::uint64_t const *>(second.offsets);
        std::uint64_t const a_begin = first_offsets[p], a_length = first_offsets[p + 1] - a_begin;
        std::uint64_t const b_begin = second_offsets[p], b_length = second_offsets[p + 1] - b_begin;
        std::int64_t score = 0;
        if (a_length == 0 || b_length == 0) {
            // Closed form of an empty side (serial.hpp:142-151, :2493-2496).
            std::uint64_t const length = a_length > b_length ? a_length : b_length;
            if (costs.kind == kind_smith_waterman_k) score = 0;
            else if (!costs.affine) score = (std::int64_t)costs.open * (std::int64_t)length;
            else score = length == 0 ? 0 : (std::int64_t)costs.open + (std::int64_t)costs.extend * (std::int64_t)(length - 1);
        }
        else {
            bool const swap = b_length < a_length;
            pair_task_t task;
            task.rows = swap ? second.base + b_begin : first.base + a_begin;
            task.cols = swap ? first.base + a_begin : second.base + b_begin;
            task.rows_length = (std::uint32_t)(swap ? b_length : a_length);
            task.cols_length = (std::uint32_t)(swap ? a_length : b_length);
            task.slot = 0;
            task.transposed = swap ? 1u : 0u;
            std::uint64_t const n = task.rows_length, m = task.cols_length;
            std::uint64_t const span = policy_::maximize_k ? n + m : m;
            bool const fits = (span + (std::uint64_t)steps_beyond_span + 1) * (std::uint64_t)magnitude < (1ull << 31) - 1;
            bool const needs_row = n > (std::uint64_t)policy_::strip_rows_k;
            if (!fits || (needs_row && m + 1 > static_scratch_columns_k)) {
                if (lane == 0) atomicOr(&control->errors, fits ? static_scratch_too_long_k : static_scratch_too_wide_k);
                score = 0; // a rejected pair's slot reads 0; the call's status says that some pair was rejected
            }
            else score = dp_score_pair_warp<policy_>(task, costs_s, row, profile);
        }
        if (lane == 0) results[p] = score;
    }
}

namespace {

std::mutex static_scratch_mutex;
unsigned char *static_scratch_address[64] = {nullptr};

/** Resolves the array's device address once per device (with that device current) and keeps it for the life of the
 *  process. The address belongs to the device's primary context: after a `cudaDeviceReset` of that device it is
 *  stale, so this entry point must not be used across a reset. */
cudaError_t static_scratch_pointer(int device, unsigned char *&pointer) {
    std::lock_guard<std::mutex> lock(static_scratch_mutex);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!static_scratch_address[device]) {
        void *address = nullptr;
        cudaError_t const status = cudaGetSymbolAddress(&address, static_scratch);
        if (status != cudaSuccess) return status;
        static_scratch_address[device] = static_cast<unsigned char *>(address);
    }
    pointer = static_scratch_address[device];
    return cudaSuccess;
}

/** Restores the calling thread's current device on every return path. */
struct current_device_guard_t {
    int saved = -1;
    current_device_guard_t() {
        if (cudaGetDevice(&saved) != cudaSuccess) {
            cudaGetLastError();
            saved = -1;
        }
    }
    ~current_device_guard_t() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

template <int kind_, bool affine_>
cudaError_t launch_static(tape_t const &first, tape_t const &second, std::uint64_t count, score_costs_t const &costs,
                          int steps, int magnitude, std::int64_t *results, unsigned char *scratch, int ctas,
                          cudaStream_t stream) {
    using policy_t = dp_policy_t<kind_, affine_, std::int32_t, 8>;
    int const shared = dp_shared_bytes<policy_t>(static_scratch_threads_k / 32, costs.classes);
    auto kernel = static_scratch_pairwise_kernel<policy_t>;
    cudaError_t status = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared);
    if (status != cudaSuccess) return status;
    kernel<<<ctas, static_scratch_threads_k, shared, stream>>>(first, second, count, costs, steps, magnitude, results,
                                                              scratch);
    return cudaGetLastError();
}

/** True for managed memory, and for device memory of `device` itself (another GPU's memory is not mapped here). */
bool on_device(void const *pointer, int device) {
    if (!pointer) return false;
    cudaPointerAttributes attributes;
    if (cudaPointerGetAttributes(&attributes, pointer) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (attributes.type == cudaMemoryTypeManaged) return true;
    return attributes.type == cudaMemoryTypeDevice && attributes.device == device;
}

} // namespace

/** Engine fields this entry point needs, filled by engine.cu (which owns the engine layout); declared identically
 *  there. */
struct static_call_t {
    score_costs_t const *costs;
    int kind;
    int magnitude;
    int device;
    cudaStream_t stream;
};

sz_status_t static_scratch_pairwise(static_call_t const &call, sz_sequence_u64tape_t const *first,
                                    sz_sequence_u64tape_t const *second, std::int64_t *results,
                                    char const **error_message) {
    auto fail = [&](sz_status_t status, char const *message) {
        if (error_message) *error_message = message;
        return status;
    };
    if (first->count != second->count) return fail(sz_unexpected_dimensions_k, "Pairwise inputs must hold the same count");
    if (first->count == 0) return fail(sz_success_k, nullptr);
    if (first->count > 0xFFFFFFFFull) return fail(sz_overflow_risk_k, "More than 2^32 pairs in one call");
    if (!on_device(first->offsets, call.device) || !on_device(second->offsets, call.device) ||
        !on_device(results, call.device) || !on_device(first->data, call.device) ||
        !on_device(second->data, call.device))
        return fail(sz_device_memory_mismatch_k,
                    "The allocation-free entry point needs tapes and results in the scope device's memory "
                    "(or managed memory), with non-null data pointers");
    current_device_guard_t const device_guard;
    cudaError_t status = cudaSetDevice(call.device);
    unsigned char *scratch = nullptr;
    if (status == cudaSuccess) status = static_scratch_pointer(call.device, scratch);
    if (status == cudaSuccess) status = cudaMemsetAsync(scratch, 0, static_scratch_control_bytes_k, call.stream);
    if (status != cudaSuccess) return fail(sz_status_unknown_k, cudaGetErrorName(status));

    tape_t a, b;
    a.base = reinterpret_cast<std::uint8_t const *>(first->data), a.offsets = first->offsets;
    a.count = first->count, a.offset_bits = 64;
    b.base = reinterpret_cast<std::uint8_t const *>(second->data), b.offsets = second->offsets;
    b.count = second->count, b.offset_bits = 64;
    int const steps = call.costs->affine ? 3 : 1;
    int const ctas = static_scratch_warps_k / (static_scratch_threads_k / 32);
    switch (call.kind * 2 + (call.costs->affine ? 1 : 0)) {
    case 0: status = launch_static<kind_levenshtein_k, false>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    case 1: status = launch_static<kind_levenshtein_k, true>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    case 2: status = launch_static<kind_needleman_wunsch_k, false>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    case 3: status = launch_static<kind_needleman_wunsch_k, true>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    case 4: status = launch_static<kind_smith_waterman_k, false>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    case 5: status = launch_static<kind_smith_waterman_k, true>(a, b, first->count, *call.costs, steps, call.magnitude, results, scratch, ctas, call.stream); break;
    default: status = cudaErrorInvalidValue; break;
    }
    static_scratch_control_t control {0};
    if (status == cudaSuccess)
        status = cudaMemcpyAsync(&control, scratch, sizeof(control), cudaMemcpyDeviceToHost, call.stream);
    if (status == cudaSuccess) status = cudaStreamSynchronize(call.stream);
    if (status != cudaSuccess) return fail(sz_status_unknown_k, cudaGetErrorName(status));
    if (control.errors & static_scratch_too_wide_k)
        return fail(sz_overflow_risk_k, "A pair's scores may overflow the 32-bit cells of the allocation-free kernel");
    if (control.errors & static_scratch_too_long_k)
        return fail(sz_overflow_risk_k, "A pair longer than 256 bytes on both sides has a side of 2,048 bytes or "
                                        "more, beyond the allocation-free kernel's fixed scratch rows");
    return fail(sz_success_k, nullptr);
}

} // namespace szs_gb300
