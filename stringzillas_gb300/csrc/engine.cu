/**
 *  @file engine.cu
 *  @brief Host orchestration of the GB300 scoring engine and its `szs_*` C-ABI.
 *
 *  One call = stage inputs that are not device-resident -> plan on the device (planner.cu) -> read the bin
 *  counts back -> launch one persistent kernel per non-empty route -> scatter results into the caller's matrix.
 *  The reference's equivalent orchestration is `cuda_weighted_cross_` / the Levenshtein cross driver
 *  (include/stringzillas/similarities/cuda.cuh:5395-5505, :3806-3936) behind the shims in
 *  c/stringzillas/{levenshtein,needleman_wunsch,smith_waterman}.cuh.
 */
#include "stringzillas_gb300.h"
#include "launchers.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

namespace szs_gb300 {

constexpr std::uint32_t engine_magic_k = 0x53475a45u; // "EZGS"
constexpr std::uint32_t scope_magic_k = 0x50435353u;
constexpr int max_devices_k = 64;

/* ---- errors --------------------------------------------------------------------------------------------------- */

struct status_t {
    sz_status_t code = sz_success_k;
    char const *message = nullptr;
    bool ok() const noexcept { return code == sz_success_k; }
};

static status_t from_cuda(cudaError_t error) noexcept {
    if (error == cudaSuccess) return {};
    if (error == cudaErrorMemoryAllocation) return {sz_bad_alloc_k, cudaGetErrorName(error)};
    if (error == cudaErrorNoDevice || error == cudaErrorInsufficientDriver || error == cudaErrorInvalidDevice)
        return {sz_missing_gpu_k, cudaGetErrorName(error)};
    return {sz_status_unknown_k, cudaGetErrorName(error)};
}

static sz_status_t report(status_t status, char const **error_message) noexcept {
    if (error_message) {
        if (status.ok()) *error_message = nullptr;
        else if (status.message) *error_message = status.message;
        else {
            switch (status.code) {
            case sz_bad_alloc_k: *error_message = "Memory allocation failed"; break;
            case sz_overflow_risk_k: *error_message = "Overflow risk detected"; break;
            case sz_unexpected_dimensions_k: *error_message = "Input/output size mismatch"; break;
            case sz_missing_gpu_k: *error_message = "GPU device not available or CUDA not initialized"; break;
            case sz_device_code_mismatch_k: *error_message = "Backend and executor mismatch"; break;
            case sz_device_memory_mismatch_k: *error_message = "Use device-reachable or unified memory"; break;
            default: *error_message = "Unknown error"; break;
            }
        }
    }
    return status.code;
}

#define SZS_TRY_CUDA(expression)                                                                                     \
    do {                                                                                                             \
        cudaError_t const szs_error_ = (expression);                                                                 \
        if (szs_error_ != cudaSuccess) return from_cuda(szs_error_);                                                 \
    } while (0)

/* ---- scopes --------------------------------------------------------------------------------------------------- */

enum scope_kind_t { scope_default_k, scope_cpu_k, scope_gpu_k };

struct scope_t {
    std::uint32_t magic = scope_magic_k;
    scope_kind_t kind = scope_default_k;
    std::size_t cpu_cores = 1;
    int device = 0;
    cudaStream_t stream = nullptr; // GPU scopes own a non-blocking stream, or borrow the caller's
    bool borrowed_stream = false;
};

static scope_t *as_scope(void *handle) noexcept {
    auto *scope = static_cast<scope_t *>(handle);
    return scope && scope->magic == scope_magic_k ? scope : nullptr;
}

static int visible_devices() noexcept {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count;
}

/* ---- device memory ---------------------------------------------------------------------------------------------- */

/** A grow-only device buffer, reused across calls. */
struct device_buffer_t {
    void *data = nullptr;
    std::size_t bytes = 0;
    status_t reserve(std::size_t needed, cudaStream_t stream) noexcept {
        if (needed <= bytes) return {};
        if (data) {
            cudaStreamSynchronize(stream);
            cudaFree(data);
            data = nullptr, bytes = 0;
        }
        std::size_t const grown = std::max(needed, std::size_t(1) << 20);
        SZS_TRY_CUDA(cudaMalloc(&data, grown));
        bytes = grown;
        return {};
    }
    void release() noexcept {
        if (data) cudaFree(data);
        data = nullptr, bytes = 0;
    }
};

/** A grow-only pinned host buffer. */
struct pinned_buffer_t {
    void *data = nullptr;
    std::size_t bytes = 0;
    status_t reserve(std::size_t needed) noexcept {
        if (needed <= bytes) return {};
        if (data) cudaFreeHost(data);
        data = nullptr, bytes = 0;
        SZS_TRY_CUDA(cudaMallocHost(&data, needed));
        bytes = needed;
        return {};
    }
    void release() noexcept {
        if (data) cudaFreeHost(data);
        data = nullptr, bytes = 0;
    }
};

static bool device_accessible(void const *pointer) noexcept {
    if (!pointer) return false;
    cudaPointerAttributes attributes;
    if (cudaPointerGetAttributes(&attributes, pointer) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attributes.type == cudaMemoryTypeDevice || attributes.type == cudaMemoryTypeManaged;
}

/**
 *  Instantiated CUDA graphs of earlier calls, keyed by every byte their launches depend on (kernel arguments,
 *  buffer addresses, grid sizes). A call whose key matches replays the graph instead of issuing its launches.
 */
struct graph_cache_t {
    static constexpr int capacity_k = 32;
    struct entry_t {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec = nullptr;
        std::uint64_t used = 0;
    };
    entry_t entries[capacity_k];
    std::uint64_t clock = 0;

    cudaGraphExec_t find(std::vector<unsigned char> const &key) noexcept {
        for (auto &entry : entries)
            if (entry.exec && entry.key == key) {
                entry.used = ++clock;
                return entry.exec;
            }
        return nullptr;
    }
    void insert(std::vector<unsigned char> key, cudaGraphExec_t exec) noexcept {
        entry_t *victim = &entries[0];
        for (auto &entry : entries)
            if (!entry.exec || entry.used < victim->used) victim = &entry;
        if (victim->exec) cudaGraphExecDestroy(victim->exec);
        victim->key = std::move(key);
        victim->exec = exec;
        victim->used = ++clock;
    }
    void release() noexcept {
        for (auto &entry : entries) {
            if (entry.exec) cudaGraphExecDestroy(entry.exec);
            entry.exec = nullptr;
            entry.key.clear();
        }
    }
};

/** Appends the object representation of @p value to a graph key. */
template <typename value_type_>
static void key_append(std::vector<unsigned char> &key, value_type_ const &value) {
    auto const *bytes = reinterpret_cast<unsigned char const *>(&value);
    key.insert(key.end(), bytes, bytes + sizeof(value_type_));
}

/** Per-device state of an engine: its stream for the default scope, buffers, plan readback, timers. */
struct device_context_t {
    bool ready = false;
    int device = -1;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    device_buffer_t control; // plan bins + alphabet
    device_buffer_t inputs;  // staged tapes
    device_buffer_t work;    // tasks + dense results
    device_buffer_t scratch; // wavefront scratch rows
    pinned_buffer_t readback;
    pinned_buffer_t results_host;
    cudaEvent_t start = nullptr, stop = nullptr;
    cudaEvent_t compute_start = nullptr, compute_stop = nullptr;
    static constexpr int lanes_k = 8; // auxiliary streams the routes of one call run on concurrently
    cudaStream_t lanes[lanes_k] = {nullptr};
    cudaEvent_t fork = nullptr;
    cudaEvent_t joins[lanes_k] = {nullptr};
    cudaEvent_t trace_events[64] = {nullptr};
    graph_cache_t prologue_graphs; // alphabet + plan + plan readback
    graph_cache_t launch_graphs;   // the scoring kernels of a plan
    // Pipelined host-input calls: every chunk's copy is queued on `copy_stream` up front, into its own slot of
    // `chunk_inputs`; chunk c is scored as soon as its copy has landed, while the later copies continue.
    static constexpr int max_chunks_k = 64;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copied[max_chunks_k] = {nullptr};
    cudaEvent_t pipe_start = nullptr, pipe_stop = nullptr, offsets_copied = nullptr;
    device_buffer_t chunk_inputs;
    static constexpr int pipeline_depth_k = 12; // chunks of a pipelined call in flight at once
    device_context_t *partners[pipeline_depth_k] = {nullptr}; // the contexts a pipelined call's chunks rotate over
    device_buffer_t utf8;                // UTF-8 calls: code-point set, counts, offsets and transcoded tapes
    device_buffer_t dense_table;         // the 256 x 256 table of the dense engine last run here over > 32 bytes
    std::uint64_t dense_table_id = 0;    // that engine's `dense_id` (0: none)
    bool deferred = false, deferred_compute = false;
    std::uint64_t deferred_launches = 0;
    int traced_jobs = 0;             // under SZS_GB300_TRACE: the deferred call's jobs, for the chunk timeline
    int traced_kind[32] = {0}, traced_variant[32] = {0};
    std::uint64_t traced_pairs[32] = {0};

    /** @p urgent: the context's own stream takes the device's highest priority (the contexts of pipelined chunks,
     *  whose planning kernels should start as soon as their chunk lands, ahead of queued scoring work). */
    status_t prepare(int device_index, bool urgent = false) noexcept {
        if (ready) return {};
        device = device_index;
        SZS_TRY_CUDA(cudaSetDevice(device));
        SZS_TRY_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
        int least = 0, greatest = 0;
        SZS_TRY_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SZS_TRY_CUDA(cudaStreamCreateWithPriority(&own_stream, cudaStreamNonBlocking, urgent ? greatest : least));
        SZS_TRY_CUDA(cudaEventCreate(&start));
        SZS_TRY_CUDA(cudaEventCreate(&stop));
        SZS_TRY_CUDA(cudaEventCreate(&compute_start));
        SZS_TRY_CUDA(cudaEventCreate(&compute_stop));
        for (auto &event : trace_events) SZS_TRY_CUDA(cudaEventCreate(&event));
        SZS_TRY_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        SZS_TRY_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
        // Timed only under SZS_GB300_TRACE or SZS_GB300_TRACE_CHUNKS, which print each pipelined chunk's timeline.
        unsigned const copied_flags = std::getenv("SZS_GB300_TRACE") || std::getenv("SZS_GB300_TRACE_CHUNKS")
                                          ? cudaEventDefault
                                          : cudaEventDisableTiming;
        for (auto &event : copied) SZS_TRY_CUDA(cudaEventCreateWithFlags(&event, copied_flags));
        SZS_TRY_CUDA(cudaEventCreate(&pipe_start));
        SZS_TRY_CUDA(cudaEventCreate(&pipe_stop));
        SZS_TRY_CUDA(cudaEventCreateWithFlags(&offsets_copied, cudaEventDisableTiming));
        for (int i = 0; i < lanes_k; ++i) {
            SZS_TRY_CUDA(cudaStreamCreateWithFlags(&lanes[i], cudaStreamNonBlocking));
            SZS_TRY_CUDA(cudaEventCreateWithFlags(&joins[i], cudaEventDisableTiming));
        }
        status_t status = control.reserve(sizeof(plan_bins_t) + sizeof(batch_alphabet_t) + 256, own_stream);
        if (!status.ok()) return status;
        // The alphabet's mark words must start at zero (each alphabet pass clears them again).
        SZS_TRY_CUDA(cudaMemsetAsync(control.data, 0, control.bytes, own_stream));
        SZS_TRY_CUDA(cudaStreamSynchronize(own_stream));
        status = readback.reserve(sizeof(plan_bins_t) + sizeof(batch_alphabet_t) + 256);
        if (!status.ok()) return status;
        ready = true;
        return {};
    }
    plan_bins_t *bins_device() const noexcept { return static_cast<plan_bins_t *>(control.data); }
    batch_alphabet_t *alphabet_device() const noexcept {
        return reinterpret_cast<batch_alphabet_t *>(static_cast<unsigned char *>(control.data) + sizeof(plan_bins_t));
    }
    plan_bins_t *bins_host() const noexcept { return static_cast<plan_bins_t *>(readback.data); }
    batch_alphabet_t *alphabet_host() const noexcept {
        return reinterpret_cast<batch_alphabet_t *>(static_cast<unsigned char *>(readback.data) + sizeof(plan_bins_t));
    }
    /** 256 spare bytes after the plan and the alphabet, on the device and in the pinned readback area. */
    std::uint32_t *spare_device() const noexcept {
        return reinterpret_cast<std::uint32_t *>(static_cast<unsigned char *>(control.data) + sizeof(plan_bins_t) +
                                                 sizeof(batch_alphabet_t));
    }
    std::uint64_t *spare_host() const noexcept {
        return reinterpret_cast<std::uint64_t *>(static_cast<unsigned char *>(readback.data) + sizeof(plan_bins_t) +
                                                 sizeof(batch_alphabet_t));
    }
    void release() noexcept {
        if (!ready) return;
        cudaSetDevice(device);
        cudaStreamSynchronize(own_stream);
        prologue_graphs.release(), launch_graphs.release();
        if (copy_stream) cudaStreamSynchronize(copy_stream), cudaStreamDestroy(copy_stream);
        for (auto &event : copied)
            if (event) cudaEventDestroy(event);
        if (pipe_start) cudaEventDestroy(pipe_start);
        if (pipe_stop) cudaEventDestroy(pipe_stop);
        if (offsets_copied) cudaEventDestroy(offsets_copied);
        chunk_inputs.release();
        utf8.release();
        dense_table.release(), dense_table_id = 0;
        for (auto &partner : partners)
            if (partner) {
                partner->release();
                delete partner;
                partner = nullptr;
            }
        control.release(), inputs.release(), work.release(), scratch.release();
        readback.release(), results_host.release();
        if (start) cudaEventDestroy(start);
        if (stop) cudaEventDestroy(stop);
        for (auto &event : trace_events)
            if (event) cudaEventDestroy(event);
        for (int i = 0; i < lanes_k; ++i) {
            if (lanes[i]) cudaStreamSynchronize(lanes[i]), cudaStreamDestroy(lanes[i]);
            if (joins[i]) cudaEventDestroy(joins[i]);
        }
        if (fork) cudaEventDestroy(fork);
        if (compute_start) cudaEventDestroy(compute_start);
        if (compute_stop) cudaEventDestroy(compute_stop);
        if (own_stream) cudaStreamDestroy(own_stream);
        ready = false;
    }
};

/* ---- engines ---------------------------------------------------------------------------------------------------- */

struct static_call_t {
    score_costs_t const *costs;
    int kind;
    int magnitude;
    int device;
    cudaStream_t stream;
};
sz_status_t static_scratch_pairwise(static_call_t const &call, sz_sequence_u64tape_t const *first,
                                    sz_sequence_u64tape_t const *second, std::int64_t *results,
                                    char const **error_message);

struct engine_t {
    std::uint32_t magic = engine_magic_k;
    int kind = kind_levenshtein_k;
    int schedule = szs_gb300_schedule_batched_k;
    score_costs_t costs {};
    int magnitude = 1;
    bool unit_levenshtein = false;
    bool packed_profile_fits = false; // every substitution cost (minus `open` for affine gaps) fits a signed byte
    szs_gb300_tuning_t tuning {};     // zeros: built-in choices
    int local_gain = -1;              // local scores with non-positive gaps: largest substitution gain (>= 0)
    std::vector<std::int8_t> dense;   // 256 x 256 [first byte][second byte] table of a dense engine, else empty
    std::uint64_t dense_id = 0;       // unique per dense engine: device contexts cache its uploaded table by it
    bool utf8 = false;                // Levenshtein over UTF-8 code points (transcoded to one-byte codes per call)
    device_context_t devices[max_devices_k];
    szs_gb300_stats_t stats {};
    ~engine_t() {
        for (auto &context : devices) context.release();
    }
};

static engine_t *as_engine(void *handle, int kind) noexcept {
    auto *engine = static_cast<engine_t *>(handle);
    if (!engine || engine->magic != engine_magic_k) return nullptr;
    if (kind >= 0 && engine->kind != kind) return nullptr;
    return engine;
}

static int cost_abs(int x) noexcept { return x < 0 ? -x : x; }

// Per plane count, built from kernels_myers.cu once per count: (words, exact, tasks, bins, key_begin, key_end,
// alphabet, results, ctas, stream), and the warp forms without `exact`.
#define SZS_DECLARE_MYERS_PLANES(planes)                                                                            \
    cudaError_t launch_myers_planes##planes(int, bool, pair_task_t const *, plan_bins_t const *, int, int,           \
                                            batch_alphabet_t const *, std::int64_t *, int, cudaStream_t);           \
    cudaError_t launch_myers_warp_planes##planes(int, pair_task_t const *, plan_bins_t *, int, int,                 \
                                                 batch_alphabet_t const *, std::int64_t *, int, cudaStream_t);
SZS_DECLARE_MYERS_PLANES(2)
SZS_DECLARE_MYERS_PLANES(3)
SZS_DECLARE_MYERS_PLANES(5)
SZS_DECLARE_MYERS_PLANES(8)
#undef SZS_DECLARE_MYERS_PLANES

int myers_planes_for(int bits_needed) {
    if (bits_needed <= 2) return 2;
    if (bits_needed <= 3) return 3;
    if (bits_needed <= 5) return 5;
    return 8;
}

int myers_threads_per_cta() { return 128; }

/** Warp-per-pair bit-parallel kernel over bins [key_begin, key_end) with `words` words per lane. */
static cudaError_t launch_myers_warp(int words, int planes, pair_task_t const *tasks, plan_bins_t *bins,
                                     int key_begin, int key_end, batch_alphabet_t const *alphabet,
                                     std::int64_t *results, int ctas, cudaStream_t stream) {
    switch (planes) {
    case 2: return launch_myers_warp_planes2(words, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 3: return launch_myers_warp_planes3(words, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 5: return launch_myers_warp_planes5(words, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 8: return launch_myers_warp_planes8(words, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_myers(int words, int planes, bool exact, pair_task_t const *tasks, plan_bins_t const *bins,
                         int key_begin, int key_end, batch_alphabet_t const *alphabet, std::int64_t *results, int ctas,
                         cudaStream_t stream) {
    switch (planes) {
    case 2: return launch_myers_planes2(words, exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 3: return launch_myers_planes3(words, exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 5: return launch_myers_planes5(words, exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    case 8: return launch_myers_planes8(words, exact, tasks, bins, key_begin, key_end, alphabet, results, ctas, stream);
    default: return cudaErrorInvalidValue;
    }
}

/** Builds the compact column classes and both orientations of the profile table from the reference's inputs. */
static void prepare_class_costs(score_costs_t &costs, std::uint8_t const *byte_to_class, std::int8_t const *table) {
    std::memcpy(costs.byte_to_class, byte_to_class, 256);
    int compact_of_class[32];
    for (int &c : compact_of_class) c = -1;
    int classes = 0;
    int class_of_compact[32];
    for (int b = 0; b < 256; ++b) {
        int const cls = byte_to_class[b] & 31; // the reference indexes a 32x32 table with the raw value
        if (compact_of_class[cls] < 0) class_of_compact[classes] = cls, compact_of_class[cls] = classes++;
        costs.byte_to_compact[b] = (std::uint8_t)compact_of_class[cls];
    }
    costs.classes = classes;
    std::memset(costs.profile_table, 0, sizeof(costs.profile_table));
    std::memset(costs.profile_table_t, 0, sizeof(costs.profile_table_t));
    for (int cc = 0; cc < classes; ++cc)
        for (int row_class = 0; row_class < 32; ++row_class) {
            int const column_class = class_of_compact[cc];
            // rows = first string: cost(first = row, second = column)
            costs.profile_table[cc * 32 + row_class] = table[row_class * 32 + column_class];
            // rows = second string: cost(first = column, second = row)
            costs.profile_table_t[cc * 32 + row_class] = table[column_class * 32 + row_class];
        }
}

/**
 *  Whether the 16x2 packed route can hold this engine's substitution costs in its int8 profiles: the costs as they
 *  are for linear gaps, `cost - open` for affine gaps (the packed affine tracks carry H + open). Only classes that
 *  some byte maps to are checked; Levenshtein engines check their match and mismatch costs.
 */
static bool packed_profile_fits(score_costs_t const &costs) {
    int const shift = costs.affine ? costs.open : 0;
    auto fits = [&](int cost) { return cost - shift >= -128 && cost - shift <= 127; };
    if (costs.kind == kind_levenshtein_k) return fits(costs.match) && fits(costs.mismatch);
    bool used[32] = {};
    for (int b = 0; b < 256; ++b) used[costs.byte_to_class[b] & 31] = true;
    for (int cc = 0; cc < costs.classes; ++cc)
        for (int row_class = 0; row_class < 32; ++row_class)
            if (used[row_class] &&
                (!fits(costs.profile_table[cc * 32 + row_class]) || !fits(costs.profile_table_t[cc * 32 + row_class])))
                return false;
    return true;
}

/* ---- inputs ----------------------------------------------------------------------------------------------------- */

/** A caller's tape in any memory, before staging. */
struct tape_view_t {
    char const *data = nullptr;
    void const *offsets = nullptr;
    std::size_t count = 0;
    int offset_bits = 64;
};

/** Owns host-side copies made for `sz_sequence_t` inputs (callbacks are host functions). */
struct gathered_tape_t {
    std::vector<char> data;
    std::vector<std::uint64_t> offsets;
    tape_view_t view() const noexcept {
        tape_view_t v;
        v.data = data.empty() ? nullptr : data.data();
        v.offsets = offsets.data();
        v.count = offsets.empty() ? 0 : offsets.size() - 1;
        v.offset_bits = 64;
        return v;
    }
};

static status_t gather_sequence(sz_sequence_t const *sequence, gathered_tape_t &out) noexcept {
    try {
        out.offsets.assign(1, 0);
        out.offsets.reserve(sequence->count + 1);
        for (sz_size_t i = 0; i < sequence->count; ++i) {
            sz_cptr_t const start = sequence->get_start(sequence->handle, i);
            sz_size_t const length = sequence->get_length(sequence->handle, i);
            out.data.insert(out.data.end(), start, start + length);
            out.offsets.push_back(out.data.size());
        }
    }
    catch (std::bad_alloc const &) {
        return {sz_bad_alloc_k, nullptr};
    }
    return {};
}

static std::uint64_t host_offset(tape_view_t const &tape, std::size_t index) noexcept {
    return tape.offset_bits == 32 ? static_cast<std::uint32_t const *>(tape.offsets)[index]
                                  : static_cast<std::uint64_t const *>(tape.offsets)[index];
}

/** Bytes of device memory staging @p tape needs (0 when fully device-resident). */
struct staging_plan_t {
    bool offsets_on_device = false, data_on_device = false;
    std::uint64_t first = 0, last = 0; // data range [first, last)
    std::size_t offsets_bytes = 0, data_bytes = 0;
};

static status_t plan_staging(tape_view_t const &tape, staging_plan_t &plan, cudaStream_t stream) noexcept {
    plan.offsets_on_device = device_accessible(tape.offsets);
    plan.data_on_device = tape.data == nullptr || device_accessible(tape.data);
    std::size_t const offset_size = tape.offset_bits == 32 ? 4 : 8;
    plan.offsets_bytes = plan.offsets_on_device ? 0 : (tape.count + 1) * offset_size;
    if (plan.offsets_on_device) {
        if (!plan.data_on_device) {
            // Read the data range from device-resident offsets.
            std::uint64_t ends[2] = {0, 0};
            if (tape.offset_bits == 32) {
                std::uint32_t e32[2];
                SZS_TRY_CUDA(cudaMemcpyAsync(&e32[0], tape.offsets, 4, cudaMemcpyDeviceToHost, stream));
                SZS_TRY_CUDA(cudaMemcpyAsync(&e32[1], static_cast<std::uint32_t const *>(tape.offsets) + tape.count,
                                             4, cudaMemcpyDeviceToHost, stream));
                SZS_TRY_CUDA(cudaStreamSynchronize(stream));
                ends[0] = e32[0], ends[1] = e32[1];
            }
            else {
                SZS_TRY_CUDA(cudaMemcpyAsync(&ends[0], tape.offsets, 8, cudaMemcpyDeviceToHost, stream));
                SZS_TRY_CUDA(cudaMemcpyAsync(&ends[1], static_cast<std::uint64_t const *>(tape.offsets) + tape.count,
                                             8, cudaMemcpyDeviceToHost, stream));
                SZS_TRY_CUDA(cudaStreamSynchronize(stream));
            }
            plan.first = ends[0], plan.last = ends[1];
        }
    }
    else {
        plan.first = host_offset(tape, 0), plan.last = host_offset(tape, tape.count);
    }
    if (plan.last < plan.first) return {sz_unexpected_dimensions_k, "Tape offsets must be non-decreasing"};
    plan.data_bytes = plan.data_on_device ? 0 : (std::size_t)(plan.last - plan.first);
    return {};
}

static std::size_t align_up(std::size_t x, std::size_t a) noexcept { return (x + a - 1) / a * a; }

/** Copies what is not device-resident into @p area (which has at least the planned bytes) and describes the
 *  result for the kernels. */
static status_t stage_tape(tape_view_t const &tape, staging_plan_t const &plan, unsigned char *area,
                           tape_t &staged, cudaStream_t stream) noexcept {
    staged.count = tape.count;
    staged.offset_bits = tape.offset_bits;
    unsigned char *cursor = area;
    if (plan.offsets_on_device) staged.offsets = tape.offsets;
    else {
        SZS_TRY_CUDA(cudaMemcpyAsync(cursor, tape.offsets, plan.offsets_bytes, cudaMemcpyHostToDevice, stream));
        staged.offsets = cursor;
        cursor += align_up(plan.offsets_bytes, 256);
    }
    if (plan.data_on_device) staged.base = reinterpret_cast<std::uint8_t const *>(tape.data);
    else {
        if (plan.data_bytes)
            SZS_TRY_CUDA(cudaMemcpyAsync(cursor, tape.data + plan.first, plan.data_bytes, cudaMemcpyHostToDevice,
                                         stream));
        // Kernels address `base + offsets[i]`; the staged copy starts at offsets[0].
        staged.base = reinterpret_cast<std::uint8_t const *>(cursor) - plan.first;
    }
    return {};
}

/* ---- one call ----------------------------------------------------------------------------------------------------- */

struct call_t {
    tape_view_t queries;
    tape_view_t candidates;
    bool has_candidates = false;
    int mode = mode_cross_k;
    std::int64_t *out = nullptr;
    std::size_t stride = 0;
    bool pre_staged = false;           // the tapes below are already on the device (a chunk of a pipelined call)
    tape_t staged_queries {}, staged_candidates {};
    bool exact_alphabet = false;       // mark every byte of the batch, no sampled guess
    // Pipelined chunks: planning waits for `plan_after` (the offsets, or the chunk's bytes when the plan reads
    // them), scoring for `scoring_after` (the chunk's bytes); a sampled alphabet comes from `sample_*` (the first
    // chunk's tapes, on the device before the later chunks), so the plan of a chunk can run before its bytes land.
    cudaEvent_t plan_after = nullptr, scoring_after = nullptr;
    tape_t const *sample_queries = nullptr, *sample_candidates = nullptr;
    // Two phases on one context: `plan_only` returns once the plan is read back and kept in the context; a later
    // call with `reuse_plan` (same tapes and costs) scores that plan without planning again.
    bool plan_only = false, reuse_plan = false;
};

static status_t resolve_scope(void *scope_handle, int &device, cudaStream_t &stream, device_context_t *contexts,
                              device_context_t *&context) noexcept {
    scope_t *scope = as_scope(scope_handle);
    if (scope_handle && !scope) return {sz_status_unknown_k, "Invalid device scope handle"};
    if (scope && scope->kind == scope_cpu_k) return {sz_device_code_mismatch_k, nullptr};
    device = scope ? scope->device : 0;
    if (device < 0 || device >= max_devices_k || device >= visible_devices()) return {sz_missing_gpu_k, nullptr};
    context = &contexts[device];
    status_t status = context->prepare(device);
    if (!status.ok()) return status;
    SZS_TRY_CUDA(cudaSetDevice(device));
    stream = scope && scope->kind == scope_gpu_k ? scope->stream : context->own_stream;
    return {};
}

/**
 *  One call on an explicit device context and stream. The engine is only read (costs, kind, schedule), so several
 *  contexts may run calls of the same engine at once; @p stats receives the call's timings and counters.
 */
static status_t finish_deferred(device_context_t *context, szs_gb300_stats_t &stats) noexcept;

/**
 *  UTF-8 Levenshtein: rewrites both device-resident tapes as codes of their code points (see utf8.cu), in place of
 *  @p queries and @p candidates: one byte each for up to 256 distinct code points, else 16 bits each (@p wide). A
 *  call may use at most 65,536 distinct code points.
 */
static status_t transcode_utf8(device_context_t *context, cudaStream_t stream, tape_t &queries, tape_t &candidates,
                               bool has_candidates, bool &wide) noexcept {
    tape_t *tapes[2] = {&queries, has_candidates ? &candidates : nullptr};
    std::uint64_t first[2] = {0, 0}, end[2] = {0, 0};
    // The tapes' extents: the transcoded data can hold no more runes than bytes.
    for (int t = 0; t < 2; ++t) {
        if (!tapes[t]) continue;
        std::size_t const size = tapes[t]->offset_bits == 32 ? 4 : 8;
        auto const *offsets = static_cast<unsigned char const *>(tapes[t]->offsets);
        SZS_TRY_CUDA(cudaMemcpyAsync(&first[t], offsets, size, cudaMemcpyDeviceToHost, stream));
        SZS_TRY_CUDA(cudaMemcpyAsync(&end[t], offsets + tapes[t]->count * size, size, cudaMemcpyDeviceToHost, stream));
    }
    SZS_TRY_CUDA(cudaStreamSynchronize(stream));
    std::size_t layout[2][3] = {}; // counts, offsets, data
    std::size_t cursor = align_up(sizeof(rune_set_t), 256);
    std::size_t scan_bytes = 0;
    for (int t = 0; t < 2; ++t) {
        if (!tapes[t]) continue;
        std::uint64_t const count = tapes[t]->count;
        layout[t][0] = cursor, cursor += align_up((count + 1) * 8, 256);
        layout[t][1] = cursor, cursor += align_up((count + 1) * 8, 256);
        // Room for two bytes per code (more than 256 code points) and a whole 8-byte chunk past the end.
        layout[t][2] = cursor, cursor += align_up(2 * (end[t] - first[t]) + 8, 256);
        scan_bytes = std::max(scan_bytes, utf8_scan_scratch_bytes(count));
    }
    std::size_t const scan_at = cursor;
    status_t status = context->utf8.reserve(cursor + align_up(scan_bytes, 256), stream);
    if (!status.ok()) return status;
    auto *area = static_cast<unsigned char *>(context->utf8.data);
    auto *set = reinterpret_cast<rune_set_t *>(area);
    SZS_TRY_CUDA(cudaMemsetAsync(set, 0, sizeof(rune_set_t), stream));
    for (int t = 0; t < 2; ++t) {
        if (!tapes[t]) continue;
        auto *counts = reinterpret_cast<std::uint64_t *>(area + layout[t][0]);
        SZS_TRY_CUDA(cudaMemsetAsync(counts, 0, (tapes[t]->count + 1) * 8, stream));
        SZS_TRY_CUDA(launch_utf8_count(*tapes[t], end[t], counts, set, context->sm_count, stream));
    }
    SZS_TRY_CUDA(launch_utf8_codes(set, stream));
    std::uint32_t seen[2] = {0, 0}; // symbols, overflow
    SZS_TRY_CUDA(cudaMemcpyAsync(seen, &set->symbols, sizeof(seen), cudaMemcpyDeviceToHost, stream));
    SZS_TRY_CUDA(cudaStreamSynchronize(stream));
    if (seen[1] || seen[0] > 65536)
        return {sz_unexpected_dimensions_k, "A UTF-8 call may use at most 65,536 distinct code points"};
    wide = seen[0] > 256; // 16-bit codes beyond 256 code points
    for (int t = 0; t < 2; ++t) {
        if (!tapes[t]) continue;
        auto const *counts = reinterpret_cast<std::uint64_t const *>(area + layout[t][0]);
        auto *offsets = reinterpret_cast<std::uint64_t *>(area + layout[t][1]);
        auto *data = reinterpret_cast<std::uint8_t *>(area + layout[t][2]);
        SZS_TRY_CUDA(launch_utf8_scan(counts, offsets, tapes[t]->count, area + scan_at, scan_bytes, stream));
        SZS_TRY_CUDA(launch_utf8_write(*tapes[t], end[t], offsets, set, data, wide, context->sm_count, stream));
        tapes[t]->base = data;
        tapes[t]->offsets = offsets;
        tapes[t]->offset_bits = 64;
    }
    if (!has_candidates) candidates = queries;
    return {};
}

/**
 *  @param defer  pairwise calls with host results only: return once the work is queued, without waiting for it;
 *                `finish_deferred` later waits and fills @p stats (the pipelined driver keeps two chunks in flight).
 */
constexpr std::uint64_t alphabet_sample_bytes_k = std::uint64_t(1) << 20; // bytes per tape of a guessed alphabet

static status_t run_on(engine_t const &engine, device_context_t *context, cudaStream_t stream, call_t const &call,
                       int schedule, szs_gb300_stats_t &stats, bool defer = false) noexcept {
    status_t status;
    std::uint64_t const queries_count = call.queries.count;
    std::uint64_t const candidates_count = call.has_candidates ? call.candidates.count : queries_count;
    plan_args_t args;
    std::memset(&args, 0, sizeof(args)); // graph keys compare its bytes, padding included
    args.mode = call.mode;
    if (call.mode == mode_pairwise_k) {
        if (call.candidates.count != call.queries.count) return {sz_unexpected_dimensions_k, nullptr};
        args.pairs = queries_count;
    }
    else if (call.mode == mode_cross_k) args.pairs = queries_count * candidates_count;
    else args.pairs = queries_count * (queries_count + 1) / 2;
    args.candidates_count = candidates_count;
    stats.last_pairs = args.pairs;
    stats.last_cells = 0;
    stats.last_launches = 0;
    stats.last_call_ms = 0;
    stats.last_compute_ms = 0;
    if (args.pairs == 0) return {};
    if (args.pairs > 0xFFFFFFFFull) return {sz_overflow_risk_k, "More than 2^32 pairs in one call"};

    // Stage inputs.
    staging_plan_t query_plan, candidate_plan;
    if (call.pre_staged) {
        query_plan.offsets_on_device = query_plan.data_on_device = true;
        candidate_plan.offsets_on_device = candidate_plan.data_on_device = true;
    }
    else {
        status = plan_staging(call.queries, query_plan, stream);
        if (!status.ok()) return status;
        if (call.has_candidates) {
            status = plan_staging(call.candidates, candidate_plan, stream);
            if (!status.ok()) return status;
        }
    }
    std::size_t const query_area = align_up(query_plan.offsets_bytes, 256) + align_up(query_plan.data_bytes, 256);
    std::size_t const candidate_area =
        call.has_candidates ? align_up(candidate_plan.offsets_bytes, 256) + align_up(candidate_plan.data_bytes, 256)
                            : 0;
    if (call.pre_staged) {
        args.queries = call.staged_queries;
        args.candidates = call.has_candidates ? call.staged_candidates : call.staged_queries;
    }
    else {
        status = context->inputs.reserve(query_area + candidate_area + 512, stream);
        if (!status.ok()) return status;
        unsigned char *inputs_area = static_cast<unsigned char *>(context->inputs.data);
        status = stage_tape(call.queries, query_plan, inputs_area, args.queries, stream);
        if (!status.ok()) return status;
        if (call.has_candidates) {
            status = stage_tape(call.candidates, candidate_plan, inputs_area + query_area, args.candidates, stream);
            if (!status.ok()) return status;
        }
        else args.candidates = args.queries;
    }
    bool wide = false; // UTF-8 calls over more than 256 code points: 16-bit codes
    if (engine.utf8) {
        status = transcode_utf8(context, stream, args.queries, args.candidates, call.has_candidates, wide);
        if (!status.ok()) return status;
        args.wide = wide ? 1 : 0;
    }

    // Cross products of short tokens under unit costs, into device-resident results: when both tapes hold at most 64
    // bytes per string on average, one kernel scores every cell in place (one thread per cell, no planning); a
    // string longer than 64 bytes raises its flag, and the general path below scores the call.
    if (engine.unit_levenshtein && !engine.utf8 && call.mode == mode_cross_k && schedule != szs_gb300_schedule_plain_k &&
        !defer && device_accessible(call.out)) {
        std::uint64_t *ends = context->spare_host(); // offsets[0] and offsets[count] of both tapes
        tape_t const *tapes[2] = {&args.queries, &args.candidates};
        for (int k = 0; k < 2; ++k) {
            std::size_t const width = tapes[k]->offset_bits == 32 ? 4 : 8;
            auto const *offsets = static_cast<unsigned char const *>(tapes[k]->offsets);
            ends[2 * k] = ends[2 * k + 1] = 0;
            SZS_TRY_CUDA(cudaMemcpyAsync(&ends[2 * k], offsets, width, cudaMemcpyDefault, stream));
            SZS_TRY_CUDA(cudaMemcpyAsync(&ends[2 * k + 1], offsets + tapes[k]->count * width, width, cudaMemcpyDefault,
                                         stream));
        }
        SZS_TRY_CUDA(cudaStreamSynchronize(stream));
        std::uint64_t const query_bytes = ends[1] - ends[0], candidate_bytes = ends[3] - ends[2];
        if (query_bytes <= 64 * queries_count && candidate_bytes <= 64 * candidates_count) {
            std::uint32_t *flag = context->spare_device();
            SZS_TRY_CUDA(cudaEventRecord(context->start, stream));
            SZS_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(std::uint32_t), stream));
            SZS_TRY_CUDA(cudaEventRecord(context->compute_start, stream));
            SZS_TRY_CUDA(launch_myers_direct(args, call.out, call.stride, flag, context->sm_count, stream));
            SZS_TRY_CUDA(cudaEventRecord(context->compute_stop, stream));
            auto *flag_host = reinterpret_cast<std::uint32_t *>(ends + 4);
            *flag_host = 0;
            SZS_TRY_CUDA(cudaMemcpyAsync(flag_host, flag, sizeof(std::uint32_t), cudaMemcpyDeviceToHost, stream));
            SZS_TRY_CUDA(cudaEventRecord(context->stop, stream));
            SZS_TRY_CUDA(cudaStreamSynchronize(stream));
            if (*flag_host == 0) {
                float elapsed = 0, compute = 0;
                cudaEventElapsedTime(&elapsed, context->start, context->stop);
                cudaEventElapsedTime(&compute, context->compute_start, context->compute_stop);
                stats.last_call_ms = elapsed, stats.last_compute_ms = compute;
                stats.last_cells = query_bytes * candidate_bytes; // sum over cells of n x m
                stats.last_launches = 1;
                stats.kernel_launches += 1;
                return {};
            }
        }
    }

    // Work buffers: tasks, then dense results.
    std::size_t const tasks_bytes = align_up(args.pairs * sizeof(pair_task_t), 256);
    std::size_t const results_bytes = align_up(args.pairs * sizeof(std::int64_t), 256);
    status = context->work.reserve(tasks_bytes + results_bytes, stream);
    if (!status.ok()) return status;
    auto *tasks = static_cast<pair_task_t *>(context->work.data);
    auto *results = reinterpret_cast<std::int64_t *>(static_cast<unsigned char *>(context->work.data) + tasks_bytes);

    score_costs_t const &costs = engine.costs;
    args.kind = engine.kind;
    args.affine = costs.affine;
    args.open = costs.open, args.extend = costs.extend;
    args.match = costs.match, args.mismatch = costs.mismatch;
    args.unit_levenshtein = engine.unit_levenshtein ? 1 : 0;
    args.magnitude = engine.magnitude;
    args.local_gain = engine.local_gain;
    args.steps_beyond_span = costs.affine ? 3 : 1;
    args.force_route = schedule == szs_gb300_schedule_plain_k ? 1 : -1;

    args.packed_allowed = engine.packed_profile_fits ? 1 : 0; // 16-bit codes (Levenshtein): compare mode
    args.dense = engine.dense.empty() ? 0 : 1;
    std::memcpy(args.packed_rows, engine.tuning.packed_rows, 16);
    std::memcpy(args.cell_bits, engine.tuning.cell_bits, 16);
    args.band_min_rows = engine.tuning.band_min_rows ? engine.tuning.band_min_rows : (std::uint32_t)band_min_rows_k;
    args.band_min_rows_packed = engine.tuning.band_min_rows_packed ? engine.tuning.band_min_rows_packed
                                                                   : (std::uint32_t)band_min_rows_packed_k;
    args.band_min_rows_compare = engine.tuning.band_min_rows_compare ? engine.tuning.band_min_rows_compare
                                                                     : (std::uint32_t)band_min_rows_compare_k;
    args.short_max_rows = engine.tuning.short_max_rows
                              ? std::min<std::uint32_t>(engine.tuning.short_max_rows, (std::uint32_t)short_max_rows_k)
                              : (std::uint32_t)short_max_rows_k;
    // A batched call with fewer pairs than one wave of the 16x2 route (two pairs per warp, about 16 resident warps
    // per SM) would leave SMs idle on the wavefront: its longer pairs spread over a band CTA's warps instead.
    if (schedule != szs_gb300_schedule_plain_k && args.pairs < 32ull * (std::uint64_t)context->sm_count) {
        std::uint32_t const few = engine.tuning.band_min_rows_few ? engine.tuning.band_min_rows_few
                                                                  : (std::uint32_t)band_min_rows_few_k;
        args.band_min_rows = std::min(args.band_min_rows, few);
        args.band_min_rows_packed = std::min(args.band_min_rows_packed, few);
        args.band_min_rows_compare = std::min(args.band_min_rows_compare, few);
    }
    for (int choice = 0; choice < 4; ++choice)
        args.packed_step_cost[choice] = engine.tuning.packed_step_cost[choice]
                                            ? engine.tuning.packed_step_cost[choice]
                                            : (std::uint16_t)packed_step_cost_k[choice];
    bool const levenshtein = engine.kind == kind_levenshtein_k;
    bool const dense = !engine.dense.empty();
    // Both score over the batch's own byte codes; 16-bit codes are already dense.
    bool const alphabet_pass = (levenshtein || dense) && !wide;
    // Unit-cost Levenshtein: the alphabet is guessed from the first bytes of each tape instead of a pass over all of
    // them, and the shared-table kernel checks every byte it reads against the guess. A guess with more than four
    // symbols, a plan with pairs on other routes, or a byte the guess missed is answered by scoring the call again
    // with the exact alphabet, so results never depend on the guess.
    // Deferred calls (pipelined chunks) guess from the sample they are given and are checked when they are settled.
    bool const speculative = alphabet_pass && engine.unit_levenshtein && !call.exact_alphabet &&
                             (!defer || call.sample_queries != nullptr);

    static bool const tracing = std::getenv("SZS_GB300_TRACE") != nullptr;
    // Device-resident inputs make every launch of the call a function of bytes the call can key on, so both phases
    // (planning, then scoring) are captured once as CUDA graphs and replayed by later calls with the same key.
    bool const graphs = !tracing && query_plan.offsets_bytes == 0 && query_plan.data_bytes == 0 &&
                        candidate_plan.offsets_bytes == 0 && candidate_plan.data_bytes == 0;
    bool prologue_replayed = false, launches_replayed = false;
    // Runs `issue(capture_stream)` directly on the call's stream, or captures it on the context's own stream into a
    // graph (once per key) and launches that graph on the call's stream.
    auto issue_or_replay = [&](graph_cache_t &cache, std::vector<unsigned char> const &key, bool &replayed,
                               auto &&issue) -> status_t {
        if (!graphs) return issue(stream);
        cudaGraphExec_t exec = cache.find(key);
        replayed = exec != nullptr;
        if (!exec) {
            cudaStream_t const capture = context->own_stream;
            SZS_TRY_CUDA(cudaStreamBeginCapture(capture, cudaStreamCaptureModeRelaxed));
            status_t const issued = issue(capture);
            cudaGraph_t graph = nullptr;
            cudaError_t const ended = cudaStreamEndCapture(capture, &graph);
            if (!issued.ok() || ended != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();
                return issued.ok() ? from_cuda(ended) : issued;
            }
            cudaError_t const made = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            SZS_TRY_CUDA(made);
            cache.insert(key, exec);
        }
        SZS_TRY_CUDA(cudaGraphLaunch(exec, stream));
        return {};
    };

    if (call.plan_after && !call.reuse_plan) SZS_TRY_CUDA(cudaStreamWaitEvent(stream, call.plan_after, 0));
    SZS_TRY_CUDA(cudaEventRecord(context->start, stream));
    std::uint64_t launches = 0;
    plan_bins_t *bins = context->bins_device();
    batch_alphabet_t *alphabet = context->alphabet_device();
    if (alphabet_pass) args.alphabet = alphabet;
    if (!call.reuse_plan) {
        std::vector<unsigned char> prologue_key;
        if (graphs) {
            key_append(prologue_key, args);
            key_append(prologue_key, bins), key_append(prologue_key, tasks), key_append(prologue_key, results);
            key_append(prologue_key, context->readback.data), key_append(prologue_key, context->sm_count);
            key_append(prologue_key, call.has_candidates), key_append(prologue_key, speculative);
            for (tape_t const *sample : {call.sample_queries, call.sample_candidates})
                if (sample) {
                    key_append(prologue_key, sample->base), key_append(prologue_key, sample->offsets);
                    key_append(prologue_key, sample->count), key_append(prologue_key, sample->offset_bits);
                }
        }
        status = issue_or_replay(context->prologue_graphs, prologue_key, prologue_replayed, [&](cudaStream_t s) -> status_t {
            // Levenshtein engines need the batch alphabet before planning: the bit-parallel route sizes its code
            // planes by it, and the 16x2 route builds its substitution profile over it (when it has at most 32
            // symbols).
            if (alphabet_pass) {
                bool const sampled_elsewhere = speculative && call.sample_queries;
                tape_t const &sample_queries = sampled_elsewhere ? *call.sample_queries : args.queries;
                tape_t const &sample_candidates = sampled_elsewhere ? *call.sample_candidates : args.candidates;
                SZS_TRY_CUDA(launch_alphabet(sample_queries, sample_candidates, call.has_candidates, alphabet,
                                             context->sm_count, s, speculative ? alphabet_sample_bytes_k : 0));
            }
            SZS_TRY_CUDA(launch_plan(args, bins, tasks, results, context->sm_count, s));
            // Read the plan (and the alphabet, stored right after it) back: which bins are non-empty, column lengths.
            SZS_TRY_CUDA(cudaMemcpyAsync(context->bins_host(), bins, sizeof(plan_bins_t) + sizeof(batch_alphabet_t),
                                         cudaMemcpyDeviceToHost, s));
            return {};
        });
        if (!status.ok()) return status;
        launches += 3 + (alphabet_pass ? 2 : 0);
        SZS_TRY_CUDA(cudaStreamSynchronize(stream));
    }
    plan_bins_t const &plan = *context->bins_host();
    batch_alphabet_t const &alphabet_host = *context->alphabet_host();
    auto run_exact = [&]() -> status_t {
        call_t exact = call;
        exact.exact_alphabet = true;
        if (exact.scoring_after) exact.plan_after = exact.scoring_after; // the exact pass reads the chunk's bytes
        return run_on(engine, context, stream, exact, schedule, stats, defer);
    };
    if (speculative) {
        bool thread_route_only = alphabet_host.bits <= 2; // at most four codes: the shared-table kernel
        for (int key = bin_dp32_begin_k; key < bin_keys_k && thread_route_only; ++key)
            thread_route_only = plan.count[key] == 0;
        if (!thread_route_only) return run_exact();
    }
    if (call.plan_only) {
        stats.last_launches = launches; // the planning launches; the scoring phase counts its own
        return {};
    }
    stats.last_cells = plan.cells;
    auto pairs_in = [&](int key_begin, int key_end) {
        std::uint64_t total = 0;
        for (int key = key_begin; key < key_end; ++key) total += plan.count[key];
        return total;
    };

    // Dense-table engines score every route over the sub-table of the bytes this batch uses (dense codes from the
    // alphabet pass), which must fit the kernels' 32 compact classes.
    score_costs_t dense_costs;
    bool direct = false;
    if (dense && alphabet_host.symbols > 32) {
        // More distinct bytes than 32 classes: the 32-bit routes read the whole table from shared memory (the plan
        // kept these pairs off the 16x2 routes, which need a 32-class profile).
        if (context->dense_table_id != engine.dense_id) {
            status = context->dense_table.reserve(engine.dense.size(), stream);
            if (!status.ok()) return status;
            SZS_TRY_CUDA(cudaMemcpyAsync(context->dense_table.data, engine.dense.data(), engine.dense.size(),
                                         cudaMemcpyHostToDevice, stream));
            context->dense_table_id = engine.dense_id;
        }
        dense_costs = engine.costs;
        dense_costs.classes = 1;
        dense_costs.direct_table = static_cast<std::int8_t const *>(context->dense_table.data);
        direct = true;
    }
    else if (dense) {
        int const symbols = (int)alphabet_host.symbols;
        dense_costs = engine.costs;
        int byte_of_code[32] = {0};
        for (int b = 0; b < 256; ++b)
            if ((alphabet_host.present[b >> 5] >> (b & 31)) & 1u) byte_of_code[alphabet_host.code[b]] = b;
        for (int b = 0; b < 256; ++b) dense_costs.byte_to_class[b] = dense_costs.byte_to_compact[b] = alphabet_host.code[b];
        dense_costs.classes = symbols < 1 ? 1 : symbols;
        std::memset(dense_costs.profile_table, 0, sizeof(dense_costs.profile_table));
        std::memset(dense_costs.profile_table_t, 0, sizeof(dense_costs.profile_table_t));
        for (int cc = 0; cc < symbols; ++cc)
            for (int rc = 0; rc < symbols; ++rc) {
                int const row_byte = byte_of_code[rc], column_byte = byte_of_code[cc];
                dense_costs.profile_table[cc * 32 + rc] = engine.dense[row_byte * 256 + column_byte];
                dense_costs.profile_table_t[cc * 32 + rc] = engine.dense[column_byte * 256 + row_byte];
            }
    }
    score_costs_t const &call_costs = dense ? dense_costs : costs;

    // 16x2 routes (packed wavefront, 16-bit band): Levenshtein engines score over the batch alphabet's codes, with a
    // profile over at most 32 of them, else by comparing the codes (the kernels' compare mode), which is also how
    // 16-bit codes are scored.
    score_costs_t packed_costs = call_costs;
    bool const packed_compare = levenshtein && (wide || alphabet_host.symbols > 32);
    // Compare mode's form: one multiply-add per row when match and mismatch, as the kernels shift them (minus `open`
    // for affine tracks), have the same sign, else a mask and a select.
    int const shift = costs.affine ? costs.open : 0;
    int const compare_mode =
        packed_compare ? compare_mode_for(costs.match - shift, costs.mismatch - shift) : (int)compare_none_k;
    if (levenshtein && (pairs_in(bin_dp16_begin_k, bin_dp16_begin_k + bin_dp16_classes_k) ||
                        pairs_in(bin_short_begin_k, bin_short_begin_k + short_shapes_k * short_m_classes_k) ||
                        pairs_in(bin_band16_begin_k, bin_band16_begin_k + bin_dp_classes_k))) {
        packed_costs.classes = packed_compare ? 1 : (int)alphabet_host.symbols;
        if (!wide) // 16-bit codes are compared as they are; no alphabet pass ran
            for (int b = 0; b < 256; ++b)
                packed_costs.byte_to_class[b] = packed_costs.byte_to_compact[b] = alphabet_host.code[b];
        for (int cc = 0; cc < 32; ++cc)
            for (int rc = 0; rc < 32; ++rc) {
                std::int8_t const cost = (std::int8_t)(cc == rc ? costs.match : costs.mismatch);
                packed_costs.profile_table[cc * 32 + rc] = packed_costs.profile_table_t[cc * 32 + rc] = cost;
            }
    }

    // The launch list, longest pairs first (64- and 32-bit wavefront, packed with the most rows per lane, then the
    // bit-parallel kernels by word count), so the routes' tails overlap each other instead of adding up.
    enum job_kind_t { job_dp_k, job_dp16_k, job_myers_k, job_band_k, job_band16_k, job_myers_warp_k, job_short_k,
                      job_myers_chain_k };
    struct job_t {
        job_kind_t kind;
        int variant; // cell bits, rows per lane, or words
        int warps;   // warps per CTA of the 16x2 launches
        int key_begin, key_end;
        std::uint64_t pairs;
        int ctas;
        std::size_t scratch_offset, scratch_bytes;
        int group_ctas = 1;            // band jobs: CTAs sharing one pair (1 = one CTA per pair)
        int rows = 8;                  // band jobs: rows per lane (4 for groups of CTAs per pair)
        std::size_t state_offset = 0;  // grouped band jobs: the groups' state records in the scratch buffer
        std::size_t state_bytes = 0;
        bool fills = true;             // the grid takes every resident CTA slot of its kernel on the device
    };
    job_t jobs[64];
    int job_count = 0;
    std::size_t const cells_per_warp = align_up(((std::size_t)plan.max_cols + 1) * 2, 64);
    std::size_t const band16_words_per_slot = align_up((std::size_t)plan.max_cols + 1, 64);
    std::size_t scratch_total = 0;
    // Long pairs: one CTA each while they fill the GPU; when fewer than half the resident CTA slots have a pair, the
    // batched form gives each pair a group of CTAs (one cooperative launch) so a few long pairs still use every SM.
    // A group never gets more warps than a pair can have strips: the shorter side is at most the longest row
    // `max_cols`, so `max_cols / strip_rows` strips bound every pair of the call.
    auto band_groups = [&](std::uint64_t pairs_here, dp_launch_shape_t const &shape, std::uint64_t strip_rows,
                           int &ctas, int &group_ctas) {
        ctas = (int)std::min<std::uint64_t>(pairs_here, (std::uint64_t)context->sm_count * shape.ctas_per_sm);
        group_ctas = 1;
        if (schedule == szs_gb300_schedule_plain_k || shape.group_ctas_per_sm <= 0) return;
        std::uint64_t const slots = (std::uint64_t)context->sm_count * shape.group_ctas_per_sm;
        if (pairs_here * 2 > slots) return;
        std::uint64_t const strips = ((std::uint64_t)plan.max_cols + strip_rows - 1) / strip_rows;
        std::uint64_t const useful = (strips + band_warps_per_cta() - 1) / band_warps_per_cta();
        std::uint64_t const size = std::min<std::uint64_t>({slots / pairs_here, (std::uint64_t)band_group_max_ctas(),
                                                            useful});
        if (size < 2) return;
        group_ctas = (int)size;
        ctas = (int)(std::min<std::uint64_t>(pairs_here, slots / group_ctas) * group_ctas);
    };
    {
        std::uint64_t const pairs_here = pairs_in(bin_band16_begin_k, bin_band16_begin_k + bin_dp_classes_k);
        if (pairs_here) {
            dp_launch_shape_t shape =
                band16_shape(engine.kind, costs.affine != 0, packed_costs.classes, compare_mode, wide, 8);
            if (shape.ctas_per_sm <= 0) return {sz_status_unknown_k, "16-bit band kernel cannot be resident"};
            int ctas = 0, group_ctas = 1;
            band_groups(pairs_here, shape, 2u * 32u * (std::uint64_t)shape.rows_per_lane, ctas, group_ctas);
            // Groups limited by their pairs' super-strips while the GPU has CTA slots to spare (a handful of long
            // pairs) take 4 rows per lane: twice the super-strips, so a pair spreads over twice the warps, each step
            // about half as long. Groups that fill the GPU keep 8 rows, which do more cells per step's overhead.
            if (group_ctas > 1 && ctas * 2 <= context->sm_count * shape.group_ctas_per_sm) {
                dp_launch_shape_t const narrow =
                    band16_shape(engine.kind, costs.affine != 0, packed_costs.classes, compare_mode, wide, 4);
                int narrow_ctas = 0, narrow_group = 1;
                if (narrow.ctas_per_sm > 0)
                    band_groups(pairs_here, narrow, 2u * 32u * 4u, narrow_ctas, narrow_group);
                if (narrow_group > group_ctas) shape = narrow, ctas = narrow_ctas, group_ctas = narrow_group;
            }
            // Local scores keep room for a 32-bit ring: a pair that reaches the 16-bit limit is scored again.
            std::size_t const ring_scale = engine.kind == kind_smith_waterman_k ? 2 : 1;
            std::size_t const bytes = align_up(band16_words_per_slot * 4 * ring_scale * (std::size_t)ctas *
                                                   (std::size_t)band_warps_per_cta(), 256);
            job_t job {job_band16_k, 16, 0, bin_band16_begin_k, bin_band16_begin_k + bin_dp_classes_k, pairs_here,
                       ctas, scratch_total, bytes};
            job.fills = group_ctas > 1 || ctas >= context->sm_count * shape.ctas_per_sm;
            job.rows = shape.rows_per_lane;
            scratch_total += bytes;
            if (group_ctas > 1) {
                job.group_ctas = group_ctas, job.state_offset = scratch_total;
                job.state_bytes = align_up((std::size_t)(ctas / group_ctas) * band_group_state_bytes(), 256);
                scratch_total += job.state_bytes;
            }
            jobs[job_count++] = job;
        }
    }
    {
        std::uint64_t const pairs_here = pairs_in(bin_band_begin_k, bin_band_begin_k + bin_dp_classes_k);
        if (pairs_here) {
            dp_launch_shape_t shape =
                band_shape(engine.kind, call_costs.affine != 0, call_costs.classes, direct, wide, 8);
            if (shape.ctas_per_sm <= 0) return {sz_status_unknown_k, "Band kernel cannot be resident"};
            int ctas = 0, group_ctas = 1;
            band_groups(pairs_here, shape, 32u * (std::uint64_t)shape.rows_per_lane, ctas, group_ctas);
            // As for the 16-bit band: 4 rows per lane only while the groups leave half the GPU's CTA slots free.
            if (group_ctas > 1 && ctas * 2 <= context->sm_count * shape.group_ctas_per_sm) {
                dp_launch_shape_t const narrow =
                    band_shape(engine.kind, call_costs.affine != 0, call_costs.classes, direct, wide, 4);
                int narrow_ctas = 0, narrow_group = 1;
                if (narrow.ctas_per_sm > 0) band_groups(pairs_here, narrow, 32u * 4u, narrow_ctas, narrow_group);
                if (narrow_group > group_ctas) shape = narrow, ctas = narrow_ctas, group_ctas = narrow_group;
            }
            std::size_t const bytes =
                align_up(cells_per_warp * 4 * (std::size_t)ctas * (std::size_t)band_warps_per_cta(), 256);
            job_t job {job_band_k, 32, 0, bin_band_begin_k, bin_band_begin_k + bin_dp_classes_k, pairs_here, ctas,
                       scratch_total, bytes};
            job.fills = group_ctas > 1 || ctas >= context->sm_count * shape.ctas_per_sm;
            job.rows = shape.rows_per_lane;
            scratch_total += bytes;
            if (group_ctas > 1) {
                job.group_ctas = group_ctas, job.state_offset = scratch_total;
                job.state_bytes = align_up((std::size_t)(ctas / group_ctas) * band_group_state_bytes(), 256);
                scratch_total += job.state_bytes;
            }
            jobs[job_count++] = job;
        }
    }
    for (int cell_bits : {64, 32}) {
        int const key_begin = cell_bits == 32 ? bin_dp32_begin_k : bin_dp64_begin_k;
        std::uint64_t const pairs_here = pairs_in(key_begin, key_begin + bin_dp_classes_k);
        if (!pairs_here) continue;
        dp_launch_shape_t const shape =
            dp_shape(engine.kind, call_costs.affine != 0, cell_bits, call_costs.classes, direct, wide);
        if (shape.ctas_per_sm <= 0) return {sz_status_unknown_k, "Wavefront kernel cannot be resident"};
        std::uint64_t const needed = (pairs_here + shape.warps_per_cta - 1) / shape.warps_per_cta;
        int const ctas = (int)std::min<std::uint64_t>(needed, (std::uint64_t)context->sm_count * shape.ctas_per_sm);
        std::size_t const bytes = align_up(cells_per_warp * (cell_bits / 8) * (std::size_t)ctas * shape.warps_per_cta, 256);
        jobs[job_count++] = {job_dp_k, cell_bits, 0, key_begin, key_begin + bin_dp_classes_k, pairs_here, ctas,
                             scratch_total, bytes};
        jobs[job_count - 1].fills = needed >= (std::uint64_t)context->sm_count * shape.ctas_per_sm;
        scratch_total += bytes;
    }
    for (int choice = dp16_row_choices_k - 1; choice >= 0; --choice) {
        int const key_begin = bin_dp16_begin_k + choice * dp16_classes_per_rows_k;
        int const key_end = key_begin + dp16_classes_per_rows_k;
        std::uint64_t const pairs_here = pairs_in(key_begin, key_end);
        if (!pairs_here) continue;
        int const rows = 4 * (choice + 1);
        int const warps = engine.tuning.packed_warps[choice] ? (int)engine.tuning.packed_warps[choice] : 4;
        dp_launch_shape_t const shape =
            dp16_shape(engine.kind, costs.affine != 0, rows, packed_costs.classes, warps, compare_mode, wide);
        if (shape.ctas_per_sm <= 0) return {sz_status_unknown_k, "Packed wavefront kernel cannot be resident"};
        std::uint64_t const warps_needed = (pairs_here + 1) / 2;
        std::uint64_t const needed = (warps_needed + shape.warps_per_cta - 1) / shape.warps_per_cta;
        int const ctas = (int)std::min<std::uint64_t>(needed, (std::uint64_t)context->sm_count * shape.ctas_per_sm);
        std::size_t const bytes = align_up(cells_per_warp * 4 * (std::size_t)ctas * shape.warps_per_cta, 256);
        jobs[job_count++] = {job_dp16_k, rows, warps, key_begin, key_end, pairs_here, ctas, scratch_total, bytes};
        jobs[job_count - 1].fills = needed >= (std::uint64_t)context->sm_count * shape.ctas_per_sm;
        scratch_total += bytes;
    }
    // Short pairs: one job per segment shape, most rows first.
    for (int shape_index : {3, 6, 2, 5, 1, 4, 0}) {
        int const key_begin = bin_short_begin_k + shape_index * short_m_classes_k;
        int const key_end = key_begin + short_m_classes_k;
        std::uint64_t const pairs_here = pairs_in(key_begin, key_end);
        if (!pairs_here) continue;
        int const warps = 4;
        dp_launch_shape_t const shape =
            short_shape(engine.kind, costs.affine != 0, shape_index, packed_costs.classes, warps, compare_mode);
        if (shape.ctas_per_sm <= 0) return {sz_status_unknown_k, "Short-pair kernel cannot be resident"};
        int const rows = short_rows_for(packed_costs.classes, compare_mode, shape_index);
        std::uint64_t const lanes = (std::uint64_t)(short_segment_rows(shape_index) / rows);
        std::uint64_t const per_warp = 2u * (32u / lanes); // pairs per warp
        std::uint64_t const warps_needed = (pairs_here + per_warp - 1) / per_warp;
        std::uint64_t const needed = (warps_needed + warps - 1) / warps;
        int const ctas = (int)std::min<std::uint64_t>(needed, (std::uint64_t)context->sm_count * shape.ctas_per_sm);
        jobs[job_count++] = {job_short_k, shape_index, warps, key_begin, key_end, pairs_here, ctas, 0, 0};
        jobs[job_count - 1].fills = needed >= (std::uint64_t)context->sm_count * shape.ctas_per_sm;
    }
    int myers_planes = 0;
    std::uint32_t chain_strips = 0, chain_wave = 0; // warps per chained pair, pairs per cooperative launch
    std::uint64_t chain_link_stride = 0;
    if (engine.unit_levenshtein) {
        myers_planes = wide ? 16 : myers_planes_for((int)alphabet_host.bits);
        // Very long patterns: a chain of warps per pair, the fewest words per lane whose chain fits the GPU at once;
        // as many pairs per cooperative launch (a wave) as fit beside each other.
        if (std::uint64_t const chained = pairs_in(bin_myers_chain_k, bin_myers_chain_k + 1)) {
            int words = 0;
            std::uint64_t capacity = 0; // resident warps of one launch
            for (int w : {1, 2, 4}) {
                std::uint32_t const strips =
                    (std::uint32_t)(((std::uint64_t)plan.max_chain_rows + 1024u * w - 1) / (1024u * w));
                capacity = (std::uint64_t)context->sm_count * myers_chain_ctas_per_sm(w, myers_planes) * 8u;
                if (strips <= capacity) {
                    words = w, chain_strips = strips;
                    break;
                }
            }
            if (!words) return {sz_status_unknown_k, "A long pattern's chain of warps does not fit the device"};
            chain_link_stride = align_up((std::size_t)plan.max_cols + 1, 256);
            chain_wave = (std::uint32_t)std::min<std::uint64_t>(chained, capacity / chain_strips);
            std::size_t const bytes =
                align_up(myers_chain_scratch_bytes(chain_strips, chain_link_stride, chain_wave), 256);
            jobs[job_count++] = {job_myers_chain_k, words, 0, bin_myers_chain_k, bin_myers_chain_k + 1, chained, 0,
                                 scratch_total, bytes};
            scratch_total += bytes;
        }
        // The plain form keeps each bit-parallel route in one bin and launches the word count of the batch's longest
        // pattern on it (the binned form launches each bin with its own word count).
        bool const plain = schedule == szs_gb300_schedule_plain_k;
        // Longer patterns first: one warp per pair, most words per lane first.
        for (int words = myers_warp_max_words_k; words >= 1; --words) {
            int const key_begin = bin_myers_warp_begin_k + (myers_warp_max_words_k - words) * myers_warp_classes_k;
            std::uint64_t const pairs_here = pairs_in(key_begin, key_begin + myers_warp_classes_k);
            if (!pairs_here) continue;
            int const launch_words =
                plain ? std::max(1, (int)((plan.max_myers_warp_rows + 32u * 32u - 1) / (32u * 32u))) : words;
            std::uint64_t const needed = (pairs_here + 7) / 8; // eight warps per CTA
            int const ctas = (int)std::min<std::uint64_t>(needed, (std::uint64_t)context->sm_count * 2);
            jobs[job_count++] = {job_myers_warp_k, launch_words, 0, key_begin, key_begin + myers_warp_classes_k,
                                 pairs_here, ctas, 0, 0};
            jobs[job_count - 1].fills = needed >= (std::uint64_t)context->sm_count * 2;
        }
        for (int words = myers_max_words_k; words >= 1; --words) {
            int const key_begin = bin_myers_begin_k + words * 16;
            std::uint64_t const pairs_here = pairs_in(key_begin, key_begin + 16);
            if (!pairs_here) continue;
            int const launch_words = plain ? std::max(1, (int)((plan.max_myers_rows + 31u) / 32u)) : words;
            int const threads = myers_threads_per_cta();
            std::uint64_t const needed = (pairs_here + threads - 1) / threads;
            int const ctas = (int)std::min<std::uint64_t>(needed, (std::uint64_t)context->sm_count * 16);
            jobs[job_count++] = {job_myers_k, launch_words, 0, key_begin, key_begin + 16, pairs_here, ctas, 0, 0};
            jobs[job_count - 1].fills = needed >= (std::uint64_t)context->sm_count * 16;
        }
    }
    // Jobs whose grids leave slots free go first: a persistent grid that fills the device holds its slots until its
    // last pair, so a small job launched after it would only start at the end and add its whole time to the call.
    // Launched first, it takes its few slots and runs beside the large grids, which balance over their cursor.
    if (schedule != szs_gb300_schedule_plain_k)
        std::stable_partition(jobs, jobs + job_count, [](job_t const &job) { return !job.fills; });
    if (scratch_total) {
        status = context->scratch.reserve(scratch_total, stream);
        if (!status.ok()) return status;
    }

    // Fork the launches over the auxiliary streams, join them back into the call's stream.
    // The plain form runs its launches one after another on one stream; the batched form spreads them.
    int const lanes_used = schedule == szs_gb300_schedule_plain_k ? std::min(job_count, 1)
                                                                   : std::min(job_count, (int)device_context_t::lanes_k);
    // Scoring kernels are bracketed by their own events so the stats isolate them from planning and copies.
    bool compute_recorded = false;
    if (call.scoring_after) SZS_TRY_CUDA(cudaStreamWaitEvent(stream, call.scoring_after, 0));
    if (job_count) {
        SZS_TRY_CUDA(cudaEventRecord(context->compute_start, stream));
        compute_recorded = true;
    }
    std::vector<unsigned char> launch_key;
    if (graphs && job_count) {
        for (int i = 0; i < job_count; ++i) { // field by field: the struct's padding bytes are indeterminate
            key_append(launch_key, (int)jobs[i].kind), key_append(launch_key, jobs[i].variant);
            key_append(launch_key, jobs[i].warps);
            key_append(launch_key, jobs[i].key_begin), key_append(launch_key, jobs[i].key_end);
            key_append(launch_key, jobs[i].ctas), key_append(launch_key, jobs[i].scratch_offset);
            key_append(launch_key, jobs[i].group_ctas), key_append(launch_key, jobs[i].state_offset);
            key_append(launch_key, jobs[i].rows);
        }
        key_append(launch_key, packed_costs), key_append(launch_key, call_costs);
        key_append(launch_key, tasks), key_append(launch_key, bins), key_append(launch_key, results);
        key_append(launch_key, context->scratch.data), key_append(launch_key, alphabet);
        key_append(launch_key, cells_per_warp), key_append(launch_key, myers_planes), key_append(launch_key, wide);
        key_append(launch_key, schedule), key_append(launch_key, lanes_used);
        key_append(launch_key, engine.kind), key_append(launch_key, compare_mode);
    }
    auto issue_jobs = [&](cudaStream_t s) -> status_t {
        SZS_TRY_CUDA(cudaEventRecord(context->fork, s));
        for (int lane = 0; lane < lanes_used; ++lane) SZS_TRY_CUDA(cudaStreamWaitEvent(context->lanes[lane], context->fork, 0));
        for (int i = 0; i < job_count; ++i) {
            job_t const &job = jobs[i];
            cudaStream_t const lane_stream = context->lanes[i % lanes_used];
            bool const traced = tracing && 2 * i + 1 < 64;
            if (traced) cudaEventRecord(context->trace_events[2 * i], lane_stream);
            void *scratch = static_cast<unsigned char *>(context->scratch.data) + job.scratch_offset;
            void *group_states = nullptr;
            if (job.group_ctas > 1) {
                group_states = static_cast<unsigned char *>(context->scratch.data) + job.state_offset;
                SZS_TRY_CUDA(cudaMemsetAsync(group_states, 0, job.state_bytes, lane_stream));
            }
            if (job.kind == job_band_k)
                SZS_TRY_CUDA(launch_band(engine.kind, costs.affine != 0, job.key_begin, job.key_end, tasks, bins,
                                         call_costs, results, scratch, cells_per_warp, job.ctas, lane_stream,
                                         group_states, job.group_ctas, wide, job.rows));
            else if (job.kind == job_band16_k)
                SZS_TRY_CUDA(launch_band16(engine.kind, costs.affine != 0, job.key_begin, job.key_end, tasks, bins,
                                           packed_costs, results, scratch, band16_words_per_slot, job.ctas,
                                           lane_stream, group_states, job.group_ctas, compare_mode, wide, job.rows));
            else if (job.kind == job_dp_k)
                SZS_TRY_CUDA(launch_dp(engine.kind, costs.affine != 0, job.variant, job.key_begin, job.key_end, tasks,
                                       bins, call_costs, results, scratch, cells_per_warp, job.ctas, lane_stream,
                                       wide));
            else if (job.kind == job_dp16_k)
                SZS_TRY_CUDA(launch_dp16(engine.kind, costs.affine != 0, job.variant, job.key_begin, job.key_end, tasks,
                                         bins, packed_costs, results, scratch, cells_per_warp, job.ctas, job.warps,
                                         lane_stream, compare_mode, wide));
            else if (job.kind == job_myers_chain_k) {
                // One cooperative launch per wave of pairs, one after another on this lane (they share the scratch).
                for (std::uint64_t first = 0; first < job.pairs; first += chain_wave)
                    SZS_TRY_CUDA(launch_myers_chain(job.variant, myers_planes, tasks, bins, job.key_begin,
                                                    (std::uint32_t)first,
                                                    (std::uint32_t)std::min<std::uint64_t>(chain_wave, job.pairs - first),
                                                    chain_strips, alphabet, results, scratch, chain_link_stride,
                                                    costs.wait_polls, lane_stream));
            }
            else if (job.kind == job_short_k)
                SZS_TRY_CUDA(launch_short(engine.kind, costs.affine != 0, job.variant, job.key_begin, job.key_end,
                                          tasks, bins, packed_costs, results, job.ctas, job.warps, lane_stream,
                                          compare_mode));
            else if (job.kind == job_myers_warp_k && wide)
                SZS_TRY_CUDA(launch_myers_warp_wide(job.variant, tasks, bins, job.key_begin, job.key_end, results,
                                                    job.ctas, lane_stream));
            else if (job.kind == job_myers_warp_k)
                SZS_TRY_CUDA(launch_myers_warp(job.variant, myers_planes, tasks, bins, job.key_begin, job.key_end,
                                               alphabet, results, job.ctas, lane_stream));
            else if (wide)
                SZS_TRY_CUDA(launch_myers_wide(job.variant, schedule != szs_gb300_schedule_plain_k, tasks, bins,
                                               job.key_begin, job.key_end, results, job.ctas, lane_stream));
            else if (myers_planes == 2)
                SZS_TRY_CUDA(launch_myers_table(job.variant, job.key_begin, job.key_end, tasks, bins, alphabet,
                                                results, job.ctas, lane_stream));
            else
                SZS_TRY_CUDA(launch_myers(job.variant, myers_planes, schedule != szs_gb300_schedule_plain_k, tasks,
                                          bins, job.key_begin, job.key_end, alphabet, results, job.ctas,
                                          lane_stream));
            if (traced) cudaEventRecord(context->trace_events[2 * i + 1], lane_stream);
        }
        for (int lane = 0; lane < lanes_used; ++lane) {
            SZS_TRY_CUDA(cudaEventRecord(context->joins[lane], context->lanes[lane]));
            SZS_TRY_CUDA(cudaStreamWaitEvent(s, context->joins[lane], 0));
        }
        return {};
    };
    if (job_count) {
        status = issue_or_replay(context->launch_graphs, launch_key, launches_replayed, issue_jobs);
        if (!status.ok()) return status;
        launches += job_count;
    }
    if (graphs && prologue_replayed && (launches_replayed || !job_count)) ++stats.graph_replays;

    if (compute_recorded) SZS_TRY_CUDA(cudaEventRecord(context->compute_stop, stream));

    // The band kernel's bounded waits report through the plan's error word; read it back with the results.
    SZS_TRY_CUDA(cudaMemcpyAsync(&context->bins_host()->error_flags, &bins->error_flags, sizeof(std::uint32_t),
                                 cudaMemcpyDeviceToHost, stream));

    // Results into the caller's matrix.
    bool const out_on_device = device_accessible(call.out);
    if (out_on_device) {
        SZS_TRY_CUDA(launch_scatter_output(args, results, call.out, call.stride, context->sm_count, stream));
        ++launches;
        SZS_TRY_CUDA(cudaEventRecord(context->stop, stream));
        SZS_TRY_CUDA(cudaStreamSynchronize(stream));
    }
    else {
        if (call.mode == mode_pairwise_k) {
            SZS_TRY_CUDA(cudaMemcpyAsync(call.out, results, args.pairs * sizeof(std::int64_t), cudaMemcpyDeviceToHost,
                                         stream));
            SZS_TRY_CUDA(cudaEventRecord(context->stop, stream));
            if (defer) {
                context->deferred = true;
                context->deferred_compute = compute_recorded;
                context->deferred_launches = launches;
                context->traced_jobs = tracing ? std::min(job_count, 32) : 0;
                for (int i = 0; i < context->traced_jobs; ++i)
                    context->traced_kind[i] = (int)jobs[i].kind, context->traced_variant[i] = jobs[i].variant,
                    context->traced_pairs[i] = jobs[i].pairs;
                return {};
            }
            SZS_TRY_CUDA(cudaStreamSynchronize(stream));
        }
        else {
            status = context->results_host.reserve(args.pairs * sizeof(std::int64_t));
            if (!status.ok()) return status;
            auto *dense = static_cast<std::int64_t *>(context->results_host.data);
            SZS_TRY_CUDA(cudaMemcpyAsync(dense, results, args.pairs * sizeof(std::int64_t), cudaMemcpyDeviceToHost,
                                         stream));
            SZS_TRY_CUDA(cudaEventRecord(context->stop, stream));
            SZS_TRY_CUDA(cudaStreamSynchronize(stream));
            if (call.mode == mode_cross_k) {
                for (std::uint64_t q = 0; q < queries_count; ++q)
                    std::memcpy(call.out + q * call.stride, dense + q * candidates_count,
                                candidates_count * sizeof(std::int64_t));
            }
            else {
                std::uint64_t p = 0;
                for (std::uint64_t q = 0; q < queries_count; ++q)
                    for (std::uint64_t c = 0; c <= q; ++c, ++p) {
                        call.out[q * call.stride + c] = dense[p];
                        call.out[c * call.stride + q] = dense[p];
                    }
            }
        }
    }
    SZS_TRY_CUDA(cudaGetLastError());
    if (context->bins_host()->error_flags & 1u)
        return {sz_status_unknown_k, "A long pair's band of warps stopped waiting for its neighbour (bounded wait "
                                     "expired); its score was not computed"};
    if (speculative && (context->bins_host()->error_flags & 2u)) return run_exact(); // the guessed alphabet missed
    float elapsed = 0;
    cudaEventElapsedTime(&elapsed, context->start, context->stop);
    stats.last_call_ms = elapsed;
    float compute = 0;
    if (compute_recorded) cudaEventElapsedTime(&compute, context->compute_start, context->compute_stop);
    stats.last_compute_ms = compute;
    if (tracing) {
        static char const *const names[] = {"wavefront bits", "packed16 rows", "bit-parallel words", "band bits",
                                            "band16 bits", "warp bit-parallel", "short shape", "chained words"};
        static_assert(sizeof(names) / sizeof(names[0]) == job_myers_chain_k + 1, "a name per job kind");
        for (int i = 0; i < job_count && 2 * i + 1 < 64; ++i) {
            float ms = 0, offset = 0;
            cudaEventElapsedTime(&ms, context->trace_events[2 * i], context->trace_events[2 * i + 1]);
            cudaEventElapsedTime(&offset, context->compute_start, context->trace_events[2 * i]);
            std::fprintf(stderr, "[szs_gb300] %-20s %3d  pairs %10llu  start %8.3f ms  took %9.3f ms\n",
                         names[jobs[i].kind], jobs[i].variant, (unsigned long long)jobs[i].pairs, offset, ms);
        }
    }
    stats.last_launches = launches;
    stats.kernel_launches += launches;
    return {};
}

/** Waits for a deferred call on @p context and reports it like `run_on` would have. */
static status_t finish_deferred(device_context_t *context, szs_gb300_stats_t &stats) noexcept {
    if (!context->deferred) return {};
    context->deferred = false;
    SZS_TRY_CUDA(cudaEventSynchronize(context->stop));
    SZS_TRY_CUDA(cudaGetLastError());
    if (context->bins_host()->error_flags & 1u)
        return {sz_status_unknown_k, "A long pair's band of warps stopped waiting for its neighbour (bounded wait "
                                     "expired); its score was not computed"};
    float elapsed = 0, compute = 0;
    cudaEventElapsedTime(&elapsed, context->start, context->stop);
    if (context->deferred_compute) cudaEventElapsedTime(&compute, context->compute_start, context->compute_stop);
    stats.last_call_ms = elapsed;
    stats.last_compute_ms = compute;
    stats.last_launches = context->deferred_launches;
    stats.kernel_launches += context->deferred_launches;
    return {};
}

static bool pinned_host(void const *pointer) noexcept {
    if (!pointer) return false;
    cudaPointerAttributes attributes;
    if (cudaPointerGetAttributes(&attributes, pointer) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attributes.type == cudaMemoryTypeHost;
}

constexpr std::size_t pipeline_chunk_bytes_k = std::size_t(64) << 20; // default input bytes per pipelined chunk

/**
 *  Pairwise calls on large pinned-host tapes: both tapes' offsets are copied first, then the strings in chunks of
 *  about `chunk_bytes` input bytes, each into its own slot, all queued at once on the context's copy stream. Chunk c
 *  is planned and scored as soon as its copy has landed, on one of `pipeline_depth_k` chunk contexts whose streams
 *  have the device's highest priority, so its planning kernels start ahead of the scoring still queued from earlier
 *  chunks while the later copies continue: the link stays busy and scoring hides behind it. The last chunks halve in
 *  size down to a quarter chunk, so little work remains once the last byte has landed. Each chunk is one ordinary
 *  call on device-resident tapes (`pre_staged`), so results equal the unchunked call's.
 */
static status_t run_pipelined(engine_t const &engine, device_context_t *context, cudaStream_t stream,
                              call_t const &call, int schedule, szs_gb300_stats_t &stats,
                              std::uint64_t chunk_bytes) noexcept {
    tape_view_t const tapes[2] = {call.queries, call.candidates};
    std::uint64_t const pairs = call.queries.count;
    auto bytes_before = [&](std::uint64_t p) { // input bytes of pairs [0, p) of both tapes
        return (host_offset(tapes[0], p) - host_offset(tapes[0], 0)) + (host_offset(tapes[1], p) - host_offset(tapes[1], 0));
    };
    std::uint64_t const total = bytes_before(pairs);
    // Chunk sizes: whole chunks while more than two remain, then halves down to a quarter chunk, then the rest.
    std::vector<std::uint64_t> targets; // byte prefix at the end of each chunk but the last
    {
        std::uint64_t done = 0, remaining = total;
        std::uint64_t const smallest = std::max<std::uint64_t>(chunk_bytes / 4, 1);
        while (remaining > 2 * chunk_bytes && targets.size() + 2 < device_context_t::max_chunks_k)
            done += chunk_bytes, remaining -= chunk_bytes, targets.push_back(done);
        while (remaining > 2 * smallest && targets.size() + 2 < device_context_t::max_chunks_k)
            done += remaining / 2, remaining -= remaining / 2, targets.push_back(done);
    }
    std::vector<std::uint64_t> cuts(1, 0);
    for (std::uint64_t const target : targets) { // first pair whose prefix reaches the target
        std::uint64_t low = cuts.back(), high = pairs;
        while (low < high) {
            std::uint64_t const mid = low + (high - low) / 2;
            if (bytes_before(mid) < target) low = mid + 1;
            else high = mid;
        }
        if (low > cuts.back() && low < pairs) cuts.push_back(low);
    }
    cuts.push_back(pairs);
    int const chunks = (int)cuts.size() - 1;
    std::size_t const offset_size = call.queries.offset_bits == 32 ? 4 : 8;
    // Slots: the offsets of both tapes, then each chunk's bytes of both tapes.
    std::size_t offsets_at[2], cursor = 0;
    for (int t = 0; t < 2; ++t) offsets_at[t] = cursor, cursor += align_up((pairs + 1) * offset_size, 256);
    std::vector<std::size_t> data_at(2 * chunks);
    for (int c = 0; c < chunks; ++c)
        for (int t = 0; t < 2; ++t)
            data_at[2 * c + t] = cursor,
                          cursor += align_up(host_offset(tapes[t], cuts[c + 1]) - host_offset(tapes[t], cuts[c]), 256);
    status_t status = context->chunk_inputs.reserve(cursor, stream);
    if (!status.ok()) return status;
    auto *area = static_cast<unsigned char *>(context->chunk_inputs.data);

    SZS_TRY_CUDA(cudaEventRecord(context->pipe_start, stream));
    auto const host_zero = std::chrono::steady_clock::now();
    auto host_ms = [&] {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_zero).count();
    };
    // Earlier work on the call's stream may still read the slots: the copies wait for it.
    SZS_TRY_CUDA(cudaStreamWaitEvent(context->copy_stream, context->pipe_start, 0));
    for (int t = 0; t < 2; ++t)
        SZS_TRY_CUDA(cudaMemcpyAsync(area + offsets_at[t], tapes[t].offsets, (pairs + 1) * offset_size,
                                     cudaMemcpyHostToDevice, context->copy_stream));
    SZS_TRY_CUDA(cudaEventRecord(context->offsets_copied, context->copy_stream));
    std::vector<tape_t> staged(2 * chunks);
    for (int c = 0; c < chunks; ++c) {
        std::uint64_t const first = cuts[c], count = cuts[c + 1] - cuts[c];
        for (int t = 0; t < 2; ++t) {
            std::uint64_t const begin = host_offset(tapes[t], first), end = host_offset(tapes[t], first + count);
            if (end > begin)
                SZS_TRY_CUDA(cudaMemcpyAsync(area + data_at[2 * c + t], tapes[t].data + begin, end - begin,
                                             cudaMemcpyHostToDevice, context->copy_stream));
            tape_t &out = staged[2 * c + t];
            out.offsets = area + offsets_at[t] + first * offset_size;
            out.count = count;
            out.offset_bits = tapes[t].offset_bits;
            out.base = reinterpret_cast<std::uint8_t const *>(area + data_at[2 * c + t]) - begin; // absolute offsets
        }
        SZS_TRY_CUDA(cudaEventRecord(context->copied[c], context->copy_stream));
    }
    double const copies_queued_ms = host_ms();
    std::vector<double> host_marks(3 * chunks, 0.0); // per chunk: plan queued from, plan read back at, scoring queued at
    int const depth = std::min(chunks, device_context_t::pipeline_depth_k);
    device_context_t *contexts[device_context_t::pipeline_depth_k] = {nullptr};
    cudaStream_t streams[device_context_t::pipeline_depth_k] = {nullptr};
    for (int i = 0; i < depth; ++i) {
        device_context_t *&partner = context->partners[i];
        if (!partner) {
            partner = new (std::nothrow) device_context_t();
            if (!partner) return {sz_bad_alloc_k, nullptr};
            status = partner->prepare(context->device, true);
            if (!status.ok()) {
                partner->release();
                delete partner;
                partner = nullptr;
                return status;
            }
        }
        contexts[i] = partner, streams[i] = partner->own_stream;
        SZS_TRY_CUDA(cudaStreamWaitEvent(streams[i], context->pipe_start, 0));
    }
    szs_gb300_stats_t chunk_stats[device_context_t::pipeline_depth_k] {};
    call_t chunk_calls[device_context_t::pipeline_depth_k];
    std::uint64_t cells = 0, launches = 0, graph_replays = 0;
    double compute_ms = 0;
    // SZS_GB300_TRACE prints each chunk's timeline and jobs (graphs off); SZS_GB300_TRACE_CHUNKS only the chunks'
    // timelines, with the graphs of ordinary calls.
    static bool const tracing =
        std::getenv("SZS_GB300_TRACE") != nullptr || std::getenv("SZS_GB300_TRACE_CHUNKS") != nullptr;
    int in_flight[device_context_t::pipeline_depth_k];
    for (int &chunk : in_flight) chunk = -1; // the chunk each context runs
    auto settle = [&](int which) -> status_t { // waits for the chunk in flight on contexts[which], if any
        if (!contexts[which]->deferred) return {};
        std::uint64_t const before = chunk_stats[which].kernel_launches;
        status_t const finished = finish_deferred(contexts[which], chunk_stats[which]);
        if (!finished.ok()) return finished;
        launches += chunk_stats[which].kernel_launches - before;
        compute_ms += chunk_stats[which].last_compute_ms;
        if (contexts[which]->bins_host()->error_flags & 2u) { // the sampled alphabet missed a byte of this chunk
            call_t exact = chunk_calls[which];
            exact.exact_alphabet = true;
            exact.plan_after = exact.scoring_after = nullptr; // its bytes landed before its scoring ran
            exact.sample_queries = exact.sample_candidates = nullptr;
            exact.plan_only = exact.reuse_plan = false;
            std::uint64_t const again = chunk_stats[which].kernel_launches;
            status_t const rescored = run_on(engine, contexts[which], streams[which], exact, schedule,
                                             chunk_stats[which], false);
            if (!rescored.ok()) return rescored;
            launches += chunk_stats[which].kernel_launches - again;
            compute_ms += chunk_stats[which].last_compute_ms;
        }
        if (tracing && in_flight[which] >= 0) { // the chunk's timeline from the start of the call, in ms
            float at[5] = {0, 0, 0, 0, 0};
            cudaEvent_t const marks[5] = {context->copied[in_flight[which]], contexts[which]->start,
                                          contexts[which]->compute_start, contexts[which]->compute_stop,
                                          contexts[which]->stop};
            for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&at[i], context->pipe_start, marks[i]);
            cudaGetLastError(); // a mark that was not recorded leaves no error behind for the next call
            std::fprintf(stderr,
                         "[szs_gb300] chunk %3d  pairs %8llu  copied %8.3f  planning %8.3f  scoring %8.3f - %8.3f  "
                         "done %8.3f\n",
                         in_flight[which], (unsigned long long)(cuts[in_flight[which] + 1] - cuts[in_flight[which]]),
                         at[0], at[1], at[2], at[3], at[4]);
            for (int i = 0; i < contexts[which]->traced_jobs; ++i) {
                float from = 0, to = 0;
                cudaEventElapsedTime(&from, context->pipe_start, contexts[which]->trace_events[2 * i]);
                cudaEventElapsedTime(&to, context->pipe_start, contexts[which]->trace_events[2 * i + 1]);
                cudaGetLastError();
                std::fprintf(stderr, "[szs_gb300]      job kind %d variant %3d  pairs %8llu  %8.3f - %8.3f\n",
                             contexts[which]->traced_kind[i], contexts[which]->traced_variant[i],
                             (unsigned long long)contexts[which]->traced_pairs[i], from, to);
            }
        }
        return {};
    };
    // A chunk is planned before its bytes land whenever its plan does not read them: engines without an alphabet
    // pass plan from the offsets alone, and unit-cost Levenshtein guesses its alphabet from the first chunk's bytes
    // (checked per pair by the kernels, a missed byte rescoring the chunk exactly). The first `depth` chunks are
    // then all planned before any scoring is queued, while the GPU only waits for the link, and only scoring waits
    // for each chunk's own copy; planning kernels queued behind scoring would wait for its CTAs to retire.
    bool const alphabet_pass = (engine.kind == kind_levenshtein_k || !engine.dense.empty()) && !engine.utf8;
    bool const sampled = alphabet_pass && engine.unit_levenshtein;
    bool const plan_ahead = !alphabet_pass || sampled;
    auto plan = [&](int c) -> status_t { // plans chunk c on context c % depth, once its previous chunk is settled
        int const which = c % depth;
        status_t settled = settle(which);
        if (!settled.ok()) return settled;
        host_marks[3 * c] = host_ms();
        call_t &chunk = chunk_calls[which];
        chunk = call;
        chunk.pre_staged = true;
        chunk.staged_queries = staged[2 * c];
        chunk.staged_candidates = staged[2 * c + 1];
        chunk.queries.count = chunk.candidates.count = cuts[c + 1] - cuts[c];
        chunk.out = call.out + cuts[c];
        chunk.scoring_after = context->copied[c];
        chunk.plan_after = !alphabet_pass ? context->offsets_copied : sampled ? context->copied[0] : context->copied[c];
        if (sampled) chunk.sample_queries = &staged[0], chunk.sample_candidates = &staged[1];
        chunk.plan_only = true;
        chunk_stats[which].graph_replays = 0;
        status_t const planned = run_on(engine, contexts[which], streams[which], chunk, schedule, chunk_stats[which]);
        launches += chunk_stats[which].last_launches;
        host_marks[3 * c + 1] = host_ms();
        return planned;
    };
    auto launch = [&](int c) -> status_t { // queues the scoring of chunk c's plan, without waiting for it
        int const which = c % depth;
        call_t &chunk = chunk_calls[which];
        chunk.plan_only = false, chunk.reuse_plan = true;
        status_t const queued = run_on(engine, contexts[which], streams[which], chunk, schedule, chunk_stats[which], true);
        if (!queued.ok()) return queued;
        in_flight[which] = c;
        cells += chunk_stats[which].last_cells, graph_replays += chunk_stats[which].graph_replays;
        host_marks[3 * c + 2] = host_ms();
        return {};
    };
    int const window = plan_ahead ? depth : 1;
    for (int c = 0; c < std::min(window, chunks) && status.ok(); ++c) status = plan(c);
    for (int c = 0; c < std::min(window, chunks) && status.ok(); ++c) status = launch(c);
    for (int c = std::min(window, chunks); c < chunks && status.ok(); ++c) {
        status = plan(c);
        if (status.ok()) status = launch(c);
    }
    for (int which = 0; which < depth; ++which) {
        status_t const settled = settle(which);
        if (status.ok()) status = settled;
    }
    if (!status.ok()) {
        cudaStreamSynchronize(context->copy_stream);
        for (int which = 0; which < depth; ++which) cudaStreamSynchronize(streams[which]);
        cudaStreamSynchronize(stream);
        return status;
    }
    for (int which = 0; which < depth; ++which) {
        SZS_TRY_CUDA(cudaEventRecord(contexts[which]->stop, streams[which]));
        SZS_TRY_CUDA(cudaStreamWaitEvent(stream, contexts[which]->stop, 0));
    }
    SZS_TRY_CUDA(cudaEventRecord(context->pipe_stop, stream));
    SZS_TRY_CUDA(cudaEventSynchronize(context->pipe_stop));
    float elapsed = 0;
    cudaEventElapsedTime(&elapsed, context->pipe_start, context->pipe_stop);
    if (tracing) { // the host's side of the timeline, in ms from the call's start
        std::fprintf(stderr, "[szs_gb300] host: copies queued %8.3f, call returns %8.3f\n", copies_queued_ms, host_ms());
        for (int c = 0; c < chunks; ++c)
            std::fprintf(stderr, "[szs_gb300] host: chunk %3d  plan queued %8.3f  read back %8.3f  scoring queued %8.3f\n",
                         c, host_marks[3 * c], host_marks[3 * c + 1], host_marks[3 * c + 2]);
    }
    stats.last_pairs = pairs, stats.last_cells = cells, stats.last_launches = launches;
    stats.last_call_ms = elapsed, stats.last_compute_ms = compute_ms;
    stats.kernel_launches += launches, stats.graph_replays += graph_replays;
    return {};
}

static status_t run_call(engine_t &engine, void *scope_handle, call_t const &call) noexcept {
    int device = 0;
    cudaStream_t stream = nullptr;
    device_context_t *context = nullptr;
    status_t status = resolve_scope(scope_handle, device, stream, engine.devices, context);
    if (!status.ok()) return status;
    if (call.mode == mode_pairwise_k && call.queries.count == call.candidates.count && call.queries.count > 1 &&
        !call.pre_staged && !engine.utf8 && pinned_host(call.queries.offsets) && pinned_host(call.candidates.offsets) &&
        pinned_host(call.queries.data) && pinned_host(call.candidates.data) && pinned_host(call.out)) {
        std::uint64_t const bytes = (host_offset(call.queries, call.queries.count) - host_offset(call.queries, 0)) +
                                    (host_offset(call.candidates, call.candidates.count) - host_offset(call.candidates, 0));
        std::size_t const chunk_bytes = engine.tuning.pipeline_chunk_kb
                                            ? std::size_t(engine.tuning.pipeline_chunk_kb) << 10
                                            : pipeline_chunk_bytes_k;
        if (bytes >= 2 * chunk_bytes)
            return run_pipelined(engine, context, stream, call, engine.schedule, engine.stats, chunk_bytes);
    }
    return run_on(engine, context, stream, call, engine.schedule, engine.stats);
}

/* ---- execution contexts for callers that run one engine from several threads (the serving loop) ---------------- */

struct exec_context_t {
    device_context_t context;
    szs_gb300_stats_t stats {};
};

sz_status_t exec_context_create(int device, void **out, char const **error_message) noexcept {
    if (device < 0 || device >= visible_devices()) return report({sz_missing_gpu_k, nullptr}, error_message);
    auto *exec = new (std::nothrow) exec_context_t();
    if (!exec) return report({sz_bad_alloc_k, nullptr}, error_message);
    status_t const status = exec->context.prepare(device);
    if (!status.ok()) {
        exec->context.release();
        delete exec;
        return report(status, error_message);
    }
    *out = exec;
    return report({}, error_message);
}

void exec_context_free(void *handle) noexcept {
    auto *exec = static_cast<exec_context_t *>(handle);
    if (!exec) return;
    exec->context.release();
    delete exec;
}

cudaStream_t exec_context_stream(void *handle) noexcept { return static_cast<exec_context_t *>(handle)->context.own_stream; }

szs_gb300_stats_t const &exec_context_stats(void *handle) noexcept { return static_cast<exec_context_t *>(handle)->stats; }

/** Pairwise scores of device-resident u64 tapes into device-resident `results`, on the context's stream. */
sz_status_t exec_pairwise(void *engine_handle, void *handle, sz_sequence_u64tape_t const *first,
                          sz_sequence_u64tape_t const *second, std::int64_t *results, int schedule,
                          char const **error_message) noexcept {
    auto *exec = static_cast<exec_context_t *>(handle);
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine || !exec) return report({sz_status_unknown_k, "Invalid engine or execution context"}, error_message);
    if (!first || !second) return report({sz_unexpected_dimensions_k, nullptr}, error_message);
    cudaError_t const selected = cudaSetDevice(exec->context.device);
    if (selected != cudaSuccess) return report(from_cuda(selected), error_message);
    auto view = [](sz_sequence_u64tape_t const *tape) {
        tape_view_t v;
        v.data = tape->data, v.offsets = tape->offsets, v.count = tape->count, v.offset_bits = 64;
        return v;
    };
    call_t call;
    call.queries = view(first);
    call.candidates = view(second);
    call.has_candidates = true;
    call.mode = mode_pairwise_k;
    call.out = results;
    call.stride = 1;
    return report(run_on(*engine, &exec->context, exec->context.own_stream, call, schedule, exec->stats),
                  error_message);
}

bool engine_handle_valid(void *engine_handle) noexcept { return as_engine(engine_handle, -1) != nullptr; }

/** The band kernels' wait bounds from the tuning: 0 keeps the built-in bounds, a smaller value lowers both (the
 *  barrier keeps four times the ring wait's polls), a larger one is clamped to the built-in bounds. */
static void apply_wait_bounds(engine_t &engine) noexcept {
    std::uint32_t const polls = engine.tuning.band_wait_polls;
    engine.costs.wait_polls = polls ? std::min(polls, band_wait_polls_default_k) : band_wait_polls_default_k;
    engine.costs.barrier_polls =
        polls ? (std::uint32_t)std::min<std::uint64_t>(4ull * polls, band_barrier_polls_default_k)
              : band_barrier_polls_default_k;
}

sz_status_t set_tuning(void *engine_handle, szs_gb300_tuning_t const *tuning, char const **error_message) noexcept {
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (!tuning) {
        engine->tuning = szs_gb300_tuning_t {};
        apply_wait_bounds(*engine);
        return report({}, error_message);
    }
    for (int k = 0; k < 16; ++k) {
        int const rows = tuning->packed_rows[k], bits = tuning->cell_bits[k];
        if (rows != 0 && rows != 4 && rows != 8 && rows != 12 && rows != 16)
            return report({sz_unexpected_dimensions_k, "Rows per lane must be 0, 4, 8, 12 or 16"}, error_message);
        if (bits != 0 && bits != 32 && bits != 64)
            return report({sz_unexpected_dimensions_k, "Cell bits must be 0, 32 or 64"}, error_message);
    }
    for (int choice = 0; choice < 4; ++choice)
        if (tuning->packed_warps[choice] > 8)
            return report({sz_unexpected_dimensions_k, "Warps per CTA must be at most 8"}, error_message);
    engine->tuning = *tuning;
    apply_wait_bounds(*engine);
    return report({}, error_message);
}

sz_status_t get_tuning(void *engine_handle, szs_gb300_tuning_t *tuning, char const **error_message) noexcept {
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine || !tuning) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    *tuning = engine->tuning;
    return report({}, error_message);
}

} // namespace szs_gb300

using namespace szs_gb300;

/* ---- C-ABI ------------------------------------------------------------------------------------------------------ */

namespace {

tape_view_t view_of(sz_sequence_u32tape_t const *tape) {
    tape_view_t v;
    v.data = tape->data, v.offsets = tape->offsets, v.count = tape->count, v.offset_bits = 32;
    return v;
}
tape_view_t view_of(sz_sequence_u64tape_t const *tape) {
    tape_view_t v;
    v.data = tape->data, v.offsets = tape->offsets, v.count = tape->count, v.offset_bits = 64;
    return v;
}

template <typename tape_type_>
sz_status_t score_cross(int kind, void *engine_handle, void *scope, tape_type_ const *queries,
                        tape_type_ const *candidates, void *results, sz_size_t stride, char const **error_message,
                        bool utf8 = false) {
    engine_t *engine = as_engine(engine_handle, kind);
    if (!engine || engine->utf8 != utf8) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (!queries || !results) return report({sz_unexpected_dimensions_k, "Queries and results must not be NULL"},
                                            error_message);
    call_t call;
    call.queries = view_of(queries);
    call.has_candidates = candidates != nullptr;
    if (candidates) call.candidates = view_of(candidates);
    call.mode = candidates ? mode_cross_k : mode_symmetric_k;
    call.out = static_cast<std::int64_t *>(results);
    call.stride = stride;
    std::size_t const columns = candidates ? candidates->count : queries->count;
    if (queries->count > 0 && columns > 0 && stride < columns)
        return report({sz_unexpected_dimensions_k, "results_row_stride is smaller than the candidates count"},
                      error_message);
    return report(run_call(*engine, scope, call), error_message);
}

sz_status_t score_cross_sequence(int kind, void *engine_handle, void *scope, sz_sequence_t const *queries,
                                 sz_sequence_t const *candidates, void *results, sz_size_t stride,
                                 char const **error_message, bool utf8 = false) {
    engine_t *engine = as_engine(engine_handle, kind);
    if (!engine || engine->utf8 != utf8) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (!queries || !results) return report({sz_unexpected_dimensions_k, "Queries and results must not be NULL"},
                                            error_message);
    gathered_tape_t q, c;
    status_t status = gather_sequence(queries, q);
    if (status.ok() && candidates) status = gather_sequence(candidates, c);
    if (!status.ok()) return report(status, error_message);
    call_t call;
    call.queries = q.view();
    call.has_candidates = candidates != nullptr;
    if (candidates) call.candidates = c.view();
    call.mode = candidates ? mode_cross_k : mode_symmetric_k;
    call.out = static_cast<std::int64_t *>(results);
    call.stride = stride;
    std::size_t const columns = candidates ? candidates->count : queries->count;
    if (queries->count > 0 && columns > 0 && stride < columns)
        return report({sz_unexpected_dimensions_k, "results_row_stride is smaller than the candidates count"},
                      error_message);
    return report(run_call(*engine, scope, call), error_message);
}

template <typename tape_type_>
sz_status_t score_pairwise(int kind, void *engine_handle, void *scope, tape_type_ const *first,
                           tape_type_ const *second, void *results, char const **error_message) {
    engine_t *engine = as_engine(engine_handle, kind);
    if (!engine) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (!first || !second || !results)
        return report({sz_unexpected_dimensions_k, "Inputs and results must not be NULL"}, error_message);
    if (first->count != second->count)
        return report({sz_unexpected_dimensions_k, "Pairwise inputs must hold the same count"}, error_message);
    call_t call;
    call.queries = view_of(first);
    call.candidates = view_of(second);
    call.has_candidates = true;
    call.mode = mode_pairwise_k;
    call.out = static_cast<std::int64_t *>(results);
    call.stride = 1;
    return report(run_call(*engine, scope, call), error_message);
}

sz_status_t create_engine(int kind, int match, int mismatch, int open, int extend, std::uint8_t const *byte_to_class,
                          std::int8_t const *table, void **engine_out, char const **error_message) {
    if (!engine_out) return report({sz_status_unknown_k, "Engine output pointer must not be NULL"}, error_message);
    if (*engine_out) return report({sz_status_unknown_k, "Engine must be uninitialized (NULL) on entry"}, error_message);
    if (kind == kind_levenshtein_k && (match < 0 || mismatch < 0 || open < 0 || extend < 0))
        return report({sz_overflow_risk_k, "Levenshtein costs must be non-negative"}, error_message);
    if (kind != kind_levenshtein_k && (!byte_to_class || !table))
        return report({sz_unexpected_dimensions_k, "Substitution tables must not be NULL"}, error_message);
    engine_t *engine = new (std::nothrow) engine_t();
    if (!engine) return report({sz_bad_alloc_k, "Failed to allocate the engine"}, error_message);
    engine->kind = kind;
    score_costs_t &costs = engine->costs;
    std::memset(&costs, 0, sizeof(costs));
    apply_wait_bounds(*engine);
    costs.kind = kind;
    costs.open = open, costs.extend = extend;
    costs.affine = open != extend; // `open == extend` selects the linear engine, as the reference's init does
    costs.match = match, costs.mismatch = mismatch;
    int magnitude = std::max(cost_abs(open), cost_abs(extend));
    if (kind == kind_levenshtein_k) {
        magnitude = std::max({magnitude, cost_abs(match), cost_abs(mismatch)});
        costs.classes = 0;
        engine->unit_levenshtein = match == 0 && mismatch == 1 && open == 1 && extend == 1;
    }
    else {
        prepare_class_costs(costs, byte_to_class, table);
        for (int i = 0; i < 1024; ++i) magnitude = std::max(magnitude, cost_abs(table[i]));
    }
    engine->magnitude = std::max(magnitude, 1);
    engine->packed_profile_fits = packed_profile_fits(costs);
    if (kind == kind_smith_waterman_k && open <= 0 && extend <= 0) {
        // The bound of a local score: every used substitution cost, at most, per diagonal step.
        bool used[32] = {};
        for (int b = 0; b < 256; ++b) used[byte_to_class[b] & 31] = true;
        int gain = 0;
        for (int row = 0; row < 32; ++row)
            for (int column = 0; column < 32; ++column)
                if (used[row] && used[column]) gain = std::max(gain, (int)table[row * 32 + column]);
        engine->local_gain = gain;
        costs.local_limit16 = 32767 - gain;
    }
    *engine_out = engine;
    return report({}, error_message);
}

/** A Needleman-Wunsch or Smith-Waterman engine over a dense 256 x 256 table (see the header's extension). */
sz_status_t create_dense_engine(int kind, int open, int extend, std::int8_t const *table, void **engine_out,
                                char const **error_message) {
    if (!engine_out) return report({sz_status_unknown_k, "Engine output pointer must not be NULL"}, error_message);
    if (*engine_out) return report({sz_status_unknown_k, "Engine must be uninitialized (NULL) on entry"}, error_message);
    if (!table) return report({sz_unexpected_dimensions_k, "The dense table must not be NULL"}, error_message);
    engine_t *engine = new (std::nothrow) engine_t();
    if (!engine) return report({sz_bad_alloc_k, "Failed to allocate the engine"}, error_message);
    engine->kind = kind;
    engine->dense.assign(table, table + 256 * 256);
    static std::atomic<std::uint64_t> dense_ids {0};
    engine->dense_id = ++dense_ids;
    score_costs_t &costs = engine->costs;
    std::memset(&costs, 0, sizeof(costs));
    apply_wait_bounds(*engine);
    costs.kind = kind;
    costs.open = open, costs.extend = extend;
    costs.affine = open != extend;
    costs.classes = 1; // replaced per call by the batch's own codes
    int magnitude = std::max(cost_abs(open), cost_abs(extend));
    int shift = costs.affine ? open : 0, gain = 0;
    bool fits = true;
    for (int i = 0; i < 256 * 256; ++i) {
        int const cost = table[i];
        magnitude = std::max(magnitude, cost_abs(cost));
        gain = std::max(gain, cost);
        fits = fits && cost - shift >= -128 && cost - shift <= 127;
    }
    engine->magnitude = std::max(magnitude, 1);
    engine->packed_profile_fits = fits;
    if (kind == kind_smith_waterman_k && open <= 0 && extend <= 0) {
        engine->local_gain = gain;
        costs.local_limit16 = 32767 - gain;
    }
    *engine_out = engine;
    return report({}, error_message);
}

void free_engine(void *handle) {
    engine_t *engine = as_engine(handle, -1);
    if (!engine) return;
    engine->magic = 0;
    delete engine;
}

/* ---- fingerprints ----------------------------------------------------------------------------------------------- */

constexpr std::uint32_t fingerprint_magic_k = 0x50524746u;

/** A Min-Hash engine: per-dimension parameters on the host, uploaded once per device. */
struct fingerprint_engine_t {
    std::uint32_t magic = fingerprint_magic_k;
    std::uint32_t dimensions = 0;
    std::vector<fingerprint_dim_t> params;
    device_context_t devices[max_devices_k];
    device_buffer_t params_device[max_devices_k];
    device_buffer_t outputs[max_devices_k];
    ~fingerprint_engine_t() {
        for (int d = 0; d < max_devices_k; ++d) {
            if (!devices[d].ready) continue;
            cudaSetDevice(d);
            params_device[d].release();
            outputs[d].release();
            devices[d].release();
        }
    }
};

fingerprint_engine_t *as_fingerprints(void *handle) {
    auto *engine = static_cast<fingerprint_engine_t *>(handle);
    return engine && engine->magic == fingerprint_magic_k ? engine : nullptr;
}

/**
 *  Dimension d's window width follows the reference's layout (c/stringzillas/fingerprints.cuh:44-139): when every
 *  width gets a whole number of 64-dimension slices, slice k has width `widths[k % count]`; otherwise dimension d
 *  has width `widths[d % count]`. Parameters are seeded by the dimension's index either way.
 */
sz_status_t create_fingerprints(std::size_t dimensions, std::size_t alphabet_size, std::size_t const *widths,
                                std::size_t widths_count, std::uint64_t seed, void **engine_out,
                                char const **error_message) {
    if (!engine_out) return report({sz_status_unknown_k, "Engine output pointer must not be NULL"}, error_message);
    if (*engine_out) return report({sz_status_unknown_k, "Engine must be uninitialized (NULL) on entry"}, error_message);
    static std::size_t const default_widths[] = {3, 4, 5, 7, 9, 11, 15, 31};
    if (!widths || !widths_count) widths = default_widths, widths_count = 8;
    if (!dimensions || dimensions > 0xFFFFFFFFull)
        return report({sz_unexpected_dimensions_k, "Fingerprints need between 1 and 2^32 - 1 dimensions"},
                      error_message);
    for (std::size_t i = 0; i < widths_count; ++i)
        if (!widths[i]) return report({sz_unexpected_dimensions_k, "Window widths must be positive"}, error_message);
    (void)alphabet_size; // the reference's double-precision hasher does not use it
    auto *engine = new (std::nothrow) fingerprint_engine_t();
    if (!engine) return report({sz_bad_alloc_k, "Failed to allocate the engine"}, error_message);
    engine->dimensions = (std::uint32_t)dimensions;
    bool const sliced = dimensions % widths_count == 0 && (dimensions / widths_count) % 64 == 0;
    engine->params.resize(dimensions);
    for (std::size_t d = 0; d < dimensions; ++d)
        engine->params[d] = fingerprint_dimension(d, widths[(sliced ? d / 64 : d) % widths_count], seed);
    *engine_out = engine;
    return report({}, error_message);
}

void free_fingerprints(void *handle) {
    fingerprint_engine_t *engine = as_fingerprints(handle);
    if (!engine) return;
    engine->magic = 0;
    delete engine;
}

sz_status_t fingerprint_call(void *engine_handle, void *scope_handle, tape_view_t const &texts,
                             std::uint32_t *hashes, std::size_t hashes_stride, std::uint32_t *counts,
                             std::size_t counts_stride, char const **error_message) {
    fingerprint_engine_t *engine = as_fingerprints(engine_handle);
    if (!engine) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    std::size_t const row_bytes = (std::size_t)engine->dimensions * 4;
    if (texts.count && (!hashes || !counts))
        return report({sz_unexpected_dimensions_k, "Outputs must not be NULL"}, error_message);
    if (texts.count && (hashes_stride < row_bytes || counts_stride < row_bytes))
        return report({sz_unexpected_dimensions_k, "Output strides (bytes) are smaller than a row"}, error_message);
    int device = 0;
    cudaStream_t stream = nullptr;
    device_context_t *context = nullptr;
    status_t status = resolve_scope(scope_handle, device, stream, engine->devices, context);
    if (!status.ok()) return report(status, error_message);
    if (!texts.count) return report({}, error_message);
    // Inputs.
    staging_plan_t plan;
    status = plan_staging(texts, plan, stream);
    if (!status.ok()) return report(status, error_message);
    status = context->inputs.reserve(align_up(plan.offsets_bytes, 256) + align_up(plan.data_bytes, 256) + 512, stream);
    if (!status.ok()) return report(status, error_message);
    tape_t staged;
    status = stage_tape(texts, plan, static_cast<unsigned char *>(context->inputs.data), staged, stream);
    if (!status.ok()) return report(status, error_message);
    // Parameters, once per device.
    device_buffer_t &params = engine->params_device[device];
    std::size_t const params_bytes = engine->params.size() * sizeof(fingerprint_dim_t);
    if (params.bytes < params_bytes) {
        status = params.reserve(params_bytes, stream);
        if (!status.ok()) return report(status, error_message);
        cudaError_t const copied = cudaMemcpyAsync(params.data, engine->params.data(), params_bytes,
                                                   cudaMemcpyHostToDevice, stream);
        if (copied != cudaSuccess) return report(from_cuda(copied), error_message);
    }
    // Outputs: in place when device-reachable, else through a dense device buffer and 2-D copies.
    bool const hashes_on_device = device_accessible(hashes), counts_on_device = device_accessible(counts);
    std::uint32_t *hashes_target = hashes, *counts_target = counts;
    std::size_t hashes_pitch = hashes_stride, counts_pitch = counts_stride;
    std::size_t const dense_bytes = align_up(texts.count * row_bytes, 256);
    if (!hashes_on_device || !counts_on_device) {
        status = engine->outputs[device].reserve(2 * dense_bytes, stream);
        if (!status.ok()) return report(status, error_message);
        auto *area = static_cast<unsigned char *>(engine->outputs[device].data);
        if (!hashes_on_device) hashes_target = reinterpret_cast<std::uint32_t *>(area), hashes_pitch = row_bytes;
        if (!counts_on_device)
            counts_target = reinterpret_cast<std::uint32_t *>(area + dense_bytes), counts_pitch = row_bytes;
    }
    cudaError_t error = launch_fingerprints(staged, static_cast<fingerprint_dim_t const *>(params.data),
                                            engine->dimensions, hashes_target, hashes_pitch, counts_target,
                                            counts_pitch, context->sm_count, stream);
    if (error == cudaSuccess && !hashes_on_device)
        error = cudaMemcpy2DAsync(hashes, hashes_stride, hashes_target, row_bytes, row_bytes, texts.count,
                                  cudaMemcpyDeviceToHost, stream);
    if (error == cudaSuccess && !counts_on_device)
        error = cudaMemcpy2DAsync(counts, counts_stride, counts_target, row_bytes, row_bytes, texts.count,
                                  cudaMemcpyDeviceToHost, stream);
    if (error == cudaSuccess) error = cudaStreamSynchronize(stream);
    if (error != cudaSuccess) return report(from_cuda(error), error_message);
    return report({}, error_message);
}

} // namespace

extern "C" {

SZS_GB300_API int szs_version_major(void) { return 5; }
SZS_GB300_API int szs_version_minor(void) { return 3; }
SZS_GB300_API int szs_version_patch(void) { return 2; }

SZS_GB300_API sz_capability_t szs_capabilities_comptime(void) { return sz_caps_ckh_k; }
SZS_GB300_API sz_capability_t szs_capabilities_runtime(void) {
    return visible_devices() > 0 ? sz_caps_ckh_k : sz_caps_none_k;
}
SZS_GB300_API sz_capability_t szs_capabilities(void) {
    static std::once_flag once;
    static sz_capability_t cached = sz_caps_none_k;
    std::call_once(once, [] { cached = (sz_capability_t)(szs_capabilities_comptime() & szs_capabilities_runtime()); });
    return cached;
}

static void *unified_allocate_(sz_size_t size, void *) { return szs_unified_alloc(size); }
static void unified_free_(void *p, sz_size_t size, void *) { szs_unified_free(p, size); }

SZS_GB300_API sz_status_t sz_memory_allocator_init_unified(sz_memory_allocator_t *alloc, char const **error_message) {
    if (!alloc) return report({sz_status_unknown_k, "Allocator must not be NULL"}, error_message);
    alloc->allocate = &unified_allocate_;
    alloc->free = &unified_free_;
    alloc->handle = nullptr;
    return report({}, error_message);
}

SZS_GB300_API void *szs_unified_alloc(sz_size_t size_bytes) {
    void *p = nullptr;
    if (cudaMallocManaged(&p, size_bytes ? size_bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
SZS_GB300_API void szs_unified_free(void *ptr, sz_size_t) {
    if (ptr) cudaFree(ptr);
}

SZS_GB300_API sz_status_t szs_device_scope_init_default(szs_device_scope_t *scope, char const **error_message) {
    if (!scope) return report({sz_status_unknown_k, "Scope must not be NULL"}, error_message);
    auto *s = new (std::nothrow) scope_t();
    if (!s) return report({sz_bad_alloc_k, "Failed to allocate device scope"}, error_message);
    *scope = s;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_device_scope_init_cpu_cores(sz_size_t cpu_cores, szs_device_scope_t *scope,
                                                          char const **error_message) {
    if (!scope) return report({sz_status_unknown_k, "Scope must not be NULL"}, error_message);
    // One core is the default scope, as in the reference (c/stringzillas/runtime.cuh:85-90).
    if (cpu_cores == 1) return szs_device_scope_init_default(scope, error_message);
    auto *s = new (std::nothrow) scope_t();
    if (!s) return report({sz_bad_alloc_k, "Failed to allocate device scope"}, error_message);
    s->kind = scope_cpu_k;
    s->cpu_cores = cpu_cores;
    *scope = s;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_device_scope_init_gpu_device(sz_size_t gpu_device, szs_device_scope_t *scope,
                                                           char const **error_message) {
    if (!scope) return report({sz_status_unknown_k, "Scope must not be NULL"}, error_message);
    if ((int)gpu_device >= visible_devices() || gpu_device >= (sz_size_t)max_devices_k)
        return report({sz_missing_gpu_k, nullptr}, error_message);
    auto *s = new (std::nothrow) scope_t();
    if (!s) return report({sz_bad_alloc_k, "Failed to allocate device scope"}, error_message);
    s->kind = scope_gpu_k;
    s->device = (int)gpu_device;
    if (cudaSetDevice(s->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaError_t const error = cudaGetLastError();
        delete s;
        return report(from_cuda(error == cudaSuccess ? cudaErrorUnknown : error), error_message);
    }
    *scope = s;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_device_scope_get_cpu_cores(szs_device_scope_t scope, sz_size_t *cpu_cores,
                                                         char const **error_message) {
    scope_t *s = as_scope(scope);
    if (!s || !cpu_cores) return report({sz_status_unknown_k, "Invalid device scope handle"}, error_message);
    if (s->kind == scope_gpu_k) return report({sz_device_code_mismatch_k, nullptr}, error_message);
    *cpu_cores = s->kind == scope_cpu_k ? s->cpu_cores : 1;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_device_scope_get_gpu_device(szs_device_scope_t scope, sz_size_t *gpu_device,
                                                          char const **error_message) {
    scope_t *s = as_scope(scope);
    if (!s || !gpu_device) return report({sz_status_unknown_k, "Invalid device scope handle"}, error_message);
    if (s->kind != scope_gpu_k) return report({sz_device_code_mismatch_k, nullptr}, error_message);
    *gpu_device = (sz_size_t)s->device;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_device_scope_get_capabilities(szs_device_scope_t scope, sz_capability_t *capabilities,
                                                            char const **error_message) {
    scope_t *s = as_scope(scope);
    if (!s || !capabilities) return report({sz_status_unknown_k, "Invalid device scope handle"}, error_message);
    if (s->kind == scope_cpu_k) *capabilities = (sz_capability_t)(sz_cap_serial_k | sz_cap_parallel_k);
    else if (s->kind == scope_gpu_k) *capabilities = sz_caps_ckh_k;
    else *capabilities = (sz_capability_t)(sz_cap_serial_k | szs_capabilities());
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_device_scope_init_stream(sz_size_t gpu_device, void *cuda_stream,
                                                             szs_device_scope_t *scope, char const **error_message) {
    if (!scope) return report({sz_status_unknown_k, "Scope must not be NULL"}, error_message);
    if ((int)gpu_device >= visible_devices() || gpu_device >= (sz_size_t)max_devices_k)
        return report({sz_missing_gpu_k, nullptr}, error_message);
    auto *s = new (std::nothrow) scope_t();
    if (!s) return report({sz_bad_alloc_k, "Failed to allocate device scope"}, error_message);
    s->kind = scope_gpu_k;
    s->device = (int)gpu_device;
    s->stream = static_cast<cudaStream_t>(cuda_stream);
    s->borrowed_stream = true;
    *scope = s;
    return report({}, error_message);
}

SZS_GB300_API void szs_device_scope_free(szs_device_scope_t scope) {
    scope_t *s = as_scope(scope);
    if (!s) return;
    if (s->stream && !s->borrowed_stream) {
        cudaSetDevice(s->device);
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    s->magic = 0;
    delete s;
}

/* Levenshtein */

SZS_GB300_API sz_status_t szs_levenshtein_distances_init(sz_error_cost_t match, sz_error_cost_t mismatch,
                                                         sz_error_cost_t open, sz_error_cost_t extend,
                                                         sz_memory_allocator_t const *, sz_capability_t,
                                                         szs_levenshtein_distances_t *engine,
                                                         char const **error_message) {
    return create_engine(kind_levenshtein_k, match, mismatch, open, extend, nullptr, nullptr, engine, error_message);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances(szs_levenshtein_distances_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                    sz_size_t *results, sz_size_t results_row_stride,
                                                    char const **error_message) {
    return score_cross_sequence(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                                error_message);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_u32tape(szs_levenshtein_distances_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u32tape_t const *queries,
                                                            sz_sequence_u32tape_t const *candidates,
                                                            sz_size_t *results, sz_size_t results_row_stride,
                                                            char const **error_message) {
    return score_cross(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_u64tape(szs_levenshtein_distances_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u64tape_t const *queries,
                                                            sz_sequence_u64tape_t const *candidates,
                                                            sz_size_t *results, sz_size_t results_row_stride,
                                                            char const **error_message) {
    return score_cross(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API void szs_levenshtein_distances_free(szs_levenshtein_distances_t engine) { free_engine(engine); }

/* UTF-8 Levenshtein: code points instead of bytes (transcoded to one-byte codes on the device, see utf8.cu) */

SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_init(sz_error_cost_t match, sz_error_cost_t mismatch,
                                                              sz_error_cost_t open, sz_error_cost_t extend,
                                                              sz_memory_allocator_t const *, sz_capability_t,
                                                              szs_levenshtein_distances_utf8_t *engine,
                                                              char const **error_message) {
    sz_status_t const status =
        create_engine(kind_levenshtein_k, match, mismatch, open, extend, nullptr, nullptr, engine, error_message);
    if (status == sz_success_k) static_cast<engine_t *>(*engine)->utf8 = true;
    return status;
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8(szs_levenshtein_distances_utf8_t engine,
                                                         szs_device_scope_t device, sz_sequence_t const *queries,
                                                         sz_sequence_t const *candidates, sz_size_t *results,
                                                         sz_size_t results_row_stride, char const **error_message) {
    return score_cross_sequence(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                                error_message, true);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_u32tape(szs_levenshtein_distances_utf8_t engine,
                                                                 szs_device_scope_t device,
                                                                 sz_sequence_u32tape_t const *queries,
                                                                 sz_sequence_u32tape_t const *candidates,
                                                                 sz_size_t *results, sz_size_t results_row_stride,
                                                                 char const **error_message) {
    return score_cross(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message, true);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_u64tape(szs_levenshtein_distances_utf8_t engine,
                                                                 szs_device_scope_t device,
                                                                 sz_sequence_u64tape_t const *queries,
                                                                 sz_sequence_u64tape_t const *candidates,
                                                                 sz_size_t *results, sz_size_t results_row_stride,
                                                                 char const **error_message) {
    return score_cross(kind_levenshtein_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message, true);
}
SZS_GB300_API void szs_levenshtein_distances_utf8_free(szs_levenshtein_distances_utf8_t engine) {
    free_engine(engine);
}

/* Needleman-Wunsch */

SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_init(sz_u8_t const *byte_to_class,
                                                           sz_error_cost_t const *class_substitution_costs,
                                                           sz_error_cost_t open, sz_error_cost_t extend,
                                                           sz_memory_allocator_t const *, sz_capability_t,
                                                           szs_needleman_wunsch_scores_t *engine,
                                                           char const **error_message) {
    return create_engine(kind_needleman_wunsch_k, 0, 0, open, extend, byte_to_class, class_substitution_costs, engine,
                         error_message);
}
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores(szs_needleman_wunsch_scores_t engine, szs_device_scope_t device,
                                                      sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                      sz_ssize_t *results, sz_size_t results_row_stride,
                                                      char const **error_message) {
    return score_cross_sequence(kind_needleman_wunsch_k, engine, device, queries, candidates, results,
                                results_row_stride, error_message);
}
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_u32tape(szs_needleman_wunsch_scores_t engine,
                                                              szs_device_scope_t device,
                                                              sz_sequence_u32tape_t const *queries,
                                                              sz_sequence_u32tape_t const *candidates,
                                                              sz_ssize_t *results, sz_size_t results_row_stride,
                                                              char const **error_message) {
    return score_cross(kind_needleman_wunsch_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_u64tape(szs_needleman_wunsch_scores_t engine,
                                                              szs_device_scope_t device,
                                                              sz_sequence_u64tape_t const *queries,
                                                              sz_sequence_u64tape_t const *candidates,
                                                              sz_ssize_t *results, sz_size_t results_row_stride,
                                                              char const **error_message) {
    return score_cross(kind_needleman_wunsch_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API void szs_needleman_wunsch_scores_free(szs_needleman_wunsch_scores_t engine) { free_engine(engine); }

/* Smith-Waterman */

SZS_GB300_API sz_status_t szs_smith_waterman_scores_init(sz_u8_t const *byte_to_class,
                                                         sz_error_cost_t const *class_substitution_costs,
                                                         sz_error_cost_t open, sz_error_cost_t extend,
                                                         sz_memory_allocator_t const *, sz_capability_t,
                                                         szs_smith_waterman_scores_t *engine,
                                                         char const **error_message) {
    return create_engine(kind_smith_waterman_k, 0, 0, open, extend, byte_to_class, class_substitution_costs, engine,
                         error_message);
}
SZS_GB300_API sz_status_t szs_smith_waterman_scores(szs_smith_waterman_scores_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                    sz_ssize_t *results, sz_size_t results_row_stride,
                                                    char const **error_message) {
    return score_cross_sequence(kind_smith_waterman_k, engine, device, queries, candidates, results,
                                results_row_stride, error_message);
}
SZS_GB300_API sz_status_t szs_smith_waterman_scores_u32tape(szs_smith_waterman_scores_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u32tape_t const *queries,
                                                            sz_sequence_u32tape_t const *candidates,
                                                            sz_ssize_t *results, sz_size_t results_row_stride,
                                                            char const **error_message) {
    return score_cross(kind_smith_waterman_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API sz_status_t szs_smith_waterman_scores_u64tape(szs_smith_waterman_scores_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u64tape_t const *queries,
                                                            sz_sequence_u64tape_t const *candidates,
                                                            sz_ssize_t *results, sz_size_t results_row_stride,
                                                            char const **error_message) {
    return score_cross(kind_smith_waterman_k, engine, device, queries, candidates, results, results_row_stride,
                       error_message);
}
SZS_GB300_API void szs_smith_waterman_scores_free(szs_smith_waterman_scores_t engine) { free_engine(engine); }

/* Fingerprints: Min-Hash over rolling hashes (see fingerprints.cu) */

SZS_GB300_API sz_status_t szs_fingerprints_init(sz_size_t dimensions, sz_size_t alphabet_size,
                                                sz_size_t const *window_widths, sz_size_t window_widths_count,
                                                sz_u64_t seed, sz_memory_allocator_t const *, sz_capability_t,
                                                szs_fingerprints_t *engine, char const **error_message) {
    return create_fingerprints(dimensions, alphabet_size, window_widths, window_widths_count, seed, engine,
                               error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_sequence(szs_fingerprints_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *texts, sz_u32_t *min_hashes,
                                                    sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                    sz_size_t min_counts_stride, char const **error_message) {
    if (!texts) return report({sz_unexpected_dimensions_k, "Texts must not be NULL"}, error_message);
    gathered_tape_t gathered;
    status_t const status = gather_sequence(texts, gathered);
    if (!status.ok()) return report(status, error_message);
    return fingerprint_call(engine, device, gathered.view(), min_hashes, min_hashes_stride, min_counts,
                            min_counts_stride, error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_u64tape(szs_fingerprints_t engine, szs_device_scope_t device,
                                                   sz_sequence_u64tape_t const *texts, sz_u32_t *min_hashes,
                                                   sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                   sz_size_t min_counts_stride, char const **error_message) {
    if (!texts) return report({sz_unexpected_dimensions_k, "Texts must not be NULL"}, error_message);
    return fingerprint_call(engine, device, view_of(texts), min_hashes, min_hashes_stride, min_counts,
                            min_counts_stride, error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_u32tape(szs_fingerprints_t engine, szs_device_scope_t device,
                                                   sz_sequence_u32tape_t const *texts, sz_u32_t *min_hashes,
                                                   sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                   sz_size_t min_counts_stride, char const **error_message) {
    if (!texts) return report({sz_unexpected_dimensions_k, "Texts must not be NULL"}, error_message);
    return fingerprint_call(engine, device, view_of(texts), min_hashes, min_hashes_stride, min_counts,
                            min_counts_stride, error_message);
}
SZS_GB300_API void szs_fingerprints_free(szs_fingerprints_t engine) { free_fingerprints(engine); }

/* UTF-8 fingerprints hash the same bytes (the reference's c/stringzillas/fingerprints.cuh:181-222 forwards them) */

SZS_GB300_API sz_status_t szs_fingerprints_utf8_init(sz_size_t dimensions, sz_size_t alphabet_size,
                                                     sz_size_t const *window_widths, sz_size_t window_widths_count,
                                                     sz_u64_t seed, sz_memory_allocator_t const *alloc,
                                                     sz_capability_t capabilities, szs_fingerprints_utf8_t *engine,
                                                     char const **error_message) {
    return szs_fingerprints_init(dimensions, alphabet_size, window_widths, window_widths_count, seed, alloc,
                                 capabilities, engine, error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_utf8_sequence(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                         sz_sequence_t const *texts, sz_u32_t *min_hashes,
                                                         sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                         sz_size_t min_counts_stride, char const **error_message) {
    return szs_fingerprints_sequence(engine, device, texts, min_hashes, min_hashes_stride, min_counts,
                                     min_counts_stride, error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_utf8_u32tape(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                        sz_sequence_u32tape_t const *texts, sz_u32_t *min_hashes,
                                                        sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                        sz_size_t min_counts_stride, char const **error_message) {
    return szs_fingerprints_u32tape(engine, device, texts, min_hashes, min_hashes_stride, min_counts,
                                    min_counts_stride, error_message);
}
SZS_GB300_API sz_status_t szs_fingerprints_utf8_u64tape(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                        sz_sequence_u64tape_t const *texts, sz_u32_t *min_hashes,
                                                        sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                        sz_size_t min_counts_stride, char const **error_message) {
    return szs_fingerprints_u64tape(engine, device, texts, min_hashes, min_hashes_stride, min_counts,
                                    min_counts_stride, error_message);
}
SZS_GB300_API void szs_fingerprints_utf8_free(szs_fingerprints_utf8_t engine) { free_fingerprints(engine); }

/* Extensions */

SZS_GB300_API sz_status_t szs_levenshtein_distances_pairwise_u32tape(szs_levenshtein_distances_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u32tape_t const *first,
                                                                     sz_sequence_u32tape_t const *second,
                                                                     sz_size_t *results, char const **error_message) {
    return score_pairwise(kind_levenshtein_k, engine, device, first, second, results, error_message);
}
SZS_GB300_API sz_status_t szs_levenshtein_distances_pairwise_u64tape(szs_levenshtein_distances_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u64tape_t const *first,
                                                                     sz_sequence_u64tape_t const *second,
                                                                     sz_size_t *results, char const **error_message) {
    return score_pairwise(kind_levenshtein_k, engine, device, first, second, results, error_message);
}
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_pairwise_u32tape(szs_needleman_wunsch_scores_t engine,
                                                                       szs_device_scope_t device,
                                                                       sz_sequence_u32tape_t const *first,
                                                                       sz_sequence_u32tape_t const *second,
                                                                       sz_ssize_t *results,
                                                                       char const **error_message) {
    return score_pairwise(kind_needleman_wunsch_k, engine, device, first, second, results, error_message);
}
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_pairwise_u64tape(szs_needleman_wunsch_scores_t engine,
                                                                       szs_device_scope_t device,
                                                                       sz_sequence_u64tape_t const *first,
                                                                       sz_sequence_u64tape_t const *second,
                                                                       sz_ssize_t *results,
                                                                       char const **error_message) {
    return score_pairwise(kind_needleman_wunsch_k, engine, device, first, second, results, error_message);
}
SZS_GB300_API sz_status_t szs_smith_waterman_scores_pairwise_u32tape(szs_smith_waterman_scores_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u32tape_t const *first,
                                                                     sz_sequence_u32tape_t const *second,
                                                                     sz_ssize_t *results, char const **error_message) {
    return score_pairwise(kind_smith_waterman_k, engine, device, first, second, results, error_message);
}
SZS_GB300_API sz_status_t szs_smith_waterman_scores_pairwise_u64tape(szs_smith_waterman_scores_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u64tape_t const *first,
                                                                     sz_sequence_u64tape_t const *second,
                                                                     sz_ssize_t *results, char const **error_message) {
    return score_pairwise(kind_smith_waterman_k, engine, device, first, second, results, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_score_pairwise_noalloc_u64tape(void *engine_handle, szs_device_scope_t device,
                                                                   sz_sequence_u64tape_t const *first,
                                                                   sz_sequence_u64tape_t const *second, void *results,
                                                                   char const **error_message) {
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (!first || !second || !results)
        return report({sz_unexpected_dimensions_k, "Inputs and results must not be NULL"}, error_message);
    // Resolve the device and stream without touching the engine's per-device buffers (which would allocate).
    scope_t *scope = as_scope(device);
    if (device && !scope) return report({sz_status_unknown_k, "Invalid device scope handle"}, error_message);
    if (scope && scope->kind == scope_cpu_k) return report({sz_device_code_mismatch_k, nullptr}, error_message);
    if (!engine->dense.empty())
        return report({sz_unexpected_dimensions_k, "Dense-table engines need the planned entry points"}, error_message);
    static_call_t call;
    call.costs = &engine->costs;
    call.kind = engine->kind;
    call.magnitude = engine->magnitude;
    call.device = scope ? scope->device : 0;
    call.stream = scope && scope->kind == scope_gpu_k ? scope->stream : nullptr;
    if (call.device >= visible_devices()) return report({sz_missing_gpu_k, nullptr}, error_message);
    return static_scratch_pairwise(call, first, second, static_cast<std::int64_t *>(results), error_message);
}

SZS_GB300_API sz_status_t szs_gb300_engine_set_schedule(void *engine_handle, szs_gb300_schedule_t schedule,
                                                        char const **error_message) {
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    if (schedule != szs_gb300_schedule_batched_k && schedule != szs_gb300_schedule_plain_k)
        return report({sz_status_unknown_k, "Unknown schedule"}, error_message);
    engine->schedule = schedule;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_engine_get_stats(void *engine_handle, szs_gb300_stats_t *stats,
                                                     char const **error_message) {
    engine_t *engine = as_engine(engine_handle, -1);
    if (!engine || !stats) return report({sz_status_unknown_k, "Invalid engine handle"}, error_message);
    *stats = engine->stats;
    return report({}, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_needleman_wunsch_scores_init_dense(sz_error_cost_t const *costs,
                                                                       sz_error_cost_t open, sz_error_cost_t extend,
                                                                       sz_memory_allocator_t const *, sz_capability_t,
                                                                       szs_needleman_wunsch_scores_t *engine,
                                                                       char const **error_message) {
    return create_dense_engine(kind_needleman_wunsch_k, open, extend, costs, engine, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_smith_waterman_scores_init_dense(sz_error_cost_t const *costs,
                                                                     sz_error_cost_t open, sz_error_cost_t extend,
                                                                     sz_memory_allocator_t const *, sz_capability_t,
                                                                     szs_smith_waterman_scores_t *engine,
                                                                     char const **error_message) {
    return create_dense_engine(kind_smith_waterman_k, open, extend, costs, engine, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_engine_set_tuning(void *engine, szs_gb300_tuning_t const *tuning,
                                                      char const **error_message) {
    return set_tuning(engine, tuning, error_message);
}

SZS_GB300_API sz_status_t szs_gb300_engine_get_tuning(void *engine, szs_gb300_tuning_t *tuning,
                                                      char const **error_message) {
    return get_tuning(engine, tuning, error_message);
}

} // extern "C"
