/**
 *  @file server.cu
 *  @brief Serving loop: requests of mixed kind and size in, merged batches in a device-resident arena, results out.
 *
 *  The reference has no serving layer: every `szs_*` call is synchronous and scores one caller's batch
 *  (c/stringzillas/stringzillas.cuh:182-321). Here one admission thread and `lanes` lane threads share one device
 *  arena:
 *
 *  - Requests wait in arrival order. Whenever a lane is free, the admission thread takes the first waiting request
 *    (with `aging_ms` set: the smallest by cells, unless the oldest has waited that long - size-aware admission, so
 *    small requests are not queued behind large ones while no request starves)
 *    and every later waiting request of the same engine that still fits the batch caps (requests, pairs, cells) and
 *    the arena (continuous batching: whatever arrived while the other lanes were busy rides along; the cells cap
 *    keeps small requests out of a large request's batch), reserves one contiguous arena region
 *    for the merged batch and hands it to the lane. A batch that does not fit waits until a finishing batch returns
 *    its region (admission by HBM budget); a request larger than the whole arena fails alone.
 *  - A lane lays the batch out as one pair of u64 tapes over the region - offsets of all first strings, offsets of
 *    all second strings, results, then the first strings' bytes and the second strings' bytes back to back - and
 *    fills it without staging what needs none: the offsets (rebased onto the region) and the bytes of pageable host
 *    inputs go through a pinned host image, one copy per run of consecutive pageable requests; the bytes of pinned
 *    host inputs (Arrow or torch buffers in page-locked memory) are copied straight from the caller's buffers, and
 *    device or managed inputs device-to-device. It scores the batch with one planned pairwise call on its own stream
 *    and device context, and copies the results out. Lanes run concurrently, so several batches are on the
 *    device at once and their kernels overlap.
 *
 *  Every pair is scored by the same planned call as a direct `szs_*_pairwise_*` call, and the routes' results do not
 *  depend on which other pairs share the batch, so each request's results equal those of scoring it alone.
 */
#include "stringzillas_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

namespace szs_gb300 {

sz_status_t exec_context_create(int device, void **out, char const **error_message) noexcept;
void exec_context_free(void *handle) noexcept;
cudaStream_t exec_context_stream(void *handle) noexcept;
szs_gb300_stats_t const &exec_context_stats(void *handle) noexcept;
sz_status_t exec_pairwise(void *engine_handle, void *handle, sz_sequence_u64tape_t const *first,
                          sz_sequence_u64tape_t const *second, std::int64_t *results, int schedule,
                          char const **error_message) noexcept;
bool engine_handle_valid(void *engine_handle) noexcept;

namespace {

using steady_t = std::chrono::steady_clock;
constexpr std::uint32_t server_magic_k = 0x56524553u; // "SERV"

double ms_between(steady_t::time_point a, steady_t::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}
std::size_t align_up(std::size_t x, std::size_t a) { return (x + a - 1) / a * a; }

bool device_accessible(void const *pointer) {
    if (!pointer) return false;
    cudaPointerAttributes attributes;
    if (cudaPointerGetAttributes(&attributes, pointer) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attributes.type == cudaMemoryTypeDevice || attributes.type == cudaMemoryTypeManaged;
}

bool pinned_host(void const *pointer) {
    if (!pointer) return false;
    cudaPointerAttributes attributes;
    if (cudaPointerGetAttributes(&attributes, pointer) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attributes.type == cudaMemoryTypeHost;
}

/** One side of a request: its offsets (copied at submission) and where its bytes live. */
struct side_t {
    char const *data = nullptr;
    std::vector<std::uint64_t> offsets; // count + 1 entries, as the caller gave them
    bool on_device = false;
    bool pinned = false; // page-locked host memory: copied into the arena without staging
    std::uint64_t bytes() const { return offsets.back() - offsets.front(); }
};

struct request_t {
    std::uint64_t ticket = 0;
    void *engine = nullptr;
    side_t first, second;
    void *results = nullptr;
    bool results_on_device = false;
    std::uint64_t pairs = 0, cells = 0;
    steady_t::time_point submitted, admitted, finished;
    sz_status_t status = sz_success_k;
    bool done = false;
    std::uint64_t batch = 0, batch_requests = 0, batch_pairs = 0;
};

/** Byte layout of one batch inside its arena region. */
struct batch_layout_t {
    std::uint64_t pairs = 0;
    std::size_t first_offsets = 0, second_offsets = 0, results = 0, first_data = 0, second_data = 0, total = 0;
    static batch_layout_t of(std::uint64_t pairs, std::uint64_t first_bytes, std::uint64_t second_bytes) {
        batch_layout_t l;
        l.pairs = pairs;
        std::size_t const offsets_bytes = align_up((pairs + 1) * 8, 256);
        l.first_offsets = 0;
        l.second_offsets = offsets_bytes;
        l.results = 2 * offsets_bytes;
        l.first_data = l.results + align_up(pairs * 8, 256);
        l.second_data = l.first_data + align_up(first_bytes, 256);
        l.total = l.second_data + align_up(second_bytes, 256);
        return l;
    }
};

/** First-fit allocator over the arena's byte range, coalescing on free. */
struct arena_allocator_t {
    std::map<std::size_t, std::size_t> free_blocks; // offset -> size
    std::size_t capacity = 0, held = 0, peak = 0;
    void reset(std::size_t bytes) {
        capacity = bytes;
        free_blocks.clear();
        free_blocks[0] = bytes;
        held = peak = 0;
    }
    static constexpr std::size_t none_k = ~std::size_t(0);
    std::size_t allocate(std::size_t bytes) {
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second < bytes) continue;
            std::size_t const offset = it->first, size = it->second;
            free_blocks.erase(it);
            if (size > bytes) free_blocks[offset + bytes] = size - bytes;
            held += bytes;
            peak = std::max(peak, held);
            return offset;
        }
        return none_k;
    }
    void release(std::size_t offset, std::size_t bytes) {
        held -= bytes;
        auto next = free_blocks.lower_bound(offset);
        if (next != free_blocks.end() && offset + bytes == next->first) {
            bytes += next->second;
            next = free_blocks.erase(next);
        }
        if (next != free_blocks.begin()) {
            auto previous = std::prev(next);
            if (previous->first + previous->second == offset) {
                previous->second += bytes;
                return;
            }
        }
        free_blocks[offset] = bytes;
    }
};

struct batch_t {
    std::vector<request_t *> requests;
    void *engine = nullptr;
    batch_layout_t layout;
    std::size_t region = 0;
    std::uint64_t id = 0;
    std::uint64_t first_bytes = 0, second_bytes = 0;
};

struct server_t;

struct lane_t {
    server_t *server = nullptr;
    void *exec = nullptr;
    std::thread thread;
    std::unique_ptr<batch_t> work;
    void *staging = nullptr; // pinned, grow-only
    std::size_t staging_bytes = 0;
    cudaEvent_t start = nullptr, stop = nullptr;
    ~lane_t() {
        if (staging) cudaFreeHost(staging);
    }
    bool reserve_staging(std::size_t bytes) {
        if (bytes <= staging_bytes) return true;
        if (staging) cudaFreeHost(staging);
        staging = nullptr, staging_bytes = 0;
        if (cudaMallocHost(&staging, bytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        staging_bytes = bytes;
        return true;
    }
};

struct server_t {
    std::uint32_t magic = server_magic_k;
    szs_gb300_server_config_t config {};
    int device = 0;
    unsigned char *arena = nullptr;
    arena_allocator_t allocator;

    std::mutex mutex;
    std::condition_variable admission_cv; // new request, freed lane or region, stop
    std::condition_variable lane_cv;      // work handed to a lane, stop
    std::condition_variable done_cv;      // a request finished
    std::list<request_t *> waiting;
    std::unordered_map<std::uint64_t, request_t *> tickets;
    std::uint64_t next_ticket = 1, next_batch = 1;
    std::uint64_t arena_generation = 0, blocked_generation = ~0ull;
    std::vector<std::unique_ptr<lane_t>> lanes;
    std::vector<lane_t *> idle_lanes;
    std::size_t inflight = 0;
    bool stopping = false, lanes_stopping = false;
    std::thread admission;
    szs_gb300_server_stats_t stats {};

    void admit_loop();
    void lane_loop(lane_t *lane);
    sz_status_t run_batch(lane_t *lane, batch_t &batch);
    void finish(std::vector<request_t *> const &requests, sz_status_t status, std::uint64_t batch_id,
                std::uint64_t batch_pairs);
};

void server_t::finish(std::vector<request_t *> const &requests, sz_status_t status, std::uint64_t batch_id,
                      std::uint64_t batch_pairs) {
    auto const now = steady_t::now();
    for (request_t *request : requests) {
        request->status = status;
        request->finished = now;
        request->batch = batch_id;
        request->batch_requests = requests.size();
        request->batch_pairs = batch_pairs;
        request->done = true;
        ++stats.completed;
    }
    done_cv.notify_all();
}

void server_t::admit_loop() {
    std::unique_lock<std::mutex> lock(mutex);
    while (true) {
        admission_cv.wait(lock, [&] {
            if (stopping && waiting.empty()) return true;
            return !waiting.empty() && !idle_lanes.empty() && blocked_generation != arena_generation;
        });
        if (waiting.empty()) break; // stopping, nothing left

        // The batch's head: the oldest waiter, or under size-aware admission the smallest one unless the oldest has
        // waited past the aging bound.
        auto head = waiting.begin();
        if (config.aging_ms && ms_between(waiting.front()->submitted, steady_t::now()) < (double)config.aging_ms)
            head = std::min_element(waiting.begin(), waiting.end(),
                                    [](request_t const *a, request_t const *b) { return a->cells < b->cells; });
        // Merge: the head, then other waiters of the same engine in arrival order while the caps and the arena allow.
        auto batch = std::make_unique<batch_t>();
        batch->engine = (*head)->engine;
        std::uint64_t pairs = 0, first_bytes = 0, second_bytes = 0, cells = 0;
        std::size_t largest_free = 0;
        for (auto const &block : allocator.free_blocks) largest_free = std::max(largest_free, block.second);
        std::size_t const max_requests = config.max_batch_requests ? config.max_batch_requests : ~std::size_t(0);
        std::vector<std::list<request_t *>::iterator> taken;
        for (int pass = 0; pass < 2; ++pass)
        for (auto it = (pass == 0 ? head : waiting.begin()); it != waiting.end(); ++it) {
            if (pass == 0 && it != head) break; // the head first, alone
            if (pass == 1 && it == head) continue;
            request_t *request = *it;
            if (request->engine != batch->engine) continue;
            if (batch->requests.size() >= max_requests) break;
            std::uint64_t const grown_pairs = pairs + request->pairs;
            std::uint64_t const grown_first = first_bytes + request->first.bytes();
            std::uint64_t const grown_second = second_bytes + request->second.bytes();
            if (!batch->requests.empty()) {
                if (grown_pairs > config.max_batch_pairs) break;
                // The cells cap only holds while another lane is free to take the rest at once: under saturation
                // every request of the engine merges, which keeps the device full.
                if (cells + request->cells > config.max_batch_cells && idle_lanes.size() > 1) break;
                if (batch_layout_t::of(grown_pairs, grown_first, grown_second).total > largest_free) break;
            }
            batch->requests.push_back(request);
            taken.push_back(it);
            pairs = grown_pairs, first_bytes = grown_first, second_bytes = grown_second;
            cells += request->cells;
        }
        batch->layout = batch_layout_t::of(pairs, first_bytes, second_bytes);
        batch->first_bytes = first_bytes, batch->second_bytes = second_bytes;
        std::size_t const region = allocator.allocate(batch->layout.total);
        if (region == arena_allocator_t::none_k) {
            if (batch->layout.total > allocator.capacity || inflight == 0) {
                // Can never fit (or nothing in flight will ever free enough): fail the head alone.
                request_t *request = *head;
                waiting.erase(head);
                request->admitted = steady_t::now();
                finish({request}, sz_bad_alloc_k, 0, request->pairs);
                continue;
            }
            blocked_generation = arena_generation; // wait until a finishing batch returns its region
            continue;
        }
        batch->region = region;
        batch->id = next_batch++;
        auto const now = steady_t::now();
        for (request_t *request : batch->requests) request->admitted = now;
        for (auto it : taken) waiting.erase(it);
        lane_t *lane = idle_lanes.back();
        idle_lanes.pop_back();
        ++inflight;
        stats.peak_inflight = std::max<std::uint64_t>(stats.peak_inflight, inflight);
        stats.arena_peak_bytes = allocator.peak;
        lane->work = std::move(batch);
        lane_cv.notify_all();
    }
}

sz_status_t server_t::run_batch(lane_t *lane, batch_t &batch) {
    batch_layout_t const &layout = batch.layout;
    cudaStream_t const stream = exec_context_stream(lane->exec);
    unsigned char *region = arena + batch.region;

    // Host image of the region up to the end of the data: offsets of both sides, then the bytes of pageable host
    // inputs (the slots of other inputs stay unused in the image).
    std::size_t const image_bytes = layout.total;
    if (!lane->reserve_staging(image_bytes)) return sz_bad_alloc_k;
    auto *image = static_cast<unsigned char *>(lane->staging);
    auto *first_offsets = reinterpret_cast<std::uint64_t *>(image + layout.first_offsets);
    auto *second_offsets = reinterpret_cast<std::uint64_t *>(image + layout.second_offsets);
    std::uint64_t pair = 0, first_at = layout.first_data, second_at = layout.second_data;
    for (request_t *request : batch.requests) {
        std::uint64_t const first_base = request->first.offsets.front();
        std::uint64_t const second_base = request->second.offsets.front();
        for (std::uint64_t i = 0; i < request->pairs; ++i, ++pair) {
            first_offsets[pair] = first_at + (request->first.offsets[i] - first_base);
            second_offsets[pair] = second_at + (request->second.offsets[i] - second_base);
        }
        if (!request->first.on_device && !request->first.pinned && request->first.bytes())
            std::memcpy(image + first_at, request->first.data + first_base, request->first.bytes());
        if (!request->second.on_device && !request->second.pinned && request->second.bytes())
            std::memcpy(image + second_at, request->second.data + second_base, request->second.bytes());
        first_at += request->first.bytes();
        second_at += request->second.bytes();
    }
    first_offsets[pair] = first_at;
    second_offsets[pair] = second_at;

    if (cudaEventRecord(lane->start, stream) != cudaSuccess) return sz_status_unknown_k;
    // Offsets (results area skipped).
    if (cudaMemcpyAsync(region, image, layout.results, cudaMemcpyHostToDevice, stream) != cudaSuccess)
        return sz_status_unknown_k;
    // The bytes of each side: runs of consecutive pageable requests from the image, the others from their buffers.
    for (int which = 0; which < 2; ++which) {
        std::uint64_t at = which ? layout.second_data : layout.first_data, run_begin = at;
        auto flush = [&](std::uint64_t run_end) -> bool {
            bool const ok = run_end == run_begin || cudaMemcpyAsync(region + run_begin, image + run_begin,
                                                                    run_end - run_begin, cudaMemcpyHostToDevice,
                                                                    stream) == cudaSuccess;
            return ok;
        };
        for (request_t *request : batch.requests) {
            side_t const &side = which ? request->second : request->first;
            std::uint64_t const bytes = side.bytes();
            if ((side.on_device || side.pinned) && bytes) {
                if (!flush(at)) return sz_status_unknown_k;
                if (cudaMemcpyAsync(region + at, side.data + side.offsets.front(), bytes,
                                    side.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                    stream) != cudaSuccess)
                    return sz_status_unknown_k;
                run_begin = at + bytes;
            }
            at += bytes;
        }
        if (!flush(at)) return sz_status_unknown_k;
    }

    sz_sequence_u64tape_t first_tape {reinterpret_cast<sz_cptr_t>(region),
                                      reinterpret_cast<sz_u64_t const *>(region + layout.first_offsets),
                                      (sz_size_t)layout.pairs};
    sz_sequence_u64tape_t second_tape {reinterpret_cast<sz_cptr_t>(region),
                                       reinterpret_cast<sz_u64_t const *>(region + layout.second_offsets),
                                       (sz_size_t)layout.pairs};
    auto *results = reinterpret_cast<std::int64_t *>(region + layout.results);
    char const *message = nullptr;
    sz_status_t const status =
        exec_pairwise(batch.engine, lane->exec, &first_tape, &second_tape, results, config.schedule, &message);
    if (status != sz_success_k) return status;

    // Results: one copy into the image's (now free) offsets area, then out to each caller.
    auto *results_image = reinterpret_cast<std::int64_t *>(image);
    if (cudaMemcpyAsync(results_image, results, layout.pairs * 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return sz_status_unknown_k;
    pair = 0;
    for (request_t *request : batch.requests) {
        if (request->results_on_device &&
            cudaMemcpyAsync(request->results, results + pair, request->pairs * 8, cudaMemcpyDeviceToDevice, stream) !=
                cudaSuccess)
            return sz_status_unknown_k;
        pair += request->pairs;
    }
    if (cudaEventRecord(lane->stop, stream) != cudaSuccess) return sz_status_unknown_k;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return sz_status_unknown_k;
    pair = 0;
    for (request_t *request : batch.requests) {
        if (!request->results_on_device)
            std::memcpy(request->results, results_image + pair, request->pairs * 8);
        pair += request->pairs;
    }
    return sz_success_k;
}

void server_t::lane_loop(lane_t *lane) {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mutex);
    while (true) {
        lane_cv.wait(lock, [&] { return lane->work != nullptr || lanes_stopping; });
        if (!lane->work) break;
        std::unique_ptr<batch_t> batch = std::move(lane->work);
        lock.unlock();
        sz_status_t const status = run_batch(lane, *batch);
        float device_ms = 0;
        if (status == sz_success_k) cudaEventElapsedTime(&device_ms, lane->start, lane->stop);
        else cudaGetLastError();
        lock.lock();
        stats.batches += 1;
        stats.pairs += batch->layout.pairs;
        for (request_t *request : batch->requests) stats.cells += request->cells;
        stats.device_ms += device_ms;
        if (status == sz_success_k) stats.kernel_launches += exec_context_stats(lane->exec).last_launches;
        finish(batch->requests, status, batch->id, batch->layout.pairs);
        allocator.release(batch->region, batch->layout.total);
        ++arena_generation;
        --inflight;
        idle_lanes.push_back(lane);
        admission_cv.notify_all();
    }
}

server_t *as_server(void *handle) {
    auto *server = static_cast<server_t *>(handle);
    return server && server->magic == server_magic_k ? server : nullptr;
}

sz_status_t fail(sz_status_t status, char const *message, char const **error_message) {
    if (error_message) *error_message = message;
    return status;
}

/** Reads a tape's offsets into host memory (from host, managed or device memory). */
bool read_side(sz_sequence_u64tape_t const *tape, side_t &side) {
    side.data = tape->data;
    side.offsets.resize(tape->count + 1);
    if (cudaMemcpy(side.offsets.data(), tape->offsets, (tape->count + 1) * 8, cudaMemcpyDefault) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    side.on_device = device_accessible(tape->data);
    side.pinned = !side.on_device && pinned_host(tape->data);
    return true;
}

} // namespace
} // namespace szs_gb300

using namespace szs_gb300;

extern "C" {

SZS_GB300_API sz_status_t szs_gb300_server_init(szs_gb300_server_config_t const *config, szs_gb300_server_t *out,
                                                char const **error_message) {
    if (error_message) *error_message = nullptr;
    if (!config || !out) return fail(sz_unexpected_dimensions_k, "Config and output must not be NULL", error_message);
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || (int)config->gpu_device >= devices) {
        cudaGetLastError();
        return fail(sz_missing_gpu_k, "GPU device not available", error_message);
    }
    auto *server = new (std::nothrow) server_t();
    if (!server) return fail(sz_bad_alloc_k, "Failed to allocate the server", error_message);
    server->config = *config;
    if (!server->config.arena_bytes) server->config.arena_bytes = std::size_t(1) << 30;
    if (!server->config.lanes) server->config.lanes = 4;
    if (!server->config.max_batch_pairs) server->config.max_batch_pairs = std::size_t(1) << 22;
    if (!server->config.max_batch_cells) server->config.max_batch_cells = std::size_t(1) << 33;
    server->device = (int)config->gpu_device;
    if (cudaSetDevice(server->device) != cudaSuccess ||
        cudaMalloc(&server->arena, server->config.arena_bytes) != cudaSuccess) {
        cudaGetLastError();
        delete server;
        return fail(sz_bad_alloc_k, "Failed to allocate the device arena", error_message);
    }
    server->allocator.reset(server->config.arena_bytes);
    server->stats.arena_bytes = server->config.arena_bytes;
    for (std::size_t i = 0; i < server->config.lanes; ++i) {
        auto lane = std::make_unique<lane_t>();
        lane->server = server;
        sz_status_t const status = exec_context_create(server->device, &lane->exec, error_message);
        if (status != sz_success_k || cudaEventCreate(&lane->start) != cudaSuccess ||
            cudaEventCreate(&lane->stop) != cudaSuccess) {
            if (lane->exec) exec_context_free(lane->exec);
            server->lanes_stopping = server->stopping = true;
            szs_gb300_server_free(server);
            return status != sz_success_k ? status : fail(sz_status_unknown_k, "Failed to create lane events",
                                                          error_message);
        }
        server->idle_lanes.push_back(lane.get());
        server->lanes.push_back(std::move(lane));
    }
    for (auto &lane : server->lanes) lane->thread = std::thread(&server_t::lane_loop, server, lane.get());
    server->admission = std::thread(&server_t::admit_loop, server);
    *out = server;
    return sz_success_k;
}

SZS_GB300_API sz_status_t szs_gb300_server_submit(szs_gb300_server_t handle, void *engine,
                                                  sz_sequence_u64tape_t const *first,
                                                  sz_sequence_u64tape_t const *second, void *results,
                                                  sz_u64_t *ticket, char const **error_message) {
    if (error_message) *error_message = nullptr;
    server_t *server = as_server(handle);
    if (!server) return fail(sz_status_unknown_k, "Invalid server handle", error_message);
    if (!engine_handle_valid(engine)) return fail(sz_status_unknown_k, "Invalid engine handle", error_message);
    if (!first || !second || !ticket) return fail(sz_unexpected_dimensions_k, "Inputs must not be NULL", error_message);
    if (first->count != second->count)
        return fail(sz_unexpected_dimensions_k, "Pairwise tapes must have the same count", error_message);
    if (first->count && (!results || !first->offsets || !second->offsets))
        return fail(sz_unexpected_dimensions_k, "Offsets and results must not be NULL", error_message);
    auto *request = new (std::nothrow) request_t();
    if (!request) return fail(sz_bad_alloc_k, "Failed to allocate the request", error_message);
    request->engine = engine;
    request->results = results;
    request->pairs = first->count;
    request->submitted = steady_t::now();
    if (first->count) {
        cudaSetDevice(server->device);
        if (!read_side(first, request->first) || !read_side(second, request->second)) {
            delete request;
            return fail(sz_status_unknown_k, "Failed to read the tapes' offsets", error_message);
        }
        for (std::uint64_t i = 0; i < request->pairs; ++i) {
            std::uint64_t const a = request->first.offsets[i + 1] - request->first.offsets[i];
            std::uint64_t const b = request->second.offsets[i + 1] - request->second.offsets[i];
            if (request->first.offsets[i + 1] < request->first.offsets[i] ||
                request->second.offsets[i + 1] < request->second.offsets[i]) {
                delete request;
                return fail(sz_unexpected_dimensions_k, "Tape offsets must be non-decreasing", error_message);
            }
            request->cells += a * b;
        }
        request->results_on_device = device_accessible(results);
    }
    else {
        request->first.offsets.assign(1, 0);
        request->second.offsets.assign(1, 0);
    }
    std::lock_guard<std::mutex> lock(server->mutex);
    if (server->stopping) {
        delete request;
        return fail(sz_status_unknown_k, "The server is stopping", error_message);
    }
    request->ticket = server->next_ticket++;
    server->tickets[request->ticket] = request;
    ++server->stats.requests;
    if (request->pairs == 0) {
        request->admitted = request->submitted;
        server->finish({request}, sz_success_k, 0, 0);
    }
    else {
        server->waiting.push_back(request);
        server->admission_cv.notify_all();
    }
    *ticket = request->ticket;
    return sz_success_k;
}

SZS_GB300_API sz_status_t szs_gb300_server_wait(szs_gb300_server_t handle, sz_u64_t ticket,
                                                szs_gb300_request_info_t *info, char const **error_message) {
    if (error_message) *error_message = nullptr;
    server_t *server = as_server(handle);
    if (!server) return fail(sz_status_unknown_k, "Invalid server handle", error_message);
    std::unique_lock<std::mutex> lock(server->mutex);
    auto found = server->tickets.find(ticket);
    if (found == server->tickets.end()) return fail(sz_unexpected_dimensions_k, "Unknown ticket", error_message);
    request_t *request = found->second;
    server->done_cv.wait(lock, [&] { return request->done; });
    server->tickets.erase(found);
    lock.unlock();
    if (info) {
        info->status = request->status;
        info->admitted_ms = ms_between(request->submitted, request->admitted);
        info->done_ms = ms_between(request->submitted, request->finished);
        info->batch = request->batch;
        info->batch_requests = request->batch_requests;
        info->batch_pairs = request->batch_pairs;
        info->cells = request->cells;
    }
    sz_status_t const status = request->status;
    delete request;
    if (status != sz_success_k)
        return fail(status, status == sz_bad_alloc_k ? "The request does not fit the server's arena"
                                                     : "The request's batch failed",
                    error_message);
    return sz_success_k;
}

SZS_GB300_API sz_status_t szs_gb300_server_get_stats(szs_gb300_server_t handle, szs_gb300_server_stats_t *stats,
                                                     char const **error_message) {
    if (error_message) *error_message = nullptr;
    server_t *server = as_server(handle);
    if (!server || !stats) return fail(sz_status_unknown_k, "Invalid server handle", error_message);
    std::lock_guard<std::mutex> lock(server->mutex);
    *stats = server->stats;
    return sz_success_k;
}

SZS_GB300_API void szs_gb300_server_free(szs_gb300_server_t handle) {
    server_t *server = as_server(handle);
    if (!server) return;
    {
        std::lock_guard<std::mutex> lock(server->mutex);
        server->stopping = true;
        server->admission_cv.notify_all();
    }
    if (server->admission.joinable()) server->admission.join();
    {
        std::lock_guard<std::mutex> lock(server->mutex);
        server->lanes_stopping = true;
        server->lane_cv.notify_all();
    }
    for (auto &lane : server->lanes)
        if (lane->thread.joinable()) lane->thread.join();
    cudaSetDevice(server->device);
    for (auto &lane : server->lanes) {
        if (lane->exec) exec_context_free(lane->exec);
        if (lane->start) cudaEventDestroy(lane->start);
        if (lane->stop) cudaEventDestroy(lane->stop);
    }
    server->lanes.clear();
    for (auto &entry : server->tickets) delete entry.second;
    if (server->arena) cudaFree(server->arena);
    server->magic = 0;
    delete server;
}

} // extern "C"
