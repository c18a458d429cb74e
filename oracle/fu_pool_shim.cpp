/**
 *  @file oracle/fu_pool_shim.cpp
 *  @brief Test-harness thread pool that satisfies the ForkUnion C symbols the reference's `szs_*` CPU library
 *         links against, so that library can be built from its own sources as the parity oracle.
 *
 *  TEST INFRASTRUCTURE ONLY. Nothing in the product links this file: it is compiled into `oracle/_ref/`
 *  together with the reference sources by `oracle/Makefile`.
 *
 *  The reference declares the pool API in `forkunion/include/forkunion.h:474-723` and consumes it through
 *  `forkunion_executor_t` (`include/stringzillas/types.hpp:131-225`), but its build lists
 *  `forkunion/c/forkunion.cpp` (`setup.py:534`), which is absent from the reference tree. This file provides the
 *  handful of entry points that executor calls, with plain `std::thread` workers spawned per parallel region:
 *  - `for_n` / `for_n_dynamic`: tasks handed out through a shared atomic counter;
 *  - `for_slices`: one contiguous slice per thread;
 *  - `for_threads`: one callback per thread.
 *  No topology, NUMA or pinning is modelled; the reference's semantics only need "every index runs once".
 */
#include <atomic>
#include <cstddef>
#include <thread>
#include <vector>

namespace {
template <typename body_type_>
void harness_run_threads_(size_t threads, body_type_ &&body) {
    std::vector<std::thread> workers;
    workers.reserve(threads > 0 ? threads - 1 : 0);
    for (size_t t = 1; t < threads; ++t) workers.emplace_back([&body, t] { body(t); });
    body(0);
    for (auto &w : workers) w.join();
}
} // namespace

extern "C" {

typedef int fu_bool_t;
typedef void *fu_topology_t;
typedef void *fu_pool_t;
typedef void *fu_lambda_context_t;
typedef void (*fu_for_threads_t)(fu_lambda_context_t context, size_t thread, size_t compute_domain);
typedef void (*fu_for_prongs_t)(fu_lambda_context_t context, size_t task, size_t thread, size_t compute_domain);
typedef void (*fu_for_slices_t)(fu_lambda_context_t context, size_t first, size_t count, size_t thread,
                                size_t compute_domain);

struct harness_pool_t {
    size_t threads = 1;
};

static size_t harness_cores_() {
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1;
}

fu_topology_t fu_topology_new(void) { return new int(0); }
void fu_topology_delete(fu_topology_t topology) { delete static_cast<int *>(topology); }
size_t fu_logical_cores_count(fu_topology_t) { return harness_cores_(); }

fu_pool_t fu_pool_new(char const *, int) { return new harness_pool_t(); }
void fu_pool_delete(fu_pool_t pool) { delete static_cast<harness_pool_t *>(pool); }
fu_bool_t fu_pool_spawn(fu_topology_t, fu_pool_t pool, size_t threads, int) {
    static_cast<harness_pool_t *>(pool)->threads = threads ? threads : 1;
    return 1;
}
size_t fu_pool_threads_count(fu_pool_t pool) { return static_cast<harness_pool_t *>(pool)->threads; }

void fu_pool_for_threads(fu_pool_t pool, fu_for_threads_t callback, fu_lambda_context_t context) {
    harness_run_threads_(fu_pool_threads_count(pool), [&](size_t t) { callback(context, t, 0); });
}

void fu_pool_for_n_dynamic(fu_pool_t pool, size_t n, fu_for_prongs_t callback, fu_lambda_context_t context) {
    std::atomic<size_t> next {0};
    harness_run_threads_(fu_pool_threads_count(pool), [&](size_t t) {
        for (size_t task = next.fetch_add(1); task < n; task = next.fetch_add(1)) callback(context, task, t, 0);
    });
}

void fu_pool_for_n(fu_pool_t pool, size_t n, fu_for_prongs_t callback, fu_lambda_context_t context) {
    fu_pool_for_n_dynamic(pool, n, callback, context);
}

void fu_pool_for_slices(fu_pool_t pool, size_t n, fu_for_slices_t callback, fu_lambda_context_t context) {
    size_t const threads = fu_pool_threads_count(pool);
    size_t const per_thread = (n + threads - 1) / threads;
    harness_run_threads_(threads, [&](size_t t) {
        size_t const first = t * per_thread;
        if (first >= n) return;
        size_t const count = first + per_thread > n ? n - first : per_thread;
        callback(context, first, count, t, 0);
    });
}

} // extern "C"
