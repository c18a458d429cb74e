/**
 *  @file include/stringzillas_gb300.h
 *  @brief C-ABI of the GB300 batched scoring engine: a drop-in for StringZillas' `szs_*` scoring path.
 *
 *  The declarations below keep the reference's names, argument order, argument meaning, status codes and ownership
 *  rules, so a program (or FFI binding) written against the reference's `include/stringzillas/stringzillas.h`
 *  links against `libszs_gb300.so` unchanged. Each declaration cites the reference line it replaces.
 *
 *  Scope of the engine: Levenshtein distances, Needleman-Wunsch global scores and Smith-Waterman local scores over
 *  bytes, with linear or affine gaps and a class-folded int8 substitution table, computed on an NVIDIA GB300
 *  (sm_103a). There is no CPU backend: a CPU-cores scope is rejected with `sz_device_code_mismatch_k`, exactly as
 *  the reference rejects a CPU scope for a CUDA engine (`c/stringzillas/levenshtein.cuh:60-90`).
 *
 *  Inputs and outputs may live in host memory (pageable or pinned), device memory or managed memory; the engine
 *  stages whatever is not device-resident. Engines are not thread-safe (one call at a time per engine, as in the
 *  reference); scopes may be driven from any thread.
 *
 *  Functions under "Extensions" have no counterpart in the reference; each says so.
 */
#ifndef STRINGZILLAS_GB300_H_
#define STRINGZILLAS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define SZS_GB300_API __declspec(dllexport)
#else
#define SZS_GB300_API __attribute__((visibility("default")))
#endif

/*  Core types. Layout-identical to `include/stringzilla/types.h` of the reference (lines cited); skipped when the
 *  reference's own types header was included first, so both headers can coexist in one translation unit. */
#ifndef STRINGZILLA_TYPES_H_
typedef int8_t sz_i8_t;                /* types.h:530 */
typedef uint8_t sz_u8_t;               /* types.h:531 */
typedef uint16_t sz_u16_t;             /* types.h:533 */
typedef uint32_t sz_u32_t;             /* types.h:535 */
typedef uint64_t sz_u64_t;             /* types.h:536 */
typedef size_t sz_size_t;              /* types.h:538 */
typedef ptrdiff_t sz_ssize_t;          /* types.h:539 */
typedef char const *sz_cptr_t;         /* types.h:632 */
typedef sz_i8_t sz_error_cost_t;       /* types.h:634 */
typedef sz_size_t sz_sorted_idx_t;     /* types.h:644 */

/** Status codes, values as in types.h:699-721. */
typedef enum sz_status_t {
    sz_success_k = 0,
    sz_bad_alloc_k = -10,
    sz_invalid_utf8_k = -12,
    sz_contains_duplicates_k = -13,
    sz_overflow_risk_k = -14,
    sz_unexpected_dimensions_k = -15,
    sz_missing_gpu_k = -16,
    sz_device_code_mismatch_k = -17,
    sz_device_memory_mismatch_k = -18,
    sz_authentication_failed_k = -19,
    sz_status_unknown_k = -1,
} sz_status_t;

/** Capability bits, values as in types.h:728-766 (only the bits this library reports or accepts are named). */
typedef enum sz_capability_t {
    sz_cap_serial_k = 1,
    sz_cap_parallel_k = 1 << 2,
    sz_cap_any_k = 0x7FFFFFFF,
    sz_cap_cuda_k = 1 << 21,
    sz_cap_kepler_k = 1 << 22,
    sz_cap_hopper_k = 1 << 23,
    sz_caps_none_k = 0,
    sz_caps_ckh_k = (1 << 21) | (1 << 22) | (1 << 23),
} sz_capability_t;

typedef sz_cptr_t (*sz_sequence_member_start_t)(void const *, sz_sorted_idx_t);  /* types.h:1168 */
typedef sz_size_t (*sz_sequence_member_length_t)(void const *, sz_sorted_idx_t); /* types.h:1170 */

/** A collection of strings reached through callbacks (types.h:1177-1182). */
typedef struct sz_sequence_t {
    void const *handle;
    sz_size_t count;
    sz_sequence_member_start_t get_start;
    sz_sequence_member_length_t get_length;
} sz_sequence_t;

typedef void *(*sz_memory_allocate_t)(sz_size_t, void *); /* types.h:859 */
typedef void (*sz_memory_free_t)(void *, sz_size_t, void *);

/** Allocator hooks (types.h:866-870). Accepted and ignored by every `*_init`, as in the reference. */
typedef struct sz_memory_allocator_t {
    sz_memory_allocate_t allocate;
    sz_memory_free_t free;
    void *handle;
} sz_memory_allocator_t;
#endif /* STRINGZILLA_TYPES_H_ */

#ifndef STRINGZILLAS_H_
/** Arrow-like tape with 32-bit offsets, `count + 1` of them (stringzillas.h:68-72). */
typedef struct sz_sequence_u32tape_t {
    sz_cptr_t data;
    sz_u32_t const *offsets;
    sz_size_t count;
} sz_sequence_u32tape_t;

/** Arrow-like tape with 64-bit offsets, `count + 1` of them (stringzillas.h:78-82). */
typedef struct sz_sequence_u64tape_t {
    sz_cptr_t data;
    sz_u64_t const *offsets;
    sz_size_t count;
} sz_sequence_u64tape_t;

typedef void *szs_device_scope_t;             /* stringzillas.h:101 */
typedef void *szs_levenshtein_distances_t;    /* stringzillas.h:153 */
typedef void *szs_levenshtein_distances_utf8_t;
typedef void *szs_needleman_wunsch_scores_t;  /* stringzillas.h:293 */
typedef void *szs_smith_waterman_scores_t;
typedef void *szs_fingerprints_t;
typedef void *szs_fingerprints_utf8_t;
#endif /* STRINGZILLAS_H_ */

/* ---- Metadata (replaces stringzillas.h:33-62) ------------------------------------------------------------------ */

/** Version of the reference release this ABI mirrors (5.3.2). Replaces stringzillas.h:37. */
SZS_GB300_API int szs_version_major(void);
/** Replaces stringzillas.h:42. */
SZS_GB300_API int szs_version_minor(void);
/** Replaces stringzillas.h:47. */
SZS_GB300_API int szs_version_patch(void);
/** `cuda | kepler | hopper` (the engine is compiled for sm_103a). Replaces stringzillas.h:52. */
SZS_GB300_API sz_capability_t szs_capabilities_comptime(void);
/** The same bits when a CUDA device is visible, else `sz_caps_none_k`. Replaces stringzillas.h:57. */
SZS_GB300_API sz_capability_t szs_capabilities_runtime(void);
/** `comptime & runtime`, cached. Replaces stringzillas.h:62. */
SZS_GB300_API sz_capability_t szs_capabilities(void);

/** Fills @p alloc with managed-memory hooks. Replaces stringzillas.h:88. */
SZS_GB300_API sz_status_t sz_memory_allocator_init_unified(sz_memory_allocator_t *alloc, char const **error_message);

/* ---- Device scopes (replaces stringzillas.h:107-152) ----------------------------------------------------------- */

/** Default scope: GPU engines run on device 0. Replaces stringzillas.h:107. */
SZS_GB300_API sz_status_t szs_device_scope_init_default(szs_device_scope_t *scope, char const **error_message);
/** CPU-cores scope: accepted, but every scoring call on it returns `sz_device_code_mismatch_k`. Replaces :115. */
SZS_GB300_API sz_status_t szs_device_scope_init_cpu_cores(sz_size_t cpu_cores, szs_device_scope_t *scope,
                                                          char const **error_message);
/** GPU scope with its own non-blocking stream; `sz_missing_gpu_k` if the device does not exist. Replaces :123. */
SZS_GB300_API sz_status_t szs_device_scope_init_gpu_device(sz_size_t gpu_device, szs_device_scope_t *scope,
                                                           char const **error_message);
/** Replaces stringzillas.h:131. */
SZS_GB300_API sz_status_t szs_device_scope_get_cpu_cores(szs_device_scope_t scope, sz_size_t *cpu_cores,
                                                         char const **error_message);
/** Replaces stringzillas.h:139. */
SZS_GB300_API sz_status_t szs_device_scope_get_gpu_device(szs_device_scope_t scope, sz_size_t *gpu_device,
                                                          char const **error_message);
/** Replaces stringzillas.h:147. */
SZS_GB300_API sz_status_t szs_device_scope_get_capabilities(szs_device_scope_t scope, sz_capability_t *capabilities,
                                                            char const **error_message);
/** Replaces stringzillas.h:152. */
SZS_GB300_API void szs_device_scope_free(szs_device_scope_t scope);

/* ---- Levenshtein distances (replaces stringzillas.h:153-223) --------------------------------------------------- */

/**
 *  Creates an engine for `min` edit costs: `match`/`mismatch` per substitution, a gap of length k costing
 *  `open + (k-1)*extend`; `open == extend` selects linear gaps. `*engine` must be NULL on entry. Costs must be
 *  non-negative (the reference's unsigned cells wrap on negative costs; here they are rejected with
 *  `sz_overflow_risk_k`). Replaces stringzillas.h:170-173.
 */
SZS_GB300_API sz_status_t szs_levenshtein_distances_init(sz_error_cost_t match, sz_error_cost_t mismatch,
                                                         sz_error_cost_t open, sz_error_cost_t extend,
                                                         sz_memory_allocator_t const *alloc,
                                                         sz_capability_t capabilities,
                                                         szs_levenshtein_distances_t *engine,
                                                         char const **error_message);
/**
 *  Fills `results[q * results_row_stride + c]` with the distance of `queries[q]` to `candidates[c]`; with
 *  `candidates == NULL`, the symmetric self-distance matrix of `queries`. Replaces stringzillas.h:184-188.
 */
SZS_GB300_API sz_status_t szs_levenshtein_distances(szs_levenshtein_distances_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                    sz_size_t *results, sz_size_t results_row_stride,
                                                    char const **error_message);
/** Tape form with 32-bit offsets. Replaces stringzillas.h:199-203. */
SZS_GB300_API sz_status_t szs_levenshtein_distances_u32tape(szs_levenshtein_distances_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u32tape_t const *queries,
                                                            sz_sequence_u32tape_t const *candidates,
                                                            sz_size_t *results, sz_size_t results_row_stride,
                                                            char const **error_message);
/** Tape form with 64-bit offsets. Replaces stringzillas.h:214-218. */
SZS_GB300_API sz_status_t szs_levenshtein_distances_u64tape(szs_levenshtein_distances_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u64tape_t const *queries,
                                                            sz_sequence_u64tape_t const *candidates,
                                                            sz_size_t *results, sz_size_t results_row_stride,
                                                            char const **error_message);
/** Replaces stringzillas.h:223. */
SZS_GB300_API void szs_levenshtein_distances_free(szs_levenshtein_distances_t engine);

/* ---- UTF-8 Levenshtein (replaces stringzillas.h:224-292) ------------------------------------------------------- */

/**
 *  Distances over UTF-8 code points. Each call decodes both tapes on the device the way the reference does
 *  (lead-byte lengths, continuation bytes not checked) and numbers the batch's distinct code points: one-byte codes
 *  up to 256 of them, 16-bit codes up to 65,536 (more give `sz_unexpected_dimensions_k`). Replaces
 *  stringzillas.h:239.
 */
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_init(sz_error_cost_t match, sz_error_cost_t mismatch,
                                                              sz_error_cost_t open, sz_error_cost_t extend,
                                                              sz_memory_allocator_t const *alloc,
                                                              sz_capability_t capabilities,
                                                              szs_levenshtein_distances_utf8_t *engine,
                                                              char const **error_message);
/** Replaces stringzillas.h:255. */
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8(szs_levenshtein_distances_utf8_t engine,
                                                         szs_device_scope_t device, sz_sequence_t const *queries,
                                                         sz_sequence_t const *candidates, sz_size_t *results,
                                                         sz_size_t results_row_stride, char const **error_message);
/** Replaces stringzillas.h:270. */
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_u32tape(szs_levenshtein_distances_utf8_t engine,
                                                                 szs_device_scope_t device,
                                                                 sz_sequence_u32tape_t const *queries,
                                                                 sz_sequence_u32tape_t const *candidates,
                                                                 sz_size_t *results, sz_size_t results_row_stride,
                                                                 char const **error_message);
/** Replaces stringzillas.h:285. */
SZS_GB300_API sz_status_t szs_levenshtein_distances_utf8_u64tape(szs_levenshtein_distances_utf8_t engine,
                                                                 szs_device_scope_t device,
                                                                 sz_sequence_u64tape_t const *queries,
                                                                 sz_sequence_u64tape_t const *candidates,
                                                                 sz_size_t *results, sz_size_t results_row_stride,
                                                                 char const **error_message);
/** Replaces stringzillas.h:292. */
SZS_GB300_API void szs_levenshtein_distances_utf8_free(szs_levenshtein_distances_utf8_t engine);

/* ---- Needleman-Wunsch scores (replaces stringzillas.h:293-364) ------------------------------------------------- */

/**
 *  Creates a global-alignment engine maximising `sum(table[byte_to_class[a]][byte_to_class[b]]) + gaps`, the table
 *  being 32x32 row-major int8 (first string's class selects the row). Gap of length k: `open + (k-1)*extend`
 *  (pass negative values). `open == extend` selects linear gaps. Replaces stringzillas.h:310-314.
 */
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_init(sz_u8_t const *byte_to_class,
                                                           sz_error_cost_t const *class_substitution_costs,
                                                           sz_error_cost_t open, sz_error_cost_t extend,
                                                           sz_memory_allocator_t const *alloc,
                                                           sz_capability_t capabilities,
                                                           szs_needleman_wunsch_scores_t *engine,
                                                           char const **error_message);
/** Replaces stringzillas.h:325-329. */
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores(szs_needleman_wunsch_scores_t engine, szs_device_scope_t device,
                                                      sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                      sz_ssize_t *results, sz_size_t results_row_stride,
                                                      char const **error_message);
/** Replaces stringzillas.h:340-344. */
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_u32tape(szs_needleman_wunsch_scores_t engine,
                                                              szs_device_scope_t device,
                                                              sz_sequence_u32tape_t const *queries,
                                                              sz_sequence_u32tape_t const *candidates,
                                                              sz_ssize_t *results, sz_size_t results_row_stride,
                                                              char const **error_message);
/** Replaces stringzillas.h:355-359. */
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_u64tape(szs_needleman_wunsch_scores_t engine,
                                                              szs_device_scope_t device,
                                                              sz_sequence_u64tape_t const *queries,
                                                              sz_sequence_u64tape_t const *candidates,
                                                              sz_ssize_t *results, sz_size_t results_row_stride,
                                                              char const **error_message);
/** Replaces stringzillas.h:364. */
SZS_GB300_API void szs_needleman_wunsch_scores_free(szs_needleman_wunsch_scores_t engine);

/* ---- Smith-Waterman scores (replaces stringzillas.h:365-434) --------------------------------------------------- */

/** Local alignment, same arguments as Needleman-Wunsch; an empty side scores 0. Replaces stringzillas.h:380-384. */
SZS_GB300_API sz_status_t szs_smith_waterman_scores_init(sz_u8_t const *byte_to_class,
                                                         sz_error_cost_t const *class_substitution_costs,
                                                         sz_error_cost_t open, sz_error_cost_t extend,
                                                         sz_memory_allocator_t const *alloc,
                                                         sz_capability_t capabilities,
                                                         szs_smith_waterman_scores_t *engine,
                                                         char const **error_message);
/** Replaces stringzillas.h:395-399. */
SZS_GB300_API sz_status_t szs_smith_waterman_scores(szs_smith_waterman_scores_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *queries, sz_sequence_t const *candidates,
                                                    sz_ssize_t *results, sz_size_t results_row_stride,
                                                    char const **error_message);
/** Replaces stringzillas.h:410-414. */
SZS_GB300_API sz_status_t szs_smith_waterman_scores_u32tape(szs_smith_waterman_scores_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u32tape_t const *queries,
                                                            sz_sequence_u32tape_t const *candidates,
                                                            sz_ssize_t *results, sz_size_t results_row_stride,
                                                            char const **error_message);
/** Replaces stringzillas.h:425-429. */
SZS_GB300_API sz_status_t szs_smith_waterman_scores_u64tape(szs_smith_waterman_scores_t engine,
                                                            szs_device_scope_t device,
                                                            sz_sequence_u64tape_t const *queries,
                                                            sz_sequence_u64tape_t const *candidates,
                                                            sz_ssize_t *results, sz_size_t results_row_stride,
                                                            char const **error_message);
/** Replaces stringzillas.h:434. */
SZS_GB300_API void szs_smith_waterman_scores_free(szs_smith_waterman_scores_t engine);

/* ---- Fingerprints (replaces stringzillas.h:435-536) ------------------------------------------------------------ */

/**
 *  Min-Hash engine of @p dimensions rolling hashers. Dimension `d` rolls a hash over windows of
 *  `window_widths[(d / 64) % count]` bytes when `dimensions` is a multiple of `64 * count` (the reference's sliced
 *  layout), else of `window_widths[d % count]`; NULL / zero widths select {3, 4, 5, 7, 9, 11, 15, 31}. Modulus and
 *  multiplier come from `seed + d` as in the reference's `floating_rolling_hasher<f64_t>`. @p alphabet_size,
 *  @p alloc and @p capabilities are accepted and unused, as in the reference. `*engine` must be NULL on entry.
 *  Replaces stringzillas.h:476-480 (c/stringzillas/fingerprints.cuh:27-141).
 */
SZS_GB300_API sz_status_t szs_fingerprints_init(sz_size_t dimensions, sz_size_t alphabet_size,
                                                sz_size_t const *window_widths, sz_size_t window_widths_count,
                                                sz_u64_t seed, sz_memory_allocator_t const *alloc,
                                                sz_capability_t capabilities, szs_fingerprints_t *engine,
                                                char const **error_message);
/**
 *  Writes, for text `i` and dimension `d`, the low 32 bits of the minimum window hash to
 *  `(char *)min_hashes + i * min_hashes_stride` [d] and its number of occurrences to the same place in
 *  @p min_counts; strides are in BYTES and at least `dimensions * 4`. Texts shorter than a dimension's window get
 *  0xFFFFFFFF and 0. Outputs may be host or device memory. Replaces stringzillas.h:495.
 */
SZS_GB300_API sz_status_t szs_fingerprints_sequence(szs_fingerprints_t engine, szs_device_scope_t device,
                                                    sz_sequence_t const *texts, sz_u32_t *min_hashes,
                                                    sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                    sz_size_t min_counts_stride, char const **error_message);
/** Replaces stringzillas.h:509. */
SZS_GB300_API sz_status_t szs_fingerprints_u64tape(szs_fingerprints_t engine, szs_device_scope_t device,
                                                   sz_sequence_u64tape_t const *texts, sz_u32_t *min_hashes,
                                                   sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                   sz_size_t min_counts_stride, char const **error_message);
/** Replaces stringzillas.h:523. */
SZS_GB300_API sz_status_t szs_fingerprints_u32tape(szs_fingerprints_t engine, szs_device_scope_t device,
                                                   sz_sequence_u32tape_t const *texts, sz_u32_t *min_hashes,
                                                   sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                   sz_size_t min_counts_stride, char const **error_message);
/** Replaces stringzillas.h:536. */
SZS_GB300_API void szs_fingerprints_free(szs_fingerprints_t engine);

/** The UTF-8 entry points hash the same bytes as the byte ones; the reference's library exports them as forwards
 *  (c/stringzillas/fingerprints.cuh:181-222). */
SZS_GB300_API sz_status_t szs_fingerprints_utf8_init(sz_size_t dimensions, sz_size_t alphabet_size,
                                                     sz_size_t const *window_widths, sz_size_t window_widths_count,
                                                     sz_u64_t seed, sz_memory_allocator_t const *alloc,
                                                     sz_capability_t capabilities, szs_fingerprints_utf8_t *engine,
                                                     char const **error_message);
/** Forwards to `szs_fingerprints_sequence` (c/stringzillas/fingerprints.cuh:192-200). */
SZS_GB300_API sz_status_t szs_fingerprints_utf8_sequence(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                         sz_sequence_t const *texts, sz_u32_t *min_hashes,
                                                         sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                         sz_size_t min_counts_stride, char const **error_message);
/** Forwards to `szs_fingerprints_u32tape` (c/stringzillas/fingerprints.cuh:201-209). */
SZS_GB300_API sz_status_t szs_fingerprints_utf8_u32tape(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                        sz_sequence_u32tape_t const *texts, sz_u32_t *min_hashes,
                                                        sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                        sz_size_t min_counts_stride, char const **error_message);
/** Forwards to `szs_fingerprints_u64tape` (c/stringzillas/fingerprints.cuh:210-218). */
SZS_GB300_API sz_status_t szs_fingerprints_utf8_u64tape(szs_fingerprints_utf8_t engine, szs_device_scope_t device,
                                                        sz_sequence_u64tape_t const *texts, sz_u32_t *min_hashes,
                                                        sz_size_t min_hashes_stride, sz_u32_t *min_counts,
                                                        sz_size_t min_counts_stride, char const **error_message);
/** Forwards to `szs_fingerprints_free` (c/stringzillas/fingerprints.cuh:219-221). */
SZS_GB300_API void szs_fingerprints_utf8_free(szs_fingerprints_utf8_t engine);

/* ---- Unified memory (replaces stringzillas.h:545-551) ---------------------------------------------------------- */

/** `cudaMallocManaged`, NULL on failure. Replaces stringzillas.h:545. */
SZS_GB300_API void *szs_unified_alloc(sz_size_t size_bytes);
/** Replaces stringzillas.h:551. */
SZS_GB300_API void szs_unified_free(void *ptr, sz_size_t size_bytes);

/* ==== Extensions (no counterpart in the reference) ============================================================== */

/**
 *  Pairwise ("zip") scoring: `results[i] = score(first[i], second[i])` for `i < first->count`; both tapes must hold
 *  the same count (else `sz_unexpected_dimensions_k`). The reference only offers the cross-product, whose diagonal
 *  gives the same numbers at quadratic cost. Results are written densely (stride 1).
 */
SZS_GB300_API sz_status_t szs_levenshtein_distances_pairwise_u32tape(szs_levenshtein_distances_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u32tape_t const *first,
                                                                     sz_sequence_u32tape_t const *second,
                                                                     sz_size_t *results, char const **error_message);
SZS_GB300_API sz_status_t szs_levenshtein_distances_pairwise_u64tape(szs_levenshtein_distances_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u64tape_t const *first,
                                                                     sz_sequence_u64tape_t const *second,
                                                                     sz_size_t *results, char const **error_message);
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_pairwise_u32tape(szs_needleman_wunsch_scores_t engine,
                                                                       szs_device_scope_t device,
                                                                       sz_sequence_u32tape_t const *first,
                                                                       sz_sequence_u32tape_t const *second,
                                                                       sz_ssize_t *results,
                                                                       char const **error_message);
SZS_GB300_API sz_status_t szs_needleman_wunsch_scores_pairwise_u64tape(szs_needleman_wunsch_scores_t engine,
                                                                       szs_device_scope_t device,
                                                                       sz_sequence_u64tape_t const *first,
                                                                       sz_sequence_u64tape_t const *second,
                                                                       sz_ssize_t *results,
                                                                       char const **error_message);
SZS_GB300_API sz_status_t szs_smith_waterman_scores_pairwise_u32tape(szs_smith_waterman_scores_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u32tape_t const *first,
                                                                     sz_sequence_u32tape_t const *second,
                                                                     sz_ssize_t *results, char const **error_message);
SZS_GB300_API sz_status_t szs_smith_waterman_scores_pairwise_u64tape(szs_smith_waterman_scores_t engine,
                                                                     szs_device_scope_t device,
                                                                     sz_sequence_u64tape_t const *first,
                                                                     sz_sequence_u64tape_t const *second,
                                                                     sz_ssize_t *results, char const **error_message);

/** Scheduling forms an engine can run a batch in. */
typedef enum szs_gb300_schedule_t {
    /** Length-binned plan: pairs sorted into bins by route and size, longest first, tile shape chosen per pair,
        the routes' persistent kernels running concurrently on forked streams. */
    szs_gb300_schedule_batched_k = 0,
    /** The "plain one-launch-per-batch" form of the same kernels: one launch per route (one kernel shape, pairs in
        input order; pairs longer than one warp's strip still take the band kernel), launches one after another. */
    szs_gb300_schedule_plain_k = 1,
} szs_gb300_schedule_t;

/**
 *  Selects the scheduling form for later calls on @p engine (any of the three engine kinds). No counterpart in the
 *  reference, which always runs its own tier router.
 */
SZS_GB300_API sz_status_t szs_gb300_engine_set_schedule(void *engine, szs_gb300_schedule_t schedule,
                                                        char const **error_message);

/** Per-engine counters of the last call. No counterpart in the reference (its timer is dropped at the ABI). */
typedef struct szs_gb300_stats_t {
    double last_call_ms;       /**< CUDA-event time of the last call's device work (copies included) */
    double last_compute_ms;    /**< CUDA-event time from the first to the end of the last scoring kernel */
    sz_u64_t last_cells;       /**< sum of len(a)*len(b) over the scored pairs */
    sz_u64_t last_pairs;       /**< number of scored pairs (a symmetric call counts the triangle once) */
    sz_u64_t last_launches;    /**< kernels launched by the last call (graph nodes count one each) */
    sz_u64_t graph_replays;    /**< calls served by replaying a cached CUDA graph */
    sz_u64_t kernel_launches;  /**< kernels launched over the engine's lifetime */
} szs_gb300_stats_t;

/**
 *  GPU scope that runs every call on the caller's CUDA stream (`cudaStream_t` passed as `void *`), so callers can
 *  order the engine's work with their own and time it with events on that stream. The stream stays owned by the
 *  caller and must outlive the scope. No counterpart in the reference (its scopes always create their own stream).
 */
SZS_GB300_API sz_status_t szs_gb300_device_scope_init_stream(sz_size_t gpu_device, void *cuda_stream,
                                                             szs_device_scope_t *scope, char const **error_message);

/**
 *  Per-length-bin choices of the planner and of the launch shapes. Length class k holds the pairs whose shorter
 *  side n has floor(log2(n)) == k (class 15 also holds everything longer). Zero fields keep the built-in choice.
 *  No counterpart in the reference, whose tier thresholds are compile-time constants.
 */
typedef struct szs_gb300_tuning_t {
    sz_u8_t packed_rows[16]; /**< rows per lane of the 16x2 route (4, 8, 12 or 16); 0 = per-pair step-cost model */
    sz_u8_t cell_bits[16];   /**< 0 = the narrowest cells the length bound proves safe; 32 = never 16-bit cells;
                                  64 = 64-bit cells (the route of spans near 2^31 / magnitude) */
    sz_u32_t band_min_rows;  /**< pairs on 32-bit cells whose shorter side exceeds this take the band (0 = 1,024) */
    sz_u32_t packed_warps[4]; /**< warps per CTA (1..8) of the 16x2 launches with 4, 8, 12, 16 rows (0 = 4) */
    sz_u32_t band_min_rows_packed; /**< the same threshold for pairs that fit 16-bit cells (0 = 2,048) */
    sz_u32_t pipeline_chunk_kb;   /**< input KiB per chunk of a pipelined pinned-host pairwise call (0 = 64 MiB) */
    /** Relative cost of one lane step of the 16x2 route with 4, 8, 12, 16 rows per lane. Where `packed_rows` is 0
        the planner gives each pair the rows per lane of least `strips x (m + 31) x cost` (0 = built-in 100, 165,
        245, 330). */
    sz_u16_t packed_step_cost[4];
    /** Calls of the batched form with fewer pairs than 32 per SM (less than one wave of the 16x2 route's warps, two
        pairs each) give pairs whose shorter side exceeds this a band instead, whatever the two thresholds above say
        (0 = 1,024): a band spreads one pair over a CTA's warps, where the wavefront would leave SMs idle. */
    sz_u32_t band_min_rows_few;
    /** The 16-bit band threshold for Levenshtein pairs scored by comparing codes (more than 32 byte values, or UTF-8
        over more than 256 code points) instead of `band_min_rows_packed` (0 = 2,048: on text the band overtakes the
        wavefront only past about 2,000 rows). */
    sz_u32_t band_min_rows_compare;
    /** Polls (about 100 ns each) before a band kernel's wait for the strip above gives up, raises the call's error
        and abandons the pair; group barriers get four times as many (0 = 4,194,304, about 0.4 s, and 3 s at a
        barrier). Values above the built-in bounds are clamped to them, so every wait stays bounded; small values
        only make calls with long pairs fail early with `sz_status_unknown_k` (a wait that gives up never faults). */
    sz_u32_t band_wait_polls;
    /** Pairs on 16-bit cells whose shorter side is at most this take the short-pair kernel, several pairs per warp
        (0 = 128; larger values are clamped to 128). */
    sz_u32_t short_max_rows;
} szs_gb300_tuning_t;

/** Installs @p tuning on @p engine (NULL restores the built-in choices); out-of-range values are rejected with
 *  `sz_unexpected_dimensions_k`. No counterpart in the reference. */
SZS_GB300_API sz_status_t szs_gb300_engine_set_tuning(void *engine, szs_gb300_tuning_t const *tuning,
                                                      char const **error_message);

/** Copies the engine's current tuning into @p tuning. No counterpart in the reference. */
SZS_GB300_API sz_status_t szs_gb300_engine_get_tuning(void *engine, szs_gb300_tuning_t *tuning,
                                                      char const **error_message);

/** Copies the engine's counters into @p stats. No counterpart in the reference. */
SZS_GB300_API sz_status_t szs_gb300_engine_get_stats(void *engine, szs_gb300_stats_t *stats,
                                                     char const **error_message);

/**
 *  Pairwise scoring that allocates no memory: `results[i] = score(first[i], second[i])` for any engine made by the
 *  `*_init` functions above (8-byte results: `sz_size_t` for Levenshtein, `sz_ssize_t` for alignments). No counterpart
 *  in the reference. For callers that cannot call `cudaMalloc` / `cudaFree` - for example a host application whose
 *  own allocator already reserves the device memory, or a latency-bound loop that cannot afford the device-wide
 *  synchronisation of `cudaFree`.
 *  - Tapes (data and offsets, non-null) and `results` must already be in the scope device's memory or in managed
 *    memory, else `sz_device_memory_mismatch_k`. The engine's staging buffers are not used.
 *  - Scratch comes from a fixed 16 MiB (+ 256 B) device array inside the library, held by every GPU that loads it
 *    until exit. A pair whose two sides both exceed 256 bytes must have both sides below 2,048 bytes; longer ones
 *    fail the call with `sz_overflow_risk_k`. The other pairs' results are still written, and every rejected pair's
 *    slot is set to 0 (which is also a valid score: check the status).
 *  - The first call on each device resolves the array's address with that device current and keeps it; make that
 *    first call before any stream capture, and do not use this entry point across a `cudaDeviceReset` of the device.
 *    Every call shares the array: calls whose kernels overlap on the GPU race.
 *  - The calling thread's current device is the same after the call as before it.
 *  The default scope runs on the legacy default stream; GPU scopes use their own stream. Synchronous, like the rest.
 */
SZS_GB300_API sz_status_t szs_gb300_score_pairwise_noalloc_u64tape(void *engine, szs_device_scope_t device,
                                                                   sz_sequence_u64tape_t const *first,
                                                                   sz_sequence_u64tape_t const *second, void *results,
                                                                   char const **error_message);

/**
 *  Measures the device's sustained integer issue rates (operations per second, whole GPU) into
 *  @p ops_per_second[0..4]: LOP3, IADD3, DPX `max(a + b, c)` (32-bit), DPX `max(a, b, c)` (32-bit) and DPX
 *  `max(a + b, c)` on 16x2 lanes. These are the roofline denominators of the scoring kernels, which are bound by the
 *  integer pipes rather than by HBM or tensor cores. No counterpart in the reference.
 */
SZS_GB300_API sz_status_t szs_gb300_measure_integer_peaks(sz_size_t gpu_device, double *ops_per_second,
                                                          sz_size_t count, char const **error_message);

/* ---- dense substitution tables (no counterpart in the reference) ------------------------------------------------ */

/**
 *  Needleman-Wunsch / Smith-Waterman engines over a dense 256 x 256 table, `costs[a * 256 + b]` = cost of aligning
 *  byte a of the first string with byte b of the second, instead of the reference's 32-class fold. Every scoring
 *  entry point accepts these engines. Each call maps the bytes its batch actually uses onto dense codes on the
 *  device and scores over that sub-table; a call over more than 32 distinct byte values reads the whole table on the
 *  32-bit routes instead. The allocation-free entry point does not accept these engines. No counterpart in the
 *  reference, whose engines take `byte_to_class` + a 32 x 32 table.
 */
SZS_GB300_API sz_status_t szs_gb300_needleman_wunsch_scores_init_dense(sz_error_cost_t const *costs,
                                                                       sz_error_cost_t open, sz_error_cost_t extend,
                                                                       sz_memory_allocator_t const *alloc,
                                                                       sz_capability_t capabilities,
                                                                       szs_needleman_wunsch_scores_t *engine,
                                                                       char const **error_message);
/** The Smith-Waterman counterpart of `szs_gb300_needleman_wunsch_scores_init_dense`. */
SZS_GB300_API sz_status_t szs_gb300_smith_waterman_scores_init_dense(sz_error_cost_t const *costs,
                                                                     sz_error_cost_t open, sz_error_cost_t extend,
                                                                     sz_memory_allocator_t const *alloc,
                                                                     sz_capability_t capabilities,
                                                                     szs_smith_waterman_scores_t *engine,
                                                                     char const **error_message);

/* ---- serving loop (no counterpart in the reference) ----------------------------------------------------------- */

/** A serving loop on one GPU: requests in, merged batches on the device, results out. */
typedef void *szs_gb300_server_t;

/** How a serving loop admits and batches requests. Zero fields take the defaults given. */
typedef struct szs_gb300_server_config_t {
    sz_size_t gpu_device;         /**< device index */
    sz_size_t arena_bytes;        /**< HBM budget of the device arena that holds admitted batches' sequences,
                                       offsets and results (default 1 GiB) */
    sz_size_t lanes;              /**< batches in flight at once, each on its own stream (default 4) */
    sz_size_t max_batch_pairs;    /**< pairs merged into one batch at most (default 2^22) */
    sz_size_t max_batch_requests; /**< requests merged into one batch at most (default unlimited; 1 = per-request) */
    int schedule;                 /**< `szs_gb300_schedule_t` of the batches (default batched) */
    sz_size_t max_batch_cells;    /**< cells (sum of len(a) * len(b)) merged into one batch at most while another lane
                                       is idle, so small requests do not wait behind a large one's batch (default
                                       2^33; a larger request still runs, alone; without an idle lane all merge) */
    sz_size_t aging_ms;           /**< 0: batches start from the oldest waiting request (arrival order); otherwise from
                                       the smallest one by cells, unless the oldest has waited this many milliseconds
                                       (size-aware admission: small requests pass large ones, none waits forever) */
} szs_gb300_server_config_t;

/** What happened to one request. Times are host wall-clock milliseconds from its submission. */
typedef struct szs_gb300_request_info_t {
    sz_status_t status;     /**< the request's outcome (the batch's status) */
    double admitted_ms;     /**< submission -> its batch was admitted into the arena */
    double done_ms;         /**< submission -> its results were in the caller's buffer */
    sz_u64_t batch;         /**< sequence number of the batch it ran in */
    sz_u64_t batch_requests; /**< requests merged into that batch */
    sz_u64_t batch_pairs;   /**< pairs in that batch */
    sz_u64_t cells;         /**< sum of len(a)*len(b) over this request's pairs */
} szs_gb300_request_info_t;

/** Counters of a serving loop since it started. */
typedef struct szs_gb300_server_stats_t {
    sz_u64_t requests;            /**< requests submitted */
    sz_u64_t completed;           /**< requests whose results are delivered */
    sz_u64_t batches;             /**< batches run */
    sz_u64_t pairs;               /**< pairs scored */
    sz_u64_t cells;               /**< cells scored */
    sz_u64_t arena_bytes;         /**< the arena's size */
    sz_u64_t arena_peak_bytes;    /**< most arena bytes held by admitted batches at once */
    sz_u64_t peak_inflight;       /**< most batches on the device at once */
    sz_u64_t kernel_launches;     /**< kernels launched by all lanes */
    double device_ms;             /**< sum over batches of their CUDA-event time */
} szs_gb300_server_stats_t;

/**
 *  Starts a serving loop: one admission thread and `lanes` lane threads, each lane with its own stream and
 *  scoring buffers, all sharing one device arena of `arena_bytes`. Requests wait in arrival order; whenever a lane
 *  is free, every waiting request of the first waiter's engine that fits the arena and the batch caps is merged
 *  into one batch (continuous batching), copied into the arena and scored with one planned call while other lanes'
 *  batches are still on the device.
 */
SZS_GB300_API sz_status_t szs_gb300_server_init(szs_gb300_server_config_t const *config, szs_gb300_server_t *server,
                                                char const **error_message);

/**
 *  Queues `results[i] = score(first[i], second[i])` on @p engine (any engine of the `*_init` functions; 8-byte
 *  results). Tapes and results may be host or device memory and must stay valid until the request is waited for.
 *  Returns at once with a ticket; the engine must not be freed while requests on it are pending.
 */
SZS_GB300_API sz_status_t szs_gb300_server_submit(szs_gb300_server_t server, void *engine,
                                                  sz_sequence_u64tape_t const *first,
                                                  sz_sequence_u64tape_t const *second, void *results,
                                                  sz_u64_t *ticket, char const **error_message);

/**
 *  Blocks until request @p ticket is done, fills @p info (may be NULL) and forgets the ticket. Returns the request's
 *  status; an unknown or already-waited ticket gives `sz_unexpected_dimensions_k`.
 */
SZS_GB300_API sz_status_t szs_gb300_server_wait(szs_gb300_server_t server, sz_u64_t ticket,
                                                szs_gb300_request_info_t *info, char const **error_message);

/** Copies the loop's counters into @p stats. */
SZS_GB300_API sz_status_t szs_gb300_server_get_stats(szs_gb300_server_t server, szs_gb300_server_stats_t *stats,
                                                     char const **error_message);

/** Finishes every queued request, stops the threads and frees the arena. */
SZS_GB300_API void szs_gb300_server_free(szs_gb300_server_t server);

#ifdef __cplusplus
}
#endif

#endif /* STRINGZILLAS_GB300_H_ */
