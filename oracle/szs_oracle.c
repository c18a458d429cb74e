/**
 *  @file oracle/szs_oracle.c
 *  @brief CPU restatement of the reference's byte-level scoring recurrences. TEST INFRASTRUCTURE ONLY: the parity
 *         oracle for the GPU engine and the timed CPU baseline ("port"). The product never links this file.
 *
 *  What is restated, and from where (paths inside the reference project):
 *  - The cost model: `error_costs_32x32_t` lookup `table[b2c[a]][b2c[b]]` (include/stringzillas/similarities/
 *    serial.hpp:157-183) and uniform match/mismatch costs (serial.hpp:86-98).
 *  - The recurrences evaluated by the serial `tile_scorer`s: linear global (serial.hpp:663-749), linear local with
 *    the `max(.,0)` clamp of the whole cell (serial.hpp:756-841), affine global (serial.hpp:848-964) and affine
 *    local with the clamp on the substitution path only (serial.hpp:971-1079). The local result is the running
 *    maximum over all cells, starting from 0.
 *  - The boundaries the `diagonal_walker`s seed (serial.hpp:1150-1229, :1310-1414) through `init_score` /
 *    `init_gap`: global linear `M[i][0] = g*i`; global affine `M[i][0] = open + extend*(i-1)` (0 at the corner)
 *    and the gap-track "discard" seed `(open + extend) + M[i][0]`; local `M = 0` and gap seed `open + extend`.
 *    The horizontal-gap track is seeded along column 0 and the vertical-gap track along row 0.
 *  - Empty inputs (serial.hpp:142-151, :1153-1160, :1310-1320, :2493-2496): global scores are the all-gap
 *    boundary cell, local scores are 0. Those values are exactly what the boundary formulas give, so no special
 *    case is needed beyond the local early-out.
 *  - The engine dispatch (serial.hpp:2044-2181, :2346-2532): `open == extend` selects linear gaps; unit-cost
 *    Levenshtein (0/1/1/1) is answered by the bit-parallel method (serial.hpp:1656-1865 uses Myers' algorithm);
 *    the published algorithm is restated here from G. Myers, "A fast bit-vector algorithm for approximate string
 *    matching based on dynamic programming", JACM 46(3), 1999 (block form) with H. Hyyrö's edit-distance boundary.
 *  - The substitution orientation is always `cost(first[i], second[j])`: the reference's walkers swap the strings
 *    so the shorter one is walked first but transpose the lookup back (serial.hpp:1179, :721-722).
 *  - The cross-product drivers (serial.hpp:2540-2660): `results[q*stride + c]`, and for the symmetric form only
 *    `c <= q` is scored, then mirrored.
 *
 *  All arithmetic is 64-bit, so every value the reference can form is represented exactly.
 */
#include "szs_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef struct oracle_scratch_t {
    int64_t *rows;      /* 2 rows of (longest second + 1) cells: M and the vertical-gap track */
    size_t rows_cells;
    uint32_t *runes;    /* decoded code points of both strings (UTF-8 Levenshtein) */
    size_t runes_capacity;
    uint64_t *peq;      /* 256 x words match masks for the bit-parallel method, kept all-zero between calls */
    size_t peq_words;
    uint64_t *vectors;  /* 2 x words: Pv, Mv */
} oracle_scratch_t;

static void oracle_scratch_free_(oracle_scratch_t *s) {
    free(s->rows);
    free(s->runes);
    free(s->peq);
    free(s->vectors);
    memset(s, 0, sizeof(*s));
}

static int oracle_scratch_reserve_(oracle_scratch_t *s, size_t second_length, size_t pattern_length) {
    size_t const cells = second_length + 1;
    if (cells > s->rows_cells) {
        int64_t *rows = (int64_t *)realloc(s->rows, 2 * cells * sizeof(int64_t));
        if (!rows) return -1;
        s->rows = rows, s->rows_cells = cells;
    }
    size_t const words = (pattern_length + 63) / 64;
    if (words > s->peq_words) {
        free(s->peq), free(s->vectors);
        s->peq = (uint64_t *)calloc(256 * words, sizeof(uint64_t));
        s->vectors = (uint64_t *)malloc(2 * words * sizeof(uint64_t));
        if (!s->peq || !s->vectors) return -1;
        s->peq_words = words;
    }
    return 0;
}

static inline int64_t oracle_opt_(int maximize, int64_t a, int64_t b) {
    return maximize ? (a > b ? a : b) : (a < b ? a : b);
}

static inline int64_t oracle_cost_(oracle_costs_t const *k, uint8_t a, uint8_t b) {
    if (k->kind == oracle_levenshtein_k) return a == b ? k->match : k->mismatch;
    if (k->dense_costs) return k->dense_costs[a * 256 + b];
    return k->class_costs[k->byte_to_class[a] * 32 + k->byte_to_class[b]];
}

/**
 *  Bit-parallel unit-cost edit distance, pattern = @p p (n >= 1), text = @p t. `peq` must be all-zero on entry
 *  (256 rows of `words` masks) and is left all-zero on exit.
 */
static uint64_t oracle_myers_(uint8_t const *p, size_t n, uint8_t const *t, size_t m, uint64_t *peq,
                              uint64_t *vectors) {
    size_t const words = (n + 63) / 64;
    for (size_t i = 0; i != n; ++i) peq[(size_t)p[i] * words + i / 64] |= (uint64_t)1 << (i % 64);
    uint64_t *pv = vectors, *mv = vectors + words;
    for (size_t w = 0; w != words; ++w) pv[w] = ~(uint64_t)0, mv[w] = 0;
    unsigned const last_bit = (unsigned)((n - 1) % 64);
    int64_t score = (int64_t)n;
    for (size_t j = 0; j != m; ++j) {
        uint64_t const *eq_row = peq + (size_t)t[j] * words;
        int h_in = +1; /* the top row grows by one per column: D[0][j] = j */
        for (size_t w = 0; w != words; ++w) {
            uint64_t eq = eq_row[w], v_pos = pv[w], v_neg = mv[w];
            uint64_t const xv = eq | v_neg;
            if (h_in < 0) eq |= 1;
            uint64_t const xh = (((eq & v_pos) + v_pos) ^ v_pos) | eq;
            uint64_t h_pos = v_neg | ~(xh | v_pos);
            uint64_t h_neg = v_pos & xh;
            unsigned const out_bit = w + 1 == words ? last_bit : 63u;
            int const h_out = (int)((h_pos >> out_bit) & 1) - (int)((h_neg >> out_bit) & 1);
            h_pos <<= 1, h_neg <<= 1;
            if (h_in < 0) h_neg |= 1;
            else if (h_in > 0) h_pos |= 1;
            pv[w] = h_neg | ~(xv | h_pos);
            mv[w] = h_pos & xv;
            h_in = h_out;
        }
        score += h_in;
    }
    for (size_t i = 0; i != n; ++i) peq[(size_t)p[i] * words + i / 64] = 0;
    return (uint64_t)score;
}

/** Row-major restatement of the four `tile_scorer` recurrences with the walkers' boundary seeds. */
static int64_t oracle_dp_(oracle_costs_t const *k, uint8_t const *a, size_t n, uint8_t const *b, size_t m,
                          int64_t *rows) {
    int const maximize = k->kind != oracle_levenshtein_k;
    int const local = k->kind == oracle_smith_waterman_k;
    int const linear = k->open == k->extend;
    int64_t const open = k->open, extend = k->extend;
    int64_t *m_row = rows, *v_row = rows + (m + 1);

    /* Row 0 boundary. */
    for (size_t j = 0; j <= m; ++j) {
        int64_t boundary;
        if (local) boundary = 0;
        else if (linear) boundary = open * (int64_t)j;
        else boundary = j ? open + extend * (int64_t)(j - 1) : 0;
        m_row[j] = boundary;
        v_row[j] = local ? open + extend : open + extend + boundary;
    }
    int64_t best = 0;
    for (size_t i = 1; i <= n; ++i) {
        int64_t left_boundary;
        if (local) left_boundary = 0;
        else if (linear) left_boundary = open * (int64_t)i;
        else left_boundary = open + extend * (int64_t)(i - 1);
        int64_t diag = m_row[0];
        int64_t m_left = left_boundary;
        int64_t h_left = local ? open + extend : open + extend + left_boundary;
        m_row[0] = left_boundary;
        uint8_t const ai = a[i - 1];
        for (size_t j = 1; j <= m; ++j) {
            int64_t const up = m_row[j];
            int64_t const substitution = diag + oracle_cost_(k, ai, b[j - 1]);
            int64_t cell;
            if (linear) {
                int64_t const gap = oracle_opt_(maximize, up, m_left) + open;
                if (local) cell = oracle_opt_(maximize, gap, oracle_opt_(maximize, substitution, 0));
                else cell = oracle_opt_(maximize, gap, substitution);
            }
            else {
                int64_t const vertical = oracle_opt_(maximize, up + open, v_row[j] + extend);
                int64_t const horizontal = oracle_opt_(maximize, m_left + open, h_left + extend);
                int64_t const substitution_or_reset = local ? oracle_opt_(maximize, substitution, 0) : substitution;
                cell = oracle_opt_(maximize, oracle_opt_(maximize, vertical, horizontal), substitution_or_reset);
                v_row[j] = vertical;
                h_left = horizontal;
            }
            if (local) best = oracle_opt_(maximize, best, cell);
            diag = up;
            m_row[j] = cell;
            m_left = cell;
        }
    }
    return local ? best : m_row[m];
}

/**
 *  Decodes like the reference's `sz_rune_decode_unchecked` (include/stringzilla/utf8_runes/serial.h:101-115), which
 *  the UTF-8 distance calls rune by rune (include/stringzillas/similarities/serial.hpp:2288-2299): the length comes
 *  from the lead byte alone (1 + [lead >= 0xC0] + [lead >= 0xE0] + [lead >= 0xF0]) and continuation bytes are not
 *  checked, so a sequence cut off by the end of a string reads on into the bytes that follow it. Those bytes are the
 *  next strings of the tape; past the tape's end (`limit`) they are read as 0 here.
 */
static size_t oracle_utf8_decode_(uint8_t const *s, size_t n, uint8_t const *limit, uint32_t *out) {
    size_t runes = 0;
    for (size_t i = 0; i < n; ++runes) {
        uint8_t const lead = s[i];
        unsigned const length = 1u + (lead >= 0xC0u) + (lead >= 0xE0u) + (lead >= 0xF0u);
#define ORACLE_NEXT_(k) ((s + i + (k) < limit) ? (uint32_t)(s[i + (k)] & 0x3Fu) : 0u)
        uint32_t rune;
        switch (length) {
        case 1: rune = lead; break;
        case 2: rune = (uint32_t)(lead & 0x1Fu) << 6 | ORACLE_NEXT_(1); break;
        case 3: rune = (uint32_t)(lead & 0x0Fu) << 12 | ORACLE_NEXT_(1) << 6 | ORACLE_NEXT_(2); break;
        default: rune = (uint32_t)(lead & 0x07u) << 18 | ORACLE_NEXT_(1) << 12 | ORACLE_NEXT_(2) << 6 | ORACLE_NEXT_(3); break;
        }
#undef ORACLE_NEXT_
        out[runes] = rune;
        i += length;
    }
    return runes;
}

/** The Levenshtein recurrences of `oracle_dp_` over code points (uniform costs, global, minimised). */
static int64_t oracle_rune_dp_(oracle_costs_t const *k, uint32_t const *a, size_t n, uint32_t const *b, size_t m,
                               int64_t *rows) {
    int const linear = k->open == k->extend;
    int64_t const open = k->open, extend = k->extend;
    int64_t *m_row = rows, *v_row = rows + (m + 1);
    for (size_t j = 0; j <= m; ++j) {
        int64_t const boundary = linear ? open * (int64_t)j : (j ? open + extend * (int64_t)(j - 1) : 0);
        m_row[j] = boundary;
        v_row[j] = open + extend + boundary;
    }
    for (size_t i = 1; i <= n; ++i) {
        int64_t const left_boundary = linear ? open * (int64_t)i : open + extend * (int64_t)(i - 1);
        int64_t diag = m_row[0], m_left = left_boundary, h_left = open + extend + left_boundary;
        m_row[0] = left_boundary;
        for (size_t j = 1; j <= m; ++j) {
            int64_t const up = m_row[j];
            int64_t const substitution = diag + (a[i - 1] == b[j - 1] ? k->match : k->mismatch);
            int64_t cell;
            if (linear) cell = oracle_opt_(0, oracle_opt_(0, up, m_left) + open, substitution);
            else {
                int64_t const vertical = oracle_opt_(0, up + open, v_row[j] + extend);
                int64_t const horizontal = oracle_opt_(0, m_left + open, h_left + extend);
                cell = oracle_opt_(0, oracle_opt_(0, vertical, horizontal), substitution);
                v_row[j] = vertical;
                h_left = horizontal;
            }
            diag = up;
            m_row[j] = cell;
            m_left = cell;
        }
    }
    return m_row[m];
}

static int64_t oracle_score_utf8_(oracle_costs_t const *k, char const *first, size_t n, char const *first_limit,
                                  char const *second, size_t m, char const *second_limit, oracle_scratch_t *s,
                                  int *status) {
    if (n + m + 8 > s->runes_capacity) {
        uint32_t *runes = (uint32_t *)realloc(s->runes, (n + m + 8) * sizeof(uint32_t));
        if (!runes) return *status = -1, 0;
        s->runes = runes, s->runes_capacity = n + m + 8;
    }
    size_t const rn = oracle_utf8_decode_((uint8_t const *)first, n, (uint8_t const *)first_limit, s->runes);
    size_t const rm = oracle_utf8_decode_((uint8_t const *)second, m, (uint8_t const *)second_limit, s->runes + rn);
    if (oracle_scratch_reserve_(s, rm, 0) != 0) return *status = -1, 0;
    return oracle_rune_dp_(k, s->runes, rn, s->runes + rn, rm, s->rows);
}

static int oracle_is_unit_levenshtein_(oracle_costs_t const *k) {
    return k->kind == oracle_levenshtein_k && k->match == 0 && k->mismatch == 1 && k->open == 1 && k->extend == 1;
}

static int64_t oracle_score_with_(oracle_costs_t const *k, char const *first, size_t n, char const *second,
                                  size_t m, oracle_scratch_t *scratch, int *status) {
    uint8_t const *a = (uint8_t const *)first, *b = (uint8_t const *)second;
    if (k->kind == oracle_smith_waterman_k && (n == 0 || m == 0)) return 0;
    if (oracle_is_unit_levenshtein_(k)) {
        if (n == 0) return (int64_t)m;
        if (m == 0) return (int64_t)n;
        /* The shorter side is the bit-vector pattern; the distance is symmetric for uniform costs. */
        uint8_t const *p = a, *t = b;
        size_t pn = n, tm = m;
        if (pn > tm) p = b, t = a, pn = m, tm = n;
        if (oracle_scratch_reserve_(scratch, 0, pn) != 0) return *status = -1, 0;
        return (int64_t)oracle_myers_(p, pn, t, tm, scratch->peq, scratch->vectors);
    }
    if (oracle_scratch_reserve_(scratch, m, 0) != 0) return *status = -1, 0;
    return oracle_dp_(k, a, n, b, m, scratch->rows);
}

int64_t oracle_score_pair(oracle_costs_t const *costs, char const *first, size_t first_length, char const *second,
                          size_t second_length) {
    oracle_scratch_t scratch = {0};
    int status = 0;
    int64_t const result = oracle_score_with_(costs, first, first_length, second, second_length, &scratch, &status);
    oracle_scratch_free_(&scratch);
    return result;
}

uint64_t oracle_levenshtein_bitparallel(char const *first, size_t first_length, char const *second,
                                        size_t second_length) {
    oracle_costs_t unit;
    memset(&unit, 0, sizeof(unit));
    unit.kind = oracle_levenshtein_k, unit.match = 0, unit.mismatch = 1, unit.open = 1, unit.extend = 1;
    return (uint64_t)oracle_score_pair(&unit, first, first_length, second, second_length);
}

/* Multi-threaded drivers: tasks are handed out one at a time through an atomic counter, like the reference's
 * `for_n_dynamic` over flattened cells (serial.hpp:2631-2644). */

typedef struct oracle_job_t {
    oracle_costs_t const *costs;
    char const *q_data, *c_data;
    uint64_t const *q_offsets, *c_offsets;
    size_t q_count, c_count, tasks;
    int mode; /* 0 = pairwise, 1 = cross, 2 = symmetric */
    int64_t *results;
    size_t stride;
    atomic_size_t next;
    atomic_int status;
} oracle_job_t;

static void *oracle_worker_(void *arg) {
    oracle_job_t *job = (oracle_job_t *)arg;
    oracle_scratch_t scratch = {0};
    for (size_t task = atomic_fetch_add(&job->next, 1); task < job->tasks; task = atomic_fetch_add(&job->next, 1)) {
        size_t q, c;
        if (job->mode == 0) q = c = task;
        else q = task / job->c_count, c = task % job->c_count;
        if (job->mode == 2 && c > q) continue;
        char const *qs = job->q_data + job->q_offsets[q];
        size_t const qn = (size_t)(job->q_offsets[q + 1] - job->q_offsets[q]);
        char const *cs = job->c_data + job->c_offsets[c];
        size_t const cn = (size_t)(job->c_offsets[c + 1] - job->c_offsets[c]);
        int status = 0;
        int64_t const score =
            job->costs->utf8 ? oracle_score_utf8_(job->costs, qs, qn, job->q_data + job->q_offsets[job->q_count], cs,
                                                  cn, job->c_data + job->c_offsets[job->c_count], &scratch, &status)
                             : oracle_score_with_(job->costs, qs, qn, cs, cn, &scratch, &status);
        if (status) {
            atomic_store(&job->status, status);
            break;
        }
        if (job->mode == 0) job->results[task] = score;
        else {
            job->results[q * job->stride + c] = score;
            if (job->mode == 2 && c != q) job->results[c * job->stride + q] = score;
        }
    }
    oracle_scratch_free_(&scratch);
    return NULL;
}

static int oracle_run_(oracle_job_t *job, size_t threads) {
    if (threads == 0) {
        long online = sysconf(_SC_NPROCESSORS_ONLN);
        threads = online > 0 ? (size_t)online : 1;
    }
    if (threads > job->tasks) threads = job->tasks ? job->tasks : 1;
    atomic_init(&job->next, 0);
    atomic_init(&job->status, 0);
    pthread_t *handles = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    if (!handles) return -1;
    size_t spawned = 0;
    for (size_t t = 1; t < threads; ++t)
        if (pthread_create(&handles[spawned], NULL, oracle_worker_, job) == 0) ++spawned;
    oracle_worker_(job);
    for (size_t t = 0; t < spawned; ++t) pthread_join(handles[t], NULL);
    free(handles);
    return atomic_load(&job->status);
}

int oracle_score_pairs_u64tape(oracle_costs_t const *costs, char const *first_data, uint64_t const *first_offsets,
                               char const *second_data, uint64_t const *second_offsets, size_t count,
                               int64_t *results, size_t threads) {
    oracle_job_t job;
    memset(&job, 0, sizeof(job));
    job.costs = costs, job.q_data = first_data, job.q_offsets = first_offsets;
    job.c_data = second_data, job.c_offsets = second_offsets;
    job.q_count = job.c_count = count, job.tasks = count, job.mode = 0, job.results = results;
    return oracle_run_(&job, threads);
}

int oracle_score_cross_u64tape(oracle_costs_t const *costs, char const *queries_data, uint64_t const *queries_offsets,
                               size_t queries_count, char const *candidates_data, uint64_t const *candidates_offsets,
                               size_t candidates_count, int64_t *results, size_t results_stride, size_t threads) {
    oracle_job_t job;
    memset(&job, 0, sizeof(job));
    int const symmetric = candidates_data == NULL;
    job.costs = costs, job.q_data = queries_data, job.q_offsets = queries_offsets, job.q_count = queries_count;
    job.c_data = symmetric ? queries_data : candidates_data;
    job.c_offsets = symmetric ? queries_offsets : candidates_offsets;
    job.c_count = symmetric ? queries_count : candidates_count;
    job.tasks = job.q_count * job.c_count, job.mode = symmetric ? 2 : 1;
    job.results = results, job.stride = results_stride;
    if (job.tasks == 0) return 0;
    return oracle_run_(&job, threads);
}

/* ---- Min-Hash fingerprints ------------------------------------------------------------------------------------ */

static uint64_t oracle_splitmix64_(uint64_t state) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int oracle_fingerprints_u64tape(size_t dimensions, size_t const *window_widths, size_t window_widths_count,
                                uint64_t seed, char const *data, uint64_t const *offsets, size_t count,
                                uint32_t *min_hashes, size_t hashes_stride, uint32_t *min_counts,
                                size_t counts_stride) {
    static size_t const default_widths[] = {3, 4, 5, 7, 9, 11, 15, 31};
    if (!window_widths || !window_widths_count) window_widths = default_widths, window_widths_count = 8;
    size_t const per_width = dimensions / window_widths_count;
    int const sliced = dimensions % window_widths_count == 0 && per_width % 64 == 0;
    for (size_t dim = 0; dim < dimensions; ++dim) {
        size_t const width = window_widths[(sliced ? dim / 64 : dim) % window_widths_count];
        uint64_t const multiplier = 256u + oracle_splitmix64_(seed + dim) % 384u;
        uint64_t const modulo = 4503599626977ull - oracle_splitmix64_(oracle_splitmix64_(seed + dim)) % (1ull << 20);
        uint64_t leading = 1; /* multiplier^(width - 1) mod modulo: the weight of a window's oldest byte */
        for (size_t i = 0; i + 1 < width; ++i) leading = leading * multiplier % modulo;
        for (size_t t = 0; t < count; ++t) {
            uint8_t const *text = (uint8_t const *)data + offsets[t];
            size_t const length = (size_t)(offsets[t + 1] - offsets[t]);
            uint32_t *hash_out = (uint32_t *)((char *)min_hashes + t * hashes_stride) + dim;
            uint32_t *count_out = (uint32_t *)((char *)min_counts + t * counts_stride) + dim;
            if (length < width) {
                *hash_out = 0xFFFFFFFFu, *count_out = 0;
                continue;
            }
            uint64_t state = 0, minimum = 0;
            uint32_t occurrences = 0;
            for (size_t i = 0; i < length; ++i) {
                uint64_t const incoming = (uint64_t)text[i] + 1u;
                if (i >= width) { /* drop the oldest byte: state - leading * outgoing, kept non-negative */
                    uint64_t const outgoing = (uint64_t)text[i - width] + 1u;
                    state = (state + modulo - leading * outgoing % modulo) % modulo;
                }
                state = (state * multiplier + incoming) % modulo;
                if (i + 1 == width) minimum = state, occurrences = 1;
                else if (i + 1 > width) {
                    if (state < minimum) minimum = state, occurrences = 1;
                    else if (state == minimum) ++occurrences;
                }
            }
            *hash_out = (uint32_t)(minimum & 0xFFFFFFFFu);
            *count_out = occurrences;
        }
    }
    return 0;
}
