/**
 *  @file utf8.cu
 *  @brief UTF-8 Levenshtein: code points of both tapes transcoded to one-byte codes on the device.
 *
 *  Edit distances over code points depend only on which code points are equal, so the batch's distinct code points
 *  are numbered 0..k-1 and every string is rewritten as a string of those numbers: bytes when k <= 256 (the byte-level
 *  Levenshtein routes then score the transcoded tapes unchanged), 16-bit codes up to k = 65,536 (scored by the
 *  Levenshtein routes' 16-bit-symbol instances). The reference decodes each string rune by rune
 *  (include/stringzillas/similarities/serial.hpp:2288-2299) with `sz_rune_decode_unchecked`
 *  (include/stringzilla/utf8_runes/serial.h:101-115): the length comes from the lead byte alone and continuation
 *  bytes are not checked, so a sequence cut off by the end of a string reads on into the next string of the tape.
 *  The same rule is applied here; bytes past the end of the tape read as 0.
 *
 *  Passes: (1) one warp per string walks its runes, counts them and marks each in a bitmap of code points (a CTA
 *  marks the Basic Multilingual Plane in shared memory, 8 KB, and merges it into the global bitmap once at its end;
 *  rarer code points are marked in the global bitmap directly); (2) one CTA ranks the bitmap's words, so a code
 *  point's code is the number of distinct code points below it; (3) after an exclusive scan of the counts, one warp
 *  per string writes its codes, each the word's rank plus a population count (the Basic Multilingual Plane's ranks and
 *  bits staged in shared memory, 16 KB). A warp decodes 128 bytes at once when the string is well formed
 *  (`warp_walk`), else its first lane walks the string with the sequential rule above.
 */
#include <cub/device/device_scan.cuh>

#include "launchers.h"

namespace szs_gb300 {

namespace {

__device__ __forceinline__ std::uint32_t rune_at(std::uint8_t const *base, std::uint64_t position, std::uint64_t end,
                                                 std::uint32_t &length) {
    std::uint32_t const lead = base[position];
    length = 1u + (lead >= 0xC0u) + (lead >= 0xE0u) + (lead >= 0xF0u);
    auto next = [&](std::uint32_t k) -> std::uint32_t {
        return position + k < end ? (std::uint32_t)(base[position + k] & 0x3Fu) : 0u;
    };
    switch (length) {
    case 1: return lead;
    case 2: return (lead & 0x1Fu) << 6 | next(1);
    case 3: return (lead & 0x0Fu) << 12 | next(1) << 6 | next(2);
    default: return (lead & 0x07u) << 18 | next(1) << 12 | next(2) << 6 | next(3);
    }
}

__device__ __forceinline__ std::uint64_t tape_offset(tape_t const &tape, std::uint64_t i) {
    return tape.offset_bits == 32 ? static_cast<std::uint32_t const *>(tape.offsets)[i]
                                  : static_cast<std::uint64_t const *>(tape.offsets)[i];
}

constexpr std::uint32_t plane_words_k = 65536 / 32; // the Basic Multilingual Plane's 2,048 bitmap words
constexpr int utf8_threads_k = 128;

/** Bit k (k < 4) set where byte k of `x` is a continuation byte (10xxxxxx). */
__device__ __forceinline__ std::uint32_t continuation_bits(std::uint32_t x) {
    std::uint32_t const tops = x & ~(x << 1) & 0x80808080u; // bit 7 of a byte: its bit 7 set and bit 6 clear
    return ((tops >> 7) * 0x01020408u) >> 24;                // gather bits 0, 8, 16, 24 into bits 0..3
}

/**
 *  One warp walks the string [begin, stop) 128 bytes at a time, lane L on bytes 4L..4L+3 of each window (coalesced
 *  loads), and calls `visit(rune, index)` once per code point, on the lane holding its lead byte, `index` counting
 *  code points from the string's start. This holds only when the string is well formed in the decoder's sense: its
 *  first byte is a lead byte and every lead byte's length covers exactly the continuation bytes (10xxxxxx) that follow
 *  it, ending at `stop`; then the code points start exactly at the lead bytes, as a sequential walk would find them,
 *  and no byte past `stop` is needed. Returns false, warp-uniformly, as soon as a window breaks that (code points
 *  visited before stay visited: both passes then walk the whole string again sequentially), or for strings of 2^31
 *  bytes or more. Sets `count` to the string's code points on success. Offsets inside the string are 32-bit and the
 *  checks are mask arithmetic, without branches.
 */
template <typename visit_>
__device__ __forceinline__ bool warp_walk(tape_t const &tape, std::uint64_t begin, std::uint64_t stop,
                                          std::uint64_t &count, visit_ &&visit) {
    if (stop - begin >= (1ull << 31)) return false;
    std::uint32_t const n = (std::uint32_t)(stop - begin);
    std::uint8_t const *string = tape.base + begin;
    int const lane = threadIdx.x & 31;
    std::uint32_t const lower = (1u << lane) - 1u;
    std::uint64_t runes = 0;
    for (std::uint32_t window = 0; window < n; window += 128) {
        std::uint32_t const rel = window + 4u * (std::uint32_t)lane;
        // This lane's four bytes, and the four after them (the next lane's, or the next window's for lane 31);
        // bytes past the string read as 0 and never decide a well-formed string.
        std::uint32_t own = 0, ahead = 0;
#pragma unroll
        for (std::uint32_t k = 0; k < 4; ++k) {
            own |= (rel + k < n ? (std::uint32_t)string[rel + k] : 0u) << (8 * k);
            if (lane == 0) ahead |= (window + 128 + k < n ? (std::uint32_t)string[window + 128 + k] : 0u) << (8 * k);
        }
        std::uint32_t const next_lane = __shfl_sync(0xFFFFFFFFu, own, (lane + 1) & 31);
        std::uint32_t const next_window = __shfl_sync(0xFFFFFFFFu, ahead, 0);
        std::uint32_t const high = lane == 31 ? next_window : next_lane;
        std::uint32_t const continuation = continuation_bits(own) | continuation_bits(high) << 4;

        bool ok = !(rel == 0 && (continuation & 1u)); // the string starts on a lead byte
        std::uint32_t leads = 0, lengths = 0;          // lengths: 4 bits per byte slot
#pragma unroll
        for (std::uint32_t j = 0; j < 4; ++j) {
            std::uint32_t const position = rel + j;
            std::uint32_t const byte = (own >> (8 * j)) & 0xFFu;
            bool const lead = position < n && !((continuation >> j) & 1u);
            // Lead bytes' lengths from their leading ones: 0 -> 1, 2 -> 2, 3 -> 3, 4 or more -> 4.
            std::uint32_t const length = min(max((std::uint32_t)__clz(~(byte << 24)), 1u), 4u);
            std::uint32_t const needed = ((1u << (length - 1)) - 1u) << (j + 1);
            bool const covered = position + length <= n && (continuation & needed) == needed &&
                                 (position + length == n || !((continuation >> (j + length)) & 1u));
            ok = ok && (!lead || covered);
            leads |= (lead ? 1u : 0u) << j;
            lengths |= length << (4 * j);
        }
        if (!__all_sync(0xFFFFFFFFu, ok)) return false;
        std::uint32_t before = 0, total = 0; // code points of lower lanes in this window, and of the whole window
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            std::uint32_t const slot = __ballot_sync(0xFFFFFFFFu, (leads >> j) & 1u);
            before += __popc(slot & lower), total += __popc(slot);
        }
#pragma unroll
        for (std::uint32_t j = 0; j < 4; ++j) {
            if (!((leads >> j) & 1u)) continue;
            std::uint32_t const word = __funnelshift_r(own, high, 8 * j); // bytes j..j+3
            std::uint32_t const length = (lengths >> (4 * j)) & 0xFu;
            std::uint32_t const b0 = word & 0xFFu, c1 = (word >> 8) & 0x3Fu, c2 = (word >> 16) & 0x3Fu,
                                c3 = (word >> 24) & 0x3Fu;
            std::uint32_t const rune = length == 1   ? b0
                                       : length == 2 ? (b0 & 0x1Fu) << 6 | c1
                                       : length == 3 ? (b0 & 0x0Fu) << 12 | c1 << 6 | c2
                                                     : (b0 & 0x07u) << 18 | c1 << 12 | c2 << 6 | c3;
            visit(rune, runes + before + (std::uint64_t)__popc(leads & ((1u << j) - 1u)));
        }
        runes += total;
    }
    count = runes;
    return true;
}

/** Pass 1: rune counts per string, and the bitmap of code points: one warp per string. */
__global__ void __launch_bounds__(utf8_threads_k) utf8_count_kernel(tape_t const tape, std::uint64_t const end,
                                                                     std::uint64_t *__restrict__ counts,
                                                                     rune_set_t *__restrict__ set) {
    __shared__ std::uint32_t plane_s[plane_words_k];
    for (std::uint32_t k = threadIdx.x; k < plane_words_k; k += blockDim.x) plane_s[k] = 0u;
    __syncthreads();
    auto mark = [&](std::uint32_t rune) {
        std::uint32_t const bit = 1u << (rune & 31u);
        if (rune < 65536u) atomicOr(&plane_s[rune >> 5], bit);
        else atomicOr(&set->present[rune >> 5], bit);
    };
    int const lane = threadIdx.x & 31;
    std::uint64_t const warps = (std::uint64_t)gridDim.x * (blockDim.x >> 5);
    for (std::uint64_t i = (std::uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < tape.count;
         i += warps) {
        std::uint64_t const begin = tape_offset(tape, i), stop = tape_offset(tape, i + 1);
        std::uint64_t runes = 0;
        bool const walked = warp_walk(tape, begin, stop, runes,
                                      [&](std::uint32_t rune, std::uint64_t) { mark(rune); });
        if (!walked && lane == 0) { // the decoder's sequential rule, as the reference applies it
            runes = 0;
            for (std::uint64_t position = begin; position < stop; ++runes) {
                std::uint32_t length;
                mark(rune_at(tape.base, position, end, length));
                position += length;
            }
        }
        if (lane == 0) counts[i] = runes;
    }
    __syncthreads();
    for (std::uint32_t k = threadIdx.x; k < plane_words_k; k += blockDim.x)
        if (plane_s[k]) atomicOr(&set->present[k], plane_s[k]);
}

/** Pass 2: the rank of every bitmap word and the number of distinct code points (one CTA of 32 warps, each over a
 *  contiguous block of 2,048 words read 32 consecutive words at a time). */
__global__ void __launch_bounds__(1024) utf8_codes_kernel(rune_set_t *__restrict__ set) {
    constexpr int warps = 32;
    constexpr std::uint32_t per_warp = rune_words_k / warps;
    __shared__ std::uint32_t warp_totals[warps];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    std::uint32_t const *present = set->present + warp * per_warp;
    std::uint32_t *rank = set->rank + warp * per_warp;
    std::uint32_t sum = 0;
    for (std::uint32_t k = lane; k < per_warp; k += 32) sum += __popc(present[k]);
    sum = __reduce_add_sync(0xFFFFFFFFu, sum);
    if (lane == 0) warp_totals[warp] = sum;
    __syncthreads();
    std::uint32_t offset = 0; // distinct code points in the blocks before this warp's
    for (int w = 0; w < warp; ++w) offset += warp_totals[w];
    for (std::uint32_t base = 0; base < per_warp; base += 32) {
        std::uint32_t const own = __popc(present[base + lane]);
        std::uint32_t scan = own; // inclusive over the 32 words
#pragma unroll
        for (int distance = 1; distance < 32; distance <<= 1) {
            std::uint32_t const lower = __shfl_up_sync(0xFFFFFFFFu, scan, distance);
            if (lane >= distance) scan += lower;
        }
        rank[base + lane] = offset + scan - own;
        offset += __shfl_sync(0xFFFFFFFFu, scan, 31);
    }
    if (threadIdx.x == 0) {
        std::uint32_t symbols = 0;
        for (int w = 0; w < warps; ++w) symbols += warp_totals[w];
        set->symbols = symbols;
    }
}

/** Pass 3: each string's codes at its scanned offset (one byte each, or two for more than 256 code points): one warp
 *  per string. */
template <typename code_type_>
__global__ void __launch_bounds__(utf8_threads_k)
    utf8_write_kernel(tape_t const tape, std::uint64_t const end, std::uint64_t const *__restrict__ offsets,
                      rune_set_t const *__restrict__ set, code_type_ *__restrict__ out) {
    __shared__ std::uint32_t present_s[plane_words_k], rank_s[plane_words_k];
    for (std::uint32_t k = threadIdx.x; k < plane_words_k; k += blockDim.x)
        present_s[k] = set->present[k], rank_s[k] = set->rank[k];
    __syncthreads();
    auto code_of = [&](std::uint32_t rune) -> std::uint32_t {
        std::uint32_t const word = rune >> 5, below = (1u << (rune & 31u)) - 1u;
        return rune < 65536u ? rank_s[word] + __popc(present_s[word] & below)
                             : __ldg(set->rank + word) + __popc(__ldg(set->present + word) & below);
    };
    int const lane = threadIdx.x & 31;
    std::uint64_t const warps = (std::uint64_t)gridDim.x * (blockDim.x >> 5);
    for (std::uint64_t i = (std::uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < tape.count;
         i += warps) {
        std::uint64_t const begin = tape_offset(tape, i), stop = tape_offset(tape, i + 1);
        code_type_ *target = out + offsets[i];
        std::uint64_t runes = 0;
        bool const walked = warp_walk(tape, begin, stop, runes, [&](std::uint32_t rune, std::uint64_t index) {
            target[index] = (code_type_)code_of(rune);
        });
        if (!walked && lane == 0) // the decoder's sequential rule, as the reference applies it
            for (std::uint64_t position = begin; position < stop;) {
                std::uint32_t length;
                *target++ = (code_type_)code_of(rune_at(tape.base, position, end, length));
                position += length;
            }
    }
}

} // namespace

std::size_t utf8_scan_scratch_bytes(std::uint64_t count) {
    std::size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, static_cast<std::uint64_t *>(nullptr),
                                  static_cast<std::uint64_t *>(nullptr), (int)(count + 1));
    return bytes;
}

cudaError_t launch_utf8_count(tape_t const &tape, std::uint64_t end, std::uint64_t *counts, rune_set_t *set,
                              int sm_count, cudaStream_t stream) {
    if (!tape.count) return cudaSuccess;
    std::uint64_t const blocks = (tape.count + utf8_threads_k / 32 - 1) / (utf8_threads_k / 32); // a warp per string
    int const grid = (int)(blocks < (std::uint64_t)sm_count * 16 ? blocks : (std::uint64_t)sm_count * 16);
    utf8_count_kernel<<<grid, utf8_threads_k, 0, stream>>>(tape, end, counts, set);
    return cudaGetLastError();
}

cudaError_t launch_utf8_codes(rune_set_t *set, cudaStream_t stream) {
    utf8_codes_kernel<<<1, 1024, 0, stream>>>(set);
    return cudaGetLastError();
}

cudaError_t launch_utf8_scan(std::uint64_t const *counts, std::uint64_t *offsets, std::uint64_t count, void *scratch,
                             std::size_t scratch_bytes, cudaStream_t stream) {
    return cub::DeviceScan::ExclusiveSum(scratch, scratch_bytes, counts, offsets, (int)(count + 1), stream);
}

cudaError_t launch_utf8_write(tape_t const &tape, std::uint64_t end, std::uint64_t const *offsets,
                              rune_set_t const *set, void *out, bool wide, int sm_count, cudaStream_t stream) {
    if (!tape.count) return cudaSuccess;
    std::uint64_t const blocks = (tape.count + utf8_threads_k / 32 - 1) / (utf8_threads_k / 32); // a warp per string
    int const grid = (int)(blocks < (std::uint64_t)sm_count * 16 ? blocks : (std::uint64_t)sm_count * 16);
    if (wide)
        utf8_write_kernel<<<grid, utf8_threads_k, 0, stream>>>(tape, end, offsets, set,
                                                               static_cast<std::uint16_t *>(out));
    else
        utf8_write_kernel<<<grid, utf8_threads_k, 0, stream>>>(tape, end, offsets, set,
                                                               static_cast<std::uint8_t *>(out));
    return cudaGetLastError();
}

} // namespace szs_gb300
