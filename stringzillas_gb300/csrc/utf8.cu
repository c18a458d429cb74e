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
 *  bits staged in shared memory, 16 KB). A warp decodes 32 bytes at once when the string is well formed
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

__device__ __forceinline__ std::uint32_t tape_byte(tape_t const &tape, std::uint64_t end, std::uint64_t position) {
    return position < end ? (std::uint32_t)tape.base[position] : 0u;
}

/**
 *  One warp walks the string [begin, stop) 32 bytes at a time, lanes on consecutive bytes (coalesced loads), and
 *  calls `visit(rune, index)` on the lane of each code point's lead byte, `index` counting code points from the
 *  string's start. This holds only when the string is well formed in the decoder's sense: its first byte is a lead
 *  byte and every lead byte's length covers exactly the continuation bytes (10xxxxxx) that follow it, ending at
 *  `stop`; then the code points start exactly at the lead bytes, as a sequential walk would find them. Returns
 *  false, warp-uniformly, as soon as a window breaks that (code points visited before stay visited: both passes
 *  then walk the whole string again sequentially). Sets `count` to the string's code points on success.
 */
template <typename visit_>
__device__ __forceinline__ bool warp_walk(tape_t const &tape, std::uint64_t end, std::uint64_t begin,
                                          std::uint64_t stop, std::uint64_t &count, visit_ &&visit) {
    int const lane = threadIdx.x & 31;
    auto is_continuation = [](std::uint32_t byte) { return (byte & 0xC0u) == 0x80u; };
    std::uint64_t runes = 0;
    for (std::uint64_t window = begin; window < stop; window += 32) {
        std::uint64_t const position = window + (std::uint64_t)lane;
        std::uint32_t const here = tape_byte(tape, end, position);
        std::uint32_t const ahead = lane < 4 ? tape_byte(tape, end, window + 32 + (std::uint64_t)lane) : 0u;
        std::uint32_t following[5]; // bytes at position + 0 .. position + 4
        following[0] = here;
#pragma unroll
        for (int k = 1; k <= 4; ++k) {
            std::uint32_t const inside = __shfl_sync(0xFFFFFFFFu, here, (lane + k) & 31);
            std::uint32_t const beyond = __shfl_sync(0xFFFFFFFFu, ahead, (lane + k) & 31);
            following[k] = lane + k < 32 ? inside : beyond;
        }
        bool const active = position < stop;
        bool const lead = active && !is_continuation(here);
        std::uint32_t const length = 1u + (here >= 0xC0u) + (here >= 0xE0u) + (here >= 0xF0u);
        bool ok = !active || lead || position != begin; // the string starts on a lead byte
        if (lead) {
            ok = position + length <= stop;
#pragma unroll
            for (int k = 1; k < 4; ++k)
                if ((std::uint32_t)k < length) ok = ok && is_continuation(following[k]);
            std::uint32_t next = following[1];
#pragma unroll
            for (int k = 2; k <= 4; ++k)
                if ((std::uint32_t)k == length) next = following[k];
            ok = ok && (position + length == stop || !is_continuation(next));
        }
        if (!__all_sync(0xFFFFFFFFu, ok)) return false;
        std::uint32_t const leads = __ballot_sync(0xFFFFFFFFu, lead);
        if (lead) {
            std::uint32_t rune;
            switch (length) {
            case 1: rune = here; break;
            case 2: rune = (here & 0x1Fu) << 6 | (following[1] & 0x3Fu); break;
            case 3: rune = (here & 0x0Fu) << 12 | (following[1] & 0x3Fu) << 6 | (following[2] & 0x3Fu); break;
            default:
                rune = (here & 0x07u) << 18 | (following[1] & 0x3Fu) << 12 | (following[2] & 0x3Fu) << 6 |
                       (following[3] & 0x3Fu);
            }
            visit(rune, runes + (std::uint64_t)__popc(leads & ((1u << lane) - 1u)));
        }
        runes += (std::uint64_t)__popc(leads);
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
        if (rune < 65536u) {
            if (!(plane_s[rune >> 5] & bit)) atomicOr(&plane_s[rune >> 5], bit);
        }
        else atomicOr(&set->present[rune >> 5], bit);
    };
    int const lane = threadIdx.x & 31;
    std::uint64_t const warps = (std::uint64_t)gridDim.x * (blockDim.x >> 5);
    for (std::uint64_t i = (std::uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < tape.count;
         i += warps) {
        std::uint64_t const begin = tape_offset(tape, i), stop = tape_offset(tape, i + 1);
        std::uint64_t runes = 0;
        bool const walked = warp_walk(tape, end, begin, stop, runes,
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

/** Pass 2: the rank of every bitmap word and the number of distinct code points (one CTA of 1,024 threads, each
 *  over 64 consecutive words). */
__global__ void __launch_bounds__(1024) utf8_codes_kernel(rune_set_t *__restrict__ set) {
    constexpr int threads = 1024;
    constexpr int per_thread = rune_words_k / threads;
    static_assert(per_thread % 4 == 0, "words are read four at a time");
    __shared__ std::uint32_t scan[threads];
    int const t = threadIdx.x;
    auto const *words = reinterpret_cast<uint4 const *>(set->present + t * per_thread);
    std::uint32_t own = 0;
#pragma unroll 4
    for (int k = 0; k < per_thread / 4; ++k) {
        uint4 const w = words[k];
        own += __popc(w.x) + __popc(w.y) + __popc(w.z) + __popc(w.w);
    }
    scan[t] = own;
    __syncthreads();
    for (int offset = 1; offset < threads; offset <<= 1) {
        std::uint32_t const add = t >= offset ? scan[t - offset] : 0u;
        __syncthreads();
        scan[t] += add;
        __syncthreads();
    }
    std::uint32_t rank = scan[t] - own;
    for (int k = 0; k < per_thread; ++k) {
        std::uint32_t const word = t * per_thread + k;
        set->rank[word] = rank;
        rank += __popc(set->present[word]);
    }
    if (t == threads - 1) set->symbols = scan[t];
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
        bool const walked = warp_walk(tape, end, begin, stop, runes, [&](std::uint32_t rune, std::uint64_t index) {
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
