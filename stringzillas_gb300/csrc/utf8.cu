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
 *  Passes: (1) one thread per string walks its runes, counts them and inserts each into an open-addressing set of
 *  code points; (2) one CTA numbers the occupied slots; (3) after an exclusive scan of the counts, one thread per
 *  string writes its codes.
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

__device__ __forceinline__ std::uint32_t rune_slot(std::uint32_t rune) {
    return (rune * 2654435761u) >> (32 - rune_set_bits_k);
}

__device__ __forceinline__ std::uint64_t tape_offset(tape_t const &tape, std::uint64_t i) {
    return tape.offset_bits == 32 ? static_cast<std::uint32_t const *>(tape.offsets)[i]
                                  : static_cast<std::uint64_t const *>(tape.offsets)[i];
}

/** Pass 1: rune counts per string, and the set of code points. */
__global__ void utf8_count_kernel(tape_t const tape, std::uint64_t const end, std::uint64_t *__restrict__ counts,
                                  rune_set_t *__restrict__ set) {
    for (std::uint64_t i = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tape.count;
         i += (std::uint64_t)gridDim.x * blockDim.x) {
        std::uint64_t position = tape_offset(tape, i);
        std::uint64_t const stop = tape_offset(tape, i + 1);
        std::uint64_t runes = 0;
        std::uint32_t previous = 0xFFFFFFFFu;
        while (position < stop) {
            std::uint32_t length;
            std::uint32_t const rune = rune_at(tape.base, position, end, length);
            position += length, ++runes;
            if (rune == previous) continue; // runs of one code point insert once
            previous = rune;
            std::uint32_t const key = rune + 1;
            std::uint32_t slot = rune_slot(rune);
            for (std::uint32_t probe = 0;; ++probe) {
                if (probe == rune_set_slots_k) {
                    set->overflow = 1;
                    break;
                }
                std::uint32_t const seen = set->keys[slot];
                if (seen == key) break;
                if (seen == 0) {
                    std::uint32_t const won = atomicCAS(&set->keys[slot], 0u, key);
                    if (won == 0 || won == key) break;
                }
                slot = (slot + 1) & (rune_set_slots_k - 1);
            }
        }
        counts[i] = runes;
    }
}

/** Pass 2: dense codes for the occupied slots, in slot order (one CTA). */
__global__ void utf8_codes_kernel(rune_set_t *__restrict__ set) {
    constexpr int threads = 1024;
    constexpr int per_thread = rune_set_slots_k / threads;
    __shared__ std::uint32_t scan[threads];
    int const t = threadIdx.x;
    std::uint32_t own = 0;
    for (int k = 0; k < per_thread; ++k) own += set->keys[t * per_thread + k] != 0;
    scan[t] = own;
    __syncthreads();
    for (int offset = 1; offset < threads; offset <<= 1) {
        std::uint32_t const add = t >= offset ? scan[t - offset] : 0u;
        __syncthreads();
        scan[t] += add;
        __syncthreads();
    }
    std::uint32_t code = scan[t] - own;
    for (int k = 0; k < per_thread; ++k) {
        int const slot = t * per_thread + k;
        set->codes[slot] = set->keys[slot] != 0 ? code++ : 0u;
    }
    if (t == threads - 1) set->symbols = scan[t];
}

/** Pass 3: each string's codes at its scanned offset (one byte each, or two for more than 256 code points). */
template <typename code_type_>
__global__ void utf8_write_kernel(tape_t const tape, std::uint64_t const end, std::uint64_t const *__restrict__ offsets,
                                  rune_set_t const *__restrict__ set, code_type_ *__restrict__ out) {
    for (std::uint64_t i = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tape.count;
         i += (std::uint64_t)gridDim.x * blockDim.x) {
        std::uint64_t position = tape_offset(tape, i);
        std::uint64_t const stop = tape_offset(tape, i + 1);
        code_type_ *target = out + offsets[i];
        std::uint32_t previous = 0xFFFFFFFFu, previous_code = 0;
        while (position < stop) {
            std::uint32_t length;
            std::uint32_t const rune = rune_at(tape.base, position, end, length);
            position += length;
            if (rune != previous) {
                std::uint32_t const key = rune + 1;
                std::uint32_t slot = rune_slot(rune);
                for (std::uint32_t probe = 0; probe < rune_set_slots_k && set->keys[slot] != key; ++probe)
                    slot = (slot + 1) & (rune_set_slots_k - 1);
                previous = rune, previous_code = set->codes[slot];
            }
            *target++ = (code_type_)previous_code;
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
    std::uint64_t const blocks = (tape.count + 255) / 256;
    int const grid = (int)(blocks < (std::uint64_t)sm_count * 8 ? blocks : (std::uint64_t)sm_count * 8);
    utf8_count_kernel<<<grid, 256, 0, stream>>>(tape, end, counts, set);
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
    std::uint64_t const blocks = (tape.count + 255) / 256;
    int const grid = (int)(blocks < (std::uint64_t)sm_count * 8 ? blocks : (std::uint64_t)sm_count * 8);
    if (wide) utf8_write_kernel<<<grid, 256, 0, stream>>>(tape, end, offsets, set, static_cast<std::uint16_t *>(out));
    else utf8_write_kernel<<<grid, 256, 0, stream>>>(tape, end, offsets, set, static_cast<std::uint8_t *>(out));
    return cudaGetLastError();
}

} // namespace szs_gb300
