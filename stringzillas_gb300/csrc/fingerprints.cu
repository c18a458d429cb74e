/**
 *  @file fingerprints.cu
 *  @brief Min-Hash fingerprints (the reference's `szs_fingerprints_*`): per text and dimension, the minimum
 *         rolling hash over all windows of the dimension's width, and how often that minimum occurs.
 *
 *  Dimension d rolls a Rabin-Karp hash over bytes + 1 modulo m_d with multiplier a_d, both drawn from `splitmix64`
 *  streams of `seed + d` (include/stringzillas/fingerprints/serial.hpp:33-41, :426-432). The reference evaluates it
 *  in double precision with Barrett reductions (:1040-1050) that are exact on these magnitudes, so exact integer
 *  arithmetic gives the same residues. Each step here is one reduction of `state * a + byte_in + 1 + D *
 *  (byte_out + 1)` with D = -a^w mod m, the reference's two reductions (drop the outgoing byte, append the incoming
 *  one) folded into one.
 *
 *  Magnitudes: 2^42 < m < 2^43 and a < 640. The rolling state is kept in [0, 2m) rather than [0, m): any
 *  representative continues the recurrence, and the conditional subtraction that would make it canonical is only
 *  paid where the running minimum needs it. Then x < 2m * a + 256 * D + 256 < 2^54, every product is a 32 x 64-bit
 *  one (two multiply-adds), and the quotient is estimated from the top 32 bits of x: with t = x >> 22 and
 *  mu = floor(2^74 / m), floor(t * mu / 2^52) is q or q - 1 (the dropped low bits and mu's truncation each cost
 *  less than 2^-20 of a unit), so x - estimate * m lies in [0, 2m) again.
 *
 *  The running minimum is over canonical values c = state or state - m. A window can only reach it when the high
 *  words pass `state_hi <= min_hi || state_hi - m_hi <= min_hi + 1` (a borrow can lower state - m's high word by one),
 *  a 32-bit test that fails for nearly every window of a long text; the exact comparison runs behind it.
 *
 *  One warp scores 32 consecutive dimensions of one text: the lanes read the same byte stream (the reference's
 *  64-dimension slices share a width, so their outgoing bytes coincide too) and write 32 adjacent outputs.
 */
#include "launchers.h"

namespace szs_gb300 {

namespace {

/** A representative in [0, 2m) of x mod m, for x < 2^54 (see the file comment). */
__device__ __forceinline__ std::uint64_t reduce(std::uint64_t x, std::uint64_t modulo, std::uint32_t mu) {
    std::uint32_t const top = (std::uint32_t)(x >> 22);
    std::uint32_t const quotient = __umulhi(top, mu) >> 20;
    return x - (std::uint64_t)quotient * modulo;
}

__device__ __forceinline__ std::uint64_t canonical(std::uint64_t r, std::uint64_t modulo) {
    return r >= modulo ? r - modulo : r;
}

__device__ __forceinline__ std::uint64_t text_offset(tape_t const &tape, std::uint64_t i) {
    return tape.offset_bits == 32 ? static_cast<std::uint32_t const *>(tape.offsets)[i]
                                  : static_cast<std::uint64_t const *>(tape.offsets)[i];
}

__global__ void fingerprints_kernel(tape_t const texts, fingerprint_dim_t const *__restrict__ params,
                                    std::uint32_t const dimensions, std::uint32_t *__restrict__ hashes,
                                    std::uint64_t const hashes_stride, std::uint32_t *__restrict__ counts,
                                    std::uint64_t const counts_stride) {
    int const lane = threadIdx.x & 31;
    std::uint64_t const groups = (dimensions + 31) / 32;
    std::uint64_t const items = texts.count * groups;
    std::uint64_t const warps = (std::uint64_t)gridDim.x * (blockDim.x / 32);
    for (std::uint64_t item = (std::uint64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; item < items;
         item += warps) {
        std::uint64_t const text = item / groups;
        std::uint32_t const dim = (std::uint32_t)(item % groups) * 32 + lane;
        bool const live = dim < dimensions;
        fingerprint_dim_t const p = params[live ? dim : 0];
        std::uint64_t const start = text_offset(texts, text);
        std::uint64_t const length = text_offset(texts, text + 1) - start;
        std::uint8_t const *bytes = texts.base + start;
        std::uint32_t min_hash = 0xFFFFFFFFu, min_count = 0;
        if (length >= p.width) {
            // The first window: no outgoing bytes.
            std::uint64_t state = 0;
            for (std::uint32_t i = 0; i < p.width; ++i)
                state = reduce(state * p.multiplier + bytes[i] + 1u, p.modulo, p.mu);
            std::uint64_t minimum = canonical(state, p.modulo);
            std::uint32_t occurrences = 1;
            std::uint32_t const modulo_hi = (std::uint32_t)(p.modulo >> 32);
            std::uint32_t minimum_hi = (std::uint32_t)(minimum >> 32);
            // in + 1 + D * (out + 1) = in + D * out + (D + 1)
            std::uint64_t const constant = p.discard + 1u;
            std::uint64_t const windows = length - p.width;
#pragma unroll 8
            for (std::uint64_t i = 0; i < windows; ++i) {
                std::uint64_t const x =
                    state * p.multiplier + p.discard * bytes[i] + (constant + bytes[p.width + i]);
                state = reduce(x, p.modulo, p.mu);
                std::uint32_t const state_hi = (std::uint32_t)(state >> 32);
                if (__builtin_expect(state_hi <= minimum_hi || state_hi - modulo_hi <= minimum_hi + 1u, 0)) {
                    std::uint64_t const value = canonical(state, p.modulo);
                    if (value <= minimum) {
                        occurrences = value == minimum ? occurrences + 1u : 1u;
                        minimum = value;
                        minimum_hi = (std::uint32_t)(minimum >> 32);
                    }
                }
            }
            min_hash = (std::uint32_t)(minimum & 0xFFFFFFFFu), min_count = occurrences;
        }
        if (live) {
            reinterpret_cast<std::uint32_t *>(reinterpret_cast<unsigned char *>(hashes) + text * hashes_stride)[dim] =
                min_hash;
            reinterpret_cast<std::uint32_t *>(reinterpret_cast<unsigned char *>(counts) + text * counts_stride)[dim] =
                min_count;
        }
    }
}

std::uint64_t splitmix64(std::uint64_t state) {
    state += 0x9E3779B97F4A7C15ull;
    std::uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

} // namespace

fingerprint_dim_t fingerprint_dimension(std::uint64_t dim, std::uint64_t width, std::uint64_t seed) {
    fingerprint_dim_t p {};
    // Parameters of the reference's `floating_rolling_hasher<f64_t>` (serial.hpp:426-432).
    p.multiplier = (std::uint32_t)(256u + splitmix64(seed + dim) % 384u);
    p.modulo = 4503599626977ull - splitmix64(splitmix64(seed + dim)) % (1ull << 20);
    std::uint64_t leading = 1; // a^(w-1) mod m: the weight of a window's oldest byte
    for (std::uint64_t i = 0; i + 1 < width; ++i) leading = leading * p.multiplier % p.modulo;
    p.discard = (p.modulo - leading * p.multiplier % p.modulo) % p.modulo;
    p.mu = (std::uint32_t)(((unsigned __int128)1 << 74) / p.modulo);
    p.width = (std::uint32_t)width;
    return p;
}

cudaError_t launch_fingerprints(tape_t const &texts, fingerprint_dim_t const *params, std::uint32_t dimensions,
                                std::uint32_t *hashes, std::uint64_t hashes_stride, std::uint32_t *counts,
                                std::uint64_t counts_stride, int sm_count, cudaStream_t stream) {
    if (!texts.count || !dimensions) return cudaSuccess;
    std::uint64_t const items = texts.count * ((dimensions + 31) / 32);
    std::uint64_t const blocks = (items + 7) / 8; // 8 warps per CTA
    int const grid = (int)(blocks < (std::uint64_t)sm_count * 16 ? blocks : (std::uint64_t)sm_count * 16);
    fingerprints_kernel<<<grid, 256, 0, stream>>>(texts, params, dimensions, hashes, hashes_stride, counts,
                                                  counts_stride);
    return cudaGetLastError();
}

} // namespace szs_gb300
