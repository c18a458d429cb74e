/**
 *  @file dp_cells.cuh
 *  @brief Cell-level arithmetic for the wavefront kernels: one place that maps "optimum of" onto DPX fused
 *         instructions for 32-bit cells and onto plain min/max for 64-bit cells.
 *
 *  The recurrences are those of the reference's serial tile scorers
 *  (include/stringzillas/similarities/serial.hpp:723-725 linear, :924-930 affine, :817-818 / :1045-1046 local clamp):
 *
 *    linear:  H = opt(diag + s, opt(up, left) + g)                    local: max(., 0)
 *    affine:  E = opt(left_E + extend, left_H + open)    (horizontal gap track)
 *             F = opt(up_F + extend, up_H + open)        (vertical gap track)
 *             H = opt(diag + s, E, F)                    local: opt(E, F, max(diag + s, 0))
 *
 *  In the affine local case the reference clamps only the substitution path; since `max` is associative,
 *  `max(E, F, max(diag + s, 0)) == max(E, F, diag + s, 0)`, which is what the `_relu` DPX forms compute.
 */
#pragma once
#include <cstdint>

namespace szs_gb300 {

/** Byte `b_` of `x` as a signed 32-bit value: one byte permute whose selector copies the byte's sign bit into the
 *  three bytes above it. */
template <int b_>
__device__ __forceinline__ std::int32_t signed_byte(std::uint32_t x) {
    constexpr std::uint32_t sign = std::uint32_t(8 + b_);
    constexpr std::uint32_t selector = std::uint32_t(b_) | (sign << 4) | (sign << 8) | (sign << 12);
    std::uint32_t r;
    asm("prmt.b32 %0, %1, %1, %2;" : "=r"(r) : "r"(x), "r"(selector));
    return (std::int32_t)r;
}

template <typename cell_t, bool maximize_>
struct cell_ops_t;

/** 32-bit cells: Hopper/Blackwell DPX instructions fuse the add with the min/max. */
template <bool maximize_>
struct cell_ops_t<std::int32_t, maximize_> {
    using cell_t = std::int32_t;
    __device__ __forceinline__ static cell_t opt2(cell_t a, cell_t b) { return maximize_ ? max(a, b) : min(a, b); }
    __device__ __forceinline__ static cell_t opt3(cell_t a, cell_t b, cell_t c) {
        return maximize_ ? __vimax3_s32(a, b, c) : __vimin3_s32(a, b, c);
    }
    /** opt(a + b, c) in one DPX instruction. */
    __device__ __forceinline__ static cell_t add_opt(cell_t a, cell_t b, cell_t c) {
        return maximize_ ? __viaddmax_s32(a, b, c) : __viaddmin_s32(a, b, c);
    }
    /** max(a, b, c, 0); only used by local (maximising) scorers. */
    __device__ __forceinline__ static cell_t opt3_relu(cell_t a, cell_t b, cell_t c) { return __vimax3_s32_relu(a, b, c); }
    /** max(a + b, c, 0); only used by local (maximising) scorers. */
    __device__ __forceinline__ static cell_t add_opt_relu(cell_t a, cell_t b, cell_t c) {
        return __viaddmax_s32_relu(a, b, c);
    }
};

/** 64-bit cells: only reached when a 32-bit cell could overflow, so plain arithmetic is fine. */
template <bool maximize_>
struct cell_ops_t<std::int64_t, maximize_> {
    using cell_t = std::int64_t;
    __device__ __forceinline__ static cell_t opt2(cell_t a, cell_t b) { return maximize_ ? (a > b ? a : b) : (a < b ? a : b); }
    __device__ __forceinline__ static cell_t opt3(cell_t a, cell_t b, cell_t c) { return opt2(opt2(a, b), c); }
    __device__ __forceinline__ static cell_t add_opt(cell_t a, cell_t b, cell_t c) { return opt2(a + b, c); }
    __device__ __forceinline__ static cell_t opt3_relu(cell_t a, cell_t b, cell_t c) {
        cell_t m = opt3(a, b, c);
        return m > 0 ? m : 0;
    }
    __device__ __forceinline__ static cell_t add_opt_relu(cell_t a, cell_t b, cell_t c) {
        cell_t m = opt2(a + b, c);
        return m > 0 ? m : 0;
    }
};

/** Boundary seeds of the walkers: `init_score` / `init_gap` (serial.hpp:1150-1229, :1310-1414). */
template <typename cell_t>
struct boundary_t {
    cell_t open, extend;
    bool affine, local;
    /** M[i][0] (equally M[0][i]): the all-gap prefix. */
    __device__ __forceinline__ cell_t score(std::int64_t i) const {
        if (local || i == 0) return 0;
        if (!affine) return open * (cell_t)i;
        return open + extend * (cell_t)(i - 1);
    }
    /** Gap-track seed along the boundary: "discard" value that never beats opening from the boundary cell. */
    __device__ __forceinline__ cell_t gap(std::int64_t i) const {
        return local ? open + extend : open + extend + score(i);
    }
};

/** Reads a byte string front to back through aligned 8-byte loads. Never touches an 8-byte chunk that holds no
 *  byte of the string, so it cannot cross a page the string does not touch. */
struct byte_stream_t {
    std::uint64_t const *chunk;
    std::uint64_t window;
    int left; // bytes remaining in `window`

    __device__ __forceinline__ void open_at(std::uint8_t const *p) {
        std::uintptr_t const address = reinterpret_cast<std::uintptr_t>(p);
        chunk = reinterpret_cast<std::uint64_t const *>(address & ~std::uintptr_t(7));
        int const skip = int(address & 7);
        window = __ldg(chunk) >> (8 * skip);
        left = 8 - skip;
        ++chunk;
    }
    /** Next byte; the caller must not read past the string end by more than the chunk holding its last byte. */
    __device__ __forceinline__ std::uint32_t next() {
        if (left == 0) {
            window = __ldg(chunk);
            ++chunk;
            left = 8;
        }
        std::uint32_t const byte = std::uint32_t(window & 0xFF);
        window >>= 8;
        --left;
        return byte;
    }
};

/** Sequential reads of 16-bit codes in aligned 8-byte chunks: the `byte_stream_t` of tapes transcoded to 16-bit codes
 *  (UTF-8 calls over more than 256 code points). */
struct code16_stream_t {
    std::uint64_t const *chunk;
    std::uint64_t window;
    int left; // codes remaining in `window`

    __device__ __forceinline__ void open_at(std::uint8_t const *p) {
        std::uintptr_t const address = reinterpret_cast<std::uintptr_t>(p);
        chunk = reinterpret_cast<std::uint64_t const *>(address & ~std::uintptr_t(7));
        int const skip = int(address & 7) / 2;
        window = __ldg(chunk) >> (16 * skip);
        left = 4 - skip;
        ++chunk;
    }
    /** Next code; the caller must not read past the string end by more than the chunk holding its last code. */
    __device__ __forceinline__ std::uint32_t next() {
        if (left == 0) {
            window = __ldg(chunk);
            ++chunk;
            left = 4;
        }
        std::uint32_t const code = std::uint32_t(window & 0xFFFF);
        window >>= 16;
        --left;
        return code;
    }
};

/** Symbol `index` of a string: a byte, or a 16-bit code when `wide_`. */
template <bool wide_>
__device__ __forceinline__ std::uint32_t symbol_at(std::uint8_t const *string, std::uint64_t index) {
    if constexpr (wide_) return reinterpret_cast<std::uint16_t const *>(string)[index];
    else return string[index];
}

} // namespace szs_gb300
