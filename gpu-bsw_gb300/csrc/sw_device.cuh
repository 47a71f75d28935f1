// Device helpers shared by the pass kernels.
#pragma once
#include <cstdint>

#include "sw_common.cuh"

namespace gbsw {
namespace {

__device__ __forceinline__ uint64_t pack_fwd(int v, int i, int key) {
    return ((uint64_t)(uint32_t)v << 32) | ((uint64_t)(0xFFFF - i) << 16) | (uint64_t)(0xFFFF - key);
}

template <int G>
__device__ __forceinline__ uint64_t group_max_u64(uint64_t v, unsigned gmask) {
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        uint64_t o = __shfl_xor_sync(gmask, v, off, G);
        v = o > v ? o : v;
    }
    return v;
}
template <int G>
__device__ __forceinline__ uint64_t group_min_u64(uint64_t v, unsigned gmask) {
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        uint64_t o = __shfl_xor_sync(gmask, v, off, G);
        v = o < v ? o : v;
    }
    return v;
}

// Sign-extending byte select: the byte of `x` chosen by `sel` (from sbyte_sel),
// as int.  prmt's selector nibbles with bit 3 set replicate the chosen byte's
// sign bit.
__device__ __forceinline__ int sbyte(unsigned x, unsigned sel) {
    int r;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "r"(sel));
    return r;
}
__host__ __device__ constexpr unsigned sbyte_sel(unsigned q) { return q * 0x1111u + 0x8880u; }

// 2-bit code of A/C/G/T: A=0, C=1, T=2, G=3.
__device__ __forceinline__ int dna_code(int c) { return (c >> 1) & 3; }

// max(a + b, c, 0) and max(a, b, c, 0): Blackwell DPX forms, or plain integer ops.
template <bool DPX>
__device__ __forceinline__ int add_max_relu(int a, int b, int c) {
    if constexpr (DPX) {
        return __viaddmax_s32_relu(a, b, c);
    } else {
        return max(max(a + b, c), 0);
    }
}
template <bool DPX>
__device__ __forceinline__ int add_max(int a, int b, int c) {
    if constexpr (DPX) {
        return __viaddmax_s32(a, b, c);
    } else {
        return max(a + b, c);
    }
}
template <bool DPX>
__device__ __forceinline__ int max3_relu(int a, int b, int c) {
    if constexpr (DPX) {
        return __vimax3_s32_relu(a, b, c);
    } else {
        return max(max(a, b), max(c, 0));
    }
}
template <bool DPX>
__device__ __forceinline__ int max3(int a, int b, int c) {
    if constexpr (DPX) {
        return __vimax3_s32(a, b, c);
    } else {
        return max(max(a, b), c);
    }
}

}  // namespace
}  // namespace gbsw
