// Shared definitions of the Smith-Waterman pass kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsw {

// Large negative substitution score of padding columns: any cell fed by it
// clamps to 0, so a padded column behaves like the DP boundary.
constexpr int kNegBig = -(1 << 22);

// Alphabet size of the protein matrix (24 residues) plus one padding index.
constexpr int kAAPad = 24;
constexpr int kAADim = 25;

// Largest sequence length the packed argmax keys can hold (16-bit row/column).
constexpr int kMaxSeqLen = 65535;

struct PassParams {
    const uint8_t* ref;         // concatenated references (raw bytes or protein indices)
    const int64_t* ref_off;     // n+1 exclusive offsets
    const uint8_t* query;
    const int64_t* query_off;
    int64_t n;
    int match_p;                // DNA: match - open
    int mismatch_p;             // DNA: mismatch - open
    int open;                   // gap open  (<= 0)
    int ext;                    // gap extend (<= 0)
    const int* aa_matrix;       // protein: 25x25 int32 of (score - open), row = first index
    const int* aa_encoding;     // protein: 91-entry symbol -> matrix index table
    int32_t* score;             // results, SoA, n entries each
    int32_t* ref_begin;
    int32_t* ref_end;
    int32_t* query_begin;
    int32_t* query_end;
    int* queue;                 // work-queue counter (reset to 0 before the launch)
    int2* scratch;              // strip boundary: per group `scratch_rows` entries
    int scratch_rows;
    int* error;                 // device error flag (0 = ok)
};

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

__device__ __forceinline__ int bitrev5(int x) { return (int)(__brev((unsigned)x) >> 27); }

// Order in which the reference's two-level shfl_down argmax tree keeps full
// (value, row) ties between columns t (0-based) of the shorter sequence: the
// tree prefers the left lane at every level, so lanes are taken in bit-reversed
// order inside a warp and warps in bit-reversed order inside the block
// (kernel.cpp:47-86, 137-182 of the reference).  Columns beyond 1,024 (which
// the reference cannot run) keep the same order inside each 1,024 block and
// take blocks in increasing order.
__device__ __forceinline__ int tie_key(int t) {
    return ((t >> 10) << 10) | (bitrev5((t >> 5) & 31) << 5) | bitrev5(t & 31);
}
__device__ __forceinline__ int tie_key_inverse(int k) { return tie_key(k); }

}  // namespace gbsw
