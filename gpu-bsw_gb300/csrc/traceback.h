// Traceback kernels (host interface): one optimal path per aligned pair.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsw {

struct TraceParams {
    const uint8_t* ref;
    const int64_t* ref_off;
    const uint8_t* query;
    const int64_t* query_off;
    const int32_t* score;        // the pairs' results (int32 SoA)
    const int32_t* ref_begin;
    const int32_t* ref_end;
    const int32_t* query_begin;
    const int32_t* query_end;
    int64_t first, count;        // this launch: pairs [first, first + count)
    int protein;
    int match, mismatch, open, ext;
    const int* aa_matrix;        // protein: 25x25 padded, row = first index
    const int* aa_encoding;      // protein: 91 entries
    const int64_t* dir_off;      // per pair: first direction word within `dir` (this launch)
    uint32_t* dir;
    const int64_t* bnd_off;      // per pair: first strip-boundary entry within `bnd` (this launch)
    int2* bnd;
    const int64_t* order;        // the pairs of this launch in the order its groups take them (ids), or
                                 // nullptr: first, first + 1, ...
    const int64_t* slot_off;     // per pair: first operation slot within `ops`
    uint32_t* ops;
    int32_t* nops;               // per pair: operations written
    int32_t* path_score;         // per pair: H(k, m) of the path
    int* error;
};

// Error bit: a path's end value differs from the pair's score.
constexpr int kErrTrace = 8;

// Columns per lane of the traceback kernel (one 4-bit direction code each, so a
// lane's row is one 16- or 32-bit word), lanes per pair's group and columns per
// strip.  With one 32-lane warp per pair, 8 columns took 14.5 ms on the
// 100,000-pair DNA batch and 4 columns 15.0 ms: narrower strips waste fewer
// columns past a segment's end, but 8 columns amortise the per-row shuffles
// and stores over twice the cells.  Groups of 8 lanes (64-column strips, four
// pairs per warp) waste fewer still: a 150-300-column segment in 256-column
// strips, plus 31 fill steps per strip, computes 1.7 x its cells, in
// 64-column strips with 7 fill steps 1.2 x.
#ifndef GBSW_TRACE_COLS
#define GBSW_TRACE_COLS 8
#endif
#ifndef GBSW_TRACE_LANES
#define GBSW_TRACE_LANES 8
#endif
constexpr int kTraceColsPerLane = GBSW_TRACE_COLS;
constexpr int kTraceLanes = GBSW_TRACE_LANES;
static_assert(kTraceColsPerLane == 4 || kTraceColsPerLane == 8, "a lane's row fills a 16- or 32-bit word");
static_assert(kTraceLanes == 8 || kTraceLanes == 16 || kTraceLanes == 32, "groups of 8, 16 or 32 lanes");
constexpr int kTraceCols = kTraceLanes * kTraceColsPerLane;

// Direction memory, in 32-bit words, of a pair whose segment is m reference x k
// query symbols: per strip and row, one 4-bit code per column.
__host__ __device__ inline int64_t trace_dir_words(int m, int k) {
    return (int64_t)((m + kTraceCols - 1) / kTraceCols) * (int64_t)k * (kTraceCols / 8);
}

cudaError_t launch_trace(const TraceParams& p, cudaStream_t stream);
// Copies pair k's nops[k] operations from its slot to out + out_off[k].
cudaError_t launch_gather_ops(const uint32_t* ops, const int64_t* slot_off, const int32_t* nops,
                              const int64_t* out_off, uint32_t* out, int64_t n, cudaStream_t stream);

}  // namespace gbsw
