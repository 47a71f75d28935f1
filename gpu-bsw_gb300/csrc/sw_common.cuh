// Shared definitions of the Smith-Waterman pass kernels and their schedule.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsw {

// Pass geometry: a group of kG lanes owns one pair; each lane holds kC columns
// of a kW-column strip; rows advance in chunks of kChunk pipeline steps.
constexpr int kG = 4;
constexpr int kC = 16;
constexpr int kW = kG * kC;
constexpr int kChunk = 4;
constexpr int kThreads = 128;

// Large negative substitution score of padding columns: any cell fed by it
// clamps to 0, so a padded column behaves like the DP boundary.
constexpr int kNegBig = -(1 << 22);
// int8 form of the same, for the packed score profiles.
constexpr int kNegByte = -128;

// Protein alphabet (24 residues) plus one padding index.
constexpr int kAAPad = 24;
constexpr int kAADim = 25;
// Rows of a protein strip profile: the 24 residues, then the padding row
// (kAAPad: -128 in every column), which rows outside the pipeline read.
constexpr int kAAProfRows = kAAPad + 1;

// Largest sequence length the packed argmax keys can hold (16-bit row/column).
constexpr int kMaxSeqLen = 65535;

// Scoring modes of the pass kernels.
enum ScoreMode : int {
    kScoreDnaProfile = 0,  // DNA pairs made only of A/C/G/T: int8 profile per column, one prmt per cell
    kScoreDnaRaw = 1,      // DNA pairs with any other byte: byte compare per cell (the reference's rule)
    kScoreAaProfile = 2,   // protein: int8 profile of the strip in shared memory, one prmt per cell
    kScoreAaWide = 3,      // protein scores that do not fit int8: shared-memory matrix lookup per cell
};

// Work classes of the schedule, each a contiguous range of the schedule's
// pair order: 0 = int32 (DNA pairs whose scores do not fit the int8 profile or
// the int16x2 kernels, protein matrices outside int8), 1 = DNA raw bytes, 2 =
// nothing to do (reverse pass only), 3 = every other pair (A/C/G/T DNA,
// profile-scored protein), in two length bins by the shorter side: below
// kLongCols (kClassShort) and from kLongCols up (kClassLong), the long bin first.
// Each bin runs its own plan -- two pairs per group in the int16x2 kernels or
// one in int32, with its own lanes per group -- so that long pairs can run in
// wider groups than short ones (a long unit then finishes several times
// sooner, which keeps the longest-first queue balanced when long pairs hold
// most of a batch's cells); bins with the same plan run as one launch over the
// whole class, so that a small bin does not end in a launch of its own.
// Measured on the 200,000-pair mixed DNA batch (30% of pairs 1,000-2,048 x
// 1,500-4,096), with short pairs in 4-lane groups: 1,330 GCUPS with long pairs at
// 16 lanes (1,280 at 8, 1,309 at 32; 1,123 with every pair in 4-lane units); a
// 1,024-symbol threshold drops to 1,070.
constexpr int kClasses = 4;
constexpr int kClassIdle = 2;
constexpr int kClassBinned = 3;
// The per-pair class array marks the bins apart: kClassShort (= kClassBinned)
// and kClassLong.
constexpr int kClassShort = 3;
constexpr int kClassLong = 4;
constexpr int kBins = 2;
// Ranges of the schedule order a launch can take: the four classes, then the
// long bin and the short bin of class kClassBinned.
constexpr int kRangeLong = 4;
constexpr int kRangeShort = 5;
constexpr int kRanges = 6;
#ifndef GBSW_LONG_COLS
#define GBSW_LONG_COLS 512
#endif
#ifndef GBSW_DUAL_WIDE_LANES
#define GBSW_DUAL_WIDE_LANES 16
#endif
constexpr int kLongCols = GBSW_LONG_COLS;
// Lanes per group of the long bin when no tuning says otherwise and the short
// bin runs 4-lane dual groups.
constexpr int kDualWideLanes = GBSW_DUAL_WIDE_LANES;
__host__ __device__ constexpr bool is_bin_class(int cls) { return cls == kClassShort || cls == kClassLong; }
// Keys: each class takes a contiguous range of histogram buckets from
// class_base(cls): kClassBuckets for the int32 and raw-byte classes (longest
// first by pass cost), one bucket's range for the idle class, and for class
// kClassBinned kBinBuckets for the long bin, then kBinBuckets for the short one.
constexpr int kClassBuckets = 1 << 13;
// Block per pair: the "lanes" of a plan whose pairs each take a whole block
// (its warps share the pair, one column strip each), and the columns per lane.
constexpr int kTeamLanes = 128;
constexpr int kTeamColumns = 8;
constexpr int kBinBuckets = 1 << 13;
constexpr int kIdleBuckets = 1 << 12;
__host__ __device__ constexpr int class_base(int cls) {
    return cls <= kClassIdle ? cls * kClassBuckets : kClassIdle * kClassBuckets + kIdleBuckets;
}
constexpr int kBuckets = class_base(kClassBinned) + 2 * kBinBuckets;
static_assert(kClassBinned == kClasses - 1 && kClassIdle == kClassBinned - 1, "class layout");

struct PassParams {
    const uint8_t* ref;         // concatenated references (raw bytes)
    const int64_t* ref_off;     // n+1 exclusive offsets
    const uint8_t* query;
    const int64_t* query_off;
    int64_t n;
    int match;                  // DNA: match score
    int mismatch;               // DNA: mismatch score
    int open;                   // gap open  (<= 0)
    int ext;                    // gap extend (<= 0)
    const int* aa_matrix;       // protein: 25x25 int32 scores (row/column 24: padding), row = first index
    const int* aa_encoding;     // protein: 91-entry symbol -> matrix index table
    int32_t* score;             // results, SoA, n entries each
    int32_t* ref_begin;
    int32_t* ref_end;
    int32_t* query_begin;
    int32_t* query_end;
    const int* order;           // pair indices in schedule order
    const int* class_range;     // [begin, end) into `order` per range (cls): 2*kRanges ints
    int cls;                    // the class this launch works on
    int* queue;                 // work-queue counter (reset to 0 before the launch)
    int2* scratch;              // strip boundary: per group `scratch_rows` entries
    int scratch_rows;
    int* error;                 // device error flags (0 = ok)
    int rev_p;                  // reverse pass: column bound cost (see reverse_columns); 0 = none
    // Dual-pair forward pass: a pair whose best score exceeds dual_limit may
    // have overflowed int16; its slot in rerun (rerun[1] counts, the pair
    // indices follow from rerun[2]) queues it for the int32 pass, and its class
    // in pair_cls becomes 0 so that its reverse pass runs in int32 too.
    int dual_limit;
    int* rerun;
    uint8_t* pair_cls;
};

// Error flag bits.
constexpr int kErrSymbol = 1;    // protein byte outside the encoding table
constexpr int kErrNoHit = 2;     // reverse pass did not find the forward score
constexpr int kErrBounds = 4;    // a sequence longer than max_len, or ends out of range
constexpr int kErrTeam = 16;     // a block-per-pair team's wait for a strip edge ran out

__device__ __forceinline__ int bitrev5(int x) { return (int)(__brev((unsigned)x) >> 27); }

// Order in which the reference's two-level shfl_down argmax tree keeps full
// (value, row) ties between columns t (0-based) of the shorter sequence: the
// tree prefers the left lane at every level, so lanes are taken in bit-reversed
// order inside a warp and warps in bit-reversed order inside the block
// (kernel.cpp:47-86, 137-182 of the reference).  Columns beyond 1,024 (which
// the reference cannot run) keep the same order inside each 1,024 block and
// take blocks in increasing order.  The map is its own inverse.
__device__ __forceinline__ int tie_key(int t) {
    return ((t >> 10) << 10) | (bitrev5((t >> 5) & 31) << 5) | bitrev5(t & 31);
}

// Reverse pass: how many columns of the transposed reversed matrix can hold a
// cell reaching the forward score `target`.  The pass runs over the prefixes
// A[0:na] and B[0:nb] of a pair of lengths a and b; its columns are the longer
// prefix, its rows (nrows) the shorter.
//
// The forward pass's H(x, y) depends only on A[0:x] and B[0:y], so every
// alignment of score `target` inside the prefixes is a forward maximum, and the
// forward pass chose the smallest row of the longer sequence L among those:
// all of them end on the forward end's row of L.  When the reverse columns are
// that same sequence, each one therefore starts at reversed column 1, and the
// column c of its last cell is its extent in L: m matches plus the positions of
// L that mismatch or face a gap.  Each of those costs at least rev_p =
// min(-mismatch, -open, -extend) > 0 (DNA, all three negative; 0 disables the
// bound), and m <= nrows, so target <= match*m - rev_p*(c - m) gives
//   c <= nrows + (match * nrows - target) / rev_p.
// The begin the reverse pass looks for is such a cell, so columns past the
// bound never hold it and need no computing.
__host__ __device__ __forceinline__ int reverse_columns(int a, int b, int na, int nb, int target, int match,
                                                        int rev_p) {
    const int ncols = na < nb ? nb : na, nrows = na < nb ? na : nb;
    if (rev_p <= 0 || match <= 0 || (a < b) != (na < nb)) return ncols;
    const long long slack = (long long)match * nrows - target;
    if (slack < 0) return ncols;  // inconsistent ends: the pass's own checks report them
    const long long bound = (long long)nrows + slack / rev_p;
    return bound < ncols ? (int)bound : ncols;
}

// Reverse pass: the band.  Under the conditions of reverse_columns, take an
// alignment of score `target` inside the prefixes: it starts at reversed column
// 1 (see above) and some row r0 >= 1, with m matches, x mismatches, gL
// positions of the longer prefix facing a gap and gS of the shorter one.  At
// any of its cells (r, c), c = (r - r0 + 1) + gL' - gS' <= r + gL' for the
// counts gL', gS' up to that cell, and gL' <= gL <= (match * m - target) /
// rev_p <= (match * nrows - target) / rev_p = band, since every mismatch and
// gap position costs at least rev_p and m <= nrows.  So every cell on such an
// alignment -- and the begin the reverse pass looks for is the first of them --
// satisfies c <= r + band: a strip whose first column is f needs only its rows
// r >= f - band.  Cells outside the band may be computed from zeros instead of
// their true values: every value then stays at or below its true value, and
// the cells of those alignments, all inside the band, keep theirs exactly.
// Returns -1 when the bound does not apply (every row is needed).
__host__ __device__ __forceinline__ int reverse_band(int a, int b, int na, int nb, int target, int match,
                                                     int rev_p) {
    const int nrows = na < nb ? na : nb;
    if (rev_p <= 0 || match <= 0 || (a < b) != (na < nb)) return -1;
    const long long slack = (long long)match * nrows - target;
    if (slack < 0) return -1;  // inconsistent ends: the pass's own checks report them
    const long long band = slack / rev_p;
    return band < (1 << 30) ? (int)band : -1;
}

// First row a reverse strip whose first (1-based) column is `first_col` must
// compute under `band` (reverse_band; -1: row 1).  The band's first row there is
// first_col - band; the strip starts one row above it, rounded down to an odd
// row (the strip-boundary copies move two rows at a time from 16-byte
// boundaries).  Then even the diagonal predecessor of lane 0's first cell,
// (row0 - 1, first_col - 1), lies outside the band, so every lane may enter the
// strip from the zero state: cells above row0 are not needed.
__host__ __device__ __forceinline__ int band_first_row(int first_col, int band) {
    if (band < 0) return 1;
    const int r = first_col - band - 1;
    if (r <= 1) return 1;
    return r - ((r - 1) & 1);
}

// Strips and pipeline steps of a pass over an nrows x ncols matrix.
__host__ __device__ __forceinline__ int pass_cost(int nrows, int ncols) {
    return ((ncols + kW - 1) / kW) * (nrows + kG - 1);
}

}  // namespace gbsw
