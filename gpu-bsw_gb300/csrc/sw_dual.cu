// Dual-pair passes: two pairs per lane group, in the two 16-bit halves of
// every register (int16x2 DPX instructions), for DNA pairs made only of
// A/C/G/T (4, 8 or 16 lanes x 16 columns) and for protein pairs (16 or 32
// lanes, the widths protein batches run at).
//
// The pass kernels are bound by the integer ALU pipe; packing two pairs into
// one register halves the ALU instructions per cell.  A group of G lanes
// owns a unit of two pairs (the schedule puts pairs of the same strip count
// and nearly the same row count next to each other); lane g holds C columns
// of both pairs.  The unit is as tall as its taller pair and as many strips
// wide as its wider pair: in the forward pass each pair is left-padded to the
// unit's width with score -128 (exactly the matrix boundary, as in the int32
// kernel), in the reverse pass padded on the right (as the int32 kernel's
// reverse), and the rows past a pair's last row are simply not looked at by
// its half.
//
// Overflow: with gap values in [-16384, 0], every term the cell update forms
// stays inside int16 while the true H values stay at or below
// dual_limit = 32767 - m, where m is the largest single-cell score (DNA
// max(match, mismatch, 0), protein the matrix's largest entry).  The first cell
// whose true H exceeds dual_limit is still computed exactly (its inputs are
// exact and it exceeds them by at most m), so a pass whose best score is at
// most dual_limit was exact throughout, and a pair whose reported best exceeds
// it may have wrapped: the forward pass then writes no result for it, queues it
// for the int32 pass (PassParams::rerun) and moves it to int32 class 0, whose
// reverse pass it then takes as well.  The reverse pass never overflows: its
// scores are bounded by the forward score.
//
// Substitution scores, both halves with one prmt per cell:
//   DNA: each column keeps the packed int8 scores of its base against A, C, G,
//     T for both pairs; the two row codes pick one byte of each;
//   protein: the group keeps an int8 profile of both pairs' strips (24 residue
//     rows each) in shared memory; per row a lane loads its C scores of pair A's
//     row residue and of pair B's and interleaves byte c of each.
// Each thread builds and reads only its own slice of the profiles, laid out
// [half][residue][thread][C bytes] so that the loads of a warp stay
// conflict-free whatever residues its rows hold.
//
// Per cell (both halves at once; E = E(i,j) from the left, Ho = H + open):
//   s   = the two pairs' scores of this cell
//   F'  = max(F + ext, Ho_up, 0)
//   T   = max(F' + open, Ho_diag + s)
//   Ho  = max(E + open, T)
//   E'  = max(E + max(ext, open), T, 0)          (= max(E + ext, Ho, 0))
// which is the int32 kernel's recurrence (see sw_pass.cuh) evaluated per half.
// Argmax rules and the transposed reverse pass are also the int32 kernel's,
// band included (reverse_band): a unit's strips start at the rows its wider
// band needs (unit_band), and both halves compute every row from there.
#include <type_traits>

#include "sw_common.cuh"
#include "sw_device.cuh"
#include "sw_kernels.h"

namespace gbsw {
namespace {

// DNA geometry: 4 lanes x 16 columns.  Measured on the 100,000-pair DNA batch:
// faster than 8 lanes x 8 columns, and than 2 lanes x 32 columns at 3 blocks/SM
// (forward 6.13 vs 8.98 ms: a lane's 32-column E chain and the doubled serial
// time of a unit outweigh the halved per-step overhead).
#ifndef GBSW_DUAL_DNA_LANES
#define GBSW_DUAL_DNA_LANES 4
#endif
#ifndef GBSW_DUAL_DNA_COLS
#define GBSW_DUAL_DNA_COLS 16
#endif
constexpr int kGD = GBSW_DUAL_DNA_LANES;
constexpr int kCD = GBSW_DUAL_DNA_COLS;
// Long DNA pairs (the long bin's default plan): kDualWideLanes lanes x kCD columns.
constexpr int kGDW = kDualWideLanes;
static_assert(kGD * kCD == 64, "the schedule pairs DNA units by 64-column strips");
constexpr unsigned kNeg2 = 0x80008000u;
// Pipeline steps per loop iteration (even: boundary rows are copied in pairs;
// at most 8: one code byte each in a 64-bit word).  Longer chunks cut the
// per-iteration overhead but unroll the loop body further.  Measured on the
// 100,000-pair DNA and 30,000-pair protein batches: DNA forward 5.30 ms at 6
// steps (5.54 at 4, 5.52 at 8), DNA reverse 2.78 ms at 4 (3.32 at 6), protein
// forward 2.10 ms at 8 (2.21 at 6), protein reverse 2.67 ms at 6 (2.62 at 8,
// 2.63 at 4).
#ifndef GBSW_DUAL_CHUNK_FWD
#define GBSW_DUAL_CHUNK_FWD 6
#endif
#ifndef GBSW_DUAL_CHUNK_REV
#define GBSW_DUAL_CHUNK_REV 4
#endif
// The forward kernels of 8 or more lanes (long pairs) take 8 steps: mixed batch
// forward 63.6 against 65.5 ms; the 4-lane kernel stays at 6 (8 steps: 5.24
// against 4.96 ms on the throughput batch).
#ifndef GBSW_DUAL_CHUNK_FWD_WIDE
#define GBSW_DUAL_CHUNK_FWD_WIDE 8
#endif
#ifndef GBSW_DUAL_CHUNK_FWD_AA
#define GBSW_DUAL_CHUNK_FWD_AA 8
#endif
#ifndef GBSW_DUAL_CHUNK_REV_AA
#define GBSW_DUAL_CHUNK_REV_AA 6
#endif
// The 16-lane DNA reverse (long pairs) as well: mixed batch reverse 34.4 ms at 4
// steps, 34.5 at 6, 38.6 at 8; protein reverse 2.72 ms at 6, 2.84 at 4, 2.87 at 8.
#ifndef GBSW_DUAL_CHUNK_REV_WIDE
#define GBSW_DUAL_CHUNK_REV_WIDE 4
#endif
template <bool REVERSE, bool AA, int G>
__host__ __device__ constexpr int chunk_steps() {
    return REVERSE ? (AA ? GBSW_DUAL_CHUNK_REV_AA : (G >= 16 ? GBSW_DUAL_CHUNK_REV_WIDE : GBSW_DUAL_CHUNK_REV))
                   : (AA ? GBSW_DUAL_CHUNK_FWD_AA : (G >= 8 ? GBSW_DUAL_CHUNK_FWD_WIDE : GBSW_DUAL_CHUNK_FWD));
}
template <bool REVERSE, bool AA, int G>
constexpr bool chunk_ok() {
    return chunk_steps<REVERSE, AA, G>() % 2 == 0 && chunk_steps<REVERSE, AA, G>() <= 8;
}
static_assert(chunk_ok<false, false, 4>() && chunk_ok<false, false, 16>() && chunk_ok<true, false, 4>() &&
                  chunk_ok<true, false, 16>() &&
                  chunk_ok<false, true, 16>() && chunk_ok<true, true, 16>(),
              "chunk");

// lo half = sign-extended byte qa of a, hi half = sign-extended byte qb of b
__device__ __forceinline__ unsigned prmt2(unsigned a, unsigned b, unsigned sel) {
    unsigned r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}
__device__ __forceinline__ unsigned dual_sel(unsigned qa, unsigned qb) {
    return qa * 0x11u + qb * 0x1100u + 0xC480u;
}
// DNA row codes: base 0-3, or kPadCode for a row outside its pair.  The
// selector of a row code byte (qa | qb << 4) is one table lookup: selector
// byte of qa, and that of qb + 0x44 (bytes 4-7 hold pair B's scores).  Base q
// selects byte q sign-extended, as dual_sel; kPadCode selects the sign of byte
// 0 twice, a score of 0 or -1, so a padding row never scores above 0.
constexpr unsigned kPadCode = 4;
constexpr unsigned kSelTableLo = 0xB3A29180u, kSelTableHi = 0x88u;
__device__ __forceinline__ unsigned dna_row_sel(unsigned code) {
    return prmt2(kSelTableLo, kSelTableHi, code) + 0x4400u;  // only the low 16 bits select
}
__device__ __forceinline__ int lo16(unsigned x) { return (int)(short)(x & 0xffffu); }
__device__ __forceinline__ int hi16(unsigned x) { return (int)(short)(x >> 16); }
__device__ __forceinline__ unsigned pack16(int lo, int hi) {
    return (unsigned)(lo & 0xffff) | ((unsigned)hi << 16);
}

// One pair of a unit, as the kernel reads it.
struct Half {
    int pid;                 // -1: empty slot
    const uint8_t* rowseq;
    const uint8_t* colseq;
    int nrows, ncols, pad;
    int ncols_run;           // columns computed (reverse: bounded, see reverse_columns)
    int band;                // reverse: the band of reverse_band (-1: every row), until the unit's is set
    bool a_short;
    int target;              // reverse: the forward score
};

// The band (reverse_band) in the unit's padded column coordinates: a half's real
// column is its unit column minus its pad, so its band there is band + pad, and
// the unit's is the larger of its halves' (-1: a half without one).
__device__ __forceinline__ int unit_band(const Half& a, const Half& b) {
    const bool has_a = a.nrows > 0, has_b = b.nrows > 0;
    if ((has_a && a.band < 0) || (has_b && b.band < 0)) return -1;
    return max(has_a ? a.band + a.pad : 0, has_b ? b.band + b.pad : 0);
}

// Bytes of dynamic shared memory of a protein dual block: both pairs' strip
// profiles, kAAProfRows rows x C bytes per thread each.
template <int C>
constexpr size_t aa_dual_smem() {
    return (size_t)2 * kAAProfRows * kThreads * C;
}

// Resident 128-thread blocks per SM the dual kernels are compiled for (their
// register budget).  The DNA forward kernels hold their strip's column profiles
// in registers (32 more) at 3 blocks per SM (154 registers), which beat
// reloading them from shared memory every row step at 4 (same GPU, alternating
// builds: forward 5.13 vs 5.18 ms on the DNA throughput batch, 66.3 vs 68.2 ms
// on the mixed batch; at 4 blocks the register form spills and took 5.91 ms).
// The other kernels run at 4: 5 (96 registers, spills) measured slower.
#ifndef GBSW_DUAL_MIN_BLOCKS
#define GBSW_DUAL_MIN_BLOCKS 4
#endif
#ifndef GBSW_DUAL_FWD_DNA_MIN_BLOCKS
#define GBSW_DUAL_FWD_DNA_MIN_BLOCKS 3
#endif
#ifndef GBSW_DUAL_REV_DNA_MIN_BLOCKS
#define GBSW_DUAL_REV_DNA_MIN_BLOCKS 4
#endif
template <bool REVERSE, bool AA, int G, int C>
__global__ void __launch_bounds__(kThreads, AA ? GBSW_DUAL_MIN_BLOCKS
                                               : (REVERSE ? GBSW_DUAL_REV_DNA_MIN_BLOCKS : GBSW_DUAL_FWD_DNA_MIN_BLOCKS))
    sw_pass_dual(PassParams p) {
    constexpr int W = G * C;
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0 && C % 4 == 0 && C <= (AA ? 16 : 32),
                  "group geometry");
    constexpr int kChunkD = chunk_steps<REVERSE, AA, G>();
    // one code byte per step: a 32-bit word up to 4 steps (measured faster), else 64-bit
    using CodeWord = typename std::conditional<(kChunkD <= 4), unsigned, unsigned long long>::type;
    // Rows saved per half: forward, the row where a lane's max last grew; reverse
    // up to 8 lanes and protein, the row where a lane first reached the score (its
    // columns are searched once per strip, which keeps the unrolled step loop
    // short: with the packed hit test below, DNA reverse of the throughput batch
    // 2.28 -> 2.12 ms, protein 2.84 -> 2.70 ms).  The 16-lane DNA reverse (long
    // pairs) searches the hit row's columns at once: mixed batch reverse 34.4
    // against 34.9 ms.
#ifndef GBSW_REV_SAVE_HIT_MAX_G
#define GBSW_REV_SAVE_HIT_MAX_G 8
#endif
    constexpr bool kSaveHit = REVERSE && (AA || G <= GBSW_REV_SAVE_HIT_MAX_G);
    __shared__ __align__(16) int4 ssave[(REVERSE && !kSaveHit) ? 1 : 2][C / 4][kThreads];
    __shared__ __align__(16) int2 sbnd[kThreads / G][2][kChunkD];
    // reverse: the unit's band (unit_band), read at strip set-up only, so kept
    // out of the registers the row steps need; one slot per thread
    __shared__ int sband[REVERSE ? kThreads : 1];
    // DNA reverse: column profiles of this lane's C columns, both pairs: entry k
    // holds {A[2k], B[2k], A[2k+1], B[2k+1]}; a thread reads only its own slice
    // (the forward kernels keep them in registers, preg)
    __shared__ __align__(16) uint4 sprof[(AA || !REVERSE) ? 1 : C / 2][(AA || !REVERSE) ? 1 : kThreads];
    // protein: strip profiles (dynamic), the matrix and the symbol table
    extern __shared__ __align__(16) unsigned char sprof_aa[];
    __shared__ int smat[AA ? kAADim * kAADim : 1];
    __shared__ int senc[AA ? 128 : 1];
    if constexpr (AA) {
        // forward: rows carry the longer sequence = the matrix's first index;
        // reverse (transposed): rows carry the shorter one = the second index
        for (int k = threadIdx.x; k < kAADim * kAADim; k += blockDim.x) {
            const int r = k / kAADim, c = k % kAADim;
            smat[k] = REVERSE ? p.aa_matrix[c * kAADim + r] : p.aa_matrix[k];
        }
        // symbol -> matrix index (driver.cpp:252-258); bytes outside the table were
        // flagged by the schedule and read as 'A'
        for (int k = threadIdx.x; k < 128; k += blockDim.x) senc[k] = k < 91 ? p.aa_encoding[k] : 0;
        __syncthreads();
    }

    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane - g));
    const int group_in_block = threadIdx.x / G;
    const long long group_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    int2* bnd = p.scratch + (size_t)group_id * (size_t)p.scratch_rows;
    const int open = p.open, ext = p.ext;
    const unsigned open2 = pack16(open, open), ext2 = pack16(ext, ext);
    const unsigned gmax2 = pack16(max(open, ext), max(open, ext));  // E' = max(E + gmax, T, 0)
    const int qbegin = p.class_range[2 * p.cls], qend = p.class_range[2 * p.cls + 1];
    // Steps run without per-row checks: a row outside the pipeline (the fill
    // rows i < 1 of lanes g > 0, the drain rows past the last row, the steps
    // past the strip's end in its last chunk) reads the padding row code (DNA:
    // kPadCode; protein: the profile's padding row, -128).  From the initial
    // state (H = 0, E = F = 0), a row that scores <= 0 in every column leaves H,
    // E and F at 0 when the gap values are <= 0 (required for this class), so
    // lanes enter their first row in exactly the boundary state; rows past the
    // last one only feed later rows past it, which neither the argmax nor the
    // boundary buffer takes.
    constexpr bool kRowChecks = false;

    bool busy = false, done = false;
    Half h[2];
    int nrows = 0, nstrips = 0, strip = 0, st = 0, nsteps = 0;
    unsigned ho[C], f[C];
    uint4 preg[(!AA && !REVERSE) ? C / 2 : 1];  // forward DNA: the strip's column profiles, in registers
    unsigned ho_out = 0, e_out = 0, diag0 = 0;
    int mA = 0, mB = 0, miA = 0, miB = 0;
    unsigned tgt2 = 0x7fff7fffu;  // reverse: both halves' scores in the H + open domain
    uint64_t bestA = 0, bestB = 0;
    // row codes, one byte per step: DNA both halves (A | B << 4); protein the
    // residue index of half A in `codes` and of half B in `codesB`
    CodeWord codes = 0, codes_next = 0, codesB = 0, codesB_next = 0;
    int2* sb = &sbnd[group_in_block][0][0];
    int sbuf = 0;

    // Row codes of the rows this lane works on in the kChunkD steps from st0
    // (byte u: row st0 + u - g + 1).  Every lane fetches its own, a chunk ahead.
    auto row_code = [&](const Half& x, int i) -> unsigned {
        const int v = x.rowseq[REVERSE ? x.nrows - i : i - 1];
        if constexpr (AA) return (unsigned)senc[v & 127];
        return (unsigned)dna_code(v);
    };
    // DNA, rows well inside both pairs: each half's kChunkD row symbols come
    // from the two or three aligned words holding them (never a byte outside
    // the pair's own sequence), converted four symbols per op.  Byte u of the
    // result is the code of row i0 + u; false when a row or a word of the
    // window leaves either pair (the per-row path below then pads).
    constexpr int kWords = (kChunkD + 3 + 3) / 4;
    auto window_codes = [&](int i0, CodeWord& out) -> bool {
        CodeWord cw[2];
#pragma unroll
        for (int x = 0; x < 2; ++x) {
            const int s = REVERSE ? h[x].nrows - i0 - kChunkD + 1 : i0 - 1;  // first index read
            const int k = (int)(((uintptr_t)h[x].rowseq + (unsigned)s) & 3u);
            const int base = s - k;
            if (base < 0 || base + 4 * kWords > h[x].nrows) return false;
            const unsigned* w = reinterpret_cast<const unsigned*>(h[x].rowseq + base);
            const unsigned w0 = __ldg(w), w1 = __ldg(w + 1);
            const unsigned lo = __funnelshift_r(w0, w1, 8 * k);
            if constexpr (kChunkD <= 4) {
                // one word of symbols; reverse: rows run backwards through the sequence
                const unsigned v = REVERSE ? (__byte_perm(lo, 0, 0x0123) >> (8 * (4 - kChunkD))) : lo;
                cw[x] = (v >> 1) & 0x03030303u;  // dna_code of every byte
            } else {
                const unsigned hi = __funnelshift_r(w1, __ldg(w + 2), 8 * k);
                uint64_t v = ((uint64_t)hi << 32) | lo;
                if constexpr (REVERSE)
                    v = (((uint64_t)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123)) >>
                        (8 * (8 - kChunkD));
                cw[x] = (CodeWord)((v >> 1) & 0x0303030303030303ull);
            }
        }
        out = cw[0] | (cw[1] << 4);
        return true;
    };
    // DNA: the window words of the next chunk are loaded at the end of a chunk
    // and converted at the end of the next one, so that no step waits for the
    // loads (converting them as they are loaded stalled every chunk on them).
    // Forward pass of the 100,000-pair DNA batch 5.148 -> 4.982 ms, mixed batch
    // 66.4 -> 65.7 ms; reverse up to 8 lanes 2.122 -> 2.089 ms (same GPU,
    // alternating builds).  The 16-lane reverse, which searches its hit rows in
    // the step loop, spills with them at 4 blocks per SM.
#ifndef GBSW_SPLIT_CODES_FWD
#define GBSW_SPLIT_CODES_FWD 1
#endif
#ifndef GBSW_SPLIT_CODES_REV
#define GBSW_SPLIT_CODES_REV 1
#endif
    constexpr bool kSplitCodes = !AA && (REVERSE ? (GBSW_SPLIT_CODES_REV && G <= 8) : GBSW_SPLIT_CODES_FWD);
    unsigned rwin[2][kSplitCodes ? kWords : 1];
    int rsh[2] = {0, 0};
    bool rwin_ok = false;
    auto issue_window = [&](int st0) {
        const int i0 = st0 - g + 1;
        int base[2];
        rwin_ok = true;
#pragma unroll
        for (int x = 0; x < 2; ++x) {
            const int s = REVERSE ? h[x].nrows - i0 - kChunkD + 1 : i0 - 1;  // first index read
            const int k = (int)(((uintptr_t)h[x].rowseq + (unsigned)s) & 3u);
            base[x] = s - k;
            rsh[x] = 8 * k;
            rwin_ok = rwin_ok && base[x] >= 0 && base[x] + 4 * kWords <= h[x].nrows;
        }
        if (rwin_ok) {
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const unsigned* w = reinterpret_cast<const unsigned*>(h[x].rowseq + base[x]);
#pragma unroll
                for (int j = 0; j < kWords; ++j) rwin[x][j] = __ldg(w + j);
            }
        }
    };
    // the same conversion as window_codes
    auto take_window = [&]() -> CodeWord {
        CodeWord cw[2];
#pragma unroll
        for (int x = 0; x < 2; ++x) {
            const unsigned lo = __funnelshift_r(rwin[x][0], rwin[x][1], rsh[x]);
            if constexpr (kChunkD <= 4) {
                const unsigned v = REVERSE ? (__byte_perm(lo, 0, 0x0123) >> (8 * (4 - kChunkD))) : lo;
                cw[x] = (v >> 1) & 0x03030303u;
            } else {
                const unsigned hi = __funnelshift_r(rwin[x][1], rwin[x][kWords - 1], rsh[x]);
                uint64_t v = ((uint64_t)hi << 32) | lo;
                if constexpr (REVERSE)
                    v = (((uint64_t)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123)) >>
                        (8 * (8 - kChunkD));
                cw[x] = (CodeWord)((v >> 1) & 0x0303030303030303ull);
            }
        }
        return cw[0] | (cw[1] << 4);
    };
    auto fetch_codes = [&](int st0, CodeWord& cb) -> CodeWord {
        CodeWord cw = 0, cwb = 0;
        if constexpr (!AA && !REVERSE) {  // the reverse kernel spills with it (164 bytes)
            if (window_codes(st0 - g + 1, cw)) {
                cb = 0;
                return cw;
            }
        }
#pragma unroll
        for (int u = 0; u < kChunkD; ++u) {
            const int i = st0 + u - g + 1;
            unsigned qa = 0, qb = 0;
            qa = qb = AA ? (unsigned)kAAPad : kPadCode;
            if (i >= 1 && i <= h[0].nrows) qa = row_code(h[0], i);
            if (i >= 1 && i <= h[1].nrows) qb = row_code(h[1], i);
            if constexpr (AA) {
                cw |= (CodeWord)qa << (8 * u);
                cwb |= (CodeWord)qb << (8 * u);
            } else {
                cw |= (CodeWord)(qa | (qb << 4)) << (8 * u);
            }
        }
        cb = cwb;
        return cw;
    };
    // Lane 0 starts the copy of the boundary entries of rows [r0, r0 + kChunkD).
    auto fetch_chunk = [&](int r0, int buf) {
        if (strip > 0) {
#pragma unroll
            for (int u = 0; u < kChunkD; u += 2) {
                if (r0 + u <= nrows) {  // rows r0+u-1, r0+u: 16 bytes inside the buffer
                    const unsigned dst = (unsigned)__cvta_generic_to_shared(sb + buf * kChunkD + u);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(bnd + (r0 + u - 1)));
                }
            }
        }
        asm volatile("cp.async.commit_group;");
    };

    auto column_profile = [&](const Half& x, int t) -> unsigned {
        if (t < 0 || t >= x.ncols) return 0x80808080u;  // padding: -128 against every base
        const int idx = REVERSE ? (x.ncols - 1 - t) : t;
        const int code = dna_code(x.colseq[idx]);
        unsigned w = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) w |= ((unsigned)(code == q ? p.match : p.mismatch) & 0xffu) << (8 * q);
        return w;
    };

    // protein: this thread's C profile bytes of residue row e of half x
    auto aa_slice = [&](int x, int e) -> unsigned char* {
        return sprof_aa + (((size_t)x * kAAProfRows + e) * kThreads + threadIdx.x) * C;
    };

    auto setup_strip = [&]() {
        const int tA = strip * W + g * C - h[0].pad;
        const int tB = strip * W + g * C - h[1].pad;
        if constexpr (AA) {
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const int t0 = x ? tB : tA;
                int cc[C];  // matrix column of each of this lane's columns; -1: padding
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const int t = t0 + c;
                    cc[c] = -1;
                    if (t >= 0 && t < h[x].ncols)
                        cc[c] = senc[h[x].colseq[REVERSE ? h[x].ncols - 1 - t : t] & 127];
                }
                for (int e = 0; e < kAAProfRows; ++e) {  // the last: the padding row
                    unsigned wv[C / 4];
#pragma unroll
                    for (int k = 0; k < C / 4; ++k) {
                        unsigned w = 0;
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int c = 4 * k + j;
                            const int v = (cc[c] < 0 || e == kAAPad) ? kNegByte : smat[e * kAADim + cc[c]];
                            w |= ((unsigned)v & 0xffu) << (8 * j);
                        }
                        wv[k] = w;
                    }
                    unsigned* dst = reinterpret_cast<unsigned*>(aa_slice(x, e));
#pragma unroll
                    for (int k = 0; k < C / 4; ++k) dst[k] = wv[k];
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < C / 2; ++k) {
                const uint4 w = make_uint4(column_profile(h[0], tA + 2 * k), column_profile(h[1], tB + 2 * k),
                                           column_profile(h[0], tA + 2 * k + 1), column_profile(h[1], tB + 2 * k + 1));
                if constexpr (REVERSE) sprof[k][threadIdx.x] = w;
                else preg[k] = w;
            }
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
            ho[c] = open2;
            f[c] = 0;
        }
        diag0 = open2;
        ho_out = open2;  // what lane 0 hands on before its first step (rows i < 1 of lane 1)
        e_out = 0;
        mA = mB = 0;
        miA = miB = 0;
        st = 0;
        // reverse: the strip's steps start at its band's first row
        if constexpr (REVERSE) st = band_first_row(strip * W + 1, sband[threadIdx.x]) - 1;
        nsteps = nrows + G - 1;
        codes = fetch_codes(st, codesB);
        if constexpr (kSplitCodes) issue_window(st + kChunkD);
        else codes_next = fetch_codes(st + kChunkD, codesB_next);
        if (g == 0) {
            asm volatile("cp.async.wait_all;");
            sbuf = 0;
            fetch_chunk(st + 1, 0);
            fetch_chunk(st + 1 + kChunkD, 1);
        }
    };

    // one pair into half slot x: returns false when it needs no pass
    auto load_half = [&](int x, int pid) {
        Half& hh = h[x];
        hh.pid = pid;
        hh.nrows = hh.ncols = hh.ncols_run = 0;
        hh.rowseq = hh.colseq = p.ref;
        hh.a_short = false;
        hh.target = 0;
        hh.band = -1;
        if (pid < 0) return;
        const int64_t ra = p.ref_off[pid], rb = p.ref_off[pid + 1];
        const int64_t qa = p.query_off[pid], qb = p.query_off[pid + 1];
        const uint8_t* A = p.ref + ra;
        const uint8_t* B = p.query + qa;
        const int a = (int)(rb - ra), b = (int)(qb - qa);
        if constexpr (!REVERSE) {
            hh.a_short = a < b;  // kernel.cpp:248
            hh.colseq = hh.a_short ? A : B;
            hh.rowseq = hh.a_short ? B : A;
            hh.ncols = hh.a_short ? a : b;
            hh.ncols_run = hh.ncols;
            hh.nrows = hh.a_short ? b : a;
            if (hh.nrows > p.scratch_rows) {
                if (g == 0) atomicOr(p.error, kErrBounds);
                hh.nrows = hh.ncols = hh.ncols_run = 0;
            }
        } else {
            hh.target = p.score[pid];
            const int na = p.ref_end[pid], nb = p.query_end[pid];
            if (hh.target <= 0) {
                hh.target = 0;  // begins were written by the forward pass
                return;
            }
            if (na < 1 || na > a || nb < 1 || nb > b || a > p.scratch_rows || b > p.scratch_rows) {
                if (g == 0) atomicOr(p.error, kErrBounds);
                hh.target = 0;
                return;
            }
            hh.a_short = na < nb;  // kernel.cpp:444; transposed: rows = shorter prefix
            hh.rowseq = hh.a_short ? A : B;
            hh.colseq = hh.a_short ? B : A;
            hh.nrows = hh.a_short ? na : nb;
            hh.ncols = hh.a_short ? nb : na;
            hh.ncols_run = reverse_columns(a, b, na, nb, hh.target, p.match, p.rev_p);
            hh.band = reverse_band(a, b, na, nb, hh.target, p.match, p.rev_p);
        }
    };

    auto write_result = [&](const Half& hh, uint64_t best) {
        const int pid = hh.pid;
        if (pid < 0) return;
        if constexpr (!REVERSE) {
            const int v = (int)(best >> 32);
            if (v > p.dual_limit) {  // may have wrapped in int16: rerun in int32
                p.rerun[2 + atomicAdd(p.rerun + 1, 1)] = pid;
                p.pair_cls[pid] = 0;
                return;
            }
            if (v <= 0) {
                p.score[pid] = 0;
                p.ref_end[pid] = p.query_end[pid] = -1;
                p.ref_begin[pid] = p.query_begin[pid] = -1;
            } else {
                const int row = 0xFFFF - (int)((best >> 16) & 0xFFFF);
                const int col = tie_key(0xFFFF - (int)(best & 0xFFFF)) + 1;
                p.score[pid] = v;
                if (hh.a_short) {  // kernel.cpp:381-386
                    p.query_end[pid] = row;
                    p.ref_end[pid] = col;
                } else {           // kernel.cpp:387-392
                    p.ref_end[pid] = row;
                    p.query_end[pid] = col;
                }
            }
        } else {
            if (hh.target <= 0) {
                p.ref_begin[pid] = p.query_begin[pid] = -1;
                return;
            }
            if (best == ~0ull) {
                atomicOr(p.error, kErrNoHit);
                p.ref_begin[pid] = p.query_begin[pid] = -1;
                return;
            }
            const int r = (int)(best >> 32), qcol = (int)(best & 0xffffffffu);
            const int beginS = hh.nrows - r;   // kernel.cpp:580
            const int beginL = hh.ncols - qcol;  // kernel.cpp:579
            if (hh.a_short) {                  // kernel.cpp:591-595
                p.ref_begin[pid] = beginS;
                p.query_begin[pid] = beginL;
            } else {                           // kernel.cpp:596-600
                p.ref_begin[pid] = beginL;
                p.query_begin[pid] = beginS;
            }
        }
    };

    while (true) {
        if (!done && !busy) {
            int q = 0;
            if (g == 0) q = atomicAdd(p.queue, 1);
            q = __shfl_sync(gmask, q, 0, G);
            const int k0 = qbegin + 2 * q;
            if (k0 >= qend) {
                done = true;
            } else {
                load_half(0, p.order[k0]);
                load_half(1, k0 + 1 < qend ? p.order[k0 + 1] : -1);
                nrows = max(h[0].nrows, h[1].nrows);
                const int wA = (h[0].ncols_run + W - 1) / W, wB = (h[1].ncols_run + W - 1) / W;
                nstrips = max(wA, wB);
                if (nrows == 0 || nstrips == 0) {
                    if (g == 0) {
                        write_result(h[0], REVERSE ? ~0ull : 0ull);
                        write_result(h[1], REVERSE ? ~0ull : 0ull);
                    }
                } else {
                    // forward: left-padded (see the top of the file); reverse:
                    // padded on the right, which keeps the band's first rows
                    // (unit_band) those of the real columns
                    h[0].pad = REVERSE ? 0 : nstrips * W - h[0].ncols_run;
                    h[1].pad = REVERSE ? 0 : nstrips * W - h[1].ncols_run;
                    if constexpr (REVERSE) {
                        sband[threadIdx.x] = unit_band(h[0], h[1]);
                        tgt2 = pack16(h[0].target > 0 ? h[0].target + open : 0x7fff,
                                      h[1].target > 0 ? h[1].target + open : 0x7fff);
                    }
                    strip = 0;
                    bestA = bestB = REVERSE ? ~0ull : 0ull;
                    busy = true;
                    setup_strip();
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (done || !busy) continue;

        const bool last_strip = strip + 1 == nstrips;
        if (g == 0 && strip > 0) asm volatile("cp.async.wait_group 1;");
        // reverse: lane 0 reads its strip edge one step ahead (mixed batch reverse
        // 36.0 against 36.7 ms; in the 4-lane forward kernel the same cost 6%)
#ifndef GBSW_EDGE_AHEAD_REV
#define GBSW_EDGE_AHEAD_REV 1
#endif
        constexpr bool kEdgeAhead = REVERSE && GBSW_EDGE_AHEAD_REV;
        int2 bnext = make_int2((int)open2, 0);
        if (kEdgeAhead && g == 0 && strip > 0) bnext = sb[sbuf * kChunkD];
#pragma unroll
        for (int u = 0; u < kChunkD; ++u) {
            if (!kRowChecks || st < nsteps) {
                const int i = st - g + 1;
                unsigned ho_in = __shfl_up_sync(gmask, ho_out, 1, G);
                unsigned e_in = __shfl_up_sync(gmask, e_out, 1, G);
                // protein: a residue index; DNA: its selector ignores the bits above the byte pair
                const unsigned code = (unsigned)(codes >> (8 * u)) & (AA ? 0xffu : 0xffffffffu);
                const unsigned codeB = AA ? (unsigned)(codesB >> (8 * u)) & 0xffu : 0u;
                if (g == 0) {
                    if constexpr (kEdgeAhead) {
                        ho_in = (unsigned)bnext.x;
                        e_in = (unsigned)bnext.y;
                        if (u + 1 < kChunkD && strip > 0) bnext = sb[sbuf * kChunkD + u + 1];
                    } else if (strip == 0) {
                        ho_in = open2;
                        e_in = 0;
                    } else {
                        const int2 v = sb[sbuf * kChunkD + u];
                        ho_in = (unsigned)v.x;
                        e_in = (unsigned)v.y;
                    }
                }
                if (!kRowChecks || (unsigned)(i - 1) < (unsigned)nrows) {
                    const unsigned sel = AA ? 0u : dna_row_sel(code);
                    unsigned wa[AA ? C / 4 : 1], wb[AA ? C / 4 : 1];
                    if constexpr (AA) {
                        const unsigned char* pa = aa_slice(0, (int)code);
                        const unsigned char* pb = aa_slice(1, (int)codeB);
                        if constexpr (C == 16) {
                            const uint4 va = *reinterpret_cast<const uint4*>(pa);
                            const uint4 vb = *reinterpret_cast<const uint4*>(pb);
                            wa[0] = va.x; wa[1] = va.y; wa[2] = va.z; wa[3] = va.w;
                            wb[0] = vb.x; wb[1] = vb.y; wb[2] = vb.z; wb[3] = vb.w;
                        } else if constexpr (C == 8) {
                            const uint2 va = *reinterpret_cast<const uint2*>(pa);
                            const uint2 vb = *reinterpret_cast<const uint2*>(pb);
                            wa[0] = va.x; wa[1] = va.y;
                            wb[0] = vb.x; wb[1] = vb.y;
                        } else {
                            wa[0] = *reinterpret_cast<const unsigned*>(pa);
                            wb[0] = *reinterpret_cast<const unsigned*>(pb);
                        }
                    }
                    unsigned e = e_in, diag = diag0, hov = open2, mrow = open2;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        unsigned s2;
                        if constexpr (AA) {
                            s2 = prmt2(wa[c / 4], wb[c / 4], dual_sel(c % 4, c % 4));  // byte c%4 of each
                        } else {
                            const uint4 pw = REVERSE ? sprof[c / 2][threadIdx.x] : preg[c / 2];
                            s2 = (c & 1) ? prmt2(pw.z, pw.w, sel) : prmt2(pw.x, pw.y, sel);
                        }
                        const unsigned fv = __viaddmax_s16x2_relu(f[c], ext2, ho[c]);  // F(i,j)
                        const unsigned u2 = __viaddmax_s16x2(diag, s2, kNeg2);        // Ho_diag + s
                        const unsigned t = __viaddmax_s16x2(fv, open2, u2);           // max(F + open, .)
                        hov = __viaddmax_s16x2(e, open2, t);                          // Ho(i,j)
                        e = __viaddmax_s16x2_relu(e, gmax2, t);                       // E(i,j+1)
                        diag = ho[c];
                        ho[c] = hov;
                        f[c] = fv;
                        if (c & 1) mrow = __vimax3_s16x2(mrow, ho[c - 1], hov);
                    }
                    ho_out = hov;
                    e_out = e;
                    diag0 = ho_in;
                    if (g == G - 1 && !last_strip && (unsigned)(i - 1) < (unsigned)nrows)
                        __stcg(&bnd[i - 1], make_int2((int)ho_out, (int)e_out));
                    const int mhA = lo16(mrow) - open, mhB = hi16(mrow) - open;  // row max of H per half
                    if constexpr (!REVERSE) {
                        const bool impA = mhA > mA && (unsigned)(i - 1) < (unsigned)h[0].nrows;
                        const bool impB = mhB > mB && (unsigned)(i - 1) < (unsigned)h[1].nrows;
                        if (impA) {
                            mA = mhA;
                            miA = i;
#pragma unroll
                            for (int k = 0; k < C / 4; ++k)
                                ssave[0][k][threadIdx.x] =
                                    make_int4((int)ho[4 * k], (int)ho[4 * k + 1], (int)ho[4 * k + 2], (int)ho[4 * k + 3]);
                        }
                        if (impB) {
                            mB = mhB;
                            miB = i;
#pragma unroll
                            for (int k = 0; k < C / 4; ++k)
                                ssave[REVERSE ? 0 : 1][k][threadIdx.x] =
                                    make_int4((int)ho[4 * k], (int)ho[4 * k + 1], (int)ho[4 * k + 2], (int)ho[4 * k + 3]);
                        }
                    } else {
                        // first row reaching the score, leftmost column in it (per half);
                        // one test per row: a zero half of mrow ^ tgt2 (no H exceeds the score)
                        const unsigned dz = mrow ^ tgt2;
                        if (((dz - 0x00010001u) & ~dz & 0x80008000u) != 0) {
                            if (mhA == h[0].target && miA == 0 && (unsigned)(i - 1) < (unsigned)h[0].nrows) {
                                miA = i;
                                if constexpr (kSaveHit) {
#pragma unroll
                                    for (int k = 0; k < C / 4; ++k)
                                        ssave[0][k][threadIdx.x] = make_int4((int)ho[4 * k], (int)ho[4 * k + 1],
                                                                             (int)ho[4 * k + 2], (int)ho[4 * k + 3]);
                                } else {
                                    int cf = C;
#pragma unroll
                                    for (int c = C - 1; c >= 0; --c)
                                        if (lo16(ho[c]) == h[0].target + open) cf = c;
                                    mA = strip * W + g * C - h[0].pad + cf + 1;  // 1-based column
                                }
                            }
                            if (mhB == h[1].target && miB == 0 && (unsigned)(i - 1) < (unsigned)h[1].nrows) {
                                miB = i;
                                if constexpr (kSaveHit) {
#pragma unroll
                                    for (int k = 0; k < C / 4; ++k)
                                        ssave[kSaveHit ? 1 : 0][k][threadIdx.x] = make_int4(
                                            (int)ho[4 * k], (int)ho[4 * k + 1], (int)ho[4 * k + 2], (int)ho[4 * k + 3]);
                                } else {
                                    int cf = C;
#pragma unroll
                                    for (int c = C - 1; c >= 0; --c)
                                        if (hi16(ho[c]) == h[1].target + open) cf = c;
                                    mB = strip * W + g * C - h[1].pad + cf + 1;
                                }
                            }
                        }
                    }
                }
                ++st;
            }
        }
        if constexpr (kSplitCodes) {
            if (st < nsteps) {
                codes = rwin_ok ? take_window() : fetch_codes(st, codesB);
                issue_window(st + kChunkD);
            }
        } else {
            codes = codes_next;
            codesB = codesB_next;
            if (st < nsteps) codes_next = fetch_codes(st + kChunkD, codesB_next);
        }
        if (g == 0) {
            if (st < nsteps) fetch_chunk(st + 1 + kChunkD, sbuf);
            sbuf ^= 1;
        }
        if (st >= nsteps) {
            // ---- end of strip: this lane's candidates ----
            if constexpr (!REVERSE) {
#pragma unroll
                for (int x = 0; x < 2; ++x) {
                    const int m = x ? mB : mA;
                    if (m > 0) {
                        const int t0 = strip * W + g * C - h[x].pad;
                        const int mo = m + open;
                        int kmin = 0x7fffffff;
#pragma unroll
                        for (int k = 0; k < C / 4; ++k) {
                            const int4 v = ssave[x][k][threadIdx.x];
                            const int vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const int val = x ? hi16((unsigned)vv[j]) : lo16((unsigned)vv[j]);
                                if (val == mo) kmin = min(kmin, tie_key(t0 + 4 * k + j));
                            }
                        }
                        const uint64_t cand = pack_fwd(m, x ? miB : miA, kmin);
                        if (x) bestB = cand > bestB ? cand : bestB;
                        else bestA = cand > bestA ? cand : bestA;
                    }
                }
            } else {
                if constexpr (kSaveHit) {
                    // leftmost column of the saved hit row (1-based column of the strip)
#pragma unroll
                    for (int x = 0; x < 2; ++x) {
                        if ((x ? miB : miA) > 0) {
                            const int to = h[x].target + open;
                            int cf = C;
#pragma unroll
                            for (int k = C / 4 - 1; k >= 0; --k) {
                                const int4 v = ssave[x][k][threadIdx.x];
                                const int vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                                for (int j = 3; j >= 0; --j) {
                                    const int val = x ? hi16((unsigned)vv[j]) : lo16((unsigned)vv[j]);
                                    if (val == to) cf = 4 * k + j;
                                }
                            }
                            const int col = strip * W + g * C - h[x].pad + cf + 1;
                            if (x) mB = col;
                            else mA = col;
                        }
                    }
                }
                if (miA > 0) {
                    const uint64_t cand = ((uint64_t)(uint32_t)miA << 32) | (uint32_t)mA;
                    bestA = cand < bestA ? cand : bestA;
                }
                if (miB > 0) {
                    const uint64_t cand = ((uint64_t)(uint32_t)miB << 32) | (uint32_t)mB;
                    bestB = cand < bestB ? cand : bestB;
                }
            }
            __syncwarp(gmask);
            ++strip;
            if (strip < nstrips) {
                setup_strip();
            } else {
                uint64_t ga, gb;
                if constexpr (!REVERSE) {
                    ga = group_max_u64<G>(bestA, gmask);
                    gb = group_max_u64<G>(bestB, gmask);
                } else {
                    ga = group_min_u64<G>(bestA, gmask);
                    gb = group_min_u64<G>(bestB, gmask);
                }
                if (g == 0) {
                    write_result(h[0], ga);
                    write_result(h[1], gb);
                }
                busy = false;
            }
        }
    }
}

}  // namespace

namespace {

template <bool REVERSE, bool AA, int G, int C>
const void* dual_ptr() {
    return (const void*)sw_pass_dual<REVERSE, AA, G, C>;
}

// Kernel and dynamic shared memory of a dual variant; nullptr if none.
const void* pick_dual(bool reverse, bool aa, int width, size_t* dyn) {
    *dyn = 0;
    if (!aa) {
        if (width == 4)  // the large-batch plan
            return reverse ? dual_ptr<true, false, kGD, kCD>() : dual_ptr<false, false, kGD, kCD>();
        if (width == kDualWideLanes)  // its long pairs, and mid-size batches
            return reverse ? dual_ptr<true, false, kGDW, kCD>() : dual_ptr<false, false, kGDW, kCD>();
        if (width == 8)
            return reverse ? dual_ptr<true, false, 8, kCD>() : dual_ptr<false, false, 8, kCD>();
        return nullptr;
    }
    if (width == 16) {
        *dyn = aa_dual_smem<8>();
        return reverse ? dual_ptr<true, true, 16, 8>() : dual_ptr<false, true, 16, 8>();
    }
    if (width == 32) {
        *dyn = aa_dual_smem<4>();
        return reverse ? dual_ptr<true, true, 32, 4>() : dual_ptr<false, true, 32, 4>();
    }
    return nullptr;
}

}  // namespace

int dual_lanes(bool aa, int width) { return aa ? width : (width == 4 ? kGD : width); }

bool has_dual(bool aa, int width) {
    size_t dyn;
    return pick_dual(false, aa, width, &dyn) != nullptr;
}

cudaError_t launch_pass_dual(bool reverse, bool aa, int width, const PassParams& p, int blocks,
                             cudaStream_t stream) {
    size_t dyn = 0;
    const void* fn = pick_dual(reverse, aa, width, &dyn);
    if (!fn) return cudaErrorInvalidValue;
    if (dyn > 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    void* args[] = {(void*)&p};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(kThreads), args, dyn, stream);
}

cudaError_t pass_dual_occupancy(bool reverse, bool aa, int width, int* blocks_per_sm) {
    size_t dyn = 0;
    const void* fn = pick_dual(reverse, aa, width, &dyn);
    if (!fn) return cudaErrorInvalidValue;
    if (dyn > 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kThreads, dyn);
}

}  // namespace gbsw
