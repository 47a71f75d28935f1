// Kernel template of the int32 Smith-Waterman passes (included by the
// translation units that instantiate it: sw_kernels.cu for 4-lane groups,
// sw_wide.cu for the wider groups used on small batches).
//
// Forward (end-position) and reverse (begin-position) passes for batches of
// independent pairs, int32 scores, sm_103a.
//
// Group geometry.  Large batches run 4-lane groups of 16 columns per lane (many
// pairs at once, the fewest instructions per cell).  Small batches cannot fill
// the GPU that way: their time is the serial time of the longest pair, so they
// run 8-, 16- or 32-lane groups with 8 or 4 columns per lane, which spread each
// pair over more lanes and cut the instructions a lane issues per row.
//
// Work decomposition.  A group of G consecutive lanes owns one pair at a time
// (32/G pairs per warp).  The DP matrix is cut into column strips of
// W = G*C columns; lane g holds C consecutive columns of the strip in
// registers (the previous row's H+open and F of each column) and the rows are
// streamed through the group as a software pipeline: at step s lane g works on
// row s-g+1 and receives, for the same row, the H+open and E of the column to
// its left from lane g-1 (one shfl_up each).  Every lane reads its own row
// symbols a chunk of steps ahead; after the first strip lane 0 also copies the
// previous strip's right edge (H+open and E per row) from a per-group boundary
// buffer in global memory; the last lane writes the edge for the next strip.
//
// Scheduling.  Pairs are bucket-sorted by class and cost (schedule.cu); a
// launch serves one class and its groups pull pairs longest-first from a work
// queue (one atomicAdd per pair).  The kernel is one flat loop whose every
// iteration advances each group by kChunk pipeline steps (or sets it up on a
// new pair or strip), so groups of one warp never wait for each other at loop
// exits.
//
// Recurrence (the reference's kernel.cpp:326-372) with E and F clamped at 0:
//   F = max(F_up + ext, H_up + open, 0)
//   E = max(E_left + ext, H_left + open, 0)
//   H = max(H_diag + s, E, F, 0)
// For open, ext <= 0 the clamp leaves every H unchanged (a negative E or F never
// wins the max against 0) and reproduces the reference's boundary values
// E(i,1) = 0 and F(1,j) = max(ext, open) <= 0 exactly.  In the forward pass
// padding columns sit on the LEFT of the first strip with a large negative
// score, so their H, E and F are all 0: they act exactly like the matrix
// boundary and never hold a maximum.  The reverse pass pads on the RIGHT of the
// last strip instead, so that a strip's band (below) starts from its real
// columns.  No H exceeds the forward score, and a padding column's own score
// is negative, so a padding cell reaches the score only through E, from a cell
// left of it in the same row that reached it (F comes from rows above, which
// hold no hit before the first one): the leftmost cell reaching the score in
// the first row that holds one, the begin, is always a real cell.
//
// Each column keeps Ho = H + open of the previous row and F.  Per cell, with
// E = E(i,j) arriving from the left:
//   F'  = max(F + ext, Ho_up, 0)
//   T   = max(Ho_diag + s, F' + open)
//   Ho  = max(E + open, T)                       (>= open as E >= 0)
//   E'  = E(i, j+1) = max(E + ext, Ho, 0) = max(E + max(ext, open), T, 0)
// The last form (substituting Ho) leaves a single DPX op per cell on the row's
// serial dependency chain (E -> E'); everything else hangs off it.  A lane
// passes E(i, j0) and Ho(i, j0-1) of its first column's left neighbour on.
//
// Substitution scores:
//   DNA, A/C/G/T-only pairs: each column keeps a packed int8 profile (its score
//     against A, C, T, G); the row symbol's 2-bit code picks the byte with one
//     sign-extending prmt;
//   DNA, other bytes: byte compare and select, exactly the reference's rule;
//   protein: each group keeps an int8 profile of its strip in shared memory
//     (24 residue rows x W columns); a lane reads its C scores for the row's
//     residue with C/16 16-byte loads (one 8- or 4-byte load for C = 8 or 4)
//     and extracts them with prmt;
//   protein scores outside int8: a lookup in a shared-memory copy of the matrix.
//
// Forward argmax (the reference's kernel.cpp:368-370 plus the shfl_down trees of
// kernel.cpp:47-86, 137-182): value desc, then smallest row i of the longer
// sequence, then the tie order `tie_key` over columns.  Each lane keeps the max
// of its own cells and the first row reaching it; on rows where that max grows
// it saves the row's values to shared memory, and at the end of the strip it
// finds the columns holding the max; the group reduces the lanes' candidates.
//
// Reverse pass (kernel.cpp:397-604 with the trees of kernel.cpp:3-45, 90-135):
// the same DP over A[0:ref_end] and B[0:query_end], both reversed; the begin is
// the cell with H == score that has the smallest reversed column of the shorter
// prefix, then the smallest reversed row of the longer one.  The pass runs
// TRANSPOSED (rows = the shorter prefix, columns = the longer one), so that order
// becomes "first row reaching the score, then leftmost column in it": a lane
// checks one comparison per row, and later strips stop at the best row found.
// For DNA with every penalty negative the pass computes only the columns that
// can hold the begin (reverse_columns) and, in each strip, only the rows from
// one above the first one its columns' band needs (reverse_band,
// band_first_row): the strip's steps start at row0 - 1 instead of 0, and every
// cell the lanes pass before row0 -- the diagonal of lane 0's first row
// included -- lies outside the band, where values computed from the zero state
// are allowed.
//
// Teams (block per pair).  With TEAM > 1 the kernel's warps (32-lane groups)
// work on one pair together: warp w takes strips w, w + TEAM, w + 2 TEAM, ...,
// so that a long pair's strips run side by side instead of one after another
// (the reference runs one block per pair, driver.cpp:176, but cannot run a
// shorter side above 1,024).  Strip s + 1 needs the right edge of strip s, row
// by row: warp w writes the edges of its strips to the boundary buffer of warp
// w + 1 (mod TEAM) and publishes, after every chunk, how many rows of which
// strip are written -- (strip << 16) | rows, and row field 0xFFFF once the
// strip is complete -- in a shared-memory counter per warp, after a CTA-scope
// fence; warp w + 1 waits for the rows of a chunk before copying them in.  A
// warp writes strip s + TEAM's edge row r only after warp w + 1 has finished
// row r of strip s + 1 (the chain of strips s + 1 ... s + TEAM - 1 runs
// through every other warp), and that warp read its input row r first, so an
// edge row is never overwritten before it is read.
//
// A warp that leaves a pair publishes -(X + 2), X the first of its strips it
// did not complete: a warp waiting on a strip below X goes on (those strips are
// complete), one waiting on strip X or later leaves too.  Every wait is
// bounded: a wait that runs out sets kErrTeam and the warp leaves the pair.
// The reverse pass shares its best hit across the team (shared memory), and a
// warp stops once its next strip starts below the rows still to search; every
// later strip then has no row to search either, so a warp that started one of
// them with an older best can drop it.  A strip's row limit comes from the best
// hit at its set-up, which only ever improves, and hits found before a strip
// is set up lie in strips to its left (a strip's rows wait on the strip to its
// left); so where a strip computes rows past its left neighbour's limit R
// (edge entries of an older strip), those rows lie below R, where no hit can
// beat the one that set R.  At the end of a pair the team combines its warps'
// results in shared memory.
#pragma once
#include <climits>
#include <type_traits>

#include "sw_common.cuh"
#include "sw_device.cuh"

// Pipeline steps per loop iteration of 16- and 32-lane groups.  Measured with
// 32-lane groups: 5,000 DNA pairs 632 vs 593 GCUPS and 5,000 protein pairs 187
// vs 165 GCUPS at 8 steps against 4.
#ifndef GBSW_PASS_CHUNK_WIDE
#define GBSW_PASS_CHUNK_WIDE 8
#endif

namespace gbsw {
namespace {

// Resident 128-thread blocks per SM each variant is compiled for (its register
// budget).  Four for all: squeezing the profile variants into five blocks costs
// spills and measured slower (forward 11.6 vs 11.4 ms on the DNA throughput batch).
#ifndef GBSW_PROFILE_MIN_BLOCKS
#define GBSW_PROFILE_MIN_BLOCKS 4
#endif
template <int SCORE>
constexpr int min_blocks() {
    return (SCORE == kScoreDnaProfile || SCORE == kScoreAaProfile) ? GBSW_PROFILE_MIN_BLOCKS : 4;
}

// Team hand-off: the row field of a complete strip.
constexpr int kTeamStripDone = 0xFFFF;
// Polls of a team wait before it gives up (each poll sleeps about 100 ns, so
// about two seconds); a wait that runs out sets kErrTeam.
constexpr int kTeamSpin = 1 << 24;

template <int SCORE, bool REVERSE, bool DPX, int G, int C, int TEAM = 1>
__global__ void __launch_bounds__(kThreads, min_blocks<SCORE>()) sw_pass(PassParams p) {
    constexpr int W = G * C;
    static_assert(TEAM == 1 || (G == 32 && TEAM == kThreads / 32), "a team is every warp of the block");
    // pipeline steps per loop iteration; the row codes of the next iteration are
    // fetched one iteration ahead, so wide groups (small batches, few warps per SM
    // to hide load latency) fetch further ahead with longer iterations
    constexpr int kCh = G >= 16 ? GBSW_PASS_CHUNK_WIDE : kChunk;
    static_assert(kCh % 2 == 0 && kCh <= 8, "chunk");
    using CodeWord = typename std::conditional<(kCh <= 4), unsigned, unsigned long long>::type;
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0 && C % 4 == 0, "group geometry");
    constexpr int kProfBytes = kAAProfRows * W;  // protein strip profile of one group
    constexpr bool AA = SCORE == kScoreAaProfile || SCORE == kScoreAaWide;
    // protein profile of each group's strip (dynamic shared memory, kProfBytes
    // per group): row e holds s'(e, column) for the W columns
    extern __shared__ __align__(16) int8_t sprof_dyn[];
    // Forward pass: a lane whose running max grows saves that row's C values of
    // H + open here (layout [quad][thread], conflict-free 16-byte stores); the
    // columns holding the max are resolved once per strip, not per row.
    constexpr bool kSaveRow = !REVERSE;
    __shared__ __align__(16) int4 ssave[kSaveRow ? C / 4 : 1][kSaveRow ? kThreads : 1];
    __shared__ __align__(16) int2 sbnd[kThreads / G][2][kCh];
    __shared__ int smat[AA ? kAADim * kAADim : 1];
    __shared__ int senc[AA ? 128 : 1];
    // teams: each warp's published edge progress ((strip << 16) | rows written,
    // -1 before its first chunk, -(X + 2) once it left the pair with strip X
    // not complete), the team's best (forward: max key; reverse: min hit) and
    // its next queue slot
    __shared__ int s_prog[TEAM];
    __shared__ unsigned long long s_best;
    __shared__ int s_q;
    if constexpr (AA) {
        // forward: rows carry the longer sequence = the matrix's first index;
        // reverse (transposed): rows carry the shorter one = the second index.
        for (int k = threadIdx.x; k < kAADim * kAADim; k += blockDim.x) {
            int r = k / kAADim, c = k % kAADim;
            smat[k] = REVERSE ? p.aa_matrix[c * kAADim + r] : p.aa_matrix[k];
        }
        // symbol -> matrix index (driver.cpp:252-258); bytes outside the table
        // were flagged by the schedule and read as 'A'
        for (int k = threadIdx.x; k < 128; k += blockDim.x) senc[k] = k < 91 ? p.aa_encoding[k] : 0;
        __syncthreads();
    }

    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane - g));
    const int group_in_block = threadIdx.x / G;
    const long long group_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    // strip edges: read from bnd_in, written to bnd_out (the group's own buffer;
    // teams: warp w reads buffer w, written by warp w - 1, and writes w + 1)
    const int tw = TEAM > 1 ? (int)(threadIdx.x >> 5) : 0;
    int2* bnd_in = p.scratch + (size_t)group_id * (size_t)p.scratch_rows;
    int2* bnd_out = TEAM > 1 ? p.scratch + ((size_t)blockIdx.x * TEAM + (tw + 1) % TEAM) * (size_t)p.scratch_rows
                             : bnd_in;
    bool team_abort = false;   // teams: this warp left the pair (warp-uniform)
    bool team_finish = false;  // teams: this warp is done with the pair; the team joins at the loop's top
    const int open = p.open, ext = p.ext;
    const int gmax = max(open, ext);  // E(i,j+1) = max(E + max(ext, open), T, 0), see above
    const int qbegin = p.class_range[2 * p.cls], qend = p.class_range[2 * p.cls + 1];
    // Steps run without per-row checks except for raw DNA bytes: a row outside
    // the pipeline (the fill rows i < 1 of lanes g > 0, the rows past the last
    // one, the steps past the strip's end in its last chunk) reads the padding
    // row code, whose score is <= 0 in every column (DNA profile: code 4 selects
    // a zero byte; protein: the padding row, -128 or kNegBig).  From the initial
    // state (H = 0, E = F = 0) such a row leaves H, E and F at 0, as gap values
    // are <= 0, so every lane enters its first row in exactly the boundary state;
    // rows past the last one only feed later rows past it, which neither the
    // argmax nor the boundary buffer takes.  Raw bytes have no score <= 0 to pad
    // with (the mismatch score may be positive) and keep the checks.
    constexpr bool kRowChecks = SCORE == kScoreDnaRaw;
    constexpr unsigned kPadRow = SCORE == kScoreDnaProfile ? 4u : (unsigned)kAAPad;

    // ---- per-group pair state (identical in the G lanes) ----
    int pid = -1;
    bool done = false;
    const uint8_t* rowseq = nullptr;  // streamed sequence (forward: longer; reverse: shorter prefix)
    const uint8_t* colseq = nullptr;  // sequence held in registers
    int nrows = 0, ncols = 0, nstrips = 0, pad = 0, strip = 0, st = 0, nsteps = 0, rows = 0;
    int ncols_run = 0;                // columns computed (reverse: bounded, see reverse_columns)
    int band = -1;                    // reverse: the band of reverse_band (-1: every row)
    bool rev = false;                 // read both sequences back to front (reverse pass)
    bool a_short = false;
    int target = 0;                   // reverse: the score to find
    // ---- per-lane state ----
    int ho[C], f[C];
    unsigned prof[SCORE == kScoreDnaProfile ? C : 1];
    int sc[SCORE == kScoreDnaRaw || SCORE == kScoreAaWide ? C : 1];
    int mmv[SCORE == kScoreDnaRaw ? C : 1];
    int ho_out = 0, e_out = 0, diag0 = 0;
    int m = 0;                        // lane max in this strip (forward)
    int mi = 0;                       // row where it was first reached (saved-row forward)
    uint64_t best = 0, sbest = 0;     // forward: packed best; reverse: packed (row, col) hit
    CodeWord codes = 0, codes_next = 0;  // this lane's row symbols of this / the next chunk
    // lane 0: boundary entries of this / the next chunk, copied by cp.async into
    // a per-group double buffer (16-byte copies of two rows, L2 only)
    int2* sb = &sbnd[group_in_block][0][0];
    int sbuf = 0;

    // Row symbol as the kernels use it: 2-bit code, raw byte or residue index.
    auto row_code = [&](int i) -> unsigned {  // i: 1-based row
        int idx = rev ? (nrows - i) : (i - 1);
        int v = rowseq[idx];
        if constexpr (SCORE == kScoreDnaProfile) return (unsigned)dna_code(v);
        if constexpr (AA) return (unsigned)senc[v & 127];
        return (unsigned)v;
    };
    // Symbols of the rows this lane works on in the kCh steps from st0 (byte u:
    // row st0 + u - g + 1).  Every lane fetches its own, a chunk ahead.
    // Forward DNA profiles, rows well inside the pair: the kCh row symbols come
    // from the two or three aligned words holding them (never a byte outside the
    // pair's sequence), converted four symbols per op; byte u is the code of
    // row i0 + u.  False when a row or a word of the window leaves the pair.
    constexpr int kWords = (kCh + 3 + 3) / 4;
    auto window_codes = [&](int i0, CodeWord& out) -> bool {
        const int s = i0 - 1;  // first index read
        const int k = (int)(((uintptr_t)rowseq + (unsigned)s) & 3u);
        const int base = s - k;
        if (base < 0 || base + 4 * kWords > rows) return false;
        const unsigned* w = reinterpret_cast<const unsigned*>(rowseq + base);
        const unsigned w0 = __ldg(w), w1 = __ldg(w + 1);
        const unsigned lo = __funnelshift_r(w0, w1, 8 * k);
        if constexpr (kCh <= 4) {
            out = (CodeWord)((lo >> 1) & 0x03030303u);  // dna_code of every byte
        } else {
            const unsigned hi = __funnelshift_r(w1, __ldg(w + 2), 8 * k);
            out = (CodeWord)(((((uint64_t)hi << 32) | lo) >> 1) & 0x0303030303030303ull);
        }
        return true;
    };
    auto fetch_codes = [&](int st0) -> CodeWord {
        CodeWord cw = 0;
        if constexpr (SCORE == kScoreDnaProfile && !REVERSE) {
            if (window_codes(st0 - g + 1, cw)) return cw;
        }
#pragma unroll
        for (int u = 0; u < kCh; ++u) {
            const int i = st0 + u - g + 1;
            const unsigned v = (i >= 1 && i <= rows) ? row_code(i) : (kRowChecks ? 0u : kPadRow);
            cw |= (CodeWord)v << (8 * u);
        }
        return cw;
    };
    // Teams, lane 0: waits until the previous strip's edge holds rows up to
    // `need` ((strip - 1) << 16 | row); false when its warp left the pair or the
    // wait ran out.
    auto team_wait = [&](int need) -> bool {
        const volatile int* pp = &s_prog[(tw + TEAM - 1) % TEAM];
        for (int it = 0; it < kTeamSpin; ++it) {
            // after one wait in the grid ran out, the others give up at once
            if ((it & 1023) == 0 && (*(volatile int*)p.error & kErrTeam)) return false;
            const int v = *pp;
            if (v <= -2 && (strip - 1) >= -v - 2) return false;  // the strip will not come
            if (v >= need || v <= -2) {
                __threadfence_block();  // the edge rows before the flag
                return true;
            }
            __nanosleep(100);
        }
        atomicOr(p.error, kErrTeam);
        return false;
    };
    // Lane 0 starts the copy of the boundary entries of rows [r0, r0 + kCh)
    // into buffer `buf` (one commit group per chunk).
    auto fetch_chunk = [&](int r0, int buf) {
        if constexpr (TEAM > 1) {
            if (strip > 0 && r0 <= rows && !team_abort && !team_wait(((strip - 1) << 16) | min(r0 + kCh - 1, rows)))
                team_abort = true;
            if (team_abort) {
                asm volatile("cp.async.commit_group;");
                return;
            }
        }
        if (strip > 0) {
#pragma unroll
            for (int u = 0; u < kCh; u += 2) {
                // rows r0+u-1 and r0+u (0-based) share 16 bytes: r0-1 is even (a strip's
                // steps start at an even step, kCh is even) and scratch_rows is even,
                // so the pair stays inside the buffer
                if (r0 + u <= rows) {
                    const unsigned dst = (unsigned)__cvta_generic_to_shared(sb + buf * kCh + u);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                                 "l"(bnd_in + (r0 + u - 1)));
                }
            }
        }
        asm volatile("cp.async.commit_group;");
    };

    auto setup_strip = [&]() {
        const int t0 = strip * W + g * C - pad;  // real column of this lane's first column
        if constexpr (SCORE == kScoreAaProfile) {
            // the group's profile rows for this strip: kAAProfRows x W int8, built by its G lanes
            int8_t* gp = sprof_dyn + group_in_block * kProfBytes;
            const int tg0 = strip * W - pad;
            __syncwarp(gmask);  // lanes may still read the previous strip's profile
            for (int k = g; k < kAAProfRows * W; k += G) {
                const int e = k / W, c = k % W;
                const int t = tg0 + c;
                int v = kNegByte;
                if (e < kAAPad && t >= 0 && t < ncols) {
                    const int idx = rev ? (ncols - 1 - t) : t;
                    v = smat[e * kAADim + senc[colseq[idx] & 127]];
                }
                gp[k] = (int8_t)v;
            }
            __syncwarp(gmask);
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int t = t0 + c;
            const bool real = t >= 0 && t < ncols;
            const int idx = rev ? (ncols - 1 - t) : t;
            const int v = real ? (int)colseq[idx] : 0;
            if constexpr (SCORE == kScoreDnaProfile) {
                // bytes q = 0..3: score against the base with code q
                unsigned w = 0;
                const int code = dna_code(v);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    int s = real ? (code == q ? p.match : p.mismatch) : kNegByte;
                    w |= ((unsigned)s & 0xffu) << (8 * q);
                }
                prof[c] = w;
            } else if constexpr (SCORE == kScoreDnaRaw) {
                sc[c] = real ? v : 256;  // 256 never equals a byte
                mmv[c] = real ? p.mismatch : kNegBig;
            } else if constexpr (SCORE == kScoreAaWide) {
                sc[c] = real ? senc[v & 127] : kAAPad;
            }
            ho[c] = open;
            f[c] = 0;
        }
        diag0 = open;
        if constexpr (!kRowChecks) {
            ho_out = open;  // what lane 0 hands on before its first step (rows i < 1 of lane 1)
            e_out = 0;
        }
        m = 0;
        mi = 0;
        sbest = REVERSE ? ~0ull : 0ull;
        st = 0;
        rows = nrows;
        if constexpr (TEAM > 1 && REVERSE) best = *(volatile unsigned long long*)&s_best;
        if (REVERSE && best != ~0ull) rows = min(nrows, (int)(best >> 32) - 1);
        if constexpr (REVERSE) st = band_first_row(strip * W - pad + 1, band) - 1;
        nsteps = rows + G - 1;
        codes = fetch_codes(st);
        codes_next = fetch_codes(st + kCh);
        if (g == 0) {
            asm volatile("cp.async.wait_all;");  // nothing of an earlier strip stays in flight
            sbuf = 0;
            fetch_chunk(st + 1, 0);
            fetch_chunk(st + 1 + kCh, 1);
        }
        if constexpr (TEAM > 1) team_abort = __shfl_sync(0xffffffffu, team_abort, 0);
    };
    // Teams: this warp is done with the pair (its strips ran out, or it left
    // early): publish kTeamAbort if strips it will not run remain, fold its
    // result into the team's, and, once every warp is here, write the pair's
    // results (thread 0).
    auto team_end = [&]() {
        const uint64_t mine = REVERSE ? best : group_max_u64<G>(best, gmask);
        if (lane == 0) {
            __threadfence_block();
            *(volatile int*)&s_prog[tw] = -(strip + 2);
            if constexpr (REVERSE) {
                atomicMin(&s_best, (unsigned long long)mine);
            } else {
                atomicMax(&s_best, (unsigned long long)mine);
            }
        }
        __syncthreads();
    };

    // The pair's results from its combined key (forward: packed argmax;
    // reverse: packed first hit); one thread.
    auto write_results = [&](uint64_t key) {
        if constexpr (!REVERSE) {
            const int v = (int)(key >> 32);
            if (v <= 0) {
                p.score[pid] = 0;
                p.ref_end[pid] = -1;
                p.query_end[pid] = -1;
                p.ref_begin[pid] = -1;
                p.query_begin[pid] = -1;
            } else {
                const int row = 0xFFFF - (int)((key >> 16) & 0xFFFF);
                const int tkey = 0xFFFF - (int)(key & 0xFFFF);
                const int col = tie_key(tkey) + 1;
                p.score[pid] = v;
                if (a_short) {  // kernel.cpp:381-386
                    p.query_end[pid] = row;
                    p.ref_end[pid] = col;
                } else {        // kernel.cpp:387-392
                    p.ref_end[pid] = row;
                    p.query_end[pid] = col;
                }
            }
        } else {
            if (key == ~0ull) {
                atomicOr(p.error, kErrNoHit);
                p.ref_begin[pid] = -1;
                p.query_begin[pid] = -1;
            } else {
                const int r = (int)(key >> 32);              // row of the shorter prefix
                const int qcol = (int)(key & 0xffffffffu);   // column of the longer prefix
                const int beginS = nrows - r;                // kernel.cpp:580
                const int beginL = ncols - qcol;             // kernel.cpp:579
                if (a_short) {                               // kernel.cpp:591-595
                    p.ref_begin[pid] = beginS;
                    p.query_begin[pid] = beginL;
                } else {                                     // kernel.cpp:596-600
                    p.ref_begin[pid] = beginL;
                    p.query_begin[pid] = beginS;
                }
            }
        }
    };

    while (true) {
        if constexpr (TEAM > 1) {
            // the one place where a team joins at the end of a pair (every warp
            // passes the same barrier instructions, in the same order)
            if (team_finish) {
                team_end();
                if (threadIdx.x == 0) write_results(s_best);
                team_finish = false;
                pid = -1;
            }
        }
        if (!done && pid < 0) {
            // ---- fetch and set up the next pair (group-uniform; teams: block-uniform) ----
            int q = 0;
            if constexpr (TEAM > 1) {
                __syncthreads();  // every warp is past the previous pair's results
                if (threadIdx.x == 0) {
                    s_q = atomicAdd(p.queue, 1);
                    for (int k = 0; k < TEAM; ++k) s_prog[k] = -1;
                    s_best = REVERSE ? ~0ull : 0ull;
                }
                __syncthreads();
                q = s_q;
                team_abort = false;
            } else {
                if (g == 0) q = atomicAdd(p.queue, 1);
                q = __shfl_sync(gmask, q, 0, G);
            }
            if (qbegin + q >= qend) {
                done = true;
            } else {
                pid = p.order[qbegin + q];
                const int64_t ra = p.ref_off[pid], rb = p.ref_off[pid + 1];
                const int64_t qa = p.query_off[pid], qb = p.query_off[pid + 1];
                const uint8_t* A = p.ref + ra;
                const uint8_t* B = p.query + qa;
                const int a = (int)(rb - ra), b = (int)(qb - qa);
                bool skip = false;
                if constexpr (!REVERSE) {
                    a_short = a < b;  // kernel.cpp:248
                    colseq = a_short ? A : B;
                    rowseq = a_short ? B : A;
                    ncols = a_short ? a : b;
                    nrows = a_short ? b : a;
                    rev = false;
                    if (nrows > p.scratch_rows || ncols == 0) {
                        skip = true;
                        if (g == 0) {
                            if (nrows > p.scratch_rows) atomicOr(p.error, kErrBounds);
                            p.score[pid] = 0;
                            p.ref_end[pid] = -1;
                            p.query_end[pid] = -1;
                            p.ref_begin[pid] = -1;
                            p.query_begin[pid] = -1;
                        }
                    }
                } else {
                    target = p.score[pid];
                    const int na = p.ref_end[pid], nb = p.query_end[pid];
                    if (target <= 0) {
                        skip = true;  // begins were written by the forward pass
                    } else if (na < 1 || na > a || nb < 1 || nb > b || a > p.scratch_rows ||
                               b > p.scratch_rows) {
                        skip = true;  // ends inconsistent with the pair: never read past it
                        if (g == 0) {
                            atomicOr(p.error, kErrBounds);
                            p.ref_begin[pid] = -1;
                            p.query_begin[pid] = -1;
                        }
                    } else {
                        a_short = na < nb;  // kernel.cpp:444
                        // transposed: rows = shorter prefix, columns = longer prefix
                        rowseq = a_short ? A : B;
                        colseq = a_short ? B : A;
                        nrows = a_short ? na : nb;
                        ncols = a_short ? nb : na;
                        ncols_run = reverse_columns(a, b, na, nb, target, p.match, p.rev_p);
                        band = reverse_band(a, b, na, nb, target, p.match, p.rev_p);
                        rev = true;
                    }
                }
                if (skip) {
                    pid = -1;
                } else {
                    if constexpr (!REVERSE) ncols_run = ncols;
                    nstrips = (ncols_run + W - 1) / W;
                    pad = REVERSE ? 0 : nstrips * W - ncols_run;  // reverse: padded on the right
                    strip = tw;
                    best = REVERSE ? ~0ull : 0ull;
                    if (strip < nstrips) {
                        setup_strip();
                    } else {
                        team_finish = true;  // teams: more warps than strips, this one has none
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (done || pid < 0) continue;
        if constexpr (TEAM > 1) {
            // done with the pair, or the strip's input will not come (or the
            // wait ran out): join the team at the loop's top
            if (team_finish || team_abort) {
                team_finish = true;
                continue;
            }
        }

        // ---- kCh pipeline steps ----
        const bool last_strip = strip + 1 == nstrips;
        if (g == 0 && strip > 0) asm volatile("cp.async.wait_group 1;");  // this chunk's entries
#pragma unroll
        for (int u = 0; u < kCh; ++u) {
            if (!kRowChecks || st < nsteps) {  // group-uniform
                const int i = st - g + 1;
                int ho_in = __shfl_up_sync(gmask, ho_out, 1, G);
                int e_in = __shfl_up_sync(gmask, e_out, 1, G);
                const unsigned code = (unsigned)(codes >> (8 * u)) & 0xffu;
                if (g == 0) {
                    if (strip == 0) {
                        ho_in = open;
                        e_in = 0;
                    } else {
                        const int2 v = sb[sbuf * kCh + u];
                        ho_in = v.x;
                        e_in = v.y;
                    }
                }
                if (!kRowChecks || (unsigned)(i - 1) < (unsigned)rows) {
                    const bool row_ok = kRowChecks || (unsigned)(i - 1) < (unsigned)rows;
                    unsigned sel = 0;
                    unsigned pw[SCORE == kScoreAaProfile ? C / 4 : 1];
                    if constexpr (SCORE == kScoreDnaProfile) sel = sbyte_sel(code);
                    if constexpr (SCORE == kScoreAaProfile) {
                        // this lane's C scores of the row's residue: C/16 16-byte loads
                        // (or one 8- or 4-byte load for C = 8 or 4)
                        const int8_t* src = sprof_dyn + group_in_block * kProfBytes + code * W + g * C;
                        if constexpr (C % 16 == 0) {
#pragma unroll
                            for (int v = 0; v < C / 16; ++v) {
                                const uint4 w = reinterpret_cast<const uint4*>(src)[v];
                                pw[4 * v + 0] = w.x;
                                pw[4 * v + 1] = w.y;
                                pw[4 * v + 2] = w.z;
                                pw[4 * v + 3] = w.w;
                            }
                        } else if constexpr (C == 8) {
                            const uint2 w = *reinterpret_cast<const uint2*>(src);
                            pw[0] = w.x;
                            pw[1] = w.y;
                        } else {
                            pw[0] = *reinterpret_cast<const unsigned*>(src);
                        }
                    }
                    int e = e_in, diag = diag0, hov = open;
                    int mrow = open;  // H + open of an all-zero row
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        int sp;
                        if constexpr (SCORE == kScoreDnaProfile) {
                            sp = sbyte(prof[c], sel);
                        } else if constexpr (SCORE == kScoreDnaRaw) {
                            sp = ((int)code == sc[c]) ? p.match : mmv[c];
                        } else if constexpr (SCORE == kScoreAaProfile) {
                            sp = sbyte(pw[c / 4], sbyte_sel(c % 4));
                        } else {
                            sp = smat[code * kAADim + sc[c]];
                        }
                        const int fv = add_max_relu<DPX>(f[c], ext, ho[c]);  // F(i,j)
                        const int t = add_max<DPX>(fv, open, diag + sp);     // max(F + open, Ho_diag + s)
                        hov = add_max<DPX>(e, open, t);                      // Ho(i,j)
                        e = add_max_relu<DPX>(e, gmax, t);                   // E(i,j+1)
                        diag = ho[c];
                        ho[c] = hov;
                        f[c] = fv;
                        if (c & 1) mrow = max3<DPX>(mrow, ho[c - 1], hov);
                    }
                    ho_out = hov;
                    e_out = e;
                    diag0 = ho_in;
                    if (g == G - 1 && !last_strip && row_ok) __stcg(&bnd_out[i - 1], make_int2(ho_out, e_out));
                    const int mh = mrow - open;  // row max of H (>= 0)
                    if constexpr (kSaveRow) {
                        if (mh > m && row_ok) {
                            m = mh;
                            mi = i;
#pragma unroll
                            for (int k = 0; k < C / 4; ++k)
                                ssave[k][threadIdx.x] = make_int4(ho[4 * k], ho[4 * k + 1], ho[4 * k + 2], ho[4 * k + 3]);
                        }
                    } else if constexpr (!REVERSE) {
                        if (mh > m && row_ok) {
                            m = mh;
                            // columns of this row holding the new lane max, in tie order
                            const int t0 = strip * W + g * C - pad;
                            unsigned hits = 0;
#pragma unroll
                            for (int c = 0; c < C; ++c) hits |= (ho[c] == mrow) ? (1u << c) : 0u;
                            int kmin = 0x7fffffff;
                            while (hits) {  // usually one column
                                const int c = __ffs(hits) - 1;
                                hits &= hits - 1;
                                kmin = min(kmin, tie_key(t0 + c));
                            }
                            sbest = pack_fwd(m, i, kmin);
                        }
                    } else {
                        if (mh == target && sbest == ~0ull && row_ok) {
                            const int t0 = strip * W + g * C - pad;
                            int cfirst = C;
#pragma unroll
                            for (int c = C - 1; c >= 0; --c) {
                                if (ho[c] == mrow) cfirst = c;
                            }
                            const int qcol = t0 + cfirst + 1;  // 1-based column of the longer prefix
                            sbest = ((uint64_t)(uint32_t)i << 32) | (uint32_t)qcol;
                        }
                    }
                }
                ++st;
            }
        }
        if constexpr (TEAM > 1) {
            // publish the rows of this strip's edge written so far
            if (g == G - 1 && !last_strip) {
                const int written = st >= nsteps ? kTeamStripDone : max(0, min(st - (G - 1), rows));
                __threadfence_block();
                *(volatile int*)&s_prog[tw] = (strip << 16) | written;
            }
        }
        // next chunk's row symbols; start fetching the chunk after it
        codes = codes_next;
        if (st < nsteps) codes_next = fetch_codes(st + kCh);
        if (g == 0) {
            if (st < nsteps) fetch_chunk(st + 1 + kCh, sbuf);
            sbuf ^= 1;
        }
        if constexpr (TEAM > 1) team_abort = __shfl_sync(0xffffffffu, team_abort, 0);
        if (st >= nsteps) {
            // ---- end of strip ----
            if constexpr (kSaveRow) {
                if (m > 0) {
                    // columns of the saved row holding the lane max, in tie order
                    const int t0 = strip * W + g * C - pad;
                    const int mo = m + open;
                    int kmin = 0x7fffffff;
#pragma unroll
                    for (int k = 0; k < C / 4; ++k) {
                        const int4 v = ssave[k][threadIdx.x];
                        if (v.x == mo) kmin = min(kmin, tie_key(t0 + 4 * k));
                        if (v.y == mo) kmin = min(kmin, tie_key(t0 + 4 * k + 1));
                        if (v.z == mo) kmin = min(kmin, tie_key(t0 + 4 * k + 2));
                        if (v.w == mo) kmin = min(kmin, tie_key(t0 + 4 * k + 3));
                    }
                    sbest = pack_fwd(m, mi, kmin);
                }
                best = sbest > best ? sbest : best;
            } else if constexpr (!REVERSE) {
                best = sbest > best ? sbest : best;
            } else {
                best = group_min_u64<G>(sbest < best ? sbest : best, gmask);
                if constexpr (TEAM > 1) {
                    // the team's best so far, which also bounds this warp's next strips
                    if (lane == 0) atomicMin(&s_best, (unsigned long long)best);
                    __syncwarp();
                    best = *(volatile unsigned long long*)&s_best;
                }
            }
            __syncwarp(gmask);  // boundary writes of this strip before the next strip reads
            strip += TEAM;
            bool more = strip < nstrips && (!REVERSE || best == ~0ull || (int)(best >> 32) > 1);
            if (REVERSE && more) {
                // the band moves down the rows strip by strip: stop once it starts
                // below the rows still to search
                const int limit = best == ~0ull ? nrows : (int)(best >> 32) - 1;
                more = band_first_row(strip * W - pad + 1, band) <= limit;
            }
            if (more) {
                setup_strip();
            } else {
                // ---- end of pair: group argmax and results (teams: at the loop's top) ----
                if constexpr (TEAM > 1) {
                    team_finish = true;
                } else {
                    const uint64_t key = REVERSE ? best : group_max_u64<G>(best, gmask);
                    if (g == 0) write_results(key);
                    pid = -1;
                }
            }
        }
    }
}

template <int SCORE, bool REVERSE, bool DPX, int G, int C, int TEAM = 1>
const void* kernel_ptr() {
    return (const void*)sw_pass<SCORE, REVERSE, DPX, G, C, TEAM>;
}

}  // namespace
}  // namespace gbsw
