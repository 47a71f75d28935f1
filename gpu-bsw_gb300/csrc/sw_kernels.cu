// Forward (end-position) and reverse (begin-position) Smith-Waterman passes
// for batches of independent pairs, int32 scores, sm_103a.
//
// Work decomposition.  A group of G consecutive lanes of a warp owns one pair
// at a time (32/G pairs per warp).  The DP matrix is cut into column strips of
// W = G*C columns; lane g holds C consecutive columns of the strip in
// registers (the previous row's H+open and F of each column) and the rows are
// streamed through the group as a software pipeline: at step s lane g works
// on row s-g+1, receiving the H+open and E of the column to its left for the
// same row from lane g-1 by one shfl_up each.  The right edge of a strip
// (H+open and E per row) goes through a per-group boundary buffer in global
// memory to the next strip.  Groups pull pairs from a global work queue
// (one atomicAdd per pair) and run independently of the other groups of the
// warp: the kernel is one flat loop in which every iteration advances each
// group by one pipeline step, so no group waits for another at loop exits.
//
// Recurrence (the reference's kernel.cpp:326-372) with E and F clamped at 0:
//   F = max(F_up + ext, H_up + open, 0)
//   E = max(E_left + ext, H_left + open, 0)
//   H = max(H_diag + s, E, F, 0)
// For open, ext <= 0 the clamp leaves every H unchanged (a negative E or F never
// wins the max against 0) and reproduces the reference's boundary values
// E(i,1) = 0 and F(1,j) = max(ext, open) <= 0 exactly.  Padding columns sit on
// the LEFT of the first strip with a score of kNegBig, so their H, E and F are
// all 0: they act exactly like the matrix boundary and never hold a maximum.
//
// Forward argmax (the reference's kernel.cpp:368-370 plus the shfl_down trees
// of kernel.cpp:47-86, 137-182): value desc, then smallest row i of the longer
// sequence, then the tie order `tie_key` over columns.  Each lane keeps the
// max of its own cells; only on rows where that max grows does it look for
// which of its columns hold the new max.
//
// Reverse pass (kernel.cpp:397-604 with the trees of kernel.cpp:3-45, 90-135):
// the same DP over A[0:ref_end] and B[0:query_end], both reversed; the begin is
// the cell with H == score that has the smallest reversed column of the shorter
// prefix, then the smallest reversed row of the longer one.  The pass runs
// TRANSPOSED (rows = the shorter prefix, columns = the longer one), so that order
// becomes "first row reaching the score, then leftmost column in it": a lane
// checks one comparison per row, and later strips stop at the best row found.
#include "sw_common.cuh"
#include "sw_kernels.h"

namespace gbsw {

namespace {

constexpr int kThreads = 256;

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

// Lane state of one column strip.
template <int C>
struct Strip {
    int ho[C];    // H(i-1, j) + open
    int f[C];     // F(i-1, j)
    int sc[C];    // column symbol (DNA byte, 256 = padding) or protein index (24 = padding)
    int mm[C];    // DNA: mismatch - open, kNegBig for padding
};

template <int G, int C, bool PROTEIN, bool REVERSE, bool DPX>
__global__ void __launch_bounds__(kThreads) sw_pass(PassParams p) {
    constexpr int W = G * C;
    __shared__ int smat[kAADim * kAADim];
    __shared__ int senc[128];
    if constexpr (PROTEIN) {
        // forward: rows carry the longer sequence = the matrix's first index;
        // reverse (transposed): rows carry the shorter one = second index.
        for (int k = threadIdx.x; k < kAADim * kAADim; k += blockDim.x) {
            int r = k / kAADim, c = k % kAADim;
            smat[k] = REVERSE ? p.aa_matrix[c * kAADim + r] : p.aa_matrix[k];
        }
        // symbol -> matrix index (driver.cpp:252-258); -1 marks bytes outside the table
        for (int k = threadIdx.x; k < 128; k += blockDim.x) senc[k] = k < 91 ? p.aa_encoding[k] : -1;
        __syncthreads();
    }

    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane - g));
    const long long group_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    int2* bnd = p.scratch + (size_t)group_id * (size_t)p.scratch_rows;
    const int open = p.open, ext = p.ext;

    // ---- per-group pair state (identical in the G lanes) ----
    int pid = -1;
    bool done = false;
    const uint8_t* rowseq = nullptr;  // streamed sequence (forward: longer; reverse: shorter prefix)
    const uint8_t* colseq = nullptr;  // sequence in registers
    int nrows = 0, ncols = 0, nstrips = 0, pad = 0, strip = 0, st = 0, nsteps = 0;
    int row_limit = 0;
    bool rev_rows = false, rev_cols = false;  // read back to front
    bool a_short = false;
    int target = 0;                           // reverse: the score to find
    int na = 0, nb = 0;
    // ---- per-lane state ----
    Strip<C> s;
    int ho_out = 0, e_out = 0, diag0 = 0;
    int m = 0;                        // lane max in this strip
    uint64_t best = 0;                // forward: packed best; reverse: packed (row, col) hit
    uint64_t sbest = 0;
    int lc_next = 0;
    int2 bnd_next = make_int2(0, 0);

    // protein symbol -> matrix index; a byte outside the encoding table flags
    // error bit 0 and is scored as 'A' (the reference would read past its table)
    auto encode = [&](int v) -> int {
        int e = v < 128 ? senc[v] : -1;
        if (e < 0) {
            atomicOr(p.error, 1);
            e = 0;
        }
        return e;
    };
    auto row_symbol = [&](int i) -> int {  // i: 1-based row
        int idx = rev_rows ? (nrows - i) : (i - 1);
        int v = rowseq[idx];
        if constexpr (PROTEIN) return encode(v) * kAADim;
        return v;
    };

    auto setup_strip = [&]() {
        const int t0 = strip * W + g * C - pad;  // real column of this lane's first column
#pragma unroll
        for (int c = 0; c < C; ++c) {
            int t = t0 + c;
            if (t >= 0 && t < ncols) {
                int idx = rev_cols ? (ncols - 1 - t) : t;
                if constexpr (PROTEIN) {
                    s.sc[c] = encode(colseq[idx]);
                } else {
                    s.sc[c] = colseq[idx];
                }
                s.mm[c] = p.mismatch_p;
            } else {
                s.sc[c] = PROTEIN ? kAAPad : 256;
                s.mm[c] = kNegBig;
            }
            s.ho[c] = open;
            s.f[c] = 0;
        }
        diag0 = open;
        m = 0;
        sbest = REVERSE ? ~0ull : 0ull;
        st = 0;
        int rows = REVERSE ? row_limit : nrows;
        nsteps = rows + G - 1;
        // prefetch for step 0 (row 1 - g)
        int i1 = 1 - g;
        if (i1 >= 1 && i1 <= rows) lc_next = row_symbol(i1);
        if (g == 0 && strip > 0 && rows >= 1) bnd_next = __ldcg(&bnd[0]);
    };

    while (true) {
        if (!done && pid < 0) {
            // ---- fetch and set up the next pair (group-uniform) ----
            int q = 0;
            if (g == 0) q = atomicAdd(p.queue, 1);
            q = __shfl_sync(gmask, q, 0, G);
            if (q >= p.n) {
                done = true;
            } else {
                pid = q;
                const int64_t ra = p.ref_off[pid], rb = p.ref_off[pid + 1];
                const int64_t qa = p.query_off[pid], qb = p.query_off[pid + 1];
                const uint8_t* A = p.ref + ra;
                const uint8_t* B = p.query + qa;
                int a = (int)(rb - ra), b = (int)(qb - qa);
                bool skip = false;
                if constexpr (!REVERSE) {
                    a_short = a < b;  // kernel.cpp:248
                    colseq = a_short ? A : B;
                    rowseq = a_short ? B : A;
                    ncols = a_short ? a : b;
                    nrows = a_short ? b : a;
                    rev_rows = rev_cols = false;
                    if (nrows > p.scratch_rows) {  // longer than the caller's max_len
                        skip = true;
                        if (g == 0) {
                            atomicOr(p.error, 4);
                            p.score[pid] = 0;
                            p.ref_end[pid] = -1;
                            p.query_end[pid] = -1;
                        }
                    } else if (ncols == 0) {
                        skip = true;
                        if (g == 0) {
                            p.score[pid] = 0;
                            p.ref_end[pid] = -1;
                            p.query_end[pid] = -1;
                        }
                    }
                } else {
                    target = p.score[pid];
                    na = p.ref_end[pid];
                    nb = p.query_end[pid];
                    if (target <= 0) {
                        skip = true;
                        if (g == 0) {
                            p.ref_begin[pid] = -1;
                            p.query_begin[pid] = -1;
                        }
                    } else if (na < 1 || na > a || nb < 1 || nb > b || a > p.scratch_rows ||
                               b > p.scratch_rows) {
                        skip = true;  // ends inconsistent with the pair: never read past it
                        if (g == 0) {
                            atomicOr(p.error, 4);
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
                        rev_rows = rev_cols = true;
                    }
                }
                if (skip) {
                    pid = -1;
                } else {
                    nstrips = (ncols + W - 1) / W;
                    pad = nstrips * W - ncols;
                    strip = 0;
                    row_limit = nrows;
                    best = REVERSE ? ~0ull : 0ull;
                    setup_strip();
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (done || pid < 0) continue;

        // ---- one pipeline step ----
        const int i = st - g + 1;
        const int rows = REVERSE ? row_limit : nrows;
        int ho_in = __shfl_up_sync(gmask, ho_out, 1, G);
        int e_in = __shfl_up_sync(gmask, e_out, 1, G);
        if (g == 0) {
            if (strip == 0) {
                ho_in = open;
                e_in = 0;
            } else {
                ho_in = bnd_next.x;
                e_in = bnd_next.y;
            }
        }
        const bool active = (i >= 1) && (i <= rows);
        if (active) {
            const int lc = lc_next;
            int hleft = ho_in, e = e_in, diag = diag0;
            int mrow = open;  // H + open of an all-zero row
#pragma unroll
            for (int c = 0; c < C; ++c) {
                int sp;
                if constexpr (PROTEIN) {
                    sp = smat[lc + s.sc[c]];
                } else {
                    sp = (lc == s.sc[c]) ? p.match_p : s.mm[c];
                }
                int f = add_max_relu<DPX>(s.f[c], ext, s.ho[c]);
                e = add_max_relu<DPX>(e, ext, hleft);
                int h = max3_relu<DPX>(diag + sp, e, f);
                diag = s.ho[c];
                int ho = h + open;
                s.ho[c] = ho;
                s.f[c] = f;
                hleft = ho;
                mrow = (c & 1) ? max3<DPX>(mrow, s.ho[c - 1], ho) : mrow;
            }
            if constexpr (C & 1) mrow = max(mrow, s.ho[C - 1]);
            ho_out = hleft;
            e_out = e;
            diag0 = ho_in;
            if (g == G - 1 && strip + 1 < nstrips) __stcg(&bnd[i - 1], make_int2(ho_out, e_out));
            const int mh = mrow - open;  // row max of H (>= 0)
            if constexpr (!REVERSE) {
                if (mh > m) {
                    m = mh;
                    // columns of this row holding the new lane max, in tie order
                    const int t0 = strip * W + g * C - pad;
                    unsigned hits = 0;
#pragma unroll
                    for (int c = 0; c < C; ++c) hits |= (s.ho[c] == mrow) ? (1u << c) : 0u;
                    int kmin = 0x7fffffff;
                    while (hits) {  // usually one column
                        const int c = __ffs(hits) - 1;
                        hits &= hits - 1;
                        kmin = min(kmin, tie_key(t0 + c));
                    }
                    sbest = pack_fwd(m, i, kmin);
                }
            } else {
                if (mh == target && sbest == ~0ull) {
                    const int t0 = strip * W + g * C - pad;
                    int cfirst = C;
#pragma unroll
                    for (int c = C - 1; c >= 0; --c) {
                        if (s.ho[c] == mrow) cfirst = c;
                    }
                    const int qcol = t0 + cfirst + 1;  // 1-based column of the longer prefix
                    sbest = ((uint64_t)(uint32_t)i << 32) | (uint32_t)qcol;
                }
            }
        }
        // prefetch the next step's row symbol and boundary
        {
            const int in = i + 1;
            if (in >= 1 && in <= rows) lc_next = row_symbol(in);
            if (g == 0 && strip > 0 && in >= 1 && in <= rows) bnd_next = __ldcg(&bnd[in - 1]);
        }
        ++st;
        if (st == nsteps) {
            // ---- end of strip ----
            if constexpr (!REVERSE) {
                best = sbest > best ? sbest : best;
            } else {
                best = sbest < best ? sbest : best;
                uint64_t gb = group_min_u64<G>(best, gmask);
                if (gb != ~0ull) row_limit = (int)(gb >> 32) - 1;
            }
            __syncwarp(gmask);  // boundary writes of this strip before the next strip reads
            ++strip;
            if (strip < nstrips && (!REVERSE || row_limit >= 1)) {
                setup_strip();
            } else {
                // ---- end of pair: group argmax and results ----
                if constexpr (!REVERSE) {
                    uint64_t gb = group_max_u64<G>(best, gmask);
                    if (g == 0) {
                        int v = (int)(gb >> 32);
                        if (v <= 0) {
                            p.score[pid] = 0;
                            p.ref_end[pid] = -1;
                            p.query_end[pid] = -1;
                        } else {
                            int row = 0xFFFF - (int)((gb >> 16) & 0xFFFF);
                            int key = 0xFFFF - (int)(gb & 0xFFFF);
                            int col = tie_key_inverse(key) + 1;
                            p.score[pid] = v;
                            if (a_short) {  // kernel.cpp:381-386
                                p.query_end[pid] = row;
                                p.ref_end[pid] = col;
                            } else {        // kernel.cpp:387-392
                                p.ref_end[pid] = row;
                                p.query_end[pid] = col;
                            }
                        }
                    }
                } else {
                    uint64_t gb = group_min_u64<G>(best, gmask);
                    if (g == 0) {
                        if (gb == ~0ull) {
                            atomicOr(p.error, 2);  // reverse pass did not find the forward score
                            p.ref_begin[pid] = -1;
                            p.query_begin[pid] = -1;
                        } else {
                            int r = (int)(gb >> 32);              // row of the shorter prefix
                            int qcol = (int)(gb & 0xffffffffu);   // column of the longer prefix
                            int beginS = nrows - r;               // kernel.cpp:580
                            int beginL = ncols - qcol;            // kernel.cpp:579
                            if (a_short) {                        // kernel.cpp:591-595
                                p.ref_begin[pid] = beginS;
                                p.query_begin[pid] = beginL;
                            } else {                              // kernel.cpp:596-600
                                p.ref_begin[pid] = beginL;
                                p.query_begin[pid] = beginS;
                            }
                        }
                    }
                }
                pid = -1;
            }
        }
    }
}

template <int G, int C, bool PROTEIN, bool REVERSE, bool DPX>
cudaError_t launch_t(const PassParams& p, int blocks, cudaStream_t stream) {
    sw_pass<G, C, PROTEIN, REVERSE, DPX><<<blocks, kThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace

int pass_threads() { return kThreads; }

int pass_group_lanes(const PassConfig&) { return kGroupLanes; }

cudaError_t pass_occupancy(const PassConfig& cfg, bool reverse, int* blocks_per_sm) {
    const void* fn = nullptr;
#define GBSW_PICK(PROT, REV, DPXV)                                                            \
    if (cfg.protein == PROT && reverse == REV && cfg.dpx == DPXV)                              \
        fn = (const void*)sw_pass<kGroupLanes, kColsPerLane, PROT, REV, DPXV>;
    GBSW_PICK(false, false, false)
    GBSW_PICK(false, false, true)
    GBSW_PICK(false, true, false)
    GBSW_PICK(false, true, true)
    GBSW_PICK(true, false, false)
    GBSW_PICK(true, false, true)
    GBSW_PICK(true, true, false)
    GBSW_PICK(true, true, true)
#undef GBSW_PICK
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kThreads, 0);
}

cudaError_t launch_pass(const PassConfig& cfg, bool reverse, const PassParams& p, int blocks,
                        cudaStream_t stream) {
    constexpr int G = kGroupLanes, C = kColsPerLane;
    if (cfg.protein) {
        if (reverse)
            return cfg.dpx ? launch_t<G, C, true, true, true>(p, blocks, stream)
                           : launch_t<G, C, true, true, false>(p, blocks, stream);
        return cfg.dpx ? launch_t<G, C, true, false, true>(p, blocks, stream)
                       : launch_t<G, C, true, false, false>(p, blocks, stream);
    }
    if (reverse)
        return cfg.dpx ? launch_t<G, C, false, true, true>(p, blocks, stream)
                       : launch_t<G, C, false, true, false>(p, blocks, stream);
    return cfg.dpx ? launch_t<G, C, false, false, true>(p, blocks, stream)
                   : launch_t<G, C, false, false, false>(p, blocks, stream);
}

}  // namespace gbsw
