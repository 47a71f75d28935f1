// Traceback: one optimal alignment path per aligned pair, as run-length
// operations (no counterpart in the reference, which declares a traceback at
// kernel.hpp:36-39 and never implements it).
//
// For a pair with score > 0, begins rb, qb and ends re, qe, the path is a
// global affine alignment of R = ref[rb:re] (m symbols, columns j) and
// Q = query[qb:qe] (k symbols, rows i):
//   H(0,0) = 0, H(0,j) = open + (j-1)*ext, H(i,0) = open + (i-1)*ext,
//   E(i,0) = F(0,j) = -inf,
//   E(i,j) = max(E(i,j-1) + ext, H(i,j-1) + open)    reference symbol vs gap: 'D'
//   F(i,j) = max(F(i-1,j) + ext, H(i-1,j) + open)    query symbol vs gap:     'I'
//   H(i,j) = max(H(i-1,j-1) + s, F(i,j), E(i,j))
// An optimal local alignment starts and ends with an aligned pair, so H(k, m)
// is the pair's score; the kernel checks that.  Ties: H takes the diagonal if
// it is >= both gaps, else F if F >= E, else E; E and F extend when extending
// is >= opening.  s is the passes' substitution score (DNA: raw byte compare;
// protein: matrix[enc(x)][enc(y)], x from the longer whole sequence).
//
// A group of kTraceLanes lanes per pair, 32 / kTraceLanes pairs per warp.  The
// segment is cut into strips of kTraceCols columns: lane l of the group holds
// the kTraceColsPerLane consecutive columns from l * kTraceColsPerLane, and the
// rows stream through the group as a pipeline: at step t lane l works on row
// t - l + 1 and receives H(i, j0 - 1), E(i, j0 - 1) of its first column's left
// neighbour from lane l - 1 by shfl_up.  Per cell it keeps 4 direction bits (H
// source in bits 0-1: 0 diagonal, 1 E, 2 F; bit 2: E extended; bit 3: F
// extended); a lane's cells of a row make one word, stored
// [strip][row][lane] so that a group's words of a row are contiguous.  Each max
// also yields its comparison (DPX __vibmax_s32), which gives the bits.  The
// group's last lane hands the strip's last column to the next strip through a
// per-pair boundary buffer.  The groups of a warp advance together in one flat
// loop (one row step each per iteration, or a strip set-up), and the host
// hands them pairs in order of cost, so that a warp's pairs end close
// together; then the first lane of every group walks its path back from
// (k, m) and writes its runs into the pair's slot, the warp's walks side by side.
#include <type_traits>

#include "sw_common.cuh"
#include "traceback.h"

namespace gbsw {
namespace {

constexpr int kTraceThreads = 256;
constexpr int kNeg = -(1 << 30);
constexpr uint32_t kOpI = 1, kOpD = 2, kOpEq = 7, kOpX = 8;
// a lane's direction codes of one row
using DirWord = std::conditional<kTraceColsPerLane == 8, uint32_t, uint16_t>::type;

// A gap of len >= 1 symbols, clamped far below any path score.
__device__ __forceinline__ int gap_cost(int open, int ext, int len) {
    const long long v = (long long)open + (long long)(len - 1) * ext;
    return v < kNeg ? kNeg : (int)v;
}

template <bool PROTEIN>
__global__ void __launch_bounds__(kTraceThreads) trace_pairs(TraceParams p) {
    constexpr int C = kTraceColsPerLane, TG = kTraceLanes, W = kTraceCols;
    __shared__ int smat[PROTEIN ? kAADim * kAADim : 1];
    __shared__ int senc[PROTEIN ? 128 : 1];
    if constexpr (PROTEIN) {
        for (int k = threadIdx.x; k < kAADim * kAADim; k += blockDim.x) smat[k] = p.aa_matrix[k];
        for (int k = threadIdx.x; k < 128; k += blockDim.x) senc[k] = k < 91 ? p.aa_encoding[k] : 0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int g = lane % TG;
    const unsigned gmask = (TG == 32) ? 0xffffffffu : (((1u << TG) - 1u) << (lane - g));
    const int64_t slot_idx = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TG;
    if (__all_sync(0xffffffffu, slot_idx >= p.count)) return;  // whole warps past the launch
    // ---- the group's pair (group-uniform) ----
    int64_t pid = -1, local = 0;
    int score = 0, m = 0, k = 0, strips = 0;
    const uint8_t* R = nullptr;
    const uint8_t* Q = nullptr;
    bool ref_longer = false;
    DirWord* dir = nullptr;
    int2* bnd = nullptr;
    if (slot_idx < p.count) {
        pid = p.order ? p.order[slot_idx] : p.first + slot_idx;
        local = pid - p.first;
        score = p.score[pid];
        if (score <= 0) {
            if (g == 0) {
                p.nops[pid] = 0;
                p.path_score[pid] = 0;
            }
        } else {
            const int a = (int)(p.ref_off[pid + 1] - p.ref_off[pid]);
            const int b = (int)(p.query_off[pid + 1] - p.query_off[pid]);
            const int rb = p.ref_begin[pid], re = p.ref_end[pid], qb = p.query_begin[pid], qe = p.query_end[pid];
            m = re - rb;
            k = qe - qb;
            R = p.ref + p.ref_off[pid] + rb;
            Q = p.query + p.query_off[pid] + qb;
            ref_longer = a >= b;
            strips = (m + W - 1) / W;
            dir = reinterpret_cast<DirWord*>(p.dir + p.dir_off[local]);
            bnd = p.bnd + p.bnd_off[local];
        }
    }
    const int open = p.open, ext = p.ext;

    int hup[C], fup[C], rcode[C];
    int s = 0, t = 0, diag0 = 0, h_out = 0, e_out = kNeg;
    bool running = strips > 0;  // group-uniform
    auto setup_strip = [&]() {
        const int j0 = s * W + g * C + 1;  // this lane's first column (1-based)
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int j = j0 + c;
            const int v = j <= m ? (int)R[j - 1] : 0;
            rcode[c] = PROTEIN ? senc[v & 127] : (j <= m ? v : 256);  // 256 matches no byte
            hup[c] = gap_cost(open, ext, j);  // H(0, j)
            fup[c] = kNeg;                    // F(0, j)
        }
        diag0 = (j0 == 1) ? 0 : gap_cost(open, ext, j0 - 1);  // H(0, j0 - 1)
        h_out = 0;
        e_out = kNeg;
        t = 0;
    };
    if (running) setup_strip();
    // ---- the DP: every group of the warp one row step per iteration ----
    while (__any_sync(0xffffffffu, running)) {
        if (!running) continue;
        int hl = __shfl_up_sync(gmask, h_out, 1, TG);
        int el = __shfl_up_sync(gmask, e_out, 1, TG);
        const int i = t - g + 1;
        if (i >= 1 && i <= k) {
            if (g == 0) {
                if (s == 0) {
                    hl = gap_cost(open, ext, i);  // H(i, 0)
                    el = kNeg;                    // E(i, 0)
                } else {
                    const int2 v = bnd[i];
                    hl = v.x;
                    el = v.y;
                }
            }
            const int qc = Q[i - 1];
            const int qcode = PROTEIN ? senc[qc & 127] : qc;
            int diag = diag0, hprev = hl, eprev = el;
            uint32_t word = 0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                int sub;
                if constexpr (PROTEIN)
                    sub = ref_longer ? smat[rcode[c] * kAADim + qcode] : smat[qcode * kAADim + rcode[c]];
                else
                    sub = rcode[c] == qcode ? p.match : p.mismatch;
                bool eb, fb, pf, pd;
                const int e = __vibmax_s32(eprev + ext, hprev + open, &eb);  // E(i, j), eb: extended
                const int f = __vibmax_s32(fup[c] + ext, hup[c] + open, &fb);  // F(i, j), fb: extended
                const int ef = __vibmax_s32(f, e, &pf);                        // pf: F >= E
                const int h = __vibmax_s32(diag + sub, ef, &pd);               // pd: diagonal >= both
                const uint32_t nib = (pd ? 0u : (pf ? 2u : 1u)) | (eb ? 4u : 0u) | (fb ? 8u : 0u);
                word |= nib << (4 * c);
                diag = hup[c];
                hup[c] = h;
                fup[c] = f;
                hprev = h;
                eprev = e;
            }
            dir[((int64_t)s * k + (i - 1)) * TG + g] = (DirWord)word;
            if (g == TG - 1 && s + 1 < strips) bnd[i] = make_int2(hprev, eprev);
            diag0 = hl;
            h_out = hprev;
            e_out = eprev;
        }
        if (++t == k + TG - 1) {  // end of strip
            __syncwarp(gmask);    // its boundary and direction words before the next strip reads
            if (++s < strips) {
                setup_strip();
            } else {
                running = false;
                --s;  // the last strip's values stay in hup
            }
        }
    }
    if (strips == 0) return;
    // H(k, m) sits in column (m - 1) % W of the lane holding column m, last strip
    const int mc = (m - 1) % W;
    int final_h = kNeg;
#pragma unroll
    for (int c = 0; c < C; ++c)
        if (c == mc % C) final_h = hup[c];
    final_h = __shfl_sync(gmask, final_h, mc / C, TG);
    if (g != 0) return;
    p.path_score[pid] = final_h;
    uint32_t* out = p.ops + p.slot_off[pid];
    if (final_h != score) {
        atomicOr(p.error, kErrTrace);
        p.nops[pid] = 0;
        return;
    }
    // ---- the walk (the warp's groups side by side) ----
    int i = k, jj = m, state = 0, n = 0;
    uint32_t run = 0;  // the run being extended (len << 4 | op), kept out of memory
    auto push = [&](uint32_t op) {
        if ((run & 15u) == op) {
            run += 16u;
        } else {
            if (run) out[n++] = run;
            run = 16u | op;
        }
    };
    while (i > 0 || jj > 0) {
        if (i == 0) {
            push(kOpD);
            --jj;
            continue;
        }
        if (jj == 0) {
            push(kOpI);
            --i;
            continue;
        }
        const int st = (jj - 1) / W, col = (jj - 1) % W;
        const DirWord* wp = dir + ((int64_t)st * k + (i - 1)) * TG + col / C;
        // the walk climbs the rows: ask for the line four rows up (rows are TG
        // words, a line 128 bytes) before the walk needs it, within this strip
        // (100,000 DNA pairs: kernel 7.36 against 7.44 ms)
        if (i > 4) asm volatile("prefetch.global.L1 [%0];" ::"l"(wp - 4 * TG));
        const uint32_t w = *wp;  // a lane's codes of row i
        const uint32_t nib = (w >> (4 * (col % C))) & 15u;
        if (state == 0) {
            const int src = (int)(nib & 3u);
            if (src == 0) {
                push(R[jj - 1] == Q[i - 1] ? kOpEq : kOpX);
                --i;
                --jj;
            } else {
                state = src;
            }
        } else if (state == 1) {
            push(kOpD);
            if (!(nib & 4u)) state = 0;
            --jj;
        } else {
            push(kOpI);
            if (!(nib & 8u)) state = 0;
            --i;
        }
    }
    if (run) out[n++] = run;
    for (int x = 0, y = n - 1; x < y; ++x, --y) {
        const uint32_t tmp = out[x];
        out[x] = out[y];
        out[y] = tmp;
    }
    p.nops[pid] = n;
}

__global__ void gather_ops(const uint32_t* ops, const int64_t* slot_off, const int32_t* nops,
                           const int64_t* out_off, uint32_t* out, int64_t n) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += warps) {
        const uint32_t* src = ops + slot_off[k];
        uint32_t* dst = out + out_off[k];
        for (int x = lane; x < nops[k]; x += 32) dst[x] = src[x];
    }
}

}  // namespace

cudaError_t launch_trace(const TraceParams& p, cudaStream_t stream) {
    if (p.count <= 0) return cudaSuccess;
    const int64_t blocks = (p.count * kTraceLanes + kTraceThreads - 1) / kTraceThreads;
    if (p.protein)
        trace_pairs<true><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(p);
    else
        trace_pairs<false><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_gather_ops(const uint32_t* ops, const int64_t* slot_off, const int32_t* nops,
                              const int64_t* out_off, uint32_t* out, int64_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n * 32 + 255) / 256;
    if (blocks > 65535) blocks = 65535;
    gather_ops<<<(unsigned)blocks, 256, 0, stream>>>(ops, slot_off, nops, out_off, out, n);
    return cudaGetLastError();
}

}  // namespace gbsw
