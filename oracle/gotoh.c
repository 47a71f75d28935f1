/*
 * oracle/gotoh.c -- CPU restatement of the ADEPT (GPU-BSW) batched Smith-Waterman
 * forward (end-position) and reverse (begin-position) passes.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle of the CUDA path: it is
 * called by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg,
 * never by the product library.  It is deliberately plain: one full O(|L|*|S|)
 * Gotoh matrix sweep per pass, int32 arithmetic, no SIMD.
 *
 * What it restates, with the reference line it follows (paths within the
 * reference project):
 *
 *   role rule            kernel.cpp:248-259   |A| < |B|  ->  S = A (columns), L = B (rows);
 *                                             otherwise  S = B, L = A (ties: A is L)
 *   recurrence           kernel.cpp:326-372   F(i,j) = max(F(i-1,j)+ext, H(i-1,j)+open)
 *                                             E(i,j) = max(E(i,j-1)+ext, H(i,j-1)+open)
 *                                             H(i,j) = max(H(i-1,j-1)+s, E, F, 0)
 *   boundaries           kernel.cpp:270-272,  H(0,.) = H(.,0) = 0, F(0,.) = 0 (register
 *                        kernel.cpp:346-350   initialisation) and E(i,1) = 0 (thread 0
 *                                             forces eVal = heVal = 0)
 *   DNA substitution     kernel.cpp:366       raw byte compare: L==S ? match : mismatch
 *   protein substitution kernel.cpp:785-788   matrix[enc(L)*24 + enc(S)], enc = the 91-entry
 *                                             ASCII table of driver.cpp:252-258
 *   per-column argmax    kernel.cpp:368-370   first strict '>' down the column (init 0,0,0)
 *   warp/block argmax    kernel.cpp:47-86,    a shfl_down tree (offsets 16..1) in every warp,
 *                        kernel.cpp:137-182   then the same tree over the warp winners; a
 *                                             lane takes its partner's candidate only if the
 *                                             partner is strictly better; padding lanes of
 *                                             the second level carry (0,-1,-1)
 *   forward tie order    kernel.cpp:72-80     value desc, then smaller row index i
 *   forward output       kernel.cpp:379-393   1-based ends; (i,j) mapped back to (ref,query)
 *   reverse pass         kernel.cpp:397-604   same DP on A[0:ref_end], B[0:query_end], both
 *                                             reversed, roles re-decided on those lengths
 *   reverse tie order    kernel.cpp:3-45      value desc, then larger ind2 (= S start)
 *   reverse output       kernel.cpp:589-601   0-based begins, mapped back by role
 *
 * The reduction trees are simulated lane by lane, exactly as the shuffles
 * execute, with the block size equal to the pair's own shorter length (runs
 * of 1,024 columns beyond the reference's limit, see block_tree).  The
 * reference sizes its blocks from whole-batch maxima; that only changes the
 * result when every cell of a pair scores 0, a case the reference cannot
 * finish (its reverse pass then sizes shared memory from an end of -1).  For
 * such pairs (and for empty sequences) this oracle defines the result as
 * score 0 with all four positions -1.
 *
 * Scores are computed in int32.  The reference stores them in int16; the
 * oracle reports, per pair, whether any H value exceeded 32767 (flag bit 0),
 * in which case the int16 reference result is not meaningful.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_DNA 0
#define ORACLE_AA 1

#define ORACLE_OK 0
#define ORACLE_EBADARG -1
#define ORACLE_EBADCHAR -2
#define ORACLE_ENOMEM -3

typedef struct {
    int kind;                /* ORACLE_DNA or ORACLE_AA                          */
    int match, mismatch;     /* DNA scores (scores[0], scores[1] of the driver)  */
    int open, extend;        /* startGap, extendGap (scores[2], scores[3])       */
    const int16_t* matrix;   /* protein: 24x24 row-major, 576 entries            */
    const int16_t* encoding; /* protein: 91-entry ASCII -> matrix index table    */
} oracle_scoring;

typedef struct {
    int v;  /* value                                 */
    int a;  /* first index  (reference "ind")       */
    int b;  /* second index (reference "ind2")      */
} cand_t;

/* One shfl_down tree over 32 lanes (kernel.cpp:59-81 forward, :15-40 reverse).
 * All lanes read their partner's values from before the step, as the shuffles do. */
static cand_t warp_tree(const cand_t* in, int reverse) {
    cand_t cur[32], nxt[32];
    memcpy(cur, in, sizeof(cur));
    for (int off = 16; off > 0; off >>= 1) {
        for (int l = 0; l < 32; ++l) {
            cand_t me = cur[l];
            cand_t other = (l + off < 32) ? cur[l + off] : cur[l];
            int val = me.v > other.v ? me.v : other.v;
            if (val != me.v) {
                me = other;
            } else if (val == other.v) {
                if (!reverse) {
                    if (other.a < me.a) me = other;   /* kernel.cpp:76 */
                } else {
                    if (other.b > me.b) me = other;   /* kernel.cpp:34 */
                }
            }
            nxt[l] = me;
        }
        memcpy(cur, nxt, sizeof(cur));
    }
    return cur[0];
}

/* Block reduction of kernel.cpp:90-182 for `n` <= 1024 column candidates
 * (one thread per column, at most 32 warps). */
static cand_t block_tree_1024(const cand_t* cols, int n, int reverse) {
    int nwarps = (n + 31) / 32;
    cand_t lanes[32], winners[32];
    for (int w = 0; w < nwarps; ++w) {
        for (int l = 0; l < 32; ++l) {
            int t = w * 32 + l;
            if (t < n) {
                lanes[l] = cols[t];
            } else {
                /* threads beyond the pair's shorter length never update their
                 * (0,0,0) initial candidate (kernel.cpp:263-266) */
                lanes[l].v = 0;
                lanes[l].a = 0;
                lanes[l].b = 0;
            }
        }
        winners[w] = warp_tree(lanes, reverse);
    }
    for (int l = nwarps; l < 32; ++l) {   /* kernel.cpp:119-124 / 166-171 */
        winners[l].v = 0;
        winners[l].a = -1;
        winners[l].b = -1;
    }
    return warp_tree(winners, reverse);
}

/* The reference cannot run a shorter sequence above 1,024 (its block size).
 * Beyond that this oracle (and the CUDA path) extends the same order: the
 * tree above over each run of 1,024 columns, then the run winners in
 * increasing column order, a later run replacing an earlier one only when
 * strictly better by the same comparison. */
static cand_t block_tree(const cand_t* cols, int n, int reverse) {
    cand_t best = block_tree_1024(cols, n < 1024 ? n : 1024, reverse);
    for (int start = 1024; start < n; start += 1024) {
        int len = n - start < 1024 ? n - start : 1024;
        cand_t c = block_tree_1024(cols + start, len, reverse);
        int better = c.v > best.v ||
                     (c.v == best.v && (reverse ? c.b > best.b : c.a < best.a));
        if (better) best = c;
    }
    return best;
}

static inline int max2(int x, int y) { return x > y ? x : y; }

/* Substitution score s(Lc, Sc). */
static inline int subst(const oracle_scoring* sc, unsigned char lc, unsigned char scc) {
    if (sc->kind == ORACLE_DNA) return lc == scc ? sc->match : sc->mismatch;
    return sc->matrix[sc->encoding[lc] * 24 + sc->encoding[scc]];
}

/*
 * One DP sweep.  Rows i = 1..nL take L char Lrow(i), columns j = 1..nS take
 * S char Scol(j).  For the forward pass Lrow(i) = L[i-1], Scol(j) = S[j-1];
 * for the reverse pass both strings are read back to front.  Fills the per-
 * column candidates: colv[j-1] = column max, colrow[j-1] = first row reaching
 * it (0 when the column max is 0).  Returns the max H seen (for the overflow flag).
 */
static int sweep(const oracle_scoring* sc, const unsigned char* L, int nL, const unsigned char* S,
                 int nS, int reversed, int* Hrow, int* Frow, int* colv, int* colrow) {
    int hmax = 0;
    for (int j = 0; j <= nS; ++j) {
        Hrow[j] = 0;
        Frow[j] = 0;
    }
    for (int j = 0; j < nS; ++j) {
        colv[j] = 0;
        colrow[j] = 0;
    }
    for (int i = 1; i <= nL; ++i) {
        unsigned char lc = reversed ? L[nL - i] : L[i - 1];
        int diag = 0;   /* H(i-1, 0) */
        int Hleft = 0;  /* H(i, 0)   */
        int Eleft = 0;
        for (int j = 1; j <= nS; ++j) {
            unsigned char scc = reversed ? S[nS - j] : S[j - 1];
            int F = max2(Frow[j] + sc->extend, Hrow[j] + sc->open);
            int E = (j == 1) ? 0 : max2(Eleft + sc->extend, Hleft + sc->open);
            int H = diag + subst(sc, lc, scc);
            H = max2(H, F);
            H = max2(H, E);
            H = max2(H, 0);
            if (H > colv[j - 1]) {  /* kernel.cpp:368-370: keep on >=, move on > */
                colv[j - 1] = H;
                colrow[j - 1] = i;
            }
            if (H > hmax) hmax = H;
            diag = Hrow[j];
            Hrow[j] = H;
            Frow[j] = F;
            Eleft = E;
            Hleft = H;
        }
    }
    return hmax;
}

typedef struct {
    int* Hrow;
    int* Frow;
    int* colv;
    int* colrow;
    cand_t* cands;
    int cap;
} workspace;

static int ws_reserve(workspace* ws, int n) {
    if (n <= ws->cap) return 0;
    free(ws->Hrow);
    free(ws->Frow);
    free(ws->colv);
    free(ws->colrow);
    free(ws->cands);
    ws->Hrow = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    ws->Frow = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    ws->colv = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    ws->colrow = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    ws->cands = (cand_t*)malloc(sizeof(cand_t) * (size_t)(n + 1));
    ws->cap = n;
    if (!ws->Hrow || !ws->Frow || !ws->colv || !ws->colrow || !ws->cands) {
        ws->cap = 0;
        return -1;
    }
    return 0;
}

static void ws_free(workspace* ws) {
    free(ws->Hrow);
    free(ws->Frow);
    free(ws->colv);
    free(ws->colrow);
    free(ws->cands);
    memset(ws, 0, sizeof(*ws));
}

static int check_chars(const oracle_scoring* sc, const unsigned char* s, int n) {
    if (sc->kind != ORACLE_AA) return 0;
    for (int k = 0; k < n; ++k)
        if (s[k] > 90) return -1;  /* outside the 91-entry encoding table */
    return 0;
}

/*
 * out[0..4] = score, ref_begin, ref_end, query_begin, query_end  (A = ref /
 * contig = seqA, B = query / read = seqB, as in driver.cpp:16 and main.cpp:213).
 * Ends are 1-based inclusive, begins 0-based, like the reference's arrays.
 * *flags: bit 0 = some H exceeded 32767.
 */
static int align_pair_ws(const char* A_, int a, const char* B_, int b, const oracle_scoring* sc,
                         int32_t* out, int* flags, workspace* ws) {
    const unsigned char* A = (const unsigned char*)A_;
    const unsigned char* B = (const unsigned char*)B_;
    *flags = 0;
    if (a < 0 || b < 0) return ORACLE_EBADARG;
    if (check_chars(sc, A, a) || check_chars(sc, B, b)) return ORACLE_EBADCHAR;
    int nmax = a > b ? a : b;
    if (ws_reserve(ws, nmax)) return ORACLE_ENOMEM;

    /* ---- forward pass (kernel.cpp:198-394) ---- */
    int a_is_short = a < b;                 /* kernel.cpp:248 */
    const unsigned char* S = a_is_short ? A : B;
    const unsigned char* L = a_is_short ? B : A;
    int nS = a_is_short ? a : b;
    int nL = a_is_short ? b : a;
    int hmax = 0;
    if (nS > 0) {
        hmax = sweep(sc, L, nL, S, nS, 0, ws->Hrow, ws->Frow, ws->colv, ws->colrow);
    }
    if (hmax > 32767) *flags |= 1;
    if (hmax <= 0) {
        out[0] = 0;
        out[1] = out[2] = out[3] = out[4] = -1;
        return ORACLE_OK;
    }
    for (int t = 0; t < nS; ++t) {
        ws->cands[t].v = ws->colv[t];
        ws->cands[t].a = ws->colrow[t];               /* thread_max_i */
        ws->cands[t].b = ws->colv[t] > 0 ? t + 1 : 0; /* thread_max_j */
    }
    cand_t fw = block_tree(ws->cands, nS, 0);
    int ref_end, query_end;
    if (a_is_short) {                               /* kernel.cpp:381-386 */
        query_end = fw.a;
        ref_end = fw.b;
    } else {                                        /* kernel.cpp:387-392 */
        ref_end = fw.a;
        query_end = fw.b;
    }

    /* ---- reverse pass (kernel.cpp:397-604) ---- */
    int na = ref_end, nb = query_end;               /* kernel.cpp:426-427 */
    int a2_is_short = na < nb;                      /* kernel.cpp:444 */
    const unsigned char* S2 = a2_is_short ? A : B;
    const unsigned char* L2 = a2_is_short ? B : A;
    int nS2 = a2_is_short ? na : nb;
    int nL2 = a2_is_short ? nb : na;
    sweep(sc, L2, nL2, S2, nS2, 1, ws->Hrow, ws->Frow, ws->colv, ws->colrow);
    for (int t = 0; t < nS2; ++t) {
        int v = ws->colv[t];
        ws->cands[t].v = v;
        ws->cands[t].a = v > 0 ? nL2 - ws->colrow[t] : 0; /* kernel.cpp:579 */
        ws->cands[t].b = v > 0 ? nS2 - t - 1 : 0;         /* kernel.cpp:580 */
    }
    cand_t rv = block_tree(ws->cands, nS2, 1);
    int ref_begin, query_begin;
    if (a2_is_short) {                              /* kernel.cpp:591-595 */
        query_begin = rv.a;
        ref_begin = rv.b;
    } else {                                        /* kernel.cpp:596-600 */
        ref_begin = rv.a;
        query_begin = rv.b;
    }
    out[0] = fw.v;
    out[1] = ref_begin;
    out[2] = ref_end;
    out[3] = query_begin;
    out[4] = query_end;
    return ORACLE_OK;
}

int oracle_align_pair(const char* A, int a, const char* B, int b, const oracle_scoring* sc,
                      int32_t* out5, int* flags) {
    workspace ws;
    memset(&ws, 0, sizeof(ws));
    int rc = align_pair_ws(A, a, B, b, sc, out5, flags, &ws);
    ws_free(&ws);
    return rc;
}

/*
 * Batch form.  offA / offB are exclusive prefix offsets with n+1 entries
 * (pair k is A[offA[k] : offA[k+1]]).  out is n x 5 (see oracle_align_pair),
 * flags is n entries (may be NULL).  nthreads <= 0 uses the OpenMP default.
 * Pairs are independent; a dynamic schedule balances uneven lengths.
 * Returns the first error code met, or ORACLE_OK.
 */
int oracle_align_batch(const char* A, const int64_t* offA, const char* B, const int64_t* offB,
                       int64_t n, const oracle_scoring* sc, int32_t* out, int32_t* flags,
                       int nthreads) {
    if (n < 0 || !offA || !offB || !out || !sc) return ORACLE_EBADARG;
    int err = ORACLE_OK;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#else
    (void)nthreads;
#endif
    {
        workspace ws;
        memset(&ws, 0, sizeof(ws));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t k = 0; k < n; ++k) {
            int f = 0;
            int rc = align_pair_ws(A + offA[k], (int)(offA[k + 1] - offA[k]), B + offB[k],
                                   (int)(offB[k + 1] - offB[k]), sc, out + 5 * k, &f, &ws);
            if (flags) flags[k] = f;
            if (rc != ORACLE_OK) {
#ifdef _OPENMP
#pragma omp critical
#endif
                {
                    if (err == ORACLE_OK) err = rc;
                }
            }
        }
        ws_free(&ws);
    }
    return err;
}

/* Number of OpenMP threads a batch call uses by default. */
int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
