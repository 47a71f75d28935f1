/*
 * oracle/traceback.c -- CPU statement of the traceback (CIGAR) of aligned pairs.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the library's traceback kernel, used
 * by tests/ and bench.py's CPU legs, never by the product library.
 *
 * The reference declares a traceback (kernel.hpp:36-39) but never implements
 * one, so there is no reference behaviour to restate; this file states the
 * library's own definition, which the GPU kernel must reproduce exactly.
 *
 * For a pair with score > 0, begins rb, qb (0-based) and ends re, qe (1-based
 * inclusive), the path is a global affine alignment of the segments
 * R = ref[rb:re] (m symbols, columns j) and Q = query[qb:qe] (k symbols, rows i):
 *
 *   H(0,0) = 0
 *   H(0,j) = open + (j-1)*extend   (j >= 1)        E(i,0) = F(0,j) = -inf
 *   H(i,0) = open + (i-1)*extend   (i >= 1)
 *   E(i,j) = max(E(i,j-1) + extend, H(i,j-1) + open)   a reference symbol against a gap: 'D'
 *   F(i,j) = max(F(i-1,j) + extend, H(i-1,j) + open)   a query symbol against a gap:     'I'
 *   H(i,j) = max(H(i-1,j-1) + s(R[j-1], Q[i-1]), F(i,j), E(i,j))
 *
 * An optimal local alignment starts and ends with an aligned pair, so H(k, m)
 * equals the pair's score; path_score reports H(k, m) so that callers can
 * check it.  s is the substitution score of the passes: DNA compares raw bytes;
 * protein uses matrix[enc(x)][enc(y)] with x the symbol of the longer of the
 * pair's two whole sequences (the reference on equal lengths).
 *
 * Ties: H takes the diagonal if it is >= both gaps, else F if F >= E, else E;
 * E and F extend when extending is >= opening.  The path is walked back from
 * (k, m) to (0, 0) and written forwards as run-length operations
 * (length << 4 | op) with the SAM/BAM codes 1 'I', 2 'D', 7 '=' (identical
 * bytes), 8 'X' (different bytes).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TB_OK 0
#define TB_EBADARG -1
#define TB_ENOMEM -3
#define TB_EPATH -4

#define OP_I 1u
#define OP_D 2u
#define OP_EQ 7u
#define OP_X 8u

typedef struct {
    int kind; /* 0 DNA, 1 protein (the oracle_scoring layout of gotoh.c) */
    int match, mismatch;
    int open, extend;
    const int16_t* matrix;
    const int16_t* encoding;
} tb_scoring;

static const int kNegInf = -(1 << 30);

static inline int imax(int x, int y) { return x > y ? x : y; }

/* gap of `len` >= 1 symbols, clamped far below any path score */
static int gap_cost(const tb_scoring* sc, int64_t len) {
    int64_t v = (int64_t)sc->open + (len - 1) * (int64_t)sc->extend;
    return v < kNegInf ? kNegInf : (int)v;
}

static int subst(const tb_scoring* sc, unsigned char r, unsigned char q, int ref_is_longer) {
    if (sc->kind == 0) return r == q ? sc->match : sc->mismatch;
    int er = sc->encoding[r], eq = sc->encoding[q];
    return ref_is_longer ? sc->matrix[er * 24 + eq] : sc->matrix[eq * 24 + er];
}

/* Appends op to the reversed run list. */
static void push(uint32_t* ops, int* nops, uint32_t op) {
    if (*nops > 0 && (ops[*nops - 1] & 15u) == op) {
        ops[*nops - 1] += 16u;
        return;
    }
    ops[(*nops)++] = 16u | op;
}

/* One pair.  dirs: (k+1)*(m+1) bytes of workspace. */
static int trace_pair(const unsigned char* R, int m, const unsigned char* Q, int k, int ref_is_longer,
                      const tb_scoring* sc, unsigned char* dirs, int* Hrow, int* Frow, uint32_t* ops,
                      int* nops, int* path_score) {
    const int W = m + 1;
    /* row 0 */
    Hrow[0] = 0;
    Frow[0] = kNegInf;
    for (int j = 1; j <= m; ++j) {
        Hrow[j] = gap_cost(sc, j);
        Frow[j] = kNegInf;
    }
    for (int i = 1; i <= k; ++i) {
        int diag = Hrow[0];      /* H(i-1, 0) */
        int hleft = gap_cost(sc, i); /* H(i, 0) */
        int eleft = kNegInf;     /* E(i, 0)  */
        Hrow[0] = hleft;
        for (int j = 1; j <= m; ++j) {
            const int e_ext = eleft + sc->extend, e_open = hleft + sc->open;
            const int e = imax(e_ext, e_open);
            const int f_ext = Frow[j] + sc->extend, f_open = Hrow[j] + sc->open;
            const int f = imax(f_ext, f_open);
            const int d = diag + subst(sc, R[j - 1], Q[i - 1], ref_is_longer);
            int h, src;
            if (d >= f && d >= e) {
                h = d;
                src = 0;
            } else if (f >= e) {
                h = f;
                src = 2;
            } else {
                h = e;
                src = 1;
            }
            dirs[(size_t)i * W + j] = (unsigned char)(src | (e_ext >= e_open ? 4 : 0) | (f_ext >= f_open ? 8 : 0));
            diag = Hrow[j];
            Hrow[j] = h;
            Frow[j] = f;
            hleft = h;
            eleft = e;
        }
    }
    *path_score = Hrow[m];
    /* walk back from (k, m) */
    int i = k, j = m, state = 0, n = 0;
    while (i > 0 || j > 0) {
        if (i == 0) {
            push(ops, &n, OP_D);
            --j;
            continue;
        }
        if (j == 0) {
            push(ops, &n, OP_I);
            --i;
            continue;
        }
        const unsigned char dv = dirs[(size_t)i * W + j];
        if (state == 0) {
            const int src = dv & 3;
            if (src == 0) {
                push(ops, &n, R[j - 1] == Q[i - 1] ? OP_EQ : OP_X);
                --i;
                --j;
            } else {
                state = src; /* 1: E, 2: F; no move */
            }
        } else if (state == 1) {
            push(ops, &n, OP_D);
            if (!(dv & 4)) state = 0;
            --j;
        } else {
            push(ops, &n, OP_I);
            if (!(dv & 8)) state = 0;
            --i;
        }
    }
    /* forwards */
    for (int a = 0, b = n - 1; a < b; ++a, --b) {
        uint32_t t = ops[a];
        ops[a] = ops[b];
        ops[b] = t;
    }
    *nops = n;
    return TB_OK;
}

/*
 * Pairs k = 0..n-1 with their results res[5k..5k+4] = score, ref_begin,
 * ref_end, query_begin, query_end.  ops_off[k] is the first slot of pair k in
 * `ops`; pair k may use up to (ref_end - ref_begin) + (query_end - query_begin)
 * slots.  Writes nops[k] runs and path_score[k] = H(k, m) (0 and 0 for a pair
 * with score <= 0).
 */
int oracle_traceback_batch(const char* A, const int64_t* offA, const char* B, const int64_t* offB, int64_t n,
                           const tb_scoring* sc, const int32_t* res, uint32_t* ops, const int64_t* ops_off,
                           int32_t* nops, int32_t* path_score, int nthreads) {
    if (n < 0 || !offA || !offB || !res || !ops || !ops_off || !nops || !path_score || !sc) return TB_EBADARG;
    int err = TB_OK;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#else
    (void)nthreads;
#endif
    {
        unsigned char* dirs = NULL;
        int *Hrow = NULL, *Frow = NULL;
        size_t dcap = 0, rcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t p = 0; p < n; ++p) {
            const int32_t* r = res + 5 * p;
            nops[p] = 0;
            path_score[p] = 0;
            if (r[0] <= 0) continue;
            const int a = (int)(offA[p + 1] - offA[p]), b = (int)(offB[p + 1] - offB[p]);
            const int rb = r[1], re = r[2], qb = r[3], qe = r[4];
            if (rb < 0 || re > a || rb >= re || qb < 0 || qe > b || qb >= qe) {
#ifdef _OPENMP
#pragma omp critical
#endif
                err = err ? err : TB_EBADARG;
                continue;
            }
            const int m = re - rb, k = qe - qb;
            const size_t need = (size_t)(k + 1) * (size_t)(m + 1);
            if (need > dcap) {
                free(dirs);
                dirs = (unsigned char*)malloc(need);
                dcap = dirs ? need : 0;
            }
            if ((size_t)(m + 1) > rcap) {
                free(Hrow);
                free(Frow);
                Hrow = (int*)malloc(sizeof(int) * (size_t)(m + 1));
                Frow = (int*)malloc(sizeof(int) * (size_t)(m + 1));
                rcap = (Hrow && Frow) ? (size_t)(m + 1) : 0;
            }
            if (!dirs || !rcap) {
#ifdef _OPENMP
#pragma omp critical
#endif
                err = err ? err : TB_ENOMEM;
                continue;
            }
            int nn = 0, ps = 0;
            trace_pair((const unsigned char*)A + offA[p] + rb, m, (const unsigned char*)B + offB[p] + qb, k, a >= b, sc,
                       dirs, Hrow, Frow, ops + ops_off[p], &nn, &ps);
            nops[p] = nn;
            path_score[p] = ps;
        }
        free(dirs);
        free(Hrow);
        free(Frow);
    }
    return err;
}
