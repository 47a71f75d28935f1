/*
 * gbsw.h -- C ABI of the GB300 batched Smith-Waterman library (libgbsw.so).
 *
 * Every entry point returns an int status (GBSW_OK = 0 or a negative code) and
 * never exits the process; gbsw_strerror() names a code and
 * gbsw_last_error() gives the message of the last failure on a context.
 *
 * Conventions shared with the reference (ADEPT / GPU-BSW):
 *   - A pair is a reference ("contig", seqA) and a query ("read", seqB).
 *   - Results per pair: top score, ref/query begin (0-based) and ref/query end
 *     (1-based, inclusive), exactly the five arrays of the reference's
 *     gpu_bsw_driver::alignment_results (driver.hpp:21-27).  A pair whose best
 *     local score is 0 (no positive cell; also any empty sequence) reports
 *     score 0 and -1 for all four positions.
 *   - DNA symbols are compared as raw bytes (kernel.cpp:366); protein symbols
 *     go through the reference's 91-entry ASCII table (driver.cpp:252-258)
 *     into a 24x24 matrix in the order A R N D C Q E G H I L K M F P S T W Y V
 *     B Z X *, indexed [longer-sequence symbol][shorter-sequence symbol]
 *     (kernel.cpp:785-788).
 *   - Ties between equal scores are broken exactly as the reference's kernels
 *     break them (see the library's design notes).
 *
 * Limits: gap_open and gap_extend must be <= 0; sequences at most
 * GBSW_MAX_SEQ_LEN symbols; protein symbols below 91.  Scores and positions
 * are computed in int32; the int16 result form truncates like the reference's
 * short arrays when a value exceeds 32767.
 */
#ifndef GBSW_H
#define GBSW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSW_DNA 0
#define GBSW_PROTEIN 1

#define GBSW_MAX_SEQ_LEN 65535

#define GBSW_OK 0
#define GBSW_EINVAL -1    /* bad argument (null pointer, negative count, gap > 0, bad offsets) */
#define GBSW_ESYMBOL -2   /* protein symbol outside the 91-entry encoding table              */
#define GBSW_ELENGTH -3   /* sequence longer than GBSW_MAX_SEQ_LEN                            */
#define GBSW_ECUDA -4     /* CUDA runtime error                                               */
#define GBSW_ENOMEM -5    /* device or pinned host allocation failed                          */
#define GBSW_EINTERNAL -6 /* internal consistency check failed                                */
#define GBSW_ETOOBIG -7   /* batch larger than the fixed scratch of gbsw_align_device_noalloc */
#define GBSW_ETIMEOUT -8  /* gbsw_server_wait: the job did not finish within the timeout     */

typedef struct gbsw_context gbsw_context;

typedef struct {
    int32_t kind;          /* GBSW_DNA or GBSW_PROTEIN                                  */
    int16_t match;         /* DNA: scores[0] of kernel_driver_dna (driver.cpp:18)       */
    int16_t mismatch;      /* DNA: scores[1]                                            */
    int16_t gap_open;      /* scores[2] / openGap   ("startGap" in the kernels)         */
    int16_t gap_extend;    /* scores[3] / extendGap                                     */
    const int16_t* matrix; /* protein: 576 entries, row-major 24x24 (main.cpp:70-92)    */
} gbsw_scoring;

/* Create a context bound to one CUDA device (replaces the per-GPU set-up of
 * driver.cpp:38-83: streams, device buffers, pinned staging).  Buffers grow on
 * demand and are reused across calls. */
int gbsw_create(int device, gbsw_context** out);
void gbsw_destroy(gbsw_context* ctx);
const char* gbsw_strerror(int status);
const char* gbsw_last_error(const gbsw_context* ctx);

/*
 * Host-buffer entry: the drop-in path.  Replaces the body of
 * gpu_bsw_driver::kernel_driver_dna / kernel_driver_aa (driver.cpp:15-243,
 * 245-489): copies the pairs to the GPU, runs the forward and reverse passes and
 * copies the five result arrays back.  Pair k is
 * ref[ref_off[k] : ref_off[k+1]] against query[query_off[k] : query_off[k+1]]
 * (n+1 exclusive prefix offsets each).  Synchronous.
 */
int gbsw_align_host16(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref,
                      const int64_t* ref_off, const char* query, const int64_t* query_off,
                      int64_t n, int16_t* ref_begin, int16_t* ref_end, int16_t* query_begin,
                      int16_t* query_end, int16_t* top_scores);
int gbsw_align_host32(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref,
                      const int64_t* ref_off, const char* query, const int64_t* query_off,
                      int64_t n, int32_t* ref_begin, int32_t* ref_end, int32_t* query_begin,
                      int32_t* query_end, int32_t* top_scores);

/*
 * Device-resident entry.  Replaces the launches of sequence_dna_kernel /
 * sequence_dna_reverse and sequence_aa_kernel / sequence_aa_reverse
 * (kernel.hpp:41-59; launched at driver.cpp:176-208, 422-455).  All pointers are
 * device pointers; max_len bounds every sequence length of the batch (the
 * driver's maxContigSize / maxReadSize, driver.cpp:19-20).  Work is enqueued
 * on `stream` (a cudaStream_t; NULL is the CUDA default stream, as everywhere
 * in CUDA) and the call returns without synchronising; gbsw_check(ctx, stream)
 * waits for the stream and reports device-side errors of the batch.
 */
int gbsw_align_device(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref,
                      const int64_t* ref_off, const uint8_t* query, const int64_t* query_off,
                      int64_t n, int32_t max_len, int32_t* top_scores, int32_t* ref_begin,
                      int32_t* ref_end, int32_t* query_begin, int32_t* query_end, void* stream);

/* Synchronises `stream` and reports device-side errors of the last device-entry
 * call (bad protein symbol, internal check). */
int gbsw_check(gbsw_context* ctx, void* stream);

/* Total memory of a device in bytes (gpu_bsw_driver::get_tot_gpu_mem, driver.hpp:29-30). */
int gbsw_device_memory(int device, uint64_t* bytes);

/*
 * Packed sequences: 2 bits per DNA base, 5 bits per protein residue.  The
 * reference ships raw bytes to the device (utils.cpp:30-54, driver.cpp:150-168);
 * a packed stream carries a concatenated sequence buffer -- the ref or the
 * query buffer of the entries above, with the same offsets -- in a quarter
 * (DNA) or about five eighths (protein) of its bytes.  Symbol j of the stream
 * is raw byte j.  Symbols fill 32-bit words from the lowest bits up:
 *   DNA      16 a word, the code (b >> 1) & 3 of the bases A C T G (0 1 2 3);
 *   protein   6 a word (bits 30-31 zero), the code b - 'A' of the letters A-Z.
 * Every other byte (N, lower case, '*', ...) is an escape: runs of escaped
 * bytes are kept raw next to the words (their symbols in the words are 0), so
 * any byte string packs and unpacks exactly and scores as the same bytes.
 * Escape runs are increasing and disjoint: run r is raw bytes
 * [run_at[r], run_at[r] + run_off[r+1] - run_off[r]), whose bytes are
 * run_bytes[run_off[r] : run_off[r+1]].
 */
typedef struct {
    const uint32_t* words;     /* gbsw_packed_words(kind, nsym) words              */
    int64_t nsym;              /* symbols (= raw bytes) in the stream              */
    int64_t nruns;             /* escape runs                                       */
    const int64_t* run_at;     /* nruns: first raw byte of each run                 */
    const int64_t* run_off;    /* nruns + 1 prefix offsets into run_bytes           */
    const uint8_t* run_bytes;  /* the escaped bytes, run after run                  */
} gbsw_packed;

#define GBSW_DNA_PER_WORD 16
#define GBSW_PROTEIN_PER_WORD 6
/* Words of a packed stream of nsym symbols (-1 for a bad kind or count). */
int64_t gbsw_packed_words(int kind, int64_t nsym);
/*
 * Packs nsym raw bytes on `threads` host threads (0: one per hardware thread,
 * up to 16).  Writes every word; writes the escape runs when they fit
 * run_cap runs and byte_cap bytes (run_at: run_cap entries, run_off:
 * run_cap + 1; both may be NULL when run_cap is 0).  *nruns and *nbytes always
 * receive the counts the stream needs: with run_cap = 0 a first call measures,
 * and the call returns GBSW_ETOOBIG whenever the runs did not fit.
 */
int gbsw_pack(int kind, const char* raw, int64_t nsym, int threads, uint32_t* words, int64_t run_cap,
              int64_t* run_at, int64_t* run_off, int64_t byte_cap, uint8_t* run_bytes, int64_t* nruns,
              int64_t* nbytes);
/*
 * Device-side unpack: every pointer of `packed` and `out` (nsym bytes) is
 * device memory of the current device.  Enqueued on `stream`; runs are not
 * validated beyond keeping every write inside out[0 : nsym).
 */
int gbsw_unpack_device(int kind, const gbsw_packed* packed, uint8_t* out, void* stream);
/*
 * Host entry over packed host buffers: gbsw_align_host16/32 with the ref and
 * query buffers given packed (host memory; page-locked memory copies fastest).
 * The packed words and runs are copied to the device and unpacked there before
 * the passes, so the host-to-device copy carries the packed bytes.  Offsets
 * as for gbsw_align_host16; ref_off[n] <= ref->nsym, query_off[n] <= query->nsym.
 * The streams are checked first; the pairs' offsets are checked while the
 * copies and the unpack run (a bad offset returns GBSW_EINVAL or GBSW_ELENGTH
 * as before, after those copies have finished).
 */
int gbsw_align_packed_host16(gbsw_context* ctx, const gbsw_scoring* scoring, const gbsw_packed* ref,
                             const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off,
                             int64_t n, int16_t* ref_begin, int16_t* ref_end, int16_t* query_begin,
                             int16_t* query_end, int16_t* top_scores);
int gbsw_align_packed_host32(gbsw_context* ctx, const gbsw_scoring* scoring, const gbsw_packed* ref,
                             const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off,
                             int64_t n, int32_t* ref_begin, int32_t* ref_end, int32_t* query_begin,
                             int32_t* query_end, int32_t* top_scores);

/*
 * Multi-GPU split (replaces the reference's split of a batch into equal pair
 * counts per GPU, driver.cpp:28-31).  Cuts n pairs into `parts` contiguous
 * ranges whose sums of cells[k] (|ref| * |query| of pair k) are as equal as a
 * cut between pairs allows: part r is pairs [bounds[r], bounds[r + 1]), and
 * bounds holds parts + 1 entries.  Part r ends at the first pair whose running
 * sum reaches r / parts of the total.  Host only; the C++ drop-in and the
 * Python sharding helper both use it.
 */
int gbsw_split_pairs(const int64_t* cells, int64_t n, int parts, int64_t* bounds);

/* Execution options of a context. */
typedef struct {
    int32_t use_dpx;        /* 1: Blackwell DPX max instructions (default), 0: plain integer ops */
    int32_t blocks_per_sm;  /* 0: from the occupancy calculator                                */
    int32_t lane_group;     /* lanes per pair: 0 = chosen from the batch size (default);
                               4 = large-batch kernels; 8, 16, 32 = kernels that spread each
                               pair over more lanes; 128 = block per pair (the four warps of a
                               block share one pair, a column strip each; int32, DPX only).
                               Two pairs share a group in int16x2:
                               DNA A/C/G/T pairs at 4, 8 and 16 lanes, protein at 16 and 32;
                               a pair whose score may have overflowed int16 there is aligned
                               again in int32 (gbsw_stats.reruns).  DPX only, ignored
                               without DPX.  0 also lets the tuning table choose per
                               length bin (see gbsw_tuning). */
} gbsw_options;
int gbsw_set_options(gbsw_context* ctx, const gbsw_options* opts);
int gbsw_get_options(const gbsw_context* ctx, gbsw_options* opts);

/* Length bins and pair-count buckets of the per-bin plans (see gbsw_tuning). */
#define GBSW_BINS 2
#define GBSW_COUNT_BUCKETS 6

/* Timing of the last call on a context (CUDA events on its stream).  After
 * gbsw_traceback_host: forward_ms is its traceback kernels, reverse_ms 0, and
 * h2d_ms / d2h_ms / total_ms its copies and the whole call. */
typedef struct {
    double forward_ms;   /* forward pass kernel                  */
    double reverse_ms;   /* reverse pass kernel                  */
    double h2d_ms;       /* host-buffer entry: input copies      */
    double d2h_ms;       /* host-buffer entry: result copies     */
    double total_ms;     /* whole call                           */
    int64_t cells;       /* forward cells, sum |ref| * |query|   */
    int32_t launches;    /* kernels launched by the call         */
    int32_t lane_group;  /* lanes per pair it ran with (4: the large-batch kernels) */
    int32_t dual;        /* 1: the dual-pair int16x2 kernels ran the eligible pairs  */
    int64_t reruns;      /* pairs of those whose score may have overflowed int16 and
                            that were therefore aligned again in int32           */
    int64_t bin_pairs[GBSW_BINS]; /* pairs in each length bin (-1: not read back) */
    int32_t bin_dual[GBSW_BINS];  /* forward pass: 1 = the bin ran two pairs per group in int16x2 */
    int32_t bin_lanes[GBSW_BINS]; /* forward pass: lanes per group of the bin's launch           */
    int32_t bin_tuned[GBSW_BINS]; /* 1: the bin's plans came from the tuning table               */
    int32_t rev_dual[GBSW_BINS];  /* reverse pass: as bin_dual                                   */
    int32_t rev_lanes[GBSW_BINS]; /* reverse pass: as bin_lanes                                  */
} gbsw_stats;
int gbsw_last_stats(const gbsw_context* ctx, gbsw_stats* stats);

/*
 * Per-length-bin plans and the autotuner (no counterpart in the reference,
 * which runs every pair of a batch as one block per pair with one thread per
 * column of the batch's shortest maximum, driver.cpp:169-176).
 *
 * The pairs a plan can choose for -- DNA pairs of A/C/G/T only, protein pairs
 * whose matrix fits int8, with gap values in [-16384, 0] -- fall into two length
 * bins by their shorter sequence: below 512, and from 512 up.  Each bin is its
 * own launch with its own variant, in each pass: two pairs per lane group in
 * the int16x2 kernels (dual = 1; DNA at 4, 8 or 16 lanes, protein at 16 or 32)
 * or one pair per group in int32 (dual = 0; 4, 8, 16 or 32 lanes, or 128: block
 * per pair).  With lane_group = 0 the call reads the bins' pair counts back
 * after the forward schedule (one small copy and a wait on the stream) and takes
 * each bin's forward variant from the context's tuning table, entry
 * variant[kind][bin][bucket] with buckets of up to 1,000, 3,000, 10,000, 30,000,
 * 100,000 and more pairs in the bin, and its reverse variant from
 * reverse[kind][bin][bucket] (lanes = 0 there: the forward one).  A forward
 * entry with lanes = 0 leaves the bin to the rule of gbsw_options.lane_group =
 * 0 (the batch size picks one width; long DNA pairs of a 4-lane plan run 16-lane
 * dual groups).  A context starts with a table measured on GB300 by
 * gpu-bsw_gb300/tune_sweep.py.
 */
typedef struct {
    int32_t dual;   /* 1: two pairs per group, int16x2; 0: one pair per group, int32 */
    int32_t lanes;  /* lanes per group; 0: no entry                                 */
} gbsw_variant;
typedef struct {
    gbsw_variant variant[2][GBSW_BINS][GBSW_COUNT_BUCKETS];  /* forward pass: [kind][bin][bucket] */
    gbsw_variant reverse[2][GBSW_BINS][GBSW_COUNT_BUCKETS];  /* reverse pass (lanes 0: as forward) */
} gbsw_tuning;
int gbsw_get_tuning(const gbsw_context* ctx, gbsw_tuning* tuning);
int gbsw_set_tuning(gbsw_context* ctx, const gbsw_tuning* tuning);

/*
 * Autotuner: runs the batch (device pointers, as gbsw_align_device) once per
 * candidate variant with every bin forced to it, `reps` timed runs each after
 * one warm-up, times each bin's forward and reverse launches with CUDA events,
 * and writes each non-empty bin's fastest variant into the context's tuning
 * table at that bin's pair-count bucket, for each pass on its own (the fastest
 * forward variant and the fastest reverse variant).  The report lists the
 * candidates, each bin's forward and reverse kernel times (ms, the fastest of
 * the runs), pairs, bucket and choices.  Synchronous; its results are
 * discarded.
 */
#define GBSW_TUNE_CANDIDATES 8
typedef struct {
    int32_t ncandidates;
    gbsw_variant candidates[GBSW_TUNE_CANDIDATES];
    double ms_forward[GBSW_BINS][GBSW_TUNE_CANDIDATES];
    double ms_reverse[GBSW_BINS][GBSW_TUNE_CANDIDATES];
    int64_t pairs[GBSW_BINS];
    int32_t bucket[GBSW_BINS];
    gbsw_variant chosen[GBSW_BINS];          /* forward pass */
    gbsw_variant chosen_reverse[GBSW_BINS];  /* reverse pass */
} gbsw_tune_report;
int gbsw_tune_device(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref,
                     const int64_t* ref_off, const uint8_t* query, const int64_t* query_off,
                     int64_t n, int32_t max_len, int32_t reps, void* stream,
                     gbsw_tune_report* report);

/*
 * Traceback (no counterpart in the reference, which declares one at
 * kernel.hpp:36-39 and never implements it).  For pairs aligned by this
 * library -- their five int32 result arrays as gbsw_align_host32 returns them,
 * same pairs, same scoring -- writes one optimal alignment path from each
 * pair's begin to its end as run-length operations (length << 4 | op), with the
 * SAM/BAM codes below.  Pair k's operations are (*ops)[ops_off[k] :
 * ops_off[k+1]]; the call writes all n+1 entries of ops_off.  The buffer belongs
 * to the context and stays valid until its next call.  A pair with score <= 0
 * has no operations.
 *
 * The path is the global affine alignment of ref[ref_begin:ref_end] and
 * query[query_begin:query_end]; its score is the pair's score.  Ties: a cell
 * takes the diagonal if it is >= both gaps, else the query gap ('I') if it is
 * >= the reference gap ('D'); a gap extends when extending scores >= opening.
 * With gap_open > gap_extend a run of one gap type may hold several gaps.
 * GBSW_EINVAL when results are out of range or a path does not reach its
 * pair's score (results from other inputs or another scoring).  Synchronous.
 */
#define GBSW_OP_I 1  /* query symbol against a gap (insertion)      */
#define GBSW_OP_D 2  /* reference symbol against a gap (deletion)   */
#define GBSW_OP_EQ 7 /* aligned identical symbols                   */
#define GBSW_OP_X 8  /* aligned different symbols                   */
int gbsw_traceback_host(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref,
                        const int64_t* ref_off, const char* query, const int64_t* query_off,
                        int64_t n, const int32_t* top_scores, const int32_t* ref_begin,
                        const int32_t* ref_end, const int32_t* query_begin,
                        const int32_t* query_end, int64_t* ops_off, const uint32_t** ops);

/*
 * Integer-pipe calibration (no counterpart in the reference).  Runs register-only
 * probes on `device` with every SM busy and reports applications per clock64
 * tick per SM of each instruction form used by the DP cell update and of the
 * whole cell updates, and the cell probes' throughput in cells per second
 * (CUDA events), which is the calibrated roofline of the passes.  On GB300
 * clock64 advances slower than the SM clock (about 1,270 ticks per
 * microsecond at a 2,070 MHz SM clock), so per-tick rates are not per-cycle
 * rates.  Takes about a second.
 */
typedef struct {
    int32_t sms;
    double sm_mhz;             /* clock64 ticks per microsecond in the probes  */
    double addmax_relu_s32;    /* __viaddmax_s32_relu                          */
    double max3_relu_s32;      /* __vimax3_s32_relu                            */
    double plain_addmax_s32;   /* max(a + b, c) from plain add + max           */
    double addmax_relu_s16x2;  /* __viaddmax_s16x2_relu                        */
    double max3_relu_s16x2;    /* __vimax3_s16x2_relu                          */
    double iadd_s32;           /* three-input add                              */
    double cell_dpx;           /* int32 DP cells (DPX forms)                   */
    double cell_plain;         /* int32 DP cells (plain integer ops)           */
    double cell_dual;          /* cells of the dual-pair pass's int16x2 cell
                                  block (16 columns x 2 pairs), registers only */
    double cell_dpx_gcups;     /* cell_dpx probe: 1e9 cells per second, all SMs */
    double cell_dual_gcups;    /* cell_dual probe: 1e9 cells per second, all SMs */
    double cell_int32;         /* cells of the int32 pass's cell block (16
                                  columns, profile scores), registers only     */
    double cell_int32_gcups;   /* cell_int32 probe: 1e9 cells per second       */
} gbsw_calibration;
int gbsw_calibrate(int device, gbsw_calibration* out);

/*
 * Allocation-free device entry (no counterpart in the reference, whose driver
 * allocates on every call).
 *
 * For callers that must not allocate GPU memory themselves or through this
 * library: code running inside another framework's memory pool or caching
 * allocator (which has to own every device byte), code that runs after the
 * device was filled to a fixed budget, or code that may not risk an allocation
 * failing half-way through a pipeline.  It calls no cudaMalloc, cudaFree or
 * other allocating routine: every byte of working memory comes from one
 * fixed array of GBSW_NOALLOC_SCRATCH_BYTES compiled into libgbsw.so.
 *
 * The call runs on the current CUDA device: every pointer and the stream must
 * belong to it.  Arguments and results are those of gbsw_align_device (all
 * pointers are device pointers, NULL stream = the CUDA default stream); there
 * is no context.  Limits: n <= GBSW_NOALLOC_MAX_PAIRS pairs and max_len <=
 * GBSW_NOALLOC_MAX_LEN per call, else GBSW_ETOOBIG (split larger batches).
 * The call is synchronous: it returns after the batch has finished on
 * `stream`, with the batch's device-side checks in its status.
 *
 * CUDA loads the array onto a device lazily: the first call on each device
 * (in each CUDA context) commits its GBSW_NOALLOC_SCRATCH_BYTES, and the
 * device then holds them until the process exits.  A call with n = 0 (NULL
 * pointers allowed) does only that, so a caller that is about to fill the
 * device to a budget makes one such call first.  Make that first call before
 * any stream capture.  Every call looks the array's address up again in the
 * current context.  All calls on a device share the one array and it keeps
 * the last call's contents (the call clears what must start at zero): calls
 * that overlap on the GPU -- from two host threads, or on two streams -- race,
 * so serialise them.  It is also slower than gbsw_align_device on large
 * batches, as the fixed boundary buffer caps how many pairs run at once.
 */
#define GBSW_NOALLOC_MAX_PAIRS 65536
#define GBSW_NOALLOC_MAX_LEN 8192
#define GBSW_NOALLOC_SCRATCH_BYTES (64u << 20)
int gbsw_align_device_noalloc(const gbsw_scoring* scoring, const uint8_t* ref,
                              const int64_t* ref_off, const uint8_t* query,
                              const int64_t* query_off, int64_t n, int32_t max_len,
                              int32_t* top_scores, int32_t* ref_begin, int32_t* ref_end,
                              int32_t* query_begin, int32_t* query_end, void* stream);

/*
 * Serving loop (no counterpart in the reference, which aligns one batch per
 * blocking driver call, driver.cpp:15-243).
 *
 * A server owns `slots` worker threads on one device, each with its own
 * context and stream, so several batches run on the GPU at once.  Any host
 * thread submits a job (pairs with one scoring, laid out as for
 * gbsw_align_host32); the server copies the job's inputs into page-locked
 * staging, so the caller's sequence buffers may be reused as soon as submit
 * returns.  Jobs are admitted to the device in arrival order while their
 * footprint (sequences, offsets, results and schedule, about
 * |ref| + |query| + 65 bytes a pair) fits `hbm_budget` next to the jobs
 * already there, and stay resident until their batch ends.  A free worker
 * takes the oldest resident job and merges into the same launch every other
 * resident job with the same scoring, up to `max_batch_pairs` pairs
 * (continuous batching).  A job larger than the budget is admitted alone once
 * nothing else is on the device.  The per-context working buffers (boundary
 * rows, schedule) come on top of the budget and are kept between batches.
 * Results of a pair do not depend on the jobs it was batched with.
 *
 * When the job finishes, its results are in the caller's `results` array
 * (n x 5 int32, row-major per pair: score, ref_begin, ref_end, query_begin,
 * query_end; int32, like gbsw_align_host32), which must stay valid until
 * gbsw_server_wait has returned for that job.
 */
typedef struct gbsw_server gbsw_server;

typedef struct {
    int32_t device;          /* CUDA device                                          */
    int32_t slots;           /* worker threads / concurrent batches (1..64)          */
    uint64_t hbm_budget;     /* bytes of job inputs and results on the device at once */
    int64_t max_batch_pairs; /* merge queued jobs up to this many pairs per launch    */
} gbsw_server_options;

typedef struct {
    int32_t status;     /* the job's status (GBSW_OK or the batch's error)  */
    int64_t pairs;
    int64_t cells;      /* sum |ref| * |query| of the job                    */
    double queue_ms;    /* submit -> taken by a worker                       */
    double latency_ms;  /* submit -> results written                         */
} gbsw_job_info;

typedef struct {
    int64_t jobs;        /* finished since creation or the last reset         */
    int64_t batches;     /* launches those jobs were merged into              */
    int64_t peak_running;/* most batches on the device at once                */
    int64_t pairs;
    int64_t cells;
    int64_t queued;      /* jobs waiting now                                  */
    uint64_t hbm_in_use; /* footprint of the batches running now              */
    double p50_ms;       /* job latency percentiles (submit -> results)       */
    double p99_ms;
    double max_ms;
    double gcups;        /* cells / (last finish - creation or reset) / 1e9   */
    int64_t staged;      /* of the queued jobs, those still on the host, waiting
                            for HBM (the others are on the device)           */
} gbsw_server_stats;

/* NULL options: device 0, 4 slots, 16 GiB budget, 50,000 pairs per launch.
 * Returns after every worker has created its context (or the first error). */
int gbsw_server_create(const gbsw_server_options* opts, gbsw_server** out);
/* Finishes every queued job, then stops the workers and frees the server. */
void gbsw_server_destroy(gbsw_server* server);
int gbsw_server_submit(gbsw_server* server, const gbsw_scoring* scoring, const char* ref,
                       const int64_t* ref_off, const char* query, const int64_t* query_off,
                       int64_t n, int32_t* results, uint64_t* job_id);
/* Waits for a job (timeout_s < 0: without limit) and forgets it; returns the
 * job's status, GBSW_ETIMEOUT (the job stays known) or GBSW_EINVAL for an
 * unknown id.  Each job is waited for once. */
/* A job given as packed streams (gbsw_packed, host memory; the first offsets
 * are 0: the streams are the job's own).  The job stays packed through
 * admission and in HBM, a quarter (DNA) or 5/8 (protein) of its raw bytes, and
 * is unpacked on the device when a worker gathers its batch.  Results as for
 * gbsw_server_submit. */
int gbsw_server_submit_packed(gbsw_server* server, const gbsw_scoring* scoring, const gbsw_packed* ref,
                              const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off,
                              int64_t n, int32_t* results, uint64_t* job_id);
int gbsw_server_wait(gbsw_server* server, uint64_t job_id, double timeout_s, gbsw_job_info* info);
int gbsw_server_get_stats(gbsw_server* server, gbsw_server_stats* stats);
int gbsw_server_reset_stats(gbsw_server* server);

#ifdef __cplusplus
}
#endif
#endif
