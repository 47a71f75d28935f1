// C ABI of libgbsw.so: contexts, device buffers, the host-buffer (drop-in)
// entry and the device-resident entry.  See include/gbsw.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbsw.h"
#include "pack.h"
#include "schedule.h"
#include "sw_kernels.h"
#include "results.h"
#include "traceback.h"
#include "tuning.h"

namespace {

const char* kAAOrder = "ARNDCQEGHILKMFPSTWYVBZX*";

// Device buffer that grows on demand (contents are not preserved).
template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap) return cudaSuccess;
        const size_t want = std::max<size_t>(n, cap + cap / 2);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&ptr, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

template <typename T>
struct HostBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap) return cudaSuccess;
        const size_t want = std::max<size_t>(n, cap + cap / 2);
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&ptr, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

enum { EV_START, EV_H2D, EV_FWD, EV_REV, EV_D2H, EV_COUNT };

}  // namespace

struct gbsw_context {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    gbsw_options opts{1, 0, 0};
    std::string last_error;

    DevBuf<uint8_t> d_ref, d_query;
    DevBuf<uint8_t> d_pack;  // packed host entries: both streams' words and escape runs
    DevBuf<int64_t> d_ref_off, d_query_off;
    DevBuf<int32_t> d_results;
    DevBuf<int2> d_scratch;
    DevBuf<int> d_misc;      // [3] error flags; [8 + class] forward and [16 + class] reverse work queues,
                             // [24] the int32 rerun pass's queue
    DevBuf<int> d_rerun;     // int32 rerun of dual-pair overflows: [0] = 0, [1] = count, pair indices from [2]
    DevBuf<uint8_t> d_cls;   // schedule: class of every pair
    DevBuf<int> d_keys;      // schedule: bucket of every pair
    DevBuf<int> d_order;     // schedule: pair indices in schedule order
    DevBuf<int> d_hist;      // schedule: bucket counters / offsets, then the class ranges
    DevBuf<int> d_matrix;    // 25x25 (score - open)
    DevBuf<int> d_encoding;  // 91 entries
    HostBuf<int> h_misc;
    // traceback
    DevBuf<uint32_t> d_tb_ops, d_tb_dir, d_tb_out;
    DevBuf<int2> d_tb_bnd;
    DevBuf<int64_t> d_tb_off;    // slot, direction, boundary and output offsets: 4n + 1
    DevBuf<int32_t> d_tb_count;  // operations and path score per pair: 2n
    HostBuf<int64_t> h_tb_off;
    HostBuf<int32_t> h_tb_count;
    HostBuf<uint32_t> h_tb_ops;

    cudaEvent_t ev[EV_COUNT] = {};
    cudaEvent_t ev_cls[2][gbsw::kRanges][2] = {};  // tuning: around each range launch of each pass
    bool timed_host = false;
    gbsw_stats stats{};
    gbsw_tuning tuning = gbsw::builtin_tuning();  // per (kind, length bin, pair-count bucket) plans

    int fail(int code, const std::string& msg) {
        last_error = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        last_error = std::string(what) + ": " + cudaGetErrorString(e);
        return GBSW_ECUDA;
    }
};

namespace {

int check_scoring(gbsw_context* ctx, const gbsw_scoring* sc) {
    if (!sc) return ctx->fail(GBSW_EINVAL, "scoring is NULL");
    if (sc->kind != GBSW_DNA && sc->kind != GBSW_PROTEIN)
        return ctx->fail(GBSW_EINVAL, "scoring.kind must be GBSW_DNA or GBSW_PROTEIN");
    if (sc->gap_open > 0 || sc->gap_extend > 0)
        return ctx->fail(GBSW_EINVAL, "gap_open and gap_extend must be <= 0");
    if (sc->kind == GBSW_PROTEIN && !sc->matrix)
        return ctx->fail(GBSW_EINVAL, "protein scoring needs a 576-entry matrix");
    return GBSW_OK;
}

// Upload the protein matrix (padded to 25x25 with a large negative row/column
// for padding columns) and the encoding table.
int upload_protein_tables(gbsw_context* ctx, const gbsw_scoring* sc, cudaStream_t stream) {
    cudaError_t e = ctx->d_matrix.reserve(gbsw::kAADim * gbsw::kAADim);
    if (e == cudaSuccess) e = ctx->d_encoding.reserve(91);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMalloc(protein tables)");
    e = ctx->h_misc.reserve(16 + gbsw::kAADim * gbsw::kAADim + 91);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMallocHost");
    int* hm = ctx->h_misc.ptr + 16;
    int* he = hm + gbsw::kAADim * gbsw::kAADim;
    for (int r = 0; r < gbsw::kAADim; ++r)
        for (int c = 0; c < gbsw::kAADim; ++c)
            hm[r * gbsw::kAADim + c] = (r < 24 && c < 24)
                                           ? (int)sc->matrix[r * 24 + c]
                                           : gbsw::kNegBig;
    for (int k = 0; k < 91; ++k) he[k] = 0;
    for (int k = 0; kAAOrder[k]; ++k) he[(int)kAAOrder[k]] = k;
    e = cudaMemcpyAsync(ctx->d_matrix.ptr, hm, sizeof(int) * gbsw::kAADim * gbsw::kAADim,
                        cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_encoding.ptr, he, sizeof(int) * 91, cudaMemcpyHostToDevice,
                            stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMemcpyAsync(protein tables)");
    // the host copies above read pinned staging that the next call may rewrite
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaStreamSynchronize");
    return GBSW_OK;
}

// Scoring mode of a class of pairs (see sw_common.cuh).
int score_mode(const gbsw_scoring* sc, int cls, bool dna_profile_ok, bool aa_profile_ok) {
    if (sc->kind == GBSW_PROTEIN) return aa_profile_ok ? gbsw::kScoreAaProfile : gbsw::kScoreAaWide;
    return (cls == 0 && dna_profile_ok) ? gbsw::kScoreDnaProfile : gbsw::kScoreDnaRaw;
}

bool fits_int8(int v) { return v >= -127 && v <= 127; }

// Lanes per pair when the caller leaves it to the library and no tuning entry
// applies (the fallback rule).  A batch finishes when its longest pair does
// unless there is enough work to keep every group busy until then, so small
// batches spread each pair over more lanes.  The thresholds are measured on
// GB300 (forward + reverse time of each width on the synthetic workloads, 3,000
// to 200,000 pairs; `lanes` = one wave of 4 resident 128-thread blocks per SM):
// * DNA: one pair per 32-lane group up to about 10,000 pairs; above that two
//   pairs per group (the dual-pair kernel) in the narrowest group that still
//   gets 2.5 two-pair units, i.e. pairs x lanes >= 5 x `lanes`: 4 lanes from
//   ~97,000 pairs, 8 from ~49,000, else 16.  On the DNA throughput shapes at
//   25,000 pairs: 2.57 ms at 16 lanes, 3.25 at 8, 5.38 at 4; at 50,000: 4.41 at
//   8, 5.75 at 4; at 100,000: 8.05 at 4 or 8, 8.59 at 16.
// * Protein (log-normal lengths up to 1,000): one pair per 32-lane group up to
//   about 10 waves of pairs, and two pairs per 16-lane group above (1.5x faster
//   than one pair at 60,000-120,000 pairs, slower below 24,000).
int auto_width(bool protein, int64_t n, int sms) {
    const int64_t lanes = (int64_t)sms * 4 * gbsw::pass_threads();
    if (protein) return n * 32 <= 10 * lanes ? 32 : 16;
    if (n * 64 <= 8 * lanes) return 32;
    for (int w : {gbsw::kG, 8})
        if (n * w >= 5 * lanes) return w;
    return 16;
}

// Pair-count buckets of the tuning table: (T[k-1], T[k]] pairs in a bin.
constexpr int64_t kBucketEdges[GBSW_COUNT_BUCKETS - 1] = {1000, 3000, 10000, 30000, 100000};
int count_bucket(int64_t pairs) {
    int k = 0;
    while (k < GBSW_COUNT_BUCKETS - 1 && pairs > kBucketEdges[k]) ++k;
    return k;
}

bool variant_ok(bool protein, const gbsw_variant& v, bool dual_ok) {
    if (v.lanes <= 0) return false;
    if (v.dual) return dual_ok && gbsw::has_dual(protein, v.lanes);
    return gbsw::pass_columns(v.lanes) != 0;
}

// What one call launches: the int32 width of classes 0 and 1 (and of the
// int16 overflow reruns) and the plan of each length bin in each pass.
struct Plan {
    int int32_lanes = gbsw::kG;
    gbsw_variant bin[2][gbsw::kBins] = {{{0, gbsw::kG}, {0, gbsw::kG}}, {{0, gbsw::kG}, {0, gbsw::kG}}};  // [pass][bin]
    bool binned = false;  // eligible pairs go to the bin classes (else to class 0)
    bool from_table[gbsw::kBins] = {false, false};
    bool any_dual(int rev) const { return binned && (bin[rev][0].dual || bin[rev][1].dual); }
    bool merged(int rev) const {
        return bin[rev][0].dual == bin[rev][1].dual && bin[rev][0].lanes == bin[rev][1].lanes;
    }
};

// The fallback plan: one width from the batch size (auto_width) or the
// caller's lane_group, the int16x2 kernels where they exist for it, and the
// long DNA bin in 16-lane dual groups when the short bin runs 4-lane ones.
Plan fallback_plan(bool protein, bool dpx, bool dual_ok, int forced, int64_t n, int sms) {
    Plan pl;
    int w = forced ? forced : auto_width(protein, n, sms);
    // protein: two pairs per group only pay on batches that fill the GPU (16
    // lanes); the 32-lane width of smaller batches runs one pair each
    const bool dual_wanted = forced || !protein || w == 16;
    if (!dpx) w = gbsw::kG;
    pl.int32_lanes = w;
    pl.binned = dpx && dual_ok;
    const gbsw_variant v{(dual_wanted && pl.binned && gbsw::has_dual(protein, w)) ? 1 : 0, w};
    for (auto& pass : pl.bin) {
        pass[0] = pass[1] = v;
        if (v.dual && !protein && w == gbsw::kG) pass[1] = gbsw_variant{1, gbsw::kDualWideLanes};
    }
    return pl;
}

int dual_or_pass_occupancy(gbsw_context* ctx, bool protein, int score, bool rev, bool dpx, const gbsw_variant& v,
                           int* blocks) {
    int b = ctx->opts.blocks_per_sm;
    if (b <= 0) {
        cudaError_t r = v.dual ? gbsw::pass_dual_occupancy(rev, protein, v.lanes, &b)
                               : gbsw::pass_occupancy(score, rev, dpx, v.lanes, &b);
        if (r != cudaSuccess) return ctx->cuda_fail(r, "occupancy");
    }
    *blocks = ctx->sms * std::max(1, b);
    return GBSW_OK;
}

// Enqueue the schedule and both passes for n pairs already on the device.
// `tune` (gbsw_tune_device) forces every bin to one variant and times each
// class launch with events; the result arrays are those of a normal call.
int run_passes(gbsw_context* ctx, const gbsw_scoring* sc, const uint8_t* ref, const int64_t* ref_off,
               const uint8_t* query, const int64_t* query_off, int64_t n, int max_len,
               int32_t* score, int32_t* ref_begin, int32_t* ref_end, int32_t* query_begin,
               int32_t* query_end, cudaStream_t stream, const gbsw_variant* tune = nullptr,
               const int64_t* host_bins = nullptr) {
    const bool protein = sc->kind == GBSW_PROTEIN;
    const bool dpx = ctx->opts.use_dpx != 0;
    const bool dna_profile_ok = !protein && fits_int8(sc->match) && fits_int8(sc->mismatch);
    bool aa_profile_ok = protein;
    if (protein)
        for (int k = 0; k < 576; ++k) aa_profile_ok = aa_profile_ok && fits_int8(sc->matrix[k]);
    const int nclasses = protein ? 1 : 2;
    // the int16x2 kernels: int8 profile scores and gap values in [-16384, 0]; a
    // pair whose score may have overflowed int16 is rerun in int32 (sw_dual.cu)
    const bool dual_ok = dpx && (protein ? aa_profile_ok : dna_profile_ok) && sc->gap_open >= -16384 &&
                         sc->gap_extend >= -16384 && sc->gap_open <= 0 && sc->gap_extend <= 0;
    // largest score of one aligned column: bounds every local score by it x min length
    int match_pos = std::max(0, std::max((int)sc->match, protein ? 0 : (int)sc->mismatch));
    if (protein)
        for (int k = 0; k < 576; ++k) match_pos = std::max(match_pos, (int)sc->matrix[k]);

    Plan plan = fallback_plan(protein, dpx, dual_ok, ctx->opts.lane_group, n, ctx->sms);
    if (tune) {
        for (auto& pass : plan.bin) pass[0] = pass[1] = *tune;
        plan.binned = dpx && dual_ok;
    }
    // a tuned plan per bin needs the bins' pair counts, read back after the
    // forward schedule (one small copy and a wait on the stream)
    const gbsw_tuning& table = ctx->tuning;
    bool use_table = false;
    if (!tune && ctx->opts.lane_group == 0 && dpx && plan.binned)
        for (int b = 0; b < gbsw::kBins; ++b)
            for (int k = 0; k < GBSW_COUNT_BUCKETS; ++k) use_table = use_table || table.variant[sc->kind][b][k].lanes > 0;

    cudaError_t e = ctx->d_misc.reserve(32);
    if (e == cudaSuccess) e = ctx->d_rerun.reserve((size_t)n + 2);
    if (e == cudaSuccess) e = ctx->d_cls.reserve((size_t)n);
    if (e == cudaSuccess) e = ctx->d_keys.reserve((size_t)n);
    if (e == cudaSuccess) e = ctx->d_order.reserve((size_t)n);
    if (e == cudaSuccess) e = ctx->d_hist.reserve((size_t)gbsw::kBuckets + 2 * gbsw::kRanges);
    if (e == cudaSuccess) e = ctx->h_misc.reserve(64);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    if (protein) {
        int rc = upload_protein_tables(ctx, sc, stream);
        if (rc != GBSW_OK) return rc;
    }
    e = cudaMemsetAsync(ctx->d_misc.ptr, 0, sizeof(int) * 32, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_rerun.ptr, 0, sizeof(int) * 2, stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMemsetAsync");

    gbsw::SchedParams sp{};
    sp.ref = ref;
    sp.ref_off = ref_off;
    sp.query = query;
    sp.query_off = query_off;
    sp.n = n;
    sp.protein = protein ? 1 : 0;
    sp.dna_profile_ok = dna_profile_ok ? 1 : 0;
    sp.binned = plan.binned ? 1 : 0;
    // reverse column bound (reverse_columns): DNA with every penalty negative
    const int rev_p = (!protein && sc->mismatch < 0 && sc->gap_open < 0 && sc->gap_extend < 0)
                          ? std::min({-(int)sc->mismatch, -(int)sc->gap_open, -(int)sc->gap_extend})
                          : 0;
    sp.match = sc->match;
    sp.rev_p = rev_p;
    sp.dual_limit = 32767 - match_pos;
    sp.score = score;
    sp.ref_end = ref_end;
    sp.query_end = query_end;
    sp.cls = ctx->d_cls.ptr;
    sp.keys = ctx->d_keys.ptr;
    sp.hist = ctx->d_hist.ptr;
    sp.class_range = ctx->d_hist.ptr + gbsw::kBuckets;
    sp.order = ctx->d_order.ptr;
    sp.error = ctx->d_misc.ptr + 3;

    cudaEventRecord(ctx->ev[EV_H2D], stream);
    e = gbsw::build_schedule(sp, false, ctx->sms, stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "schedule");
    int launches = 3;
    ctx->stats.bin_pairs[0] = ctx->stats.bin_pairs[1] = -1;
    // pairs of each range of the forward schedule, when read back (else -1:
    // unknown, launch anyway)
    int64_t range_pairs[gbsw::kRanges];
    for (int64_t& c : range_pairs) c = -1;
    // (reading the counts back also tells which ranges are empty: skipping
    // their launches saves more than the copy's wait costs, even on batches
    // whose plan the counts cannot change -- 1,000 pairs: 0.235 against 0.253 ms).
    // A caller that knows the bins' counts on the host (the serving loop) skips
    // the wait: the plan comes from its counts, a bin it counts empty is empty on
    // the device too, and the other ranges launch whatever they hold.
    if (host_bins && use_table && !tune) {
        for (int b = 0; b < gbsw::kBins; ++b) {
            const int64_t count = std::max<int64_t>(0, host_bins[b]);
            range_pairs[b ? gbsw::kRangeLong : gbsw::kRangeShort] = count;
            ctx->stats.bin_pairs[b] = count;
            const gbsw_variant& v = table.variant[sc->kind][b][count_bucket(count)];
            if (count > 0 && variant_ok(protein, v, dual_ok)) {
                plan.bin[0][b] = plan.bin[1][b] = v;
                const gbsw_variant& rv = table.reverse[sc->kind][b][count_bucket(count)];
                if (variant_ok(protein, rv, dual_ok)) plan.bin[1][b] = rv;
                plan.from_table[b] = true;
            }
        }
    } else if (use_table || tune) {
        int* hr = ctx->h_misc.ptr + 32;
        e = cudaMemcpyAsync(hr, sp.class_range, sizeof(int) * 2 * gbsw::kRanges, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "bin counts");
        for (int r = 0; r < gbsw::kRanges; ++r) range_pairs[r] = hr[2 * r + 1] - hr[2 * r];
        for (int b = 0; b < gbsw::kBins; ++b) {
            const int r = b ? gbsw::kRangeLong : gbsw::kRangeShort;
            const int64_t count = hr[2 * r + 1] - hr[2 * r];
            ctx->stats.bin_pairs[b] = count;
            const gbsw_variant& v = table.variant[sc->kind][b][count_bucket(count)];
            if (use_table && count > 0 && variant_ok(protein, v, dual_ok)) {
                plan.bin[0][b] = plan.bin[1][b] = v;
                const gbsw_variant& rv = table.reverse[sc->kind][b][count_bucket(count)];
                if (variant_ok(protein, rv, dual_ok)) plan.bin[1][b] = rv;
                plan.from_table[b] = true;
            }
        }
    }

    // the bins share one launch over their whole class when their plans agree
    // (the tuner times them apart)
    auto merged = [&](int rev) { return !tune && plan.merged(rev); };
    // persistent grids: each launch fills the SMs to its variant's occupancy
    // (gbsw_options.blocks_per_sm > 0 overrides); the boundary scratch holds one
    // buffer per group of the largest launch
    int grid[2][gbsw::kRanges] = {};
    int64_t groups = 0;
    for (int rev = 0; rev < 2; ++rev) {
        for (int cls = 0; cls < nclasses; ++cls) {
            int rc = dual_or_pass_occupancy(ctx, protein, score_mode(sc, cls, dna_profile_ok, aa_profile_ok), rev != 0,
                                            dpx, gbsw_variant{0, plan.int32_lanes}, &grid[rev][cls]);
            if (rc != GBSW_OK) return rc;
            groups = std::max(groups, (int64_t)grid[rev][cls] * gbsw::pass_groups_per_block(plan.int32_lanes));
        }
        if (plan.binned) {
            for (int b = 0; b < gbsw::kBins; ++b) {
                const int cls = b ? gbsw::kRangeLong : gbsw::kRangeShort;
                const gbsw_variant& v = plan.bin[rev][b];
                int rc = dual_or_pass_occupancy(ctx, protein, score_mode(sc, 0, dna_profile_ok, aa_profile_ok),
                                                rev != 0, dpx, v, &grid[rev][cls]);
                if (rc != GBSW_OK) return rc;
                const int lanes = v.dual ? gbsw::dual_lanes(protein, v.lanes) : v.lanes;
                groups = std::max(groups, (int64_t)grid[rev][cls] * gbsw::pass_groups_per_block(lanes));
            }
            grid[rev][gbsw::kClassBinned] = grid[rev][gbsw::kRangeShort];
        }
    }
    const int rows = (std::max(1, max_len) + 1) & ~1;  // even: 16-byte boundary copies stay in a group's buffer
    e = ctx->d_scratch.reserve((size_t)groups * (size_t)rows);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));

    gbsw::PassParams p{};
    p.ref = ref;
    p.ref_off = ref_off;
    p.query = query;
    p.query_off = query_off;
    p.n = n;
    p.open = sc->gap_open;
    p.ext = sc->gap_extend;
    p.match = sc->match;
    p.mismatch = sc->mismatch;
    p.aa_matrix = ctx->d_matrix.ptr;
    p.aa_encoding = ctx->d_encoding.ptr;
    p.score = score;
    p.ref_begin = ref_begin;
    p.ref_end = ref_end;
    p.query_begin = query_begin;
    p.query_end = query_end;
    p.order = sp.order;
    p.class_range = sp.class_range;
    p.scratch = ctx->d_scratch.ptr;
    p.scratch_rows = rows;
    p.error = ctx->d_misc.ptr + 3;
    p.rev_p = rev_p;
    // the dual-pair passes stay exact while every H is at most 32767 - match_pos
    // (sw_dual.cu); a pair whose best exceeds it is rerun in int32
    p.dual_limit = 32767 - match_pos;
    p.rerun = ctx->d_rerun.ptr;
    p.pair_cls = ctx->d_cls.ptr;

    // class launches, each bracketed by events when tuning
    auto timed = [&](int rev, int cls, auto&& launch) -> cudaError_t {
        if (tune) cudaEventRecord(ctx->ev_cls[rev][cls][0], stream);
        cudaError_t r = launch();
        if (tune) cudaEventRecord(ctx->ev_cls[rev][cls][1], stream);
        return r;
    };
    // dual forward launches may queue int32 reruns; a dual reverse launch
    // takes no pair whose score may exceed int16 (reverse_keys sends those to
    // class 0)
    const bool any_dual = plan.any_dual(0) || plan.any_dual(1);
    // A range known to be empty needs no launch.  A pair keeps its forward
    // range in the reverse pass, except pairs with no score (to the idle class)
    // and dual-pair pairs rerun in int32 (to class 0), so class 0's reverse
    // launch stays whenever a dual launch could have queued reruns.
    auto empty = [&](int rev, int range) {
        if (range_pairs[range] != 0) return false;
        return !(rev && range == 0 && any_dual);
    };
    for (int rev = 0; rev < 2; ++rev) {
        if (rev) {
            sp.rev_dual_bins = plan.binned ? (plan.bin[1][0].dual ? 1 : 0) | (plan.bin[1][1].dual ? 2 : 0) : 0;
            e = gbsw::build_schedule(sp, true, ctx->sms, stream);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "schedule");
            launches += 3;
        }
        auto queue = [&](int cls) { return ctx->d_misc.ptr + (rev ? 16 : 8) + cls; };
        if (plan.binned) {
            // the long bin first: its units are the heaviest work; one launch over
            // the whole class (long bin first in its order) when the plans agree
            for (int b = gbsw::kBins - 1; b >= 0; --b) {
                if (merged(rev) && b == 1) continue;
                const int cls = merged(rev) ? gbsw::kClassBinned : (b ? gbsw::kRangeLong : gbsw::kRangeShort);
                if (empty(rev, cls)) {
                    if (tune) timed(rev, cls, [] { return cudaSuccess; });  // 0 ms for the report
                    continue;
                }
                const gbsw_variant& v = plan.bin[rev][b];
                p.cls = cls;
                p.queue = queue(cls);
                e = timed(rev, cls, [&] {
                    return v.dual ? gbsw::launch_pass_dual(rev != 0, protein, v.lanes, p, grid[rev][cls], stream)
                                  : gbsw::launch_pass(score_mode(sc, 0, dna_profile_ok, aa_profile_ok), rev != 0, dpx,
                                                      v.lanes, p, grid[rev][cls], stream);
                });
                if (e != cudaSuccess) return ctx->cuda_fail(e, rev ? "reverse pass launch" : "forward pass launch");
                ++launches;
            }
        }
        for (int cls = 0; cls < nclasses; ++cls) {
            if (empty(rev, cls)) continue;
            p.cls = cls;
            p.queue = queue(cls);
            e = gbsw::launch_pass(score_mode(sc, cls, dna_profile_ok, aa_profile_ok), rev != 0, dpx, plan.int32_lanes,
                                  p, grid[rev][cls], stream);
            if (e != cudaSuccess) return ctx->cuda_fail(e, rev ? "reverse pass launch" : "forward pass launch");
            ++launches;
        }
        if (plan.any_dual(0) && !rev) {
            // the dual-pair pairs that may have overflowed int16, in the int32
            // class-0 kernel: its work list is the rerun list the dual launches
            // above filled (class range [rerun[0], rerun[1]) = [0, count))
            gbsw::PassParams pr = p;
            pr.cls = 0;
            pr.class_range = ctx->d_rerun.ptr;
            pr.order = ctx->d_rerun.ptr + 2;
            pr.queue = ctx->d_misc.ptr + 24;
            e = gbsw::launch_pass(score_mode(sc, 0, dna_profile_ok, aa_profile_ok), false, dpx, plan.int32_lanes, pr,
                                  grid[0][0], stream);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "int32 rerun launch");
            ++launches;
        }
        cudaEventRecord(ctx->ev[rev ? EV_REV : EV_FWD], stream);
    }
    ctx->stats.launches = launches;
    ctx->stats.lane_group = plan.binned ? plan.bin[0][0].lanes : plan.int32_lanes;
    ctx->stats.dual = any_dual ? 1 : 0;
    ctx->stats.reruns = plan.any_dual(0) ? -1 : 0;  // read back on demand (gbsw_last_stats)
    for (int b = 0; b < gbsw::kBins; ++b) {
        ctx->stats.bin_dual[b] = plan.binned ? plan.bin[0][b].dual : 0;
        ctx->stats.bin_lanes[b] = plan.binned ? plan.bin[0][b].lanes : plan.int32_lanes;
        ctx->stats.rev_dual[b] = plan.binned ? plan.bin[1][b].dual : 0;
        ctx->stats.rev_lanes[b] = plan.binned ? plan.bin[1][b].lanes : plan.int32_lanes;
        ctx->stats.bin_tuned[b] = plan.from_table[b] ? 1 : 0;
    }
    return GBSW_OK;
}

// Five result arrays -> rows of five (the serving loop's per-job layout).
__global__ void rows_of(const int32_t* soa, int64_t n, int32_t* rows) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int f = 0; f < 5; ++f) rows[5 * k + f] = soa[(int64_t)f * n + k];
}

// int32 results -> the narrower result type of the int16 host entry (keeps the
// low 16 bits, as the reference's short arrays do).
template <typename T>
__global__ void narrow_results(const int32_t* in, T* out, int64_t count) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (T)in[k];
}

int validate_offsets(gbsw_context* ctx, const int64_t* off, int64_t n, const char* what,
                     int* max_len, int64_t* lengths_out) {
    if (off[0] != 0) return ctx->fail(GBSW_EINVAL, std::string(what) + " offsets must start at 0");
    for (int64_t k = 0; k < n; ++k) {
        int64_t len = off[k + 1] - off[k];
        if (len < 0) return ctx->fail(GBSW_EINVAL, std::string(what) + " offsets must not decrease");
        if (len > GBSW_MAX_SEQ_LEN)
            return ctx->fail(GBSW_ELENGTH, std::string(what) + " sequence longer than 65535");
        if (len > *max_len) *max_len = (int)len;
        if (lengths_out) lengths_out[k] = len;
    }
    return GBSW_OK;
}

// Both offset arrays and the cell count in one pass over the pairs; on a bad
// entry the arrays are checked one after the other, which reports the same
// error as validate_offsets on each.
int validate_pairs(gbsw_context* ctx, const int64_t* ref_off, const int64_t* query_off, int64_t n,
                   int* max_len, int64_t* cells) {
    // branch-free (it vectorises): a negative length wraps above the limit as
    // an unsigned value, so the largest length alone tells whether all are valid
    uint64_t longest = 0, total = 0;
    for (int64_t k = 0; k < n; ++k) {
        const uint64_t a = (uint64_t)(ref_off[k + 1] - ref_off[k]), b = (uint64_t)(query_off[k + 1] - query_off[k]);
        longest = std::max(longest, std::max(a, b));
        total += a * b;
    }
    const bool ok = ref_off[0] == 0 && query_off[0] == 0 && longest <= (uint64_t)GBSW_MAX_SEQ_LEN;
    if (!ok) {
        int rc = validate_offsets(ctx, ref_off, n, "reference", max_len, nullptr);
        if (rc == GBSW_OK) rc = validate_offsets(ctx, query_off, n, "query", max_len, nullptr);
        return rc != GBSW_OK ? rc : ctx->fail(GBSW_EINTERNAL, "offset check");
    }
    *max_len = std::max(*max_len, (int)longest);
    *cells = (int64_t)total;
    return GBSW_OK;
}

int decode_device_error(gbsw_context* ctx, int flags) {
    if (flags & 1)
        return ctx->fail(GBSW_ESYMBOL, "protein symbol outside the 91-entry encoding table");
    if (flags & 2) return ctx->fail(GBSW_EINTERNAL, "reverse pass did not reach the forward score");
    if (flags & 4) return ctx->fail(GBSW_ELENGTH, "a sequence is longer than max_len, or ends are out of range");
    if (flags & gbsw::kErrTeam)
        return ctx->fail(GBSW_EINTERNAL, "a block-per-pair team waited too long for a strip edge");
    if (flags & gbsw::kErrTrace)
        return ctx->fail(GBSW_EINVAL, "traceback: a path does not reach its pair's score (results from other inputs "
                                      "or another scoring)");
    return GBSW_OK;
}

// Device bytes of direction words plus strip boundaries one traceback launch
// may hold; larger batches run in several launches.
constexpr int64_t kTraceBudget = int64_t(1) << 30;

int traceback_host(gbsw_context* ctx, const gbsw_scoring* sc, const char* ref, const int64_t* ref_off,
                   const char* query, const int64_t* query_off, int64_t n, const int32_t* top_scores,
                   const int32_t* ref_begin, const int32_t* ref_end, const int32_t* query_begin,
                   const int32_t* query_end, int64_t* ops_off, const uint32_t** ops) {
    if (!ctx) return GBSW_EINVAL;
    int rc = check_scoring(ctx, sc);
    if (rc != GBSW_OK) return rc;
    if (n < 0 || !ops_off || !ops) return ctx->fail(GBSW_EINVAL, "negative pair count or NULL output");
    ops_off[0] = 0;
    *ops = nullptr;
    if (n == 0) return GBSW_OK;
    if (!ref || !ref_off || !query || !query_off || !top_scores || !ref_begin || !ref_end || !query_begin ||
        !query_end)
        return ctx->fail(GBSW_EINVAL, "NULL buffer");
    if (n > (int64_t)0x7fffffff) return ctx->fail(GBSW_EINVAL, "too many pairs for one call");
    int max_len = 0;
    rc = validate_offsets(ctx, ref_off, n, "reference", &max_len, nullptr);
    if (rc == GBSW_OK) rc = validate_offsets(ctx, query_off, n, "query", &max_len, nullptr);
    if (rc != GBSW_OK) return rc;

    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    // per pair: operation slot (m + k), direction words and boundary entries of
    // its launch; launches cut where the budget fills
    e = ctx->h_tb_off.reserve((size_t)5 * n + 1);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, "cudaMallocHost");
    int64_t* slot = ctx->h_tb_off.ptr;       // n + 1
    int64_t* dir_off = slot + n + 1;         // n
    int64_t* bnd_off = dir_off + n;          // n
    int64_t* order = slot + 4 * n + 1;       // n: each launch's pairs by descending cost
    std::vector<int64_t> cuts{0};
    int64_t dir_max = 1, bnd_max = 1, dir_run = 0, bnd_run = 0;
    slot[0] = 0;
    for (int64_t k = 0; k < n; ++k) {
        int64_t cap = 0, dw = 0, bw = 0;
        if (top_scores[k] > 0) {
            const int64_t a = ref_off[k + 1] - ref_off[k], b = query_off[k + 1] - query_off[k];
            if (ref_begin[k] < 0 || ref_begin[k] >= ref_end[k] || ref_end[k] > a || query_begin[k] < 0 ||
                query_begin[k] >= query_end[k] || query_end[k] > b)
                return ctx->fail(GBSW_EINVAL, "traceback: begins/ends out of range for pair " + std::to_string(k));
            const int m = ref_end[k] - ref_begin[k], kk = query_end[k] - query_begin[k];
            cap = (int64_t)m + kk;
            dw = gbsw::trace_dir_words(m, kk);
            bw = (int64_t)kk + 1;
        }
        if (k > cuts.back() && (dir_run + dw) * 4 + (bnd_run + bw) * 8 > kTraceBudget) {
            cuts.push_back(k);
            dir_run = bnd_run = 0;
        }
        dir_off[k] = dir_run;
        bnd_off[k] = bnd_run;
        dir_run += dw;
        bnd_run += bw;
        dir_max = std::max(dir_max, dir_run);
        bnd_max = std::max(bnd_max, bnd_run);
        slot[k + 1] = slot[k] + cap;
    }
    cuts.push_back(n);
    // Each launch's pairs by descending row steps (strips x (rows + fill)), so
    // that the pairs a warp's groups run together end close together: a
    // counting sort over 8 buckets per doubling of the cost (the exponent and
    // the next three bits of the integer cost).
    {
        constexpr int kCostBuckets = 8 * 64;
        std::vector<uint16_t> bucket((size_t)n);
        for (int64_t k = 0; k < n; ++k) {
            int b = 0;
            if (top_scores[k] > 0) {
                const int m = ref_end[k] - ref_begin[k], kk = query_end[k] - query_begin[k];
                const uint64_t cost = (uint64_t)((m + gbsw::kTraceCols - 1) / gbsw::kTraceCols) *
                                      (uint64_t)(kk + gbsw::kTraceLanes - 1);
                const int e = 63 - __builtin_clzll(cost | 1);
                const int frac = e >= 3 ? (int)((cost >> (e - 3)) & 7) : (int)((cost << (3 - e)) & 7);
                b = std::min(kCostBuckets - 1, 1 + 8 * e + frac);
            }
            bucket[(size_t)k] = (uint16_t)(kCostBuckets - 1 - b);  // descending cost first
        }
        std::vector<int64_t> count(kCostBuckets);
        for (size_t c = 0; c + 1 < cuts.size(); ++c) {
            std::fill(count.begin(), count.end(), 0);
            for (int64_t k = cuts[c]; k < cuts[c + 1]; ++k) ++count[bucket[(size_t)k]];
            int64_t at = cuts[c];
            for (int b = 0; b < kCostBuckets; ++b) {
                const int64_t here = count[b];
                count[b] = at;
                at += here;
            }
            for (int64_t k = cuts[c]; k < cuts[c + 1]; ++k) order[count[bucket[(size_t)k]]++] = k;
        }
    }
    const int64_t ra = ref_off[n], qa = query_off[n];
    cudaStream_t stream = ctx->stream;
    e = ctx->d_ref.reserve((size_t)std::max<int64_t>(ra, 1));
    if (e == cudaSuccess) e = ctx->d_query.reserve((size_t)std::max<int64_t>(qa, 1));
    if (e == cudaSuccess) e = ctx->d_ref_off.reserve((size_t)n + 1);
    if (e == cudaSuccess) e = ctx->d_query_off.reserve((size_t)n + 1);
    if (e == cudaSuccess) e = ctx->d_results.reserve((size_t)n * 5);
    if (e == cudaSuccess) e = ctx->d_tb_ops.reserve((size_t)std::max<int64_t>(slot[n], 1));
    if (e == cudaSuccess) e = ctx->d_tb_out.reserve((size_t)std::max<int64_t>(slot[n], 1));
    if (e == cudaSuccess) e = ctx->d_tb_dir.reserve((size_t)dir_max);
    if (e == cudaSuccess) e = ctx->d_tb_bnd.reserve((size_t)bnd_max);
    if (e == cudaSuccess) e = ctx->d_tb_off.reserve((size_t)5 * n + 1);
    if (e == cudaSuccess) e = ctx->d_tb_count.reserve((size_t)2 * n);
    if (e == cudaSuccess) e = ctx->d_misc.reserve(8);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = ctx->h_tb_count.reserve((size_t)n);
    if (e == cudaSuccess) e = ctx->h_misc.reserve(16);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, "cudaMallocHost");
    if (sc->kind == GBSW_PROTEIN) {
        rc = upload_protein_tables(ctx, sc, stream);
        if (rc != GBSW_OK) return rc;
    }
    int32_t* R = ctx->d_results.ptr;
    const int32_t* res_host[5] = {top_scores, ref_begin, ref_end, query_begin, query_end};
    // phases for gbsw_last_stats: copies in (h2d_ms), the traceback kernels
    // (forward_ms), the operations back (d2h_ms)
    ctx->stats = gbsw_stats{};
    ctx->stats.launches = (int32_t)cuts.size() + 1;
    cudaEventRecord(ctx->ev[EV_START], stream);
    if (ra > 0) e = cudaMemcpyAsync(ctx->d_ref.ptr, ref, (size_t)ra, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && qa > 0)
        e = cudaMemcpyAsync(ctx->d_query.ptr, query, (size_t)qa, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_ref_off.ptr, ref_off, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice,
                            stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_query_off.ptr, query_off, sizeof(int64_t) * (size_t)(n + 1),
                            cudaMemcpyHostToDevice, stream);
    for (int f = 0; f < 5 && e == cudaSuccess; ++f)
        e = cudaMemcpyAsync(R + (size_t)f * n, res_host[f], sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice,
                            stream);
    int64_t* d_off = ctx->d_tb_off.ptr;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, slot, sizeof(int64_t) * (size_t)(3 * n + 1), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off + 4 * n + 1, order, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_misc.ptr, 0, sizeof(int) * 8, stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "traceback copies");
    cudaEventRecord(ctx->ev[EV_H2D], stream);

    gbsw::TraceParams tp{};
    tp.ref = ctx->d_ref.ptr;
    tp.ref_off = ctx->d_ref_off.ptr;
    tp.query = ctx->d_query.ptr;
    tp.query_off = ctx->d_query_off.ptr;
    tp.score = R;
    tp.ref_begin = R + n;
    tp.ref_end = R + 2 * n;
    tp.query_begin = R + 3 * n;
    tp.query_end = R + 4 * n;
    tp.protein = sc->kind == GBSW_PROTEIN;
    tp.match = sc->match;
    tp.mismatch = sc->mismatch;
    tp.open = sc->gap_open;
    tp.ext = sc->gap_extend;
    tp.aa_matrix = ctx->d_matrix.ptr;
    tp.aa_encoding = ctx->d_encoding.ptr;
    tp.dir = ctx->d_tb_dir.ptr;
    tp.bnd = ctx->d_tb_bnd.ptr;
    tp.slot_off = d_off;
    tp.ops = ctx->d_tb_ops.ptr;
    tp.nops = ctx->d_tb_count.ptr;
    tp.path_score = ctx->d_tb_count.ptr + n;
    tp.error = ctx->d_misc.ptr + 3;
    for (size_t c = 0; c + 1 < cuts.size(); ++c) {
        tp.first = cuts[c];
        tp.count = cuts[c + 1] - cuts[c];
        // offsets are per launch; the kernel indexes them by pair within the launch
        tp.dir_off = d_off + (n + 1) + cuts[c];
        tp.bnd_off = d_off + (2 * n + 1) + cuts[c];
        tp.order = d_off + (4 * n + 1) + cuts[c];
        e = gbsw::launch_trace(tp, stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "traceback launch");
    }
    cudaEventRecord(ctx->ev[EV_FWD], stream);
    cudaEventRecord(ctx->ev[EV_REV], stream);
    e = cudaMemcpyAsync(ctx->h_tb_count.ptr, tp.nops, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_misc.ptr, ctx->d_misc.ptr + 3, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "traceback");
    rc = decode_device_error(ctx, ctx->h_misc.ptr[0]);
    if (rc != GBSW_OK) return rc;
    // compact the operations
    for (int64_t k = 0; k < n; ++k) ops_off[k + 1] = ops_off[k] + ctx->h_tb_count.ptr[k];
    const int64_t total = ops_off[n];
    e = ctx->h_tb_ops.reserve((size_t)std::max<int64_t>(total, 1));
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, "cudaMallocHost");
    int64_t* d_out_off = d_off + 3 * n + 1;  // n entries
    e = cudaMemcpyAsync(d_out_off, ops_off, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = gbsw::launch_gather_ops(ctx->d_tb_ops.ptr, d_off, tp.nops, d_out_off, ctx->d_tb_out.ptr, n, stream);
    if (e == cudaSuccess && total > 0)
        e = cudaMemcpyAsync(ctx->h_tb_ops.ptr, ctx->d_tb_out.ptr, sizeof(uint32_t) * (size_t)total,
                            cudaMemcpyDeviceToHost, stream);
    cudaEventRecord(ctx->ev[EV_D2H], stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "traceback results");
    ctx->timed_host = true;
    *ops = ctx->h_tb_ops.ptr;
    return GBSW_OK;
}

// The sequence bytes of a host-entry call: raw host buffers, or packed streams
// (gbsw_packed, host memory) that are unpacked on the device.
struct HostSeqs {
    const char* ref = nullptr;
    const char* query = nullptr;
    const gbsw_packed* pref = nullptr;
    const gbsw_packed* pquery = nullptr;
    bool packed() const { return pref != nullptr; }
};

// A packed host stream that covers `need` symbols: words present, escape runs
// increasing, disjoint and inside the stream.
int validate_packed(gbsw_context* ctx, const gbsw_packed* p, int64_t need, const char* what) {
    const std::string w(what);
    if (!p) return ctx->fail(GBSW_EINVAL, w + " stream is NULL");
    if (p->nsym < need) return ctx->fail(GBSW_EINVAL, w + " stream holds fewer symbols than its offsets reach");
    if (p->nsym > 0 && !p->words) return ctx->fail(GBSW_EINVAL, w + " stream has no words");
    if (p->nruns < 0) return ctx->fail(GBSW_EINVAL, w + " stream: negative run count");
    if (p->nruns == 0) return GBSW_OK;
    if (!p->run_at || !p->run_off || !p->run_bytes) return ctx->fail(GBSW_EINVAL, w + " stream: NULL run arrays");
    if (p->run_off[0] != 0) return ctx->fail(GBSW_EINVAL, w + " stream: run offsets must start at 0");
    int64_t end = 0;
    for (int64_t r = 0; r < p->nruns; ++r) {
        const int64_t len = p->run_off[r + 1] - p->run_off[r];
        if (len < 0 || p->run_at[r] < end || p->run_at[r] + len > p->nsym)
            return ctx->fail(GBSW_EINVAL, w + " stream: escape runs must be increasing, disjoint and inside it");
        end = p->run_at[r] + len;
    }
    return GBSW_OK;
}

// Enqueues the copies of one packed host stream into ctx->d_pack at byte
// `base` and its unpack into `out`; returns the bytes the stream took there.
cudaError_t upload_packed(gbsw_context* ctx, int kind, const gbsw_packed& p, size_t base, uint8_t* out,
                          cudaStream_t stream, size_t* used) {
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t wbytes = 4 * (size_t)gbsw_packed_words(kind, p.nsym);
    const size_t rbytes = 8 * (size_t)p.nruns, obytes = 8 * (size_t)(p.nruns + 1);
    const size_t bbytes = p.nruns > 0 ? (size_t)p.run_off[p.nruns] : 0;
    uint8_t* d = ctx->d_pack.ptr + base;
    gbsw_packed dp{};
    dp.words = reinterpret_cast<const uint32_t*>(d);
    dp.nsym = p.nsym;
    dp.nruns = p.nruns;
    dp.run_at = reinterpret_cast<const int64_t*>(d + up16(wbytes));
    dp.run_off = reinterpret_cast<const int64_t*>(d + up16(wbytes) + up16(rbytes));
    dp.run_bytes = d + up16(wbytes) + up16(rbytes) + up16(obytes);
    *used = up16(wbytes) + (p.nruns > 0 ? up16(rbytes) + up16(obytes) + up16(bbytes) : 0);
    cudaError_t e = cudaSuccess;
    if (wbytes) e = cudaMemcpyAsync((void*)dp.words, p.words, wbytes, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && p.nruns > 0) {
        e = cudaMemcpyAsync((void*)dp.run_at, p.run_at, rbytes, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync((void*)dp.run_off, p.run_off, obytes, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess && bbytes)
            e = cudaMemcpyAsync((void*)dp.run_bytes, p.run_bytes, bbytes, cudaMemcpyHostToDevice, stream);
    }
    if (e == cudaSuccess) e = gbsw::launch_unpack(kind, dp, out, stream);
    return e;
}

size_t packed_device_bytes(int kind, const gbsw_packed& p) {
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    size_t b = up16(4 * (size_t)gbsw_packed_words(kind, p.nsym));
    if (p.nruns > 0)
        b += up16(8 * (size_t)p.nruns) + up16(8 * (size_t)(p.nruns + 1)) + up16((size_t)p.run_off[p.nruns]);
    return b;
}

template <typename T>
int align_host(gbsw_context* ctx, const gbsw_scoring* sc, const HostSeqs& in, const int64_t* ref_off,
               const int64_t* query_off, int64_t n, T* ref_begin, T* ref_end, T* query_begin, T* query_end,
               T* top_scores) {
    if (!ctx) return GBSW_EINVAL;
    int rc = check_scoring(ctx, sc);
    if (rc != GBSW_OK) return rc;
    if (n < 0) return ctx->fail(GBSW_EINVAL, "negative pair count");
    if (n == 0) return GBSW_OK;
    const bool seqs_ok = in.packed() ? (in.pref && in.pquery) : (in.ref && in.query);
    if (!seqs_ok || !ref_off || !query_off || !ref_begin || !ref_end || !query_begin || !query_end || !top_scores)
        return ctx->fail(GBSW_EINVAL, "NULL buffer");
    if (n > (int64_t)0x7fffffff) return ctx->fail(GBSW_EINVAL, "too many pairs for one call");
    int max_len = 0;
    int64_t cells = 0;
    // Packed input: the copies and the unpack depend only on the streams, so
    // they are enqueued first and the pairs' offsets are checked on the host
    // while they run (the check of 100,000 pairs takes a few hundred
    // microseconds); a failed check waits for the copies before returning.
    const bool check_late = in.packed();
    if (!check_late) {
        rc = validate_pairs(ctx, ref_off, query_off, n, &max_len, &cells);
        if (rc != GBSW_OK) return rc;
    }
    int64_t ra = ref_off[n], qa = query_off[n];
    if (in.packed()) {
        rc = validate_packed(ctx, in.pref, ra, "reference");
        if (rc == GBSW_OK) rc = validate_packed(ctx, in.pquery, qa, "query");
        if (rc != GBSW_OK) return rc;
        ra = in.pref->nsym;  // the unpack writes whole streams
        qa = in.pquery->nsym;
    }

    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    cudaStream_t stream = ctx->stream;
    e = ctx->d_ref.reserve((size_t)std::max<int64_t>(ra, 1));
    if (e == cudaSuccess) e = ctx->d_query.reserve((size_t)std::max<int64_t>(qa, 1));
    if (e == cudaSuccess) e = ctx->d_ref_off.reserve((size_t)n + 1);
    if (e == cudaSuccess) e = ctx->d_query_off.reserve((size_t)n + 1);
    // int32 results, then (int16 form) their narrowed copy: 5n int32 + 5n int16
    if (e == cudaSuccess) e = ctx->d_results.reserve((size_t)n * 5 + (sizeof(T) < 4 ? ((size_t)n * 5 + 1) / 2 : 0));
    if (e == cudaSuccess && in.packed())
        e = ctx->d_pack.reserve(packed_device_bytes(sc->kind, *in.pref) + packed_device_bytes(sc->kind, *in.pquery));
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));

    cudaEventRecord(ctx->ev[EV_START], stream);
    if (in.packed()) {
        size_t used = 0, used_q = 0;
        e = upload_packed(ctx, sc->kind, *in.pref, 0, ctx->d_ref.ptr, stream, &used);
        if (e == cudaSuccess) e = upload_packed(ctx, sc->kind, *in.pquery, used, ctx->d_query.ptr, stream, &used_q);
        if (e == cudaSuccess) ctx->stats.launches += 2 + (in.pref->nruns > 0) + (in.pquery->nruns > 0);
    } else {
        if (ra > 0) e = cudaMemcpyAsync(ctx->d_ref.ptr, in.ref, (size_t)ra, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess && qa > 0)
            e = cudaMemcpyAsync(ctx->d_query.ptr, in.query, (size_t)qa, cudaMemcpyHostToDevice, stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_ref_off.ptr, ref_off, sizeof(int64_t) * (size_t)(n + 1),
                            cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_query_off.ptr, query_off, sizeof(int64_t) * (size_t)(n + 1),
                            cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMemcpyAsync H2D");
    if (check_late) {
        rc = validate_pairs(ctx, ref_off, query_off, n, &max_len, &cells);
        if (rc != GBSW_OK) {
            cudaStreamSynchronize(stream);  // the copies read the caller's buffers
            return rc;
        }
    }

    int32_t* R = ctx->d_results.ptr;
    rc = run_passes(ctx, sc, ctx->d_ref.ptr, ctx->d_ref_off.ptr, ctx->d_query.ptr,
                    ctx->d_query_off.ptr, n, max_len, R, R + n, R + 2 * n, R + 3 * n, R + 4 * n,
                    stream);
    if (rc != GBSW_OK) return rc;
    // results straight into the caller's five arrays (narrowed on the device first)
    const T* D = reinterpret_cast<const T*>(R);
    if (sizeof(T) < 4) {
        T* d16 = reinterpret_cast<T*>(R + (size_t)n * 5);
        const int blocks = (int)std::min<int64_t>((n * 5 + 255) / 256, (int64_t)ctx->sms * 16);
        narrow_results<T><<<blocks, 256, 0, stream>>>(R, d16, n * 5);
        e = cudaGetLastError();
        ++ctx->stats.launches;
        D = d16;
    }
    T* outs[5] = {top_scores, ref_begin, ref_end, query_begin, query_end};
    for (int f = 0; f < 5 && e == cudaSuccess; ++f)
        e = cudaMemcpyAsync(outs[f], D + (size_t)f * (size_t)n, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost,
                            stream);
    if (e == cudaSuccess) {
        e = ctx->h_misc.reserve(16);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->h_misc.ptr, ctx->d_misc.ptr + 3, sizeof(int),
                                cudaMemcpyDeviceToHost, stream);
    }
    cudaEventRecord(ctx->ev[EV_D2H], stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "alignment");
    rc = decode_device_error(ctx, ctx->h_misc.ptr[0]);
    if (rc != GBSW_OK) return rc;
    ctx->timed_host = true;
    ctx->stats.cells = cells;
    return GBSW_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.f;
    return ms;
}

}  // namespace

cudaError_t gbsw::results_rows(const int32_t* soa, int64_t n, int32_t* rows, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    rows_of<<<blocks, 256, 0, stream>>>(soa, n, rows);
    return cudaGetLastError();
}

extern "C" {

const char* gbsw_strerror(int status) {
    switch (status) {
        case GBSW_OK: return "ok";
        case GBSW_EINVAL: return "invalid argument";
        case GBSW_ESYMBOL: return "protein symbol outside the encoding table";
        case GBSW_ELENGTH: return "sequence too long";
        case GBSW_ECUDA: return "CUDA error";
        case GBSW_ENOMEM: return "out of memory";
        case GBSW_EINTERNAL: return "internal error";
        case GBSW_ETOOBIG: return "batch larger than the fixed scratch of the allocation-free entry";
        case GBSW_ETIMEOUT: return "job not finished within the timeout";
        default: return "unknown status";
    }
}

const char* gbsw_last_error(const gbsw_context* ctx) {
    return ctx ? ctx->last_error.c_str() : "no context";
}

int gbsw_create(int device, gbsw_context** out) {
    if (!out) return GBSW_EINVAL;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return GBSW_ECUDA;
    if (device < 0 || device >= count) return GBSW_EINVAL;
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return GBSW_ECUDA;
    gbsw_context* ctx = new (std::nothrow) gbsw_context();
    if (!ctx) return GBSW_ENOMEM;
    ctx->device = device;
    e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (int k = 0; e == cudaSuccess && k < EV_COUNT; ++k) e = cudaEventCreate(&ctx->ev[k]);
    for (int r = 0; e == cudaSuccess && r < 2; ++r)
        for (int c = 0; e == cudaSuccess && c < gbsw::kRanges; ++c)
            for (int k = 0; e == cudaSuccess && k < 2; ++k) e = cudaEventCreate(&ctx->ev_cls[r][c][k]);
    if (e != cudaSuccess) {
        gbsw_destroy(ctx);
        return GBSW_ECUDA;
    }
    *out = ctx;
    return GBSW_OK;
}

void gbsw_destroy(gbsw_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->d_ref.release();
    ctx->d_query.release();
    ctx->d_pack.release();
    ctx->d_ref_off.release();
    ctx->d_query_off.release();
    ctx->d_results.release();
    ctx->d_scratch.release();
    ctx->d_misc.release();
    ctx->d_rerun.release();
    ctx->d_matrix.release();
    ctx->d_encoding.release();
    ctx->d_cls.release();
    ctx->d_keys.release();
    ctx->d_order.release();
    ctx->d_hist.release();
    ctx->h_misc.release();
    ctx->d_tb_ops.release();
    ctx->d_tb_dir.release();
    ctx->d_tb_out.release();
    ctx->d_tb_bnd.release();
    ctx->d_tb_off.release();
    ctx->d_tb_count.release();
    ctx->h_tb_off.release();
    ctx->h_tb_count.release();
    ctx->h_tb_ops.release();
    for (int k = 0; k < EV_COUNT; ++k)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    for (auto& pass : ctx->ev_cls)
        for (auto& cls : pass)
            for (cudaEvent_t ev : cls)
                if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int gbsw_align_host16(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref,
                      const int64_t* ref_off, const char* query, const int64_t* query_off,
                      int64_t n, int16_t* ref_begin, int16_t* ref_end, int16_t* query_begin,
                      int16_t* query_end, int16_t* top_scores) {
    HostSeqs in;
    in.ref = ref;
    in.query = query;
    return align_host<int16_t>(ctx, scoring, in, ref_off, query_off, n, ref_begin, ref_end, query_begin, query_end,
                               top_scores);
}

int gbsw_align_host32(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref,
                      const int64_t* ref_off, const char* query, const int64_t* query_off,
                      int64_t n, int32_t* ref_begin, int32_t* ref_end, int32_t* query_begin,
                      int32_t* query_end, int32_t* top_scores) {
    HostSeqs in;
    in.ref = ref;
    in.query = query;
    return align_host<int32_t>(ctx, scoring, in, ref_off, query_off, n, ref_begin, ref_end, query_begin, query_end,
                               top_scores);
}

int gbsw_align_packed_host16(gbsw_context* ctx, const gbsw_scoring* scoring, const gbsw_packed* ref,
                             const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off,
                             int64_t n, int16_t* ref_begin, int16_t* ref_end, int16_t* query_begin,
                             int16_t* query_end, int16_t* top_scores) {
    HostSeqs in;
    in.pref = ref;
    in.pquery = query;
    return align_host<int16_t>(ctx, scoring, in, ref_off, query_off, n, ref_begin, ref_end, query_begin, query_end,
                               top_scores);
}

int gbsw_align_packed_host32(gbsw_context* ctx, const gbsw_scoring* scoring, const gbsw_packed* ref,
                             const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off,
                             int64_t n, int32_t* ref_begin, int32_t* ref_end, int32_t* query_begin,
                             int32_t* query_end, int32_t* top_scores) {
    HostSeqs in;
    in.pref = ref;
    in.pquery = query;
    return align_host<int32_t>(ctx, scoring, in, ref_off, query_off, n, ref_begin, ref_end, query_begin, query_end,
                               top_scores);
}

int gbsw_traceback_host(gbsw_context* ctx, const gbsw_scoring* scoring, const char* ref, const int64_t* ref_off,
                        const char* query, const int64_t* query_off, int64_t n, const int32_t* top_scores,
                        const int32_t* ref_begin, const int32_t* ref_end, const int32_t* query_begin,
                        const int32_t* query_end, int64_t* ops_off, const uint32_t** ops) {
    return traceback_host(ctx, scoring, ref, ref_off, query, query_off, n, top_scores, ref_begin, ref_end,
                          query_begin, query_end, ops_off, ops);
}

int gbsw_align_device(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref,
                      const int64_t* ref_off, const uint8_t* query, const int64_t* query_off,
                      int64_t n, int32_t max_len, int32_t* top_scores, int32_t* ref_begin,
                      int32_t* ref_end, int32_t* query_begin, int32_t* query_end, void* stream) {
    if (!ctx) return GBSW_EINVAL;
    int rc = check_scoring(ctx, scoring);
    if (rc != GBSW_OK) return rc;
    if (n < 0) return ctx->fail(GBSW_EINVAL, "negative pair count");
    if (n == 0) return GBSW_OK;
    if (n > (int64_t)0x7fffffff) return ctx->fail(GBSW_EINVAL, "too many pairs for one call");
    if (max_len < 0 || max_len > GBSW_MAX_SEQ_LEN)
        return ctx->fail(GBSW_ELENGTH, "max_len outside [0, 65535]");
    if (!ref || !ref_off || !query || !query_off || !top_scores || !ref_begin || !ref_end ||
        !query_begin || !query_end)
        return ctx->fail(GBSW_EINVAL, "NULL buffer");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;  // NULL is the CUDA default stream
    cudaEventRecord(ctx->ev[EV_START], s);
    ctx->timed_host = false;
    ctx->stats.cells = 0;
    return run_passes(ctx, scoring, ref, ref_off, query, query_off, n, max_len, top_scores,
                      ref_begin, ref_end, query_begin, query_end, s);
}

int gbsw_check(gbsw_context* ctx, void* stream) {
    if (!ctx) return GBSW_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = ctx->h_misc.reserve(16);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, "cudaMallocHost");
    if (!ctx->d_misc.ptr) return GBSW_OK;
    e = cudaMemcpyAsync(ctx->h_misc.ptr, ctx->d_misc.ptr + 3, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "gbsw_check");
    return decode_device_error(ctx, ctx->h_misc.ptr[0]);
}

int gbsw_device_memory(int device, uint64_t* bytes) {
    if (!bytes) return GBSW_EINVAL;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return GBSW_ECUDA;
    *bytes = (uint64_t)prop.totalGlobalMem;
    return GBSW_OK;
}

int gbsw_set_options(gbsw_context* ctx, const gbsw_options* opts) {
    if (!ctx || !opts) return GBSW_EINVAL;
    if (opts->blocks_per_sm < 0 || opts->blocks_per_sm > 64) return ctx->fail(GBSW_EINVAL, "blocks_per_sm");
    if (opts->lane_group != 0 && gbsw::pass_columns(opts->lane_group) == 0)
        return ctx->fail(GBSW_EINVAL, "lane_group must be 0, 4, 8, 16 or 32");
    ctx->opts = *opts;
    return GBSW_OK;
}

int gbsw_get_options(const gbsw_context* ctx, gbsw_options* opts) {
    if (!ctx || !opts) return GBSW_EINVAL;
    *opts = ctx->opts;
    return GBSW_OK;
}

int gbsw_get_tuning(const gbsw_context* ctx, gbsw_tuning* tuning) {
    if (!ctx || !tuning) return GBSW_EINVAL;
    *tuning = ctx->tuning;
    return GBSW_OK;
}

int gbsw_set_tuning(gbsw_context* ctx, const gbsw_tuning* tuning) {
    if (!ctx || !tuning) return GBSW_EINVAL;
    for (int pass = 0; pass < 2; ++pass)
        for (int kind = 0; kind < 2; ++kind)
            for (int b = 0; b < GBSW_BINS; ++b)
                for (int k = 0; k < GBSW_COUNT_BUCKETS; ++k) {
                    const gbsw_variant& v = pass ? tuning->reverse[kind][b][k] : tuning->variant[kind][b][k];
                    if (v.lanes == 0) continue;  // no entry
                    if (v.dual != 0 && v.dual != 1) return ctx->fail(GBSW_EINVAL, "tuning: dual must be 0 or 1");
                    if (v.dual ? !gbsw::has_dual(kind == GBSW_PROTEIN, v.lanes) : gbsw::pass_columns(v.lanes) == 0)
                        return ctx->fail(GBSW_EINVAL, "tuning: no kernel variant with these lanes");
                }
    ctx->tuning = *tuning;
    return GBSW_OK;
}

int gbsw_tune_device(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref, const int64_t* ref_off,
                     const uint8_t* query, const int64_t* query_off, int64_t n, int32_t max_len, int32_t reps,
                     void* stream, gbsw_tune_report* report) {
    if (!ctx) return GBSW_EINVAL;
    int rc = check_scoring(ctx, scoring);
    if (rc != GBSW_OK) return rc;
    if (!report || reps < 1 || reps > 100) return ctx->fail(GBSW_EINVAL, "report is NULL or reps outside [1, 100]");
    if (n < 1 || n > (int64_t)0x7fffffff) return ctx->fail(GBSW_EINVAL, "pair count outside [1, 2^31)");
    if (max_len < 0 || max_len > GBSW_MAX_SEQ_LEN) return ctx->fail(GBSW_ELENGTH, "max_len outside [0, 65535]");
    if (!ref || !ref_off || !query || !query_off) return ctx->fail(GBSW_EINVAL, "NULL buffer");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    e = ctx->d_results.reserve((size_t)n * 5);
    if (e != cudaSuccess) return ctx->fail(GBSW_ENOMEM, "cudaMalloc");
    const bool protein = scoring->kind == GBSW_PROTEIN;
    std::memset(report, 0, sizeof(*report));
    // the candidates: the int16x2 dual-pair variants, then one pair per group in int32
    std::vector<gbsw_variant> cand;
    for (int w : {4, 8, 16, 32})
        if (gbsw::has_dual(protein, w)) cand.push_back(gbsw_variant{1, w});
    for (int w : {4, 8, 16, 32, gbsw::kTeamLanes})
        if (gbsw::pass_columns(w) != 0) cand.push_back(gbsw_variant{0, w});
    cudaStream_t s = (cudaStream_t)stream;
    int32_t* R = ctx->d_results.ptr;
    double best[2][GBSW_BINS];  // [pass][bin]
    for (auto& pass : best)
        for (double& v : pass) v = 1e30;
    int nc = 0;
    for (const gbsw_variant& v : cand) {
        if (nc == GBSW_TUNE_CANDIDATES) break;
        double t[2][GBSW_BINS] = {{1e30, 1e30}, {1e30, 1e30}};
        bool ran = false;
        for (int r = 0; r <= reps; ++r) {  // run 0 warms the variant up
            rc = run_passes(ctx, scoring, ref, ref_off, query, query_off, n, max_len, R, R + n, R + 2 * n, R + 3 * n,
                            R + 4 * n, s, &v);
            if (rc != GBSW_OK) return rc;
            rc = gbsw_check(ctx, stream);
            if (rc != GBSW_OK) return rc;
            if (!ctx->stats.dual && v.dual) break;  // the scoring keeps these pairs out of the dual kernels
            ran = true;
            if (r == 0) continue;
            for (int pass = 0; pass < 2; ++pass)
                for (int b = 0; b < GBSW_BINS; ++b) {
                    const int cls = b ? gbsw::kRangeLong : gbsw::kRangeShort;
                    const double ms = elapsed(ctx->ev_cls[pass][cls][0], ctx->ev_cls[pass][cls][1]);
                    t[pass][b] = std::min(t[pass][b], ms);
                }
        }
        if (!ran) continue;
        report->candidates[nc] = v;
        for (int b = 0; b < GBSW_BINS; ++b) {
            report->ms_forward[b][nc] = t[0][b];
            report->ms_reverse[b][nc] = t[1][b];
            for (int pass = 0; pass < 2; ++pass) {
                if (t[pass][b] < best[pass][b]) {
                    best[pass][b] = t[pass][b];
                    (pass ? report->chosen_reverse : report->chosen)[b] = v;
                }
            }
        }
        ++nc;
    }
    report->ncandidates = nc;
    if (nc == 0) return ctx->fail(GBSW_EINVAL, "no kernel variant applies to this scoring");
    // the bins' pair counts, as the forward schedule of the last run found them
    for (int b = 0; b < GBSW_BINS; ++b) {
        report->pairs[b] = ctx->stats.bin_pairs[b];
        report->bucket[b] = count_bucket(report->pairs[b]);
        if (report->pairs[b] > 0) {
            ctx->tuning.variant[scoring->kind][b][report->bucket[b]] = report->chosen[b];
            ctx->tuning.reverse[scoring->kind][b][report->bucket[b]] = report->chosen_reverse[b];
        }
    }
    return GBSW_OK;
}

int gbsw_last_stats(const gbsw_context* ctx, gbsw_stats* stats) {
    if (!ctx || !stats) return GBSW_EINVAL;
    gbsw_stats s = ctx->stats;
    if (cudaEventSynchronize(ctx->ev[EV_REV]) == cudaSuccess) {
        if (s.reruns < 0) {  // the dual-pair launches' overflow count, final once the passes are done
            int count = 0;
            s.reruns = cudaMemcpy(&count, ctx->d_rerun.ptr + 1, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess
                           ? count
                           : 0;
        }
        s.forward_ms = elapsed(ctx->ev[EV_H2D], ctx->ev[EV_FWD]);
        s.reverse_ms = elapsed(ctx->ev[EV_FWD], ctx->ev[EV_REV]);
        if (ctx->timed_host && cudaEventSynchronize(ctx->ev[EV_D2H]) == cudaSuccess) {
            s.h2d_ms = elapsed(ctx->ev[EV_START], ctx->ev[EV_H2D]);
            s.d2h_ms = elapsed(ctx->ev[EV_REV], ctx->ev[EV_D2H]);
            s.total_ms = elapsed(ctx->ev[EV_START], ctx->ev[EV_D2H]);
        } else {
            s.h2d_ms = s.d2h_ms = 0;
            s.total_ms = elapsed(ctx->ev[EV_START], ctx->ev[EV_REV]);
        }
    }
    *stats = s;
    return GBSW_OK;
}

}  // extern "C"

int gbsw::long_bin_cols() { return gbsw::kLongCols; }

int gbsw::align_device_known_bins(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref,
                                  const int64_t* ref_off, const uint8_t* query, const int64_t* query_off, int64_t n,
                                  int32_t max_len, int32_t* top_scores, int32_t* ref_begin, int32_t* ref_end,
                                  int32_t* query_begin, int32_t* query_end, cudaStream_t stream,
                                  const int64_t bin_pairs[2]) {
    if (!ctx) return GBSW_EINVAL;
    int rc = check_scoring(ctx, scoring);
    if (rc != GBSW_OK) return rc;
    if (n < 0) return ctx->fail(GBSW_EINVAL, "negative pair count");
    if (n == 0) return GBSW_OK;
    if (n > (int64_t)0x7fffffff) return ctx->fail(GBSW_EINVAL, "too many pairs for one call");
    if (max_len < 0 || max_len > GBSW_MAX_SEQ_LEN) return ctx->fail(GBSW_ELENGTH, "max_len outside [0, 65535]");
    if (!ref || !ref_off || !query || !query_off || !top_scores || !ref_begin || !ref_end || !query_begin ||
        !query_end || !bin_pairs)
        return ctx->fail(GBSW_EINVAL, "NULL buffer");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    cudaEventRecord(ctx->ev[EV_START], stream);
    ctx->timed_host = false;
    ctx->stats.cells = 0;
    return run_passes(ctx, scoring, ref, ref_off, query, query_off, n, max_len, top_scores, ref_begin, ref_end,
                      query_begin, query_end, stream, nullptr, bin_pairs);
}
