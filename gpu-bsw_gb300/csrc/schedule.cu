// Work schedule of the pass kernels: per pair a class (which kernel variant
// runs it) and a cost (strips x pipeline steps); pairs are bucket-sorted by
// (class, descending cost) so every class is one contiguous range of `order`
// that the persistent pass kernels consume longest-first through their work
// queue.  Four small kernels: keys (+ histogram), scan, scatter; the reverse
// pass recomputes keys from the forward pass's ends.
#include "schedule.h"
#include "sw_common.cuh"

namespace gbsw {
namespace {

constexpr int kKeyThreads = 256;

// Descending cost -> ascending bucket.  Costs (strips x pipeline steps) are
// binned by 64; everything from 262,080 up (very long pairs) shares the first
// bucket and so starts first.
__device__ __forceinline__ int cost_bucket(int cost) {
    int q = cost >> 6;
    return kClassBuckets - 1 - (q < kClassBuckets - 1 ? q : kClassBuckets - 1);
}

// Dual-pair class: width then rows, both descending, so that the two pairs of a
// unit have nearly the same shape.  Forward passes and protein: 64-column
// strips (the unit's strip count), rows within 32.  DNA reverse passes: width in
// GBSW_REV_KEY_COLS-column steps and rows in GBSW_REV_KEY_ROWS-row steps -- the
// reverse columns of a pair are its rows plus its band (reverse_columns), so
// pairs of like width and rows also have like bands, and the unit's band (the
// larger of its halves') wastes less.  Reverse pass of the 100,000-pair DNA
// batch: 2.343 ms with 64-column / 32-row keys, 2.316 with 32 / 32, 2.306 with
// 16 / 32, 2.265 with 16 / 16 (same GPU, alternating builds).  Finer forward
// keys measured slower (protein forward 2.23 against 2.11 ms): they order the
// units of one strip count by width before rows, against longest first.
#ifndef GBSW_REV_KEY_COLS
#define GBSW_REV_KEY_COLS 16
#endif
#ifndef GBSW_REV_KEY_ROWS
#define GBSW_REV_KEY_ROWS 16
#endif
template <int COLS, int ROWS>
__device__ __forceinline__ int dual_bucket(int nrows, int ncols) {
    int strips = (ncols + COLS - 1) / COLS;
    strips = strips < 63 ? strips : 63;
    int r = nrows / ROWS;
    r = r < 127 ? r : 127;
    return kBinBuckets - 1 - ((strips << 7) | r);
}
static_assert(64 * 128 <= kBinBuckets, "dual keys");

// Key of a pair of class `cls` (its entry of the per-pair class array): the
// bins share class kClassBinned, long bin first.  `fine`: the DNA reverse keys.
__device__ __forceinline__ int pair_key(int cls, int nrows, int ncols, bool fine = false) {
    if (is_bin_class(cls))
        return class_base(kClassBinned) + (cls == kClassShort ? kBinBuckets : 0) +
               (fine ? dual_bucket<GBSW_REV_KEY_COLS, GBSW_REV_KEY_ROWS>(nrows, ncols)
                     : dual_bucket<64, 32>(nrows, ncols));
    return class_base(cls) + cost_bucket(pass_cost(nrows, ncols));
}

__device__ __forceinline__ bool is_acgt(uint8_t c) {
    return c == 'A' || c == 'C' || c == 'G' || c == 'T';
}

// Four bytes at once.  DNA: every byte is A, C, G or T exactly when rebuilding
// each byte's letter from its code (b >> 1) & 3 gives the bytes back (with b0,
// b1 the code's bits the letter is 0x41 + 2 b0 + 0x13 b1 - 0x0f (b0 & b1): A
// 0x41, C 0x43, T 0x54, G 0x47; no byte lane carries or borrows).  Protein:
// every byte is below 91: (b & 0x7f) + 37 sets bit 7 exactly when b >= 91 for
// b < 128, and bytes >= 128 have bit 7 set already.
__device__ __forceinline__ bool word_ok(unsigned v, bool protein) {
    if (protein) return ((((v & 0x7f7f7f7fu) + 0x25252525u) | v) & 0x80808080u) == 0;
    const unsigned c = (v >> 1) & 0x03030303u;
    const unsigned b0 = c & 0x01010101u, b1 = (c >> 1) & 0x01010101u;
    return 0x41414141u + 2u * b0 + 0x13u * b1 - 0x0fu * (b0 & b1) == v;
}

// The warp's check of bytes [from, to) of `base`: the bytes before the first
// and after the last 16-byte boundary one per lane, the rest as 16-byte loads.
__device__ __forceinline__ bool span_ok(const uint8_t* base, int64_t from, int64_t to, bool protein, int lane) {
    bool ok = true;
    const uintptr_t start = reinterpret_cast<uintptr_t>(base + from);
    int64_t a0 = from + (int64_t)((16 - (start & 15u)) & 15u);  // first 16-byte boundary
    if (a0 > to) a0 = to;
    const int64_t a1 = a0 + ((to - a0) & ~(int64_t)15);          // last one
    for (int64_t t = from + lane; t < a0; t += 32) ok = ok && (protein ? base[t] < 91 : is_acgt(base[t]));
    for (int64_t t = a1 + lane; t < to; t += 32) ok = ok && (protein ? base[t] < 91 : is_acgt(base[t]));
    const uint4* v = reinterpret_cast<const uint4*>(base + a0);
    for (int64_t w = lane; w < (a1 - a0) / 16; w += 32) {
        const uint4 x = __ldg(v + w);
        ok = ok && word_ok(x.x, protein) && word_ok(x.y, protein) && word_ok(x.z, protein) && word_ok(x.w, protein);
    }
    return ok;
}

// One warp per pair: lengths, DNA alphabet class (A/C/G/T only or not) or the
// protein symbol check, key and histogram.
__global__ void forward_keys(SchedParams s) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = warp; k < s.n; k += nwarps) {
        const int64_t ra = s.ref_off[k], rb = s.ref_off[k + 1];
        const int64_t qa = s.query_off[k], qb = s.query_off[k + 1];
        const int a = (int)(rb - ra), b = (int)(qb - qa);
        // DNA: only A/C/G/T; protein: every byte inside the table
        bool ok = span_ok(s.ref, ra, rb, s.protein != 0, lane) && span_ok(s.query, qa, qb, s.protein != 0, lane);
        ok = __all_sync(0xffffffffu, ok);
        if (lane == 0) {
            int cls;
            if (s.protein) {
                if (!ok) atomicOr(s.error, kErrSymbol);
                cls = 0;
            } else {
                cls = (ok && s.dna_profile_ok) ? 0 : 1;
            }
            const int nrows = a > b ? a : b, ncols = a < b ? a : b;
            // every A/C/G/T (DNA) or profile-scored (protein) pair goes to the
            // length bin of its shorter side; a bin whose plan runs the int16x2
            // kernels detects a score that may have overflowed int16 and queues
            // that pair for the int32 pass
            if (cls == 0 && s.binned) cls = ncols >= kLongCols ? kClassLong : kClassShort;
            // bins: strips then rows, which pairs like shapes for the two-pair
            // units and is longest-first for one-pair plans as well
            const int key = pair_key(cls, nrows, ncols);
            s.cls[k] = (uint8_t)cls;
            s.keys[k] = key;
            atomicAdd(&s.hist[key], 1);
        }
    }
}

// Reverse-pass keys from the forward results: pairs with no positive score go
// to the idle class (their begins are already -1).
__global__ void reverse_keys(SchedParams s) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int key;
        if (s.score[k] <= 0) {
            key = class_base(kClassIdle);
        } else {
            const int na = s.ref_end[k], nb = s.query_end[k];
            const int nrows = na < nb ? na : nb;  // transposed: rows = shorter prefix
            const int a = (int)(s.ref_off[k + 1] - s.ref_off[k]), b = (int)(s.query_off[k + 1] - s.query_off[k]);
            const int ncols = reverse_columns(a, b, na, nb, s.score[k], s.match, s.rev_p);
            // a pair whose score may exceed the int16 range of the dual-pair
            // kernels (the forward pass ran it in int32), in a bin whose reverse
            // plan is dual, takes the int32 class
            int cls = (int)s.cls[k];
            if (is_bin_class(cls) && ((s.rev_dual_bins >> (cls == kClassLong ? 1 : 0)) & 1) &&
                s.score[k] > s.dual_limit)
                cls = 0;
            key = pair_key(cls, nrows, ncols, s.protein == 0);
        }
        s.keys[k] = key;
        atomicAdd(&s.hist[key], 1);
    }
}

// Exclusive scan of the kBuckets-entry histogram in one block (each thread owns
// kPer consecutive buckets, read and written as int4); also writes the
// [begin, end) range of every class and of the two bins of class kClassBinned.
__global__ void __launch_bounds__(1024) scan_hist(SchedParams s) {
    constexpr int kPer = kBuckets / 1024;
    static_assert(kPer % 4 == 0, "int4 access");
    __shared__ int part[1024];
    const int t = threadIdx.x;
    int4 v[kPer / 4];
    int4* h4 = reinterpret_cast<int4*>(s.hist) + t * (kPer / 4);
    int local = 0;
#pragma unroll
    for (int k = 0; k < kPer / 4; ++k) {
        v[k] = h4[k];
        local += v[k].x + v[k].y + v[k].z + v[k].w;
    }
    part[t] = local;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
        int x = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    int run = t > 0 ? part[t - 1] : 0;
#pragma unroll
    for (int k = 0; k < kPer / 4; ++k) {
        int4 o;
        o.x = run; run += v[k].x;
        o.y = run; run += v[k].y;
        o.z = run; run += v[k].z;
        o.w = run; run += v[k].w;
        h4[k] = o;
    }
    __syncthreads();
    if (t < kClasses) {
        s.class_range[2 * t] = s.hist[class_base(t)];
        s.class_range[2 * t + 1] = t + 1 < kClasses ? s.hist[class_base(t + 1)] : part[1023];
    } else if (t == kClasses) {
        const int begin = s.hist[class_base(kClassBinned)];
        const int split = s.hist[class_base(kClassBinned) + kBinBuckets];
        const int end = part[1023];  // the binned class is the last
        s.class_range[2 * kRangeLong] = begin;
        s.class_range[2 * kRangeLong + 1] = split;
        s.class_range[2 * kRangeShort] = split;
        s.class_range[2 * kRangeShort + 1] = end;
    }
}

__global__ void scatter(SchedParams s) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int pos = atomicAdd(&s.hist[s.keys[k]], 1);
        s.order[pos] = (int)k;
    }
}

int grid_for(int64_t items, int per_block, int sms) {
    int64_t want = (items + per_block - 1) / per_block;
    int64_t cap = (int64_t)sms * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

cudaError_t build_schedule(const SchedParams& s, bool reverse, int sms, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(s.hist, 0, sizeof(int) * kBuckets, stream);
    if (e != cudaSuccess) return e;
    if (!reverse) {
        forward_keys<<<grid_for(s.n * 32, kKeyThreads, sms), kKeyThreads, 0, stream>>>(s);
    } else {
        reverse_keys<<<grid_for(s.n, kKeyThreads, sms), kKeyThreads, 0, stream>>>(s);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    scan_hist<<<1, 1024, 0, stream>>>(s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    scatter<<<grid_for(s.n, kKeyThreads, sms), kKeyThreads, 0, stream>>>(s);
    return cudaGetLastError();
}

}  // namespace gbsw
