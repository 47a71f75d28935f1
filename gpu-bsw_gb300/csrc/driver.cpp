// C++ drop-in for gpu_bsw_driver::kernel_driver_dna / kernel_driver_aa
// (reference driver.hpp:18-42, driver.cpp:10-489, utils.cpp:13-28) over the
// C ABI of gbsw.h.  Like the reference (driver.cpp:23-41) one call uses every
// visible GPU -- or the devices listed in GBSW_DEVICES -- with one host thread
// each; the pairs are split into contiguous ranges balanced by cells
// (gbsw_split_pairs) rather than by pair count, and each device writes its own
// slice of the result arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbsw.h"
#include "../../include/gpu_bsw/driver.hpp"
#include "../../include/gpu_bsw/utils.hpp"
#include "pack.h"
#include "pinned_pool.h"

namespace {

// Exit like the reference's gpuAssert (utils.hpp:12-21): message on stderr,
// non-zero process status.
[[noreturn]] void die(const char* what, int status, const gbsw_context* ctx) {
    std::fprintf(stderr, "gpu_bsw_driver: %s failed: %s (%s)\n", what, gbsw_strerror(status),
                 ctx ? gbsw_last_error(ctx) : "");
    std::exit(status < 0 ? -status : (status == 0 ? 1 : status));
}

bool verbose() {
    const char* v = std::getenv("GBSW_VERBOSE");
    return v && v[0] == '1';
}

void alloc_results(gpu_bsw_driver::alignment_results* r, size_t n) {
    // utils.cpp:13-19: pinned host arrays owned by the caller's struct
    size_t bytes = sizeof(short) * (n > 0 ? n : 1);
    short** fields[5] = {&r->ref_begin, &r->ref_end, &r->query_begin, &r->query_end, &r->top_scores};
    for (short** f : fields) {
        cudaError_t e = cudaMallocHost((void**)f, bytes);
        if (e != cudaSuccess) die("cudaMallocHost", GBSW_ENOMEM, nullptr);
    }
}

// Grow-on-demand device buffer of the ingest pipeline (contents are not preserved).
template <typename T>
struct DeviceBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    bool reserve(size_t n) {
        if (n <= cap) return true;
        const size_t want = std::max(n, cap + cap / 2);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        if (cudaMalloc((void**)&ptr, want * sizeof(T)) != cudaSuccess) return false;
        cap = want;
        return true;
    }
};

// One chunk's buffers of the ingest pipeline: page-locked staging (from the
// process-wide pool shared with the serving loop) and device copies.  Two
// slots alternate, so that one chunk is packed and copied in while the
// previous one is aligned.
struct Slot {
    gbsw::PooledPinned<char> h_ref, h_query;
    gbsw::PooledPinned<int64_t> h_ref_off, h_query_off;
    gbsw::PooledPinned<int32_t> h_res;
    DeviceBuf<uint8_t> d_ref, d_query;
    DeviceBuf<int64_t> d_ref_off, d_query_off;
    DeviceBuf<int32_t> d_res;
    // packed ingest: both streams' words (ref then query), their escape runs
    // (ref positions, ref offsets, query positions, query offsets) and bytes
    gbsw::PooledPinned<uint32_t> h_words;
    gbsw::PooledPinned<int64_t> h_runs;
    gbsw::PooledPinned<uint8_t> h_run_bytes;
    DeviceBuf<uint32_t> d_words;
    DeviceBuf<int64_t> d_runs;
    DeviceBuf<uint8_t> d_run_bytes;
    gbsw_packed pref{}, pquery{};  // device pointers, unpacked into d_ref / d_query
    bool packed = false;
    int kind = GBSW_DNA;
    cudaEvent_t copied = nullptr;  // the chunk's inputs are on the device
    size_t begin = 0, end = 0, max_len = 0;
};

// Per-device state of the drop-in: a library context, a compute stream for the
// passes and the results, a copy stream for the inputs, and the two pipeline
// slots, kept between calls.  One per entry of the device list (a device
// listed twice gets two).
struct DeviceState {
    int device = 0;
    gbsw_context* ctx = nullptr;
    cudaStream_t stream = nullptr;  // passes and result copies
    cudaStream_t copy = nullptr;    // input copies of the next chunk
    std::mutex mu;  // one call at a time per device
    Slot slot[2];
};

// State of slot `slot` of the device list, on device `dev` (the calling
// thread's current device becomes `dev`).
DeviceState* state_for(int dev, int slot) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, DeviceState*> states;
    if (cudaSetDevice(dev) != cudaSuccess) die("cudaSetDevice", GBSW_ECUDA, nullptr);
    std::lock_guard<std::mutex> lock(mu);
    auto it = states.find({dev, slot});
    if (it != states.end()) return it->second;
    DeviceState* st = new DeviceState();
    st->device = dev;
    int rc = gbsw_create(dev, &st->ctx);
    if (rc != GBSW_OK) die("gbsw_create", rc, nullptr);
    if (cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st->copy, cudaStreamNonBlocking) != cudaSuccess)
        die("cudaStreamCreate", GBSW_ECUDA, st->ctx);
    for (Slot& sl : st->slot)
        if (cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming) != cudaSuccess)
            die("cudaEventCreate", GBSW_ECUDA, st->ctx);
    states[{dev, slot}] = st;
    return st;
}

// The devices one call spreads over: GBSW_DEVICES ("0,2,3"; a device may be
// listed more than once) or every visible device (driver.cpp:23-25).
std::vector<int> device_list() {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) die("cudaGetDeviceCount", GBSW_ECUDA, nullptr);
    std::vector<int> devs;
    if (const char* env = std::getenv("GBSW_DEVICES")) {
        const char* p = env;
        while (*p) {
            char* end = nullptr;
            const long d = std::strtol(p, &end, 10);
            if (end == p || d < 0 || d >= count) {
                std::fprintf(stderr, "gpu_bsw_driver: GBSW_DEVICES=%s names no visible device list\n", env);
                std::exit(1);
            }
            devs.push_back((int)d);
            p = (*end == ',') ? end + 1 : end;
            if (*end && *end != ',') {
                std::fprintf(stderr, "gpu_bsw_driver: GBSW_DEVICES=%s: expected comma-separated device numbers\n",
                             env);
                std::exit(1);
            }
        }
    }
    if (devs.empty())
        for (int d = 0; d < count; ++d) devs.push_back(d);
    return devs;
}

// Threads that pack one chunk.  The host side of the reference driver packs the
// strings on one thread into pageable buffers and copies them afterwards
// (driver.cpp:115-168); here worker threads copy slices of the chunk into
// page-locked staging and the calling thread starts each slice's host-to-device
// copy as soon as the slice is packed, so the copies overlap the packing.
unsigned pack_threads() {
    const unsigned hw = std::thread::hardware_concurrency();
    return std::max(1u, std::min(8u, hw ? hw : 1u));
}

// Whether the ingest packs the sequences (2-bit DNA / 5-bit protein, unpacked
// on the device) rather than copying raw bytes: GBSW_DROPIN_PACK=0 turns it off.
bool pack_ingest() {
    const char* v = std::getenv("GBSW_DROPIN_PACK");
    return !(v && v[0] == '0');
}

// Packs symbols [s0, s1) of the concatenation of seqs[first + k] (offsets
// `off`, relative to the chunk) into stream words from words[s0 / per word];
// s0 is a multiple of the symbols per word.  The bytes are gathered through a
// small buffer in whole words.
void gather_pack(int kind, const std::vector<std::string>& seqs, size_t first, const int64_t* off, size_t n,
                 int64_t s0, int64_t s1, uint32_t* words, gbsw::EscapeRuns* esc) {
    constexpr int64_t kTmp = 48 * 1024;  // a multiple of 16 and of 6 symbols
    char tmp[kTmp];
    const int64_t per = gbsw::symbols_per_word(kind);
    size_t k = (size_t)(std::upper_bound(off, off + n + 1, s0) - off) - 1;  // the pair holding symbol s0
    for (int64_t pos = s0; pos < s1;) {
        const int64_t m = std::min(kTmp, s1 - pos);
        for (int64_t got = 0; got < m;) {
            while (off[k + 1] <= pos + got) ++k;  // empty pairs and finished ones
            const int64_t at = pos + got - off[k], take = std::min(off[k + 1] - (pos + got), m - got);
            std::memcpy(tmp + got, seqs[first + k].data() + at, (size_t)take);
            got += take;
        }
        gbsw::pack_span(kind, tmp, m, pos, words + pos / per, esc);
        pos += m;
    }
}

// Wall time of the phases of the drop-in calls (GBSW_VERBOSE=1 report).
struct Phases {
    double offsets = 0, pack = 0, align = 0, results = 0;
    int chunks = 0;
};

double ms_since(std::chrono::steady_clock::time_point& t) {
    const auto now = std::chrono::steady_clock::now();
    const double d = std::chrono::duration<double, std::milli>(now - t).count();
    t = now;
    return d;
}

// Joins the slices' escape runs of both streams into the slot's page-locked
// run arrays, starts their copies on `s` and points the slot's device-side
// packed streams at the copies.  False when a buffer cannot be had.
bool copy_escapes(Slot& sl, const std::vector<gbsw::EscapeRuns>& resc, const std::vector<gbsw::EscapeRuns>& qesc,
                  int64_t ra, int64_t qa, size_t rw, cudaStream_t s) {
    gbsw::EscapeRuns r, q;
    for (const auto& e : resc) r.append(e);
    for (const auto& e : qesc) q.append(e);
    const size_t nr = r.at.size(), nq = q.at.size();
    const size_t nruns = 2 * nr + 1 + 2 * nq + 1, nbytes = r.bytes.size() + q.bytes.size();
    if (!sl.h_runs.reserve(nruns) || !sl.d_runs.reserve(nruns) ||
        !sl.h_run_bytes.reserve(std::max<size_t>(nbytes, 1)) || !sl.d_run_bytes.reserve(std::max<size_t>(nbytes, 1)))
        return false;
    int64_t* h = sl.h_runs.ptr;
    auto lay = [](const gbsw::EscapeRuns& x, int64_t* at, int64_t* off) {
        off[0] = 0;
        for (size_t k = 0; k < x.at.size(); ++k) {
            at[k] = x.at[k];
            off[k + 1] = off[k] + x.len[k];
        }
    };
    lay(r, h, h + nr);
    lay(q, h + 2 * nr + 1, h + 2 * nr + 1 + nq);
    if (!r.bytes.empty()) std::memcpy(sl.h_run_bytes.ptr, r.bytes.data(), r.bytes.size());
    if (!q.bytes.empty()) std::memcpy(sl.h_run_bytes.ptr + r.bytes.size(), q.bytes.data(), q.bytes.size());
    if (nr + nq > 0) {
        if (cudaMemcpyAsync(sl.d_runs.ptr, h, 8 * nruns, cudaMemcpyHostToDevice, s) != cudaSuccess) return false;
        if (nbytes && cudaMemcpyAsync(sl.d_run_bytes.ptr, sl.h_run_bytes.ptr, nbytes, cudaMemcpyHostToDevice, s) !=
                          cudaSuccess)
            return false;
    }
    const int64_t* d = sl.d_runs.ptr;
    sl.pref = gbsw_packed{sl.d_words.ptr, ra, (int64_t)nr, d, d + nr, sl.d_run_bytes.ptr};
    sl.pquery = gbsw_packed{sl.d_words.ptr + rw, qa, (int64_t)nq, d + 2 * nr + 1, d + 2 * nr + 1 + nq,
                            sl.d_run_bytes.ptr + r.bytes.size()};
    return true;
}

// Packs pairs [begin, end) of the caller's vectors into slot `sl` and starts
// their host-to-device copies on the copy stream (recorded in sl.copied).
void pack_chunk(DeviceState* st, Slot& sl, const std::vector<std::string>& contigs,
                const std::vector<std::string>& reads, size_t begin, size_t end, int kind, Phases* ph) {
    auto t = std::chrono::steady_clock::now();
    const size_t n = end - begin;
    sl.begin = begin;
    sl.end = end;
    sl.kind = kind;
    sl.packed = pack_ingest();
    if (!sl.h_ref_off.reserve(n + 1) || !sl.h_query_off.reserve(n + 1) || !sl.h_res.reserve(5 * n))
        die("cudaMallocHost", GBSW_ENOMEM, st->ctx);
    int64_t* ro = sl.h_ref_off.ptr;
    int64_t* qo = sl.h_query_off.ptr;
    ro[0] = qo[0] = 0;
    size_t max_len = 0;
    for (size_t k = 0; k < n; ++k) {
        const size_t a = contigs[begin + k].size(), b = reads[begin + k].size();
        if (a > GBSW_MAX_SEQ_LEN || b > GBSW_MAX_SEQ_LEN) die("alignment", GBSW_ELENGTH, st->ctx);
        ro[k + 1] = ro[k] + (int64_t)a;
        qo[k + 1] = qo[k] + (int64_t)b;
        max_len = std::max(max_len, std::max(a, b));
    }
    sl.max_len = max_len;
    const size_t ra = (size_t)ro[n], qa = (size_t)qo[n];
    ph->offsets += ms_since(t);
    const int64_t per = gbsw::symbols_per_word(kind);
    const size_t rw = (ra + per - 1) / per, qw = (qa + per - 1) / per;
    if (sl.packed ? !sl.h_words.reserve(std::max<size_t>(rw + qw, 1))
                  : (!sl.h_ref.reserve(std::max<size_t>(ra, 1)) || !sl.h_query.reserve(std::max<size_t>(qa, 1))))
        die("cudaMallocHost", GBSW_ENOMEM, st->ctx);
    if (sl.packed && !sl.d_words.reserve(std::max<size_t>(rw + qw, 1))) die("cudaMalloc", GBSW_ENOMEM, st->ctx);
    if (!sl.d_ref.reserve(std::max<size_t>(ra, 1)) || !sl.d_query.reserve(std::max<size_t>(qa, 1)) ||
        !sl.d_ref_off.reserve(n + 1) || !sl.d_query_off.reserve(n + 1) || !sl.d_res.reserve(5 * n))
        die("cudaMalloc", GBSW_ENOMEM, st->ctx);
    cudaStream_t s = st->copy;
    if (cudaMemcpyAsync(sl.d_ref_off.ptr, ro, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(sl.d_query_off.ptr, qo, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s) != cudaSuccess)
        die("cudaMemcpyAsync", GBSW_ECUDA, st->ctx);

    // slices of about 4 MB of sequence each, packed by the workers in order
    const size_t total = ra + qa;
    const size_t slices = std::max<size_t>(1, std::min<size_t>(n, total / (4u << 20) + 1));
    std::vector<size_t> cut(slices + 1, n);
    cut[0] = 0;
    for (size_t j = 1, k = 0; j < slices; ++j) {
        const size_t target = total * j / slices;
        while (k < n && (size_t)(ro[k] + qo[k]) < target) ++k;
        cut[j] = k;
    }
    // packed: slice j covers the symbols from its first pair's start, rounded
    // down to a whole word, to the next slice's (the last one to the end), so
    // no two slices share a word
    std::vector<int64_t> rcut(slices + 1), qcut(slices + 1);
    for (size_t j = 0; j <= slices; ++j) {
        rcut[j] = j == slices ? (int64_t)ra : (j == 0 ? 0 : ro[cut[j]] / per * per);
        qcut[j] = j == slices ? (int64_t)qa : (j == 0 ? 0 : qo[cut[j]] / per * per);
    }
    std::vector<gbsw::EscapeRuns> resc(sl.packed ? slices : 0), qesc(sl.packed ? slices : 0);
    uint32_t* rwords = sl.h_words.ptr;
    uint32_t* qwords = sl.h_words.ptr + rw;
    std::vector<char> done(slices, 0);
    std::mutex mu;
    std::condition_variable cv;
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t j; (j = next.fetch_add(1)) < slices;) {
            if (sl.packed) {
                gather_pack(kind, contigs, begin, ro, n, rcut[j], rcut[j + 1], rwords, &resc[j]);
                gather_pack(kind, reads, begin, qo, n, qcut[j], qcut[j + 1], qwords, &qesc[j]);
            } else {
                for (size_t k = cut[j]; k < cut[j + 1]; ++k) {
                    const std::string& a = contigs[begin + k];
                    const std::string& b = reads[begin + k];
                    if (!a.empty()) std::memcpy(sl.h_ref.ptr + ro[k], a.data(), a.size());
                    if (!b.empty()) std::memcpy(sl.h_query.ptr + qo[k], b.data(), b.size());
                }
            }
            {
                std::lock_guard<std::mutex> lock(mu);
                done[j] = 1;
            }
            cv.notify_one();
        }
    };
    const unsigned nthreads = (unsigned)std::min<size_t>(pack_threads(), slices);
    std::vector<std::thread> pool;
    for (unsigned th = 1; th < nthreads; ++th) pool.emplace_back(worker);
    if (nthreads == 1) worker();
    cudaError_t e = cudaSuccess;
    for (size_t j = 0; j < slices; ++j) {
        {
            std::unique_lock<std::mutex> lock(mu);
            cv.wait(lock, [&] { return done[j] != 0; });
        }
        if (sl.packed) {
            // the slice's words: [first word, first word of the next slice)
            const size_t r0 = (size_t)rcut[j] / per, r1 = ((size_t)rcut[j + 1] + per - 1) / per;
            const size_t q0 = (size_t)qcut[j] / per, q1 = ((size_t)qcut[j + 1] + per - 1) / per;
            if (e == cudaSuccess && r1 > r0)
                e = cudaMemcpyAsync(sl.d_words.ptr + r0, rwords + r0, 4 * (r1 - r0), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess && q1 > q0)
                e = cudaMemcpyAsync(sl.d_words.ptr + rw + q0, qwords + q0, 4 * (q1 - q0), cudaMemcpyHostToDevice,
                                    s);
            continue;
        }
        const size_t r0 = (size_t)ro[cut[j]], r1 = (size_t)ro[cut[j + 1]];
        const size_t q0 = (size_t)qo[cut[j]], q1 = (size_t)qo[cut[j + 1]];
        if (e == cudaSuccess && r1 > r0)
            e = cudaMemcpyAsync(sl.d_ref.ptr + r0, sl.h_ref.ptr + r0, r1 - r0, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && q1 > q0)
            e = cudaMemcpyAsync(sl.d_query.ptr + q0, sl.h_query.ptr + q0, q1 - q0, cudaMemcpyHostToDevice, s);
    }
    for (auto& th : pool) th.join();
    if (sl.packed && e == cudaSuccess && !copy_escapes(sl, resc, qesc, (int64_t)ra, (int64_t)qa, rw, s))
        die("escape runs", GBSW_ENOMEM, st->ctx);
    if (e == cudaSuccess) e = cudaEventRecord(sl.copied, s);
    if (e != cudaSuccess) die("cudaMemcpyAsync", GBSW_ECUDA, st->ctx);
    ph->pack += ms_since(t);
}

// Enqueues slot `sl`'s passes and result copy on the compute stream, after its
// input copies.
void launch_chunk(DeviceState* st, Slot& sl, const gbsw_scoring& sc) {
    const size_t n = sl.end - sl.begin;
    cudaStream_t s = st->stream;
    if (cudaStreamWaitEvent(s, sl.copied, 0) != cudaSuccess) die("cudaStreamWaitEvent", GBSW_ECUDA, st->ctx);
    if (sl.packed) {
        int rc = gbsw_unpack_device(sl.kind, &sl.pref, sl.d_ref.ptr, (void*)s);
        if (rc == GBSW_OK) rc = gbsw_unpack_device(sl.kind, &sl.pquery, sl.d_query.ptr, (void*)s);
        if (rc != GBSW_OK) die("unpack", rc, st->ctx);
    }
    int32_t* R = sl.d_res.ptr;
    int rc = gbsw_align_device(st->ctx, &sc, sl.d_ref.ptr, sl.d_ref_off.ptr, sl.d_query.ptr, sl.d_query_off.ptr,
                               (int64_t)n, (int32_t)std::max<size_t>(sl.max_len, 1), R, R + n, R + 2 * n, R + 3 * n,
                               R + 4 * n, (void*)s);
    if (rc != GBSW_OK) die("alignment", rc, st->ctx);
    if (cudaMemcpyAsync(sl.h_res.ptr, R, sizeof(int32_t) * 5 * n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        die("cudaMemcpyAsync", GBSW_ECUDA, st->ctx);
}

// Waits for slot `sl`'s chunk (and reports its device-side input errors), then
// writes its results into the reference's short arrays.
void finish_chunk(DeviceState* st, Slot& sl, gpu_bsw_driver::alignment_results* out, Phases* ph) {
    auto t = std::chrono::steady_clock::now();
    const int rc = gbsw_check(st->ctx, (void*)st->stream);
    if (rc != GBSW_OK) die("alignment", rc, st->ctx);
    ph->align += ms_since(t);
    const size_t n = sl.end - sl.begin, begin = sl.begin;
    const int32_t* h = sl.h_res.ptr;
    for (size_t k = 0; k < n; ++k) {  // the reference's short result arrays
        out->top_scores[begin + k] = (short)h[k];
        out->ref_begin[begin + k] = (short)h[n + k];
        out->ref_end[begin + k] = (short)h[2 * n + k];
        out->query_begin[begin + k] = (short)h[3 * n + k];
        out->query_end[begin + k] = (short)h[4 * n + k];
    }
    ph->results += ms_since(t);
}

// Pairs per pipeline chunk of a large call: large enough to fill the GPU (a
// chunk's passes end in a last wave of their own), small enough that packing
// the next chunk on the host threads hides behind the current one's passes.
constexpr size_t kPipePairs = size_t(1) << 17;

// Pairs [first, last) on slot `slot` of the device list, in chunks that stay
// within `factor` of the device's memory (driver.cpp:36, 51-55) and, for large
// calls, in pipeline chunks of about kPipePairs: chunk k + 1 is packed and
// copied in while chunk k's passes run.
void run_range(int dev, int slot, const std::vector<std::string>& reads, const std::vector<std::string>& contigs,
               size_t first, size_t last, gpu_bsw_driver::alignment_results* out, const gbsw_scoring& sc,
               float factor, Phases* ph) {
    DeviceState* st = state_for(dev, slot);
    std::lock_guard<std::mutex> lock(st->mu);
    // bytes of both sequences plus offsets and results, for both slots
    uint64_t mem = 0;
    if (gbsw_device_memory(st->device, &mem) != GBSW_OK) die("get_tot_gpu_mem", GBSW_ECUDA, st->ctx);
    double f = factor > 0 && factor <= 1 ? factor : 1.0;
    // leave room for the strip boundary buffers (sized by the longest sequence)
    const double budget = (double)mem * f * 0.25;
    const size_t n = last - first;
    const size_t pieces = n > kPipePairs + kPipePairs / 2 ? (n + kPipePairs / 2) / kPipePairs : 1;
    const size_t per_piece = (n + pieces - 1) / pieces;
    std::vector<std::pair<size_t, size_t>> chunks;
    size_t begin = first;
    while (begin < last) {
        size_t end = begin;
        double bytes = 0;
        while (end < last && end - begin < per_piece) {
            double need = (double)contigs[end].size() + (double)reads[end].size() + 16.0 + 20.0;
            if (end > begin && bytes + need > budget) break;
            bytes += need;
            ++end;
        }
        chunks.emplace_back(begin, end);
        begin = end;
    }
    ph->chunks += (int)chunks.size();
    pack_chunk(st, st->slot[0], contigs, reads, chunks[0].first, chunks[0].second, sc.kind, ph);
    for (size_t k = 0; k < chunks.size(); ++k) {
        Slot& cur = st->slot[k % 2];
        launch_chunk(st, cur, sc);
        // the other slot's previous chunk finished in the last finish_chunk
        if (k + 1 < chunks.size())
            pack_chunk(st, st->slot[(k + 1) % 2], contigs, reads, chunks[k + 1].first, chunks[k + 1].second, sc.kind,
                       ph);
        finish_chunk(st, cur, out, ph);
    }
}

void run(const std::vector<std::string>& reads, const std::vector<std::string>& contigs,
         gpu_bsw_driver::alignment_results* out, const gbsw_scoring& sc, float factor) {
    auto t0 = std::chrono::steady_clock::now();
    if (!out) die("kernel_driver", GBSW_EINVAL, nullptr);
    if (reads.size() != contigs.size()) {
        std::fprintf(stderr, "gpu_bsw_driver: reads and contigs differ in count (%zu vs %zu)\n",
                     reads.size(), contigs.size());
        std::exit(1);
    }
    const size_t n = contigs.size();
    alloc_results(out, n);  // driver.cpp:33
    if (n == 0) return;
    const std::vector<int> devs = device_list();
    int caller_dev = 0;
    if (cudaGetDevice(&caller_dev) != cudaSuccess) die("cudaGetDevice", GBSW_ECUDA, nullptr);

    // contiguous ranges balanced by cells, one per listed device (replaces the
    // equal pair counts of driver.cpp:28-31)
    std::vector<int64_t> cells(n), bounds(devs.size() + 1);
    for (size_t k = 0; k < n; ++k) cells[k] = (int64_t)contigs[k].size() * (int64_t)reads[k].size();
    if (gbsw_split_pairs(cells.data(), (int64_t)n, (int)devs.size(), bounds.data()) != GBSW_OK)
        die("gbsw_split_pairs", GBSW_EINVAL, nullptr);
    std::vector<Phases> ph(devs.size());
    std::vector<std::thread> workers;
    for (size_t d = 1; d < devs.size(); ++d)
        if (bounds[d + 1] > bounds[d])
            workers.emplace_back(run_range, devs[d], (int)d, std::cref(reads), std::cref(contigs),
                                 (size_t)bounds[d], (size_t)bounds[d + 1], out, std::cref(sc), factor, &ph[d]);
    if (bounds[1] > bounds[0])
        run_range(devs[0], 0, reads, contigs, (size_t)bounds[0], (size_t)bounds[1], out, sc, factor, &ph[0]);
    for (auto& w : workers) w.join();
    cudaSetDevice(caller_dev);  // the caller's current device is left as it was
    if (verbose()) {
        std::chrono::duration<double> d = std::chrono::steady_clock::now() - t0;
        size_t maxA = 0, maxB = 0;
        for (size_t k = 0; k < n; ++k) {
            maxA = contigs[k].size() > maxA ? contigs[k].size() : maxA;
            maxB = reads[k].size() > maxB ? reads[k].size() : maxB;
        }
        // same report as driver.cpp:242
        std::printf("Total Alignments:%zu\nMax Reference Size:%zu\nMax Query Size:%zu\n"
                    "Total Execution Time (seconds):%g\n",
                    n, maxA, maxB, d.count());
        for (size_t d = 0; d < devs.size(); ++d)
            std::printf("Device %d: pairs %lld-%lld in %d chunks, phases (ms): offsets %.3f, pack and copy in "
                        "%.3f (%u threads), align %.3f, results %.3f\n",
                        devs[d], (long long)bounds[d], (long long)bounds[d + 1], ph[d].chunks, ph[d].offsets,
                        ph[d].pack, pack_threads(), ph[d].align, ph[d].results);
    }
}

}  // namespace

extern "C" int gbsw_split_pairs(const int64_t* cells, int64_t n, int parts, int64_t* bounds) {
    if (!cells && n > 0) return GBSW_EINVAL;
    if (n < 0 || parts < 1 || !bounds) return GBSW_EINVAL;
    // range r ends at the first pair whose running cell sum reaches r/parts of
    // the total (the first pair past it starts range r + 1)
    std::vector<int64_t> csum((size_t)n + 1, 0);
    for (int64_t k = 0; k < n; ++k) {
        if (cells[k] < 0) return GBSW_EINVAL;
        csum[(size_t)k + 1] = csum[(size_t)k] + cells[k];
    }
    const double total = (double)csum[(size_t)n];
    bounds[0] = 0;
    for (int r = 1; r < parts; ++r) {
        const double target = total * r / parts;
        int64_t k = (int64_t)(std::lower_bound(csum.begin(), csum.end(), target,
                                               [](int64_t a, double t) { return (double)a < t; }) -
                              csum.begin());
        bounds[r] = std::min(std::max(k, bounds[r - 1]), n);
    }
    bounds[parts] = n;
    return GBSW_OK;
}

size_t gpu_bsw_driver::get_tot_gpu_mem(int id) {
    uint64_t bytes = 0;
    int rc = gbsw_device_memory(id, &bytes);
    if (rc != GBSW_OK) die("get_tot_gpu_mem", rc, nullptr);
    return (size_t)bytes;
}

void gpu_bsw_driver::kernel_driver_dna(std::vector<std::string> reads,
                                       std::vector<std::string> contigs,
                                       gpu_bsw_driver::alignment_results* alignments,
                                       short scores[4], float factor) {
    gbsw_scoring sc{};
    sc.kind = GBSW_DNA;
    sc.match = scores[0];  // driver.cpp:18
    sc.mismatch = scores[1];
    sc.gap_open = scores[2];
    sc.gap_extend = scores[3];
    run(reads, contigs, alignments, sc, factor);
}

void gpu_bsw_driver::kernel_driver_aa(std::vector<std::string> reads,
                                      std::vector<std::string> contigs,
                                      gpu_bsw_driver::alignment_results* alignments,
                                      short scoring_matrix[], short openGap, short extendGap,
                                      float factor) {
    gbsw_scoring sc{};
    sc.kind = GBSW_PROTEIN;
    sc.gap_open = openGap;
    sc.gap_extend = extendGap;
    sc.matrix = scoring_matrix;
    run(reads, contigs, alignments, sc, factor);
}

void free_alignments(gpu_bsw_driver::alignment_results* alignments) {
    // utils.cpp:21-28
    if (!alignments) return;
    short* fields[5] = {alignments->ref_begin, alignments->ref_end, alignments->query_begin,
                        alignments->query_end, alignments->top_scores};
    for (short* f : fields) {
        if (!f) continue;
        cudaError_t e = cudaFreeHost(f);
        if (e != cudaSuccess) die("cudaFreeHost", GBSW_ECUDA, nullptr);
    }
    std::memset(alignments, 0, sizeof(*alignments));
}
