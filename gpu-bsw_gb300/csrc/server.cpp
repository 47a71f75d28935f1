// Serving loop: continuous batching of alignment jobs on one GPU (see gbsw.h).
//
// A job is a set of pairs with one scoring, submitted from any host thread.
// `slots` worker threads each own a library context (device buffers, stream).
// A free worker takes the oldest queued job that fits the HBM budget and, in
// the same launch, every other queued job with the same scoring that still
// fits, up to max_batch_pairs: jobs that arrive while others run are admitted
// as soon as a slot and memory free up, and the slots' launches overlap on the
// device.  Each job's results are written to its caller-owned array when its
// batch completes; the pair-by-pair results do not depend on which jobs share
// a launch (pairs are independent and the passes are deterministic).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbsw.h"
#include "pinned_pool.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    gbsw_scoring sc{};
    std::vector<int16_t> matrix;  // owned copy of the protein matrix
    std::vector<char> ref, query;
    std::vector<int64_t> ref_off, query_off;
    int64_t n = 0;
    int64_t cells = 0;
    uint64_t footprint = 0;
    int32_t* out = nullptr;  // caller's n x 5 array
    Clock::time_point t_submit, t_admit, t_done;
    int status = 1;  // 1 pending, 0 ok, < 0 error
};

bool same_scoring(const gbsw_scoring& a, const std::vector<int16_t>& ma, const gbsw_scoring& b,
                  const std::vector<int16_t>& mb) {
    if (a.kind != b.kind || a.gap_open != b.gap_open || a.gap_extend != b.gap_extend) return false;
    if (a.kind == GBSW_DNA) return a.match == b.match && a.mismatch == b.mismatch;
    return ma == mb;
}

// True when any byte of buf is >= 91 (outside the protein encoding table).
// Eight bytes per step: for a byte b < 128, (b & 0x7f) + 37 sets bit 7 exactly
// when b >= 91 and never carries into the next byte; bytes >= 128 have bit 7
// set already.
bool any_byte_at_least_91(const char* buf, size_t len) {
    const uint64_t low7 = 0x7f7f7f7f7f7f7f7full, add = 0x2525252525252525ull, hi = 0x8080808080808080ull;
    uint64_t acc = 0;
    size_t k = 0;
    for (; k + 8 <= len; k += 8) {
        uint64_t x;
        std::memcpy(&x, buf + k, 8);
        acc |= ((x & low7) + add) | x;
    }
    for (; k < len; ++k) acc |= (uint64_t)((unsigned char)buf[k] >= 91) << 7;
    return (acc & hi) != 0;
}

// Device bytes one pair holds while its batch runs: both sequences, two
// offsets, int32 results, schedule entries.
uint64_t pair_footprint(int64_t a, int64_t b) { return (uint64_t)(a + b) + 16 + 20 + 9; }

// Bytes of job buffers a server keeps for reuse.
constexpr size_t kPoolBytes = size_t(512) << 20;

// Latency percentiles cover at most this many most recent jobs.
constexpr size_t kLatencySamples = size_t(1) << 20;

}  // namespace

struct gbsw_server {
    gbsw_server_options opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Job>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Job>> jobs;
    std::vector<std::thread> workers;
    std::vector<double> latencies_ms;
    uint64_t next_id = 1;
    uint64_t used = 0;
    bool stop = false;
    int64_t done_jobs = 0, done_pairs = 0, done_cells = 0, done_batches = 0;
    int64_t running = 0, peak_running = 0;
    Clock::time_point t0 = Clock::now(), t_last_done = Clock::now();
    int create_status = GBSW_OK;
    int ready = 0;  // workers that finished creating their context (or failed to)
    // Recycled job buffers (guarded by mu).  Buffers of a few MB come straight
    // from the kernel in common allocators: without reuse every job pays page
    // faults on its first touch and every finished job an unmap, which stall
    // the submitting threads under load.
    std::vector<std::vector<char>> free_bytes;
    std::vector<std::vector<int64_t>> free_offsets;
    size_t pooled = 0;

    std::vector<char> take_bytes() {
        if (free_bytes.empty()) return {};
        std::vector<char> v = std::move(free_bytes.back());
        free_bytes.pop_back();
        pooled -= v.capacity();
        return v;
    }
    std::vector<int64_t> take_offsets() {
        if (free_offsets.empty()) return {};
        std::vector<int64_t> v = std::move(free_offsets.back());
        free_offsets.pop_back();
        pooled -= v.capacity() * sizeof(int64_t);
        return v;
    }
    void recycle(Job& j) {
        for (std::vector<char>* v : {&j.ref, &j.query}) {
            if (pooled + v->capacity() <= kPoolBytes && v->capacity() > 0) {
                pooled += v->capacity();
                v->clear();
                free_bytes.push_back(std::move(*v));
            }
            std::vector<char>().swap(*v);
        }
        for (std::vector<int64_t>* v : {&j.ref_off, &j.query_off}) {
            if (pooled + v->capacity() * sizeof(int64_t) <= kPoolBytes && v->capacity() > 0) {
                pooled += v->capacity() * sizeof(int64_t);
                v->clear();
                free_offsets.push_back(std::move(*v));
            }
            std::vector<int64_t>().swap(*v);
        }
    }

    // hidden: only the extern "C" functions below leave the library
    __attribute__((visibility("hidden"))) void worker();
};

void gbsw_server::worker() {
    gbsw_context* ctx = nullptr;
    int rc = gbsw_create(opts.device, &ctx);
    {
        std::lock_guard<std::mutex> lock(mu);
        if (rc != GBSW_OK) create_status = rc;
        ++ready;
    }
    cv_done.notify_all();
    if (rc != GBSW_OK) return;
    // the batch is gathered into page-locked buffers from the process-wide pool
    // the C++ drop-in's ingest also draws from, so the copies run as DMA
    gbsw::PooledPinned<char> ref, query;
    gbsw::PooledPinned<int64_t> ref_off, query_off;
    gbsw::PooledPinned<int32_t> res;
    while (true) {
        std::vector<std::shared_ptr<Job>> batch;
        uint64_t reserved = 0;
        {
            std::unique_lock<std::mutex> lock(mu);
            cv_work.wait(lock, [&] {
                if (stop) return true;
                if (queue.empty()) return false;
                const auto& h = queue.front();
                // a job larger than the whole budget runs alone once nothing else holds memory
                return used + h->footprint <= opts.hbm_budget || used == 0;
            });
            if (stop && queue.empty()) break;
            if (queue.empty()) continue;
            std::shared_ptr<Job> head = queue.front();
            queue.pop_front();
            batch.push_back(head);
            reserved = head->footprint;
            int64_t pairs = head->n;
            for (auto it = queue.begin(); it != queue.end() && pairs < opts.max_batch_pairs;) {
                const auto& j = *it;
                if (same_scoring(j->sc, j->matrix, head->sc, head->matrix) &&
                    used + reserved + j->footprint <= opts.hbm_budget && pairs + j->n <= opts.max_batch_pairs) {
                    batch.push_back(j);
                    reserved += j->footprint;
                    pairs += j->n;
                    it = queue.erase(it);
                } else {
                    ++it;
                }
            }
            used += reserved;
            peak_running = std::max(peak_running, ++running);
            const auto now = Clock::now();
            for (auto& j : batch) j->t_admit = now;
        }
        // ---- concatenate, align, split ----
        int64_t n = 0, ra = 0, qa = 0;
        for (auto& j : batch) {
            n += j->n;
            ra += j->ref_off[j->n];
            qa += j->query_off[j->n];
        }
        if (!ref.reserve((size_t)std::max<int64_t>(ra, 1)) || !query.reserve((size_t)std::max<int64_t>(qa, 1)) ||
            !ref_off.reserve((size_t)n + 1) || !query_off.reserve((size_t)n + 1) || !res.reserve((size_t)n * 5)) {
            rc = GBSW_ENOMEM;
        } else {
            ref_off.ptr[0] = query_off.ptr[0] = 0;
            int64_t k = 0, rp = 0, qp = 0;
            for (auto& j : batch) {
                if (j->ref_off[j->n] > 0) std::memcpy(ref.ptr + rp, j->ref.data(), (size_t)j->ref_off[j->n]);
                if (j->query_off[j->n] > 0) std::memcpy(query.ptr + qp, j->query.data(), (size_t)j->query_off[j->n]);
                for (int64_t p = 0; p < j->n; ++p) {
                    ref_off.ptr[k + p + 1] = rp + j->ref_off[(size_t)p + 1];
                    query_off.ptr[k + p + 1] = qp + j->query_off[(size_t)p + 1];
                }
                k += j->n;
                rp += j->ref_off[j->n];
                qp += j->query_off[j->n];
            }
            int32_t* R = res.ptr;
            rc = gbsw_align_host32(ctx, &batch[0]->sc, ref.ptr, ref_off.ptr, query.ptr, query_off.ptr, n, R + n,
                                   R + 2 * n, R + 3 * n, R + 4 * n, R);
        }
        // results to the callers' arrays (each job's array is touched by this worker only)
        const int32_t* R = res.ptr;
        int64_t off = 0;
        for (auto& j : batch) {
            if (rc == GBSW_OK) {
                for (int64_t p = 0; p < j->n; ++p)
                    for (int f = 0; f < 5; ++f) j->out[p * 5 + f] = R[(size_t)f * (size_t)n + (size_t)(off + p)];
            }
            off += j->n;
        }
        {
            std::lock_guard<std::mutex> lock(mu);
            const auto now = Clock::now();
            for (auto& j : batch) {
                recycle(*j);
                j->status = rc == GBSW_OK ? 0 : rc;
                j->t_done = now;
                const double ms = std::chrono::duration<double, std::milli>(now - j->t_submit).count();
                if (latencies_ms.size() < kLatencySamples)
                    latencies_ms.push_back(ms);
                else
                    latencies_ms[(size_t)done_jobs % kLatencySamples] = ms;
                ++done_jobs;
                done_pairs += j->n;
                done_cells += j->cells;
            }
            t_last_done = now;
            used -= reserved;
            --running;
            ++done_batches;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
    gbsw_destroy(ctx);
}

extern "C" {

int gbsw_server_create(const gbsw_server_options* opts, gbsw_server** out) {
    if (!out) return GBSW_EINVAL;
    *out = nullptr;
    gbsw_server_options o{};
    o.device = 0;
    o.slots = 4;
    o.hbm_budget = 16ull << 30;
    o.max_batch_pairs = 50000;
    if (opts) o = *opts;
    if (o.slots < 1 || o.slots > 64 || o.max_batch_pairs < 1 || o.hbm_budget == 0) return GBSW_EINVAL;
    gbsw_server* s = new (std::nothrow) gbsw_server();
    if (!s) return GBSW_ENOMEM;
    s->opts = o;
    for (int k = 0; k < o.slots; ++k) s->workers.emplace_back([s] { s->worker(); });
    int rc;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv_done.wait(lock, [&] { return s->ready == o.slots; });
        rc = s->create_status;
    }
    if (rc != GBSW_OK) {
        gbsw_server_destroy(s);
        return rc;
    }
    *out = s;
    return GBSW_OK;
}

void gbsw_server_destroy(gbsw_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
}

int gbsw_server_submit(gbsw_server* s, const gbsw_scoring* sc, const char* ref, const int64_t* ref_off,
                       const char* query, const int64_t* query_off, int64_t n, int32_t* results,
                       uint64_t* job_id) {
    if (!s || !sc || !ref_off || !query_off || !job_id || n < 0) return GBSW_EINVAL;
    if (n > 0 && (!ref || !query || !results)) return GBSW_EINVAL;
    if (sc->kind != GBSW_DNA && sc->kind != GBSW_PROTEIN) return GBSW_EINVAL;
    if (sc->gap_open > 0 || sc->gap_extend > 0) return GBSW_EINVAL;
    if (sc->kind == GBSW_PROTEIN && !sc->matrix) return GBSW_EINVAL;
    auto j = std::make_shared<Job>();
    j->sc = *sc;
    if (sc->kind == GBSW_PROTEIN) {
        j->matrix.assign(sc->matrix, sc->matrix + 576);
        j->sc.matrix = j->matrix.data();
    }
    j->n = n;
    j->out = results;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        j->ref = s->take_bytes();
        j->query = s->take_bytes();
        j->ref_off = s->take_offsets();
        j->query_off = s->take_offsets();
    }
    j->ref_off.assign(ref_off, ref_off + n + 1);
    j->query_off.assign(query_off, query_off + n + 1);
    for (int64_t k = 0; k < n; ++k) {
        const int64_t a = ref_off[k + 1] - ref_off[k], b = query_off[k + 1] - query_off[k];
        if (a < 0 || b < 0) return GBSW_EINVAL;
        if (a > GBSW_MAX_SEQ_LEN || b > GBSW_MAX_SEQ_LEN) return GBSW_ELENGTH;
        j->cells += a * b;
        j->footprint += pair_footprint(a, b);
    }
    // job-local offsets from 0
    const int64_t r0 = ref_off[0], q0 = query_off[0];
    for (auto& v : j->ref_off) v -= r0;
    for (auto& v : j->query_off) v -= q0;
    if (j->ref_off[n] > 0) j->ref.assign(ref + r0, ref + r0 + j->ref_off[n]);
    if (j->query_off[n] > 0) j->query.assign(query + q0, query + q0 + j->query_off[n]);
    // Inputs are checked here, on the submitting thread, so that a job with a
    // bad symbol is refused alone instead of failing the batch it would share.
    if (sc->kind == GBSW_PROTEIN && (any_byte_at_least_91(j->ref.data(), j->ref.size()) ||
                                     any_byte_at_least_91(j->query.data(), j->query.size())))
        return GBSW_ESYMBOL;
    j->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        j->id = s->next_id++;
        *job_id = j->id;
        if (n == 0) {
            j->status = 0;
            j->t_admit = j->t_done = j->t_submit;
            s->jobs[j->id] = j;
            return GBSW_OK;
        }
        s->jobs[j->id] = j;
        s->queue.push_back(j);
    }
    s->cv_work.notify_one();
    return GBSW_OK;
}

int gbsw_server_wait(gbsw_server* s, uint64_t job_id, double timeout_s, gbsw_job_info* info) {
    if (!s) return GBSW_EINVAL;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return GBSW_EINVAL;
    std::shared_ptr<Job> j = it->second;
    auto finished = [&] { return j->status != 1; };
    if (timeout_s < 0) {
        s->cv_done.wait(lock, finished);
    } else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), finished)) {
        return GBSW_ETIMEOUT;
    }
    if (info) {
        info->status = j->status;
        info->pairs = j->n;
        info->cells = j->cells;
        info->queue_ms = std::chrono::duration<double, std::milli>(j->t_admit - j->t_submit).count();
        info->latency_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
    }
    s->jobs.erase(job_id);
    return j->status;
}

int gbsw_server_get_stats(gbsw_server* s, gbsw_server_stats* st) {
    if (!s || !st) return GBSW_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->jobs = s->done_jobs;
    st->batches = s->done_batches;
    st->peak_running = s->peak_running;
    st->pairs = s->done_pairs;
    st->cells = s->done_cells;
    st->queued = (int64_t)s->queue.size();
    st->hbm_in_use = s->used;
    std::vector<double> v = s->latencies_ms;
    if (!v.empty()) {
        auto pct = [&](double q) {
            size_t k = (size_t)(q * (double)(v.size() - 1) + 0.5);
            std::nth_element(v.begin(), v.begin() + (ptrdiff_t)k, v.end());
            return v[k];
        };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        st->max_ms = *std::max_element(v.begin(), v.end());
    }
    const double secs = std::chrono::duration<double>(s->t_last_done - s->t0).count();
    st->gcups = secs > 0 ? (double)s->done_cells / secs / 1e9 : 0.0;
    return GBSW_OK;
}

int gbsw_server_reset_stats(gbsw_server* s) {
    if (!s) return GBSW_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    s->latencies_ms.clear();
    s->done_jobs = s->done_pairs = s->done_cells = s->done_batches = 0;
    s->peak_running = s->running;
    s->t0 = s->t_last_done = Clock::now();
    return GBSW_OK;
}

}  // extern "C"
