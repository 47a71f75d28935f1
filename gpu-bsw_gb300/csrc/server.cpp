// Serving loop: continuous batching of alignment jobs on one GPU, with the
// jobs' sequences and results resident on the device (see gbsw.h).
//
// A job is a set of pairs with one scoring, submitted from any host thread.
// The submitting thread copies the job into page-locked staging (from the
// process-wide pool the C++ drop-in also uses) and returns.  An uploader thread
// admits staged jobs in arrival order as the HBM budget allows: each admitted
// job gets a device block from the server's own stream-ordered memory pool and
// its sequences are copied in on the upload stream, overlapping whatever the
// workers are running.  `slots` worker threads each own a library context and
// a stream.  A free worker takes the oldest resident job and every other
// resident job with the same scoring, up to max_batch_pairs, and builds one
// launch from them on the device: device-to-device copies into its batch
// buffers (after each job's upload event; the job's device block is freed in
// stream order right after), the passes, and a kernel that turns the results
// into each job's rows; the batch's rows come back in one copy into the
// worker's page-locked buffer, from which each job's rows go to its caller.
// Jobs that arrive while others run are admitted as soon as memory frees and a
// slot takes them, and the slots' launches overlap on the device.  A pair's
// results do not depend on which jobs share its launch (pairs are independent
// and the passes are deterministic).
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
#include "pack.h"
#include "pinned_pool.h"
#include "results.h"

namespace {

using Clock = std::chrono::steady_clock;

// Where a packed job's parts sit in its staging and device block (byte
// offsets, each 16-byte aligned): both streams' words, run positions, run
// offsets and run bytes.
struct PackedLayout {
    size_t words[2] = {0, 0}, run_at[2] = {0, 0}, run_off[2] = {0, 0}, run_bytes[2] = {0, 0};
    int64_t nsym[2] = {0, 0}, nruns[2] = {0, 0};
};

struct Job {
    uint64_t id = 0;
    gbsw_scoring sc{};
    std::vector<int16_t> matrix;  // owned copy of the protein matrix
    gbsw::PooledPinned<char> h_seq;  // page-locked staging: references, then queries (packed jobs: PackedLayout)
    size_t stage_bytes = 0;          // bytes of h_seq the device block holds
    bool packed = false;             // the sequences travel and stay packed, unpacked by the gather
    PackedLayout lay;
    std::vector<int64_t> ref_off, query_off;  // job-local, from 0
    int64_t n = 0;
    int64_t cells = 0;
    int64_t long_pairs = 0;  // pairs of the long length bin (shorter side >= gbsw::long_bin_cols())
    int64_t ref_bytes = 0, query_bytes = 0;
    int max_len = 0;
    uint64_t footprint = 0;
    uint8_t* d_seq = nullptr;          // device copy of h_seq (while admitted)
    cudaEvent_t uploaded = nullptr;    // its copy is done
    int32_t* out = nullptr;            // caller's n x 5 array
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

// Device bytes one pair holds from admission to its launch's end: both
// sequences, two offsets, int32 results and their rows, schedule entries.
uint64_t pair_footprint(int64_t a, int64_t b) { return (uint64_t)(a + b) + 16 + 40 + 9; }

// Latency percentiles cover at most this many most recent jobs.
constexpr size_t kLatencySamples = size_t(1) << 20;

template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    bool reserve(size_t count) {
        if (count <= cap) return true;
        const size_t want = std::max(count, cap + cap / 2);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        if (cudaMalloc((void**)&ptr, want * sizeof(T)) != cudaSuccess) return false;
        cap = want;
        return true;
    }
    ~DevBuf() {
        if (ptr) cudaFree(ptr);
    }
};

}  // namespace

struct gbsw_server {
    gbsw_server_options opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_upload;
    std::deque<std::shared_ptr<Job>> staged;    // on the host, waiting for HBM
    std::deque<std::shared_ptr<Job>> resident;  // on the device, waiting for a slot
    std::unordered_map<uint64_t, std::shared_ptr<Job>> jobs;
    std::vector<std::thread> workers;
    std::thread uploader;
    std::vector<double> latencies_ms;
    uint64_t next_id = 1;
    uint64_t used = 0;  // footprint of the admitted jobs
    bool stop = false;          // no more jobs: the uploader admits what is staged, then ends
    bool stop_workers = false;  // set once the uploader has ended: workers drain, then end
    int64_t done_jobs = 0, done_pairs = 0, done_cells = 0, done_batches = 0;
    int64_t running = 0, peak_running = 0;
    Clock::time_point t0 = Clock::now(), t_last_done = Clock::now();
    int create_status = GBSW_OK;
    int ready = 0;  // workers that finished creating their context (or failed to)
    cudaStream_t upload_stream = nullptr;
    cudaMemPool_t pool = nullptr;  // device blocks of admitted jobs, stream-ordered

    // hidden: only the extern "C" functions below leave the library
    __attribute__((visibility("hidden"))) void worker();
    __attribute__((visibility("hidden"))) void upload_loop();
    __attribute__((visibility("hidden"))) void finish(std::vector<std::shared_ptr<Job>>& batch, int rc);
};

// Admits staged jobs in arrival order while the budget allows (a job larger
// than the whole budget once nothing else is admitted) and starts their copies.
void gbsw_server::upload_loop() {
    cudaSetDevice(opts.device);
    while (true) {
        std::shared_ptr<Job> j;
        {
            std::unique_lock<std::mutex> lock(mu);
            cv_upload.wait(lock, [&] {
                if (stop && staged.empty()) return true;
                if (staged.empty()) return false;
                const auto& h = staged.front();
                return used + h->footprint <= opts.hbm_budget || used == 0;
            });
            if (staged.empty()) break;
            j = staged.front();
            staged.pop_front();
            used += j->footprint;
        }
        const size_t bytes = std::max<size_t>(j->stage_bytes, 1);
        cudaError_t e = cudaMallocFromPoolAsync((void**)&j->d_seq, bytes, pool, upload_stream);
        if (e == cudaSuccess && j->stage_bytes > 0)
            e = cudaMemcpyAsync(j->d_seq, j->h_seq.ptr, j->stage_bytes, cudaMemcpyHostToDevice, upload_stream);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j->uploaded, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(j->uploaded, upload_stream);
        std::vector<std::shared_ptr<Job>> failed;
        {
            std::lock_guard<std::mutex> lock(mu);
            j->t_admit = Clock::now();
            if (e == cudaSuccess) {
                resident.push_back(j);
            } else {
                failed.push_back(j);
            }
        }
        if (!failed.empty()) {
            cudaGetLastError();
            finish(failed, GBSW_ENOMEM);
        }
        cv_work.notify_one();
    }
}

// Results, statistics and the device blocks of a finished batch.
void gbsw_server::finish(std::vector<std::shared_ptr<Job>>& batch, int rc) {
    std::lock_guard<std::mutex> lock(mu);
    const auto now = Clock::now();
    for (auto& j : batch) {
        j->h_seq.release();
        if (j->uploaded) cudaEventDestroy(j->uploaded);
        j->uploaded = nullptr;
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
        used -= j->footprint;
    }
    t_last_done = now;
    cv_done.notify_all();
    cv_upload.notify_one();
}

void gbsw_server::worker() {
    gbsw_context* ctx = nullptr;
    cudaStream_t stream = nullptr;
    int rc = gbsw_create(opts.device, &ctx);
    if (rc == GBSW_OK && cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) rc = GBSW_ECUDA;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (rc != GBSW_OK) create_status = rc;
        ++ready;
    }
    cv_done.notify_all();
    if (rc != GBSW_OK) {
        if (ctx) gbsw_destroy(ctx);
        return;
    }
    cudaSetDevice(opts.device);
    DevBuf<uint8_t> d_ref, d_query;
    DevBuf<int64_t> d_off;
    DevBuf<int32_t> d_res, d_rows;
    gbsw::PooledPinned<int64_t> h_off;
    gbsw::PooledPinned<int32_t> h_rows;
    while (true) {
        std::vector<std::shared_ptr<Job>> batch;
        {
            std::unique_lock<std::mutex> lock(mu);
            cv_work.wait(lock, [&] { return stop_workers || !resident.empty(); });
            if (resident.empty()) break;
            std::shared_ptr<Job> head = resident.front();
            resident.pop_front();
            batch.push_back(head);
            int64_t pairs = head->n;
            for (auto it = resident.begin(); it != resident.end() && pairs < opts.max_batch_pairs;) {
                const auto& j = *it;
                if (same_scoring(j->sc, j->matrix, head->sc, head->matrix) && pairs + j->n <= opts.max_batch_pairs) {
                    batch.push_back(j);
                    pairs += j->n;
                    it = resident.erase(it);
                } else {
                    ++it;
                }
            }
            peak_running = std::max(peak_running, ++running);
        }
        // ---- one launch from resident jobs, on the device ----
        int64_t n = 0, ra = 0, qa = 0, n_long = 0;
        int max_len = 1;
        for (auto& j : batch) {
            n += j->n;
            n_long += j->long_pairs;
            ra += j->ref_bytes;
            qa += j->query_bytes;
            max_len = std::max(max_len, j->max_len);
        }
        rc = GBSW_OK;
        if (!d_ref.reserve((size_t)std::max<int64_t>(ra, 1)) || !d_query.reserve((size_t)std::max<int64_t>(qa, 1)) ||
            !d_off.reserve(2 * (size_t)n + 2) || !d_res.reserve(5 * (size_t)n) || !d_rows.reserve(5 * (size_t)n) ||
            !h_off.reserve(2 * (size_t)n + 2) || !h_rows.reserve(5 * (size_t)n))
            rc = GBSW_ENOMEM;
        cudaError_t e = cudaSuccess;
        if (rc == GBSW_OK) {
            int64_t* ro = h_off.ptr;
            int64_t* qo = h_off.ptr + n + 1;
            ro[0] = qo[0] = 0;
            int64_t k = 0, rp = 0, qp = 0;
            for (auto& j : batch) {
                for (int64_t p = 0; p < j->n; ++p) {
                    ro[k + p + 1] = rp + j->ref_off[(size_t)p + 1];
                    qo[k + p + 1] = qp + j->query_off[(size_t)p + 1];
                }
                e = cudaStreamWaitEvent(stream, j->uploaded, 0);
                if (j->packed) {
                    // unpack both streams straight into the batch buffers
                    for (int x = 0; x < 2 && e == cudaSuccess; ++x) {
                        const PackedLayout& L = j->lay;
                        gbsw_packed dp{};
                        dp.words = reinterpret_cast<const uint32_t*>(j->d_seq + L.words[x]);
                        dp.nsym = L.nsym[x];
                        dp.nruns = L.nruns[x];
                        dp.run_at = reinterpret_cast<const int64_t*>(j->d_seq + L.run_at[x]);
                        dp.run_off = reinterpret_cast<const int64_t*>(j->d_seq + L.run_off[x]);
                        dp.run_bytes = reinterpret_cast<const uint8_t*>(j->d_seq + L.run_bytes[x]);
                        e = gbsw::launch_unpack(j->sc.kind, dp, x ? d_query.ptr + qp : d_ref.ptr + rp, stream);
                    }
                } else {
                    if (e == cudaSuccess && j->ref_bytes > 0)
                        e = cudaMemcpyAsync(d_ref.ptr + rp, j->d_seq, (size_t)j->ref_bytes, cudaMemcpyDeviceToDevice,
                                            stream);
                    if (e == cudaSuccess && j->query_bytes > 0)
                        e = cudaMemcpyAsync(d_query.ptr + qp, j->d_seq + j->ref_bytes, (size_t)j->query_bytes,
                                            cudaMemcpyDeviceToDevice, stream);
                }
                // the job's block goes back to the pool once these copies are done
                if (e == cudaSuccess) e = cudaFreeAsync(j->d_seq, stream);
                if (e != cudaSuccess) break;
                j->d_seq = nullptr;
                k += j->n;
                rp += j->ref_bytes;
                qp += j->query_bytes;
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_off.ptr, h_off.ptr, sizeof(int64_t) * (2 * (size_t)n + 2), cudaMemcpyHostToDevice,
                                    stream);
            if (e != cudaSuccess) rc = GBSW_ECUDA;
        }
        if (rc == GBSW_OK) {
            int32_t* R = d_res.ptr;
            // the bins' pair counts are known here, so the passes need not wait
            // for the device's own between the schedule and the launches
            const int64_t bins[2] = {n - n_long, n_long};
            rc = gbsw::align_device_known_bins(ctx, &batch[0]->sc, d_ref.ptr, d_off.ptr, d_query.ptr, d_off.ptr + n + 1,
                                               n, max_len, R, R + n, R + 2 * n, R + 3 * n, R + 4 * n, stream, bins);
        }
        if (rc == GBSW_OK && gbsw::results_rows(d_res.ptr, n, d_rows.ptr, stream) != cudaSuccess) rc = GBSW_ECUDA;
        if (rc == GBSW_OK && cudaMemcpyAsync(h_rows.ptr, d_rows.ptr, sizeof(int32_t) * 5 * (size_t)n,
                                             cudaMemcpyDeviceToHost, stream) != cudaSuccess)
            rc = GBSW_ECUDA;
        for (auto& j : batch) {  // blocks a failed gather did not reach, in stream order
            if (j->d_seq) cudaFreeAsync(j->d_seq, stream);
            j->d_seq = nullptr;
        }
        const int rc_check = gbsw_check(ctx, (void*)stream);  // waits for the stream; device-side input errors
        if (rc == GBSW_OK) rc = rc_check;
        if (rc != GBSW_OK) cudaGetLastError();
        if (rc == GBSW_OK) {
            int64_t off = 0;
            for (auto& j : batch) {  // each job's rows into its caller's array
                if (j->n > 0) std::memcpy(j->out, h_rows.ptr + 5 * off, sizeof(int32_t) * 5 * (size_t)j->n);
                off += j->n;
            }
        }
        {
            std::lock_guard<std::mutex> lock(mu);
            --running;
            ++done_batches;
        }
        finish(batch, rc);
    }
    cudaStreamDestroy(stream);
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
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return GBSW_ECUDA;  // no device can be opened
    }
    if (o.device < 0 || o.device >= count) return GBSW_EINVAL;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(o.device) != cudaSuccess) return GBSW_ECUDA;
    gbsw_server* s = new (std::nothrow) gbsw_server();
    if (!s) return GBSW_ENOMEM;
    s->opts = o;
    // the server's own pool for admitted jobs' device blocks: freed blocks stay
    // cached up to the budget instead of going back to the driver
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = o.device;
    cudaError_t e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = o.hbm_budget;
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) {
        // a block freed on a worker's stream is reused for an upload only once
        // its free has happened; the pool must not make the upload stream wait
        // for the freeing batch instead (which would chain every admission,
        // and so every next batch, behind the batches running now)
        int no = 0;
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->upload_stream, cudaStreamNonBlocking);
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        gbsw_server_destroy(s);
        return GBSW_ECUDA;
    }
    for (int k = 0; k < o.slots; ++k) s->workers.emplace_back([s] { s->worker(); });
    int rc;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv_done.wait(lock, [&] { return s->ready == o.slots; });
        rc = s->create_status;
    }
    s->uploader = std::thread([s] { s->upload_loop(); });
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
    s->cv_upload.notify_all();
    if (s->uploader.joinable()) s->uploader.join();  // every staged job is admitted by now
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop_workers = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    if (s->upload_stream) {
        cudaStreamSynchronize(s->upload_stream);
        cudaStreamDestroy(s->upload_stream);
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
}

}  // extern "C"

namespace {

// The checks and job-local offsets shared by both submit forms; nullptr and a
// status on a bad argument.
std::shared_ptr<Job> new_job(const gbsw_scoring* sc, const int64_t* ref_off, const int64_t* query_off, int64_t n,
                             int32_t* results, int* rc) {
    *rc = GBSW_EINVAL;
    if (!sc || !ref_off || !query_off || n < 0 || (n > 0 && !results)) return nullptr;
    if (sc->kind != GBSW_DNA && sc->kind != GBSW_PROTEIN) return nullptr;
    if (sc->gap_open > 0 || sc->gap_extend > 0) return nullptr;
    if (sc->kind == GBSW_PROTEIN && !sc->matrix) return nullptr;
    auto j = std::make_shared<Job>();
    j->sc = *sc;
    if (sc->kind == GBSW_PROTEIN) {
        j->matrix.assign(sc->matrix, sc->matrix + 576);
        j->sc.matrix = j->matrix.data();
    }
    j->n = n;
    j->out = results;
    j->ref_off.assign(ref_off, ref_off + n + 1);
    j->query_off.assign(query_off, query_off + n + 1);
    const int64_t long_cols = gbsw::long_bin_cols();
    for (int64_t k = 0; k < n; ++k) {
        const int64_t a = ref_off[k + 1] - ref_off[k], b = query_off[k + 1] - query_off[k];
        if (a < 0 || b < 0) return nullptr;
        j->long_pairs += std::min(a, b) >= long_cols ? 1 : 0;
        if (a > GBSW_MAX_SEQ_LEN || b > GBSW_MAX_SEQ_LEN) {
            *rc = GBSW_ELENGTH;
            return nullptr;
        }
        j->cells += a * b;
        j->footprint += pair_footprint(a, b);
        j->max_len = std::max(j->max_len, (int)std::max(a, b));
    }
    // job-local offsets from 0
    const int64_t r0 = ref_off[0], q0 = query_off[0];
    for (auto& v : j->ref_off) v -= r0;
    for (auto& v : j->query_off) v -= q0;
    j->ref_bytes = j->ref_off[(size_t)n];
    j->query_bytes = j->query_off[(size_t)n];
    *rc = GBSW_OK;
    return j;
}

// Queues a staged job (an empty one finishes at once).
int enqueue(gbsw_server* s, const std::shared_ptr<Job>& j, uint64_t* job_id) {
    j->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        j->id = s->next_id++;
        *job_id = j->id;
        s->jobs[j->id] = j;
        if (j->n == 0) {
            j->status = 0;
            j->t_admit = j->t_done = j->t_submit;
            return GBSW_OK;
        }
        s->staged.push_back(j);
    }
    s->cv_upload.notify_one();
    return GBSW_OK;
}

// A packed stream covering `need` symbols: words present, escape runs
// increasing, disjoint and inside it.
bool packed_ok(const gbsw_packed* p, int64_t need) {
    if (!p || p->nsym < need || p->nruns < 0 || (p->nsym > 0 && !p->words)) return false;
    if (p->nruns == 0) return true;
    if (!p->run_at || !p->run_off || !p->run_bytes || p->run_off[0] != 0) return false;
    int64_t end = 0;
    for (int64_t r = 0; r < p->nruns; ++r) {
        const int64_t len = p->run_off[r + 1] - p->run_off[r];
        if (len < 0 || p->run_at[r] < end || p->run_at[r] + len > p->nsym) return false;
        end = p->run_at[r] + len;
    }
    return true;
}

}  // namespace

extern "C" {

int gbsw_server_submit(gbsw_server* s, const gbsw_scoring* sc, const char* ref, const int64_t* ref_off,
                       const char* query, const int64_t* query_off, int64_t n, int32_t* results,
                       uint64_t* job_id) {
    if (!s || !job_id || (n > 0 && (!ref || !query))) return GBSW_EINVAL;
    int rc = GBSW_OK;
    auto j = new_job(sc, ref_off, query_off, n, results, &rc);
    if (!j) return rc;
    const int64_t r0 = ref_off[0], q0 = query_off[0];
    // Inputs are checked here, on the submitting thread, so that a job with a
    // bad symbol is refused alone instead of failing the batch it would share.
    if (sc->kind == GBSW_PROTEIN && (any_byte_at_least_91(ref + r0, (size_t)j->ref_bytes) ||
                                     any_byte_at_least_91(query + q0, (size_t)j->query_bytes)))
        return GBSW_ESYMBOL;
    j->stage_bytes = (size_t)(j->ref_bytes + j->query_bytes);
    if (n > 0) {
        if (!j->h_seq.reserve(std::max<size_t>(j->stage_bytes, 1))) return GBSW_ENOMEM;
        if (j->ref_bytes > 0) std::memcpy(j->h_seq.ptr, ref + r0, (size_t)j->ref_bytes);
        if (j->query_bytes > 0) std::memcpy(j->h_seq.ptr + j->ref_bytes, query + q0, (size_t)j->query_bytes);
    }
    return enqueue(s, j, job_id);
}

int gbsw_server_submit_packed(gbsw_server* s, const gbsw_scoring* scoring, const gbsw_packed* ref,
                              const int64_t* ref_off, const gbsw_packed* query, const int64_t* query_off, int64_t n,
                              int32_t* results, uint64_t* job_id) {
    if (!s || !job_id || !ref_off || !query_off || n < 0) return GBSW_EINVAL;
    if (ref_off[0] != 0 || query_off[0] != 0) return GBSW_EINVAL;  // the streams are the job's own
    int rc = GBSW_OK;
    auto j = new_job(scoring, ref_off, query_off, n, results, &rc);
    if (!j) return rc;
    if (n > 0 && (!packed_ok(ref, j->ref_bytes) || !packed_ok(query, j->query_bytes))) return GBSW_EINVAL;
    if (n == 0) return enqueue(s, j, job_id);
    // escaped bytes are the only ones that can fall outside the protein table
    const gbsw_packed* ps[2] = {ref, query};
    if (scoring->kind == GBSW_PROTEIN)
        for (const gbsw_packed* p : ps)
            if (p->nruns > 0 &&
                any_byte_at_least_91(reinterpret_cast<const char*>(p->run_bytes), (size_t)p->run_off[p->nruns]))
                return GBSW_ESYMBOL;
    // staging: both streams' words, run positions, offsets and bytes, each part 16-byte aligned
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    PackedLayout& L = j->lay;
    size_t at = 0;
    for (int x = 0; x < 2; ++x) {
        const gbsw_packed* p = ps[x];
        L.nsym[x] = x ? j->query_bytes : j->ref_bytes;
        L.nruns[x] = p->nruns;
        L.words[x] = at;
        at += up16(4 * (size_t)gbsw_packed_words(scoring->kind, L.nsym[x]));
        L.run_at[x] = at;
        at += up16(8 * (size_t)p->nruns);
        L.run_off[x] = at;
        at += up16(8 * (size_t)(p->nruns + 1));
        L.run_bytes[x] = at;
        at += up16(p->nruns > 0 ? (size_t)p->run_off[p->nruns] : 0);
    }
    j->stage_bytes = at;
    j->packed = true;
    if (!j->h_seq.reserve(std::max<size_t>(at, 1))) return GBSW_ENOMEM;
    for (int x = 0; x < 2; ++x) {
        const gbsw_packed* p = ps[x];
        const size_t wbytes = 4 * (size_t)gbsw_packed_words(scoring->kind, L.nsym[x]);
        if (wbytes) std::memcpy(j->h_seq.ptr + L.words[x], p->words, wbytes);
        if (p->nruns > 0) {
            std::memcpy(j->h_seq.ptr + L.run_at[x], p->run_at, 8 * (size_t)p->nruns);
            std::memcpy(j->h_seq.ptr + L.run_off[x], p->run_off, 8 * (size_t)(p->nruns + 1));
            std::memcpy(j->h_seq.ptr + L.run_bytes[x], p->run_bytes, (size_t)p->run_off[p->nruns]);
        } else {
            const int64_t zero = 0;
            std::memcpy(j->h_seq.ptr + L.run_off[x], &zero, 8);
        }
    }
    return enqueue(s, j, job_id);
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
    st->queued = (int64_t)(s->staged.size() + s->resident.size());
    st->hbm_in_use = s->used;
    st->staged = (int64_t)s->staged.size();
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
