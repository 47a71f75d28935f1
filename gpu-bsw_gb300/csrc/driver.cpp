// C++ drop-in for gpu_bsw_driver::kernel_driver_dna / kernel_driver_aa
// (reference driver.hpp:18-42, driver.cpp:10-489, utils.cpp:13-28) over the
// C ABI of gbsw.h, on the current CUDA device.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbsw.h"
#include "../../include/gpu_bsw/driver.hpp"
#include "../../include/gpu_bsw/utils.hpp"

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

// One context per device for the life of the process.
gbsw_context* context_for_current_device() {
    static std::mutex mu;
    static std::map<int, gbsw_context*> contexts;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) die("cudaGetDevice", GBSW_ECUDA, nullptr);
    std::lock_guard<std::mutex> lock(mu);
    auto it = contexts.find(dev);
    if (it != contexts.end()) return it->second;
    gbsw_context* ctx = nullptr;
    int rc = gbsw_create(dev, &ctx);
    if (rc != GBSW_OK) die("gbsw_create", rc, nullptr);
    contexts[dev] = ctx;
    return ctx;
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

struct Packed {
    std::vector<char> ref, query;
    std::vector<int64_t> ref_off, query_off;
};

void pack(const std::vector<std::string>& contigs, const std::vector<std::string>& reads,
          size_t begin, size_t end, Packed* p) {
    size_t n = end - begin;
    p->ref_off.assign(n + 1, 0);
    p->query_off.assign(n + 1, 0);
    size_t ra = 0, qa = 0;
    for (size_t k = 0; k < n; ++k) {
        ra += contigs[begin + k].size();
        qa += reads[begin + k].size();
        p->ref_off[k + 1] = (int64_t)ra;
        p->query_off[k + 1] = (int64_t)qa;
    }
    p->ref.resize(ra ? ra : 1);
    p->query.resize(qa ? qa : 1);
    for (size_t k = 0; k < n; ++k) {
        const std::string& a = contigs[begin + k];
        const std::string& b = reads[begin + k];
        if (!a.empty()) std::memcpy(p->ref.data() + p->ref_off[k], a.data(), a.size());
        if (!b.empty()) std::memcpy(p->query.data() + p->query_off[k], b.data(), b.size());
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
    gbsw_context* ctx = context_for_current_device();

    // Chunk so that one call stays within `factor` of device memory
    // (driver.cpp:36, 51-55): bytes of both sequences plus offsets and results.
    int dev = 0;
    cudaGetDevice(&dev);
    uint64_t mem = 0;
    if (gbsw_device_memory(dev, &mem) != GBSW_OK) die("get_tot_gpu_mem", GBSW_ECUDA, ctx);
    double f = factor > 0 && factor <= 1 ? factor : 1.0;
    // leave room for the strip boundary buffers (sized by the longest sequence)
    const double budget = (double)mem * f * 0.5;
    Packed pk;
    size_t begin = 0;
    while (begin < n) {
        size_t end = begin;
        double bytes = 0;
        while (end < n) {
            double need = (double)contigs[end].size() + (double)reads[end].size() + 16.0 + 20.0;
            if (end > begin && bytes + need > budget) break;
            bytes += need;
            ++end;
        }
        pack(contigs, reads, begin, end, &pk);
        int rc = gbsw_align_host16(ctx, &sc, pk.ref.data(), pk.ref_off.data(), pk.query.data(),
                                   pk.query_off.data(), (int64_t)(end - begin), out->ref_begin + begin,
                                   out->ref_end + begin, out->query_begin + begin,
                                   out->query_end + begin, out->top_scores + begin);
        if (rc != GBSW_OK) die("alignment", rc, ctx);
        begin = end;
    }
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
    }
}

}  // namespace

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
