// ref_harness -- drives the reference's own driver (gpu_bsw_driver::kernel_driver_dna /
// kernel_driver_aa, compiled from the reference sources by oracle/build_ref.sh) on
// pairs read from a file, and writes its five result arrays.
//
// TEST INFRASTRUCTURE ONLY: used to produce golden fixtures and to time the
// reference's kernels on the same GPU.  Never linked into the product.
//
// usage: ref_harness dna <pairs.tsv> <out.tsv> <match> <mismatch> <open> <extend>
//        ref_harness aa  <pairs.tsv> <out.tsv> <matrix.txt> <open> <extend>
// pairs.tsv: one pair per line, "reference<TAB>query".
// out.tsv:   "score ref_begin ref_end query_begin query_end" per pair (raw arrays).
// stderr:    one JSON line {"pairs":..,"cells":..,"seconds":..,"kernel_seconds":..,"launches":..,
//            "reps":..} -- the fastest wall time of GBSW_REF_REPS (default 1) calls, after CUDA
//            context creation, and the fastest kernel time of those calls.
//
// Kernel time.  Built by oracle/build_ref.sh, the harness is linked with
// -Wl,--wrap=__cudaLaunchKernel: every kernel launch the reference's driver
// compiles to (the runtime's launch entry, declared in crt/device_functions.h)
// reaches __wrap___cudaLaunchKernel below, which brackets it with two events on
// the launch's own stream and then launches it unchanged.  A call's kernel time
// is the union of those [start, end] intervals on the GPU timeline (its two
// streams overlap), so it leaves out the driver's host packing, copies and host
// synchronisation.  Built against another driver (GBSW_REF_WRAP_LAUNCH undefined)
// it reports kernel_seconds = -1.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "driver.hpp"
#include "utils.hpp"

namespace {
constexpr int kMaxLaunches = 2048;
cudaEvent_t g_ev[2 * kMaxLaunches];
int g_launches = 0;
bool g_timing = false;
}  // namespace

#ifdef GBSW_REF_WRAP_LAUNCH
extern "C" cudaError_t __real___cudaLaunchKernel(cudaKernel_t, dim3, dim3, void**, size_t, cudaStream_t);
extern "C" cudaError_t __wrap___cudaLaunchKernel(cudaKernel_t kernel, dim3 grid, dim3 block, void** args,
                                                 size_t smem, cudaStream_t stream) {
    if (!g_timing || g_launches >= kMaxLaunches) return __real___cudaLaunchKernel(kernel, grid, block, args, smem, stream);
    cudaEventRecord(g_ev[2 * g_launches], stream);
    const cudaError_t r = __real___cudaLaunchKernel(kernel, grid, block, args, smem, stream);
    cudaEventRecord(g_ev[2 * g_launches + 1], stream);
    ++g_launches;
    return r;
}
#endif

// Union of the recorded launch intervals, in seconds (-1 when nothing was recorded).
static double kernel_union_seconds() {
    if (g_launches == 0) return -1.0;
    cudaDeviceSynchronize();
    std::vector<std::pair<float, float>> iv;
    for (int k = 0; k < g_launches; ++k) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, g_ev[0], g_ev[2 * k]);
        cudaEventElapsedTime(&b, g_ev[0], g_ev[2 * k + 1]);
        iv.push_back({a, b});
    }
    std::sort(iv.begin(), iv.end());
    double total = 0.0, lo = iv[0].first, hi = iv[0].second;
    for (size_t k = 1; k < iv.size(); ++k) {
        if (iv[k].first > hi) {
            total += hi - lo;
            lo = iv[k].first;
            hi = iv[k].second;
        } else if (iv[k].second > hi) {
            hi = iv[k].second;
        }
    }
    total += hi - lo;
    return total / 1e3;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s dna|aa pairs.tsv out.tsv ...\n", argv[0]);
        return 2;
    }
    std::string mode = argv[1];
    std::ifstream in(argv[2]);
    if (!in) {
        std::fprintf(stderr, "cannot read %s\n", argv[2]);
        return 2;
    }
    std::vector<std::string> contigs, reads;
    std::string line;
    long long cells = 0;
    while (std::getline(in, line)) {
        size_t tab = line.find('\t');
        if (tab == std::string::npos) continue;
        contigs.push_back(line.substr(0, tab));
        reads.push_back(line.substr(tab + 1));
        cells += (long long)contigs.back().size() * (long long)reads.back().size();
    }
    gpu_bsw_driver::alignment_results res;
    int reps = std::getenv("GBSW_REF_REPS") ? std::atoi(std::getenv("GBSW_REF_REPS")) : 1;
    if (reps < 1) reps = 1;
    cudaFree(0);  // create the CUDA context outside the timed calls
    for (int k = 0; k < 2 * kMaxLaunches; ++k) cudaEventCreate(&g_ev[k]);
    std::vector<short> mat;
    if (mode != "dna") {
        if (argc < 7) return 2;
        std::ifstream mf(argv[4]);
        int v;
        while (mf >> v) mat.push_back((short)v);
        if (mat.size() != 576) {
            std::fprintf(stderr, "matrix file must hold 576 integers\n");
            return 2;
        }
    } else if (argc < 8) {
        return 2;
    }
    double best = 1e30, best_kernel = -1.0;
    int launches = 0;
    for (int r = 0; r < reps; ++r) {
        if (r > 0) free_alignments(&res);
        g_launches = 0;
        g_timing = true;
        auto t0 = std::chrono::steady_clock::now();
        if (mode == "dna") {
            short scores[4] = {(short)std::atoi(argv[4]), (short)std::atoi(argv[5]),
                               (short)std::atoi(argv[6]), (short)std::atoi(argv[7])};
            gpu_bsw_driver::kernel_driver_dna(reads, contigs, &res, scores, 0.5);
        } else {
            gpu_bsw_driver::kernel_driver_aa(reads, contigs, &res, mat.data(),
                                             (short)std::atoi(argv[5]), (short)std::atoi(argv[6]), 0.5);
        }
        std::chrono::duration<double> dt = std::chrono::steady_clock::now() - t0;
        g_timing = false;
        if (dt.count() < best) best = dt.count();
        const double kt = kernel_union_seconds();
        if (kt >= 0 && (best_kernel < 0 || kt < best_kernel)) best_kernel = kt;
        launches = g_launches;
    }
    FILE* out = std::fopen(argv[3], "w");
    if (!out) return 2;
    for (size_t k = 0; k < contigs.size(); ++k)
        std::fprintf(out, "%d\t%d\t%d\t%d\t%d\n", res.top_scores[k], res.ref_begin[k], res.ref_end[k],
                     res.query_begin[k], res.query_end[k]);
    std::fclose(out);
    std::fprintf(stderr,
                 "{\"pairs\": %zu, \"cells\": %lld, \"seconds\": %.6f, \"kernel_seconds\": %.6f, "
                 "\"launches\": %d, \"reps\": %d}\n",
                 contigs.size(), cells, best, best_kernel, launches, reps);
    return 0;
}
