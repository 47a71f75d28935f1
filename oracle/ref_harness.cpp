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
// stderr:    one JSON line {"pairs":..,"cells":..,"seconds":..,"reps":..} -- the fastest wall
//            time of GBSW_REF_REPS (default 1) calls, after CUDA context creation.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "driver.hpp"
#include "utils.hpp"

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
    double best = 1e30;
    for (int r = 0; r < reps; ++r) {
        if (r > 0) free_alignments(&res);
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
        if (dt.count() < best) best = dt.count();
    }
    FILE* out = std::fopen(argv[3], "w");
    if (!out) return 2;
    for (size_t k = 0; k < contigs.size(); ++k)
        std::fprintf(out, "%d\t%d\t%d\t%d\t%d\n", res.top_scores[k], res.ref_begin[k], res.ref_end[k],
                     res.query_begin[k], res.query_end[k]);
    std::fclose(out);
    std::fprintf(stderr, "{\"pairs\": %zu, \"cells\": %lld, \"seconds\": %.6f, \"reps\": %d}\n",
                 contigs.size(), cells, best, reps);
    return 0;
}
