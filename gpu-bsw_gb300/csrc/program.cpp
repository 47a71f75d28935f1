// program_gpu -- command-line front end with the reference's I/O conventions
// (main.cpp:13-248 of ADEPT / GPU-BSW), over the C++ drop-in gpu_bsw/driver.hpp.
//
//   program_gpu dna|aa REF.fasta QUERY.fasta OUT.tsv [--scores M,X,O,E] [--gaps O,E] [--factor F]
//
// Input, as the reference reads it: every line that does not start with '>' is
// one sequence (single-line FASTA; an empty line is an empty sequence; nothing
// is stripped from a line).  Pair k is the k-th reference sequence against the
// k-th query sequence.
// Output: one line per pair, tab-separated: score, ref_begin, ref_end - 1,
// query_begin, query_end - 1 (main.cpp:130-137, 214-221); a pair without a
// positive score prints 0 -1 -2 -1 -2.  Then "Total Cells:N" on stdout, N the
// sum of |ref| * |query| (main.cpp:141-146, 226-230).
// Scoring defaults are the reference program's: DNA match 1, mismatch -3, gap
// open -3, extend -1 (main.cpp:210); protein BLOSUM62 with open -6, extend -1
// (main.cpp:70-123); memory factor 0.5.  --scores / --gaps / --factor change them.
// Differences: the mode must be "dna" or "aa" (the reference runs anything but
// "aa" as DNA); a usage error or unequal sequence counts exit with status 2.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "gpu_bsw/driver.hpp"
#include "gpu_bsw/utils.hpp"

namespace {

// BLOSUM62, rows and columns in the order A R N D C Q E G H I L K M F P S T W Y V B Z X *
// (the reference program's matrix, main.cpp:70-92).
short kBlosum62[576] = {
     4, -1, -2, -2,  0, -1, -1,  0, -2, -1, -1, -1, -1, -2, -1,  1,  0, -3, -2,  0, -2, -1,  0, -4,  // A
    -1,  5,  0, -2, -3,  1,  0, -2,  0, -3, -2,  2, -1, -3, -2, -1, -1, -3, -2, -3, -1,  0, -1, -4,  // R
    -2,  0,  6,  1, -3,  0,  0,  0,  1, -3, -3,  0, -2, -3, -2,  1,  0, -4, -2, -3,  3,  0, -1, -4,  // N
    -2, -2,  1,  6, -3,  0,  2, -1, -1, -3, -4, -1, -3, -3, -1,  0, -1, -4, -3, -3,  4,  1, -1, -4,  // D
     0, -3, -3, -3,  9, -3, -4, -3, -3, -1, -1, -3, -1, -2, -3, -1, -1, -2, -2, -1, -3, -3, -2, -4,  // C
    -1,  1,  0,  0, -3,  5,  2, -2,  0, -3, -2,  1,  0, -3, -1,  0, -1, -2, -1, -2,  0,  3, -1, -4,  // Q
    -1,  0,  0,  2, -4,  2,  5, -2,  0, -3, -3,  1, -2, -3, -1,  0, -1, -3, -2, -2,  1,  4, -1, -4,  // E
     0, -2,  0, -1, -3, -2, -2,  6, -2, -4, -4, -2, -3, -3, -2,  0, -2, -2, -3, -3, -1, -2, -1, -4,  // G
    -2,  0,  1, -1, -3,  0,  0, -2,  8, -3, -3, -1, -2, -1, -2, -1, -2, -2,  2, -3,  0,  0, -1, -4,  // H
    -1, -3, -3, -3, -1, -3, -3, -4, -3,  4,  2, -3,  1,  0, -3, -2, -1, -3, -1,  3, -3, -3, -1, -4,  // I
    -1, -2, -3, -4, -1, -2, -3, -4, -3,  2,  4, -2,  2,  0, -3, -2, -1, -2, -1,  1, -4, -3, -1, -4,  // L
    -1,  2,  0, -1, -3,  1,  1, -2, -1, -3, -2,  5, -1, -3, -1,  0, -1, -3, -2, -2,  0,  1, -1, -4,  // K
    -1, -1, -2, -3, -1,  0, -2, -3, -2,  1,  2, -1,  5,  0, -2, -1, -1, -1, -1,  1, -3, -1, -1, -4,  // M
    -2, -3, -3, -3, -2, -3, -3, -3, -1,  0,  0, -3,  0,  6, -4, -2, -2,  1,  3, -1, -3, -3, -1, -4,  // F
    -1, -2, -2, -1, -3, -1, -1, -2, -2, -3, -3, -1, -2, -4,  7, -1, -1, -4, -3, -2, -2, -1, -2, -4,  // P
     1, -1,  1,  0, -1,  0,  0,  0, -1, -2, -2,  0, -1, -2, -1,  4,  1, -3, -2, -2,  0,  0,  0, -4,  // S
     0, -1,  0, -1, -1, -1, -1, -2, -2, -1, -1, -1, -1, -2, -1,  1,  5, -2, -2,  0, -1, -1,  0, -4,  // T
    -3, -3, -4, -4, -2, -2, -3, -2, -2, -3, -2, -3, -1,  1, -4, -3, -2, 11,  2, -3, -4, -3, -2, -4,  // W
    -2, -2, -2, -3, -2, -1, -2, -3,  2, -1, -1, -2, -1,  3, -3, -2, -2,  2,  7, -1, -3, -2, -1, -4,  // Y
     0, -3, -3, -3, -1, -2, -2, -3, -3,  3,  1, -2,  1, -1, -2, -2,  0, -3, -1,  4, -3, -2, -1, -4,  // V
    -2, -1,  3,  4, -3,  0,  1, -1,  0, -3, -4,  0, -3, -3, -2,  0, -1, -4, -3, -3,  4,  1, -1, -4,  // B
    -1,  0,  0,  1, -3,  3,  4, -2,  0, -3, -3,  1, -1, -3, -1,  0, -1, -3, -2, -2,  1,  4, -1, -4,  // Z
     0, -1, -1, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2,  0,  0, -2, -1, -1, -1, -1, -1, -4,  // X
    -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4,  1,  // *
};

int usage(const char* why) {
    std::fprintf(stderr,
                 "program_gpu: %s\n"
                 "usage: program_gpu dna|aa REF.fasta QUERY.fasta OUT.tsv [--scores M,X,O,E] [--gaps O,E] "
                 "[--factor F]\n",
                 why);
    return 2;
}

bool read_sequences(const char* path, std::vector<std::string>* out) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line[0] == '>') continue;
        out->push_back(line);
    }
    return true;
}

// "a,b,c" -> n shorts; false on a malformed list
bool parse_shorts(const char* s, short* v, int n) {
    for (int k = 0; k < n; ++k) {
        char* end = nullptr;
        long x = std::strtol(s, &end, 10);
        if (end == s || x < -32768 || x > 32767) return false;
        v[k] = (short)x;
        if (k + 1 < n) {
            if (*end != ',') return false;
            s = end + 1;
        } else if (*end != '\0') {
            return false;
        }
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) return usage("missing arguments");
    const std::string mode = argv[1];
    if (mode != "dna" && mode != "aa") return usage("mode must be dna or aa");
    short scores[4] = {1, -3, -3, -1};
    short gaps[2] = {-6, -1};
    float factor = 0.5f;
    for (int k = 5; k < argc; ++k) {
        const std::string a = argv[k];
        if (a == "--scores" && k + 1 < argc) {
            if (!parse_shorts(argv[++k], scores, 4)) return usage("--scores wants M,X,O,E");
        } else if (a == "--gaps" && k + 1 < argc) {
            if (!parse_shorts(argv[++k], gaps, 2)) return usage("--gaps wants O,E");
        } else if (a == "--factor" && k + 1 < argc) {
            factor = std::strtof(argv[++k], nullptr);
            if (!(factor > 0.0f && factor <= 1.0f)) return usage("--factor wants a value in (0, 1]");
        } else {
            return usage(("unknown option " + a).c_str());
        }
    }
    std::vector<std::string> refs, queries;
    if (!read_sequences(argv[2], &refs)) return usage((std::string("cannot read ") + argv[2]).c_str());
    if (!read_sequences(argv[3], &queries)) return usage((std::string("cannot read ") + argv[3]).c_str());
    if (refs.size() != queries.size()) {
        std::fprintf(stderr, "program_gpu: %zu reference sequences but %zu query sequences\n", refs.size(),
                     queries.size());
        return 2;
    }
    std::ofstream out(argv[4]);
    if (!out.is_open()) return usage((std::string("cannot write ") + argv[4]).c_str());

    gpu_bsw_driver::alignment_results r;
    if (mode == "aa")
        gpu_bsw_driver::kernel_driver_aa(queries, refs, &r, kBlosum62, gaps[0], gaps[1], factor);
    else
        gpu_bsw_driver::kernel_driver_dna(queries, refs, &r, scores, factor);

    std::string buf;
    buf.reserve(1 << 20);
    char line[96];
    long long cells = 0;
    for (size_t k = 0; k < refs.size(); ++k) {
        std::snprintf(line, sizeof line, "%d\t%d\t%d\t%d\t%d\n", r.top_scores[k], r.ref_begin[k], r.ref_end[k] - 1,
                      r.query_begin[k], r.query_end[k] - 1);
        buf += line;
        if (buf.size() > (1u << 20) - 128) {
            out << buf;
            buf.clear();
        }
        cells += (long long)refs[k].size() * (long long)queries[k].size();
    }
    out << buf;
    out.close();
    free_alignments(&r);
    if (!out) {
        std::fprintf(stderr, "program_gpu: error writing %s\n", argv[4]);
        return 1;
    }
    std::cout << "Total Cells:" << cells << std::endl;
    return 0;
}
