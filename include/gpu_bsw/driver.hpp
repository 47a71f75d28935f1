/*
 * gpu_bsw/driver.hpp -- source-compatible drop-in for the reference's driver
 * API (driver.hpp:18-42 of ADEPT / GPU-BSW), implemented over the C ABI of
 * gbsw.h.  Like the reference (driver.cpp:23-41), a call spreads over every
 * visible GPU, one host thread each; GBSW_DEVICES="0,2" restricts it to a list.
 *
 * Same namespace, struct and signatures.  Behaviour kept:
 *   - reads are the queries (seqB), contigs the references (seqA), pair k is
 *     contigs[k] against reads[k]; the vectors must have the same length;
 *   - the five result arrays are allocated with cudaMallocHost into the
 *     caller's struct and released by free_alignments() (utils.hpp:25);
 *   - `factor` is the share of device memory one call may use; larger batches
 *     run in chunks (driver.cpp:51-55);
 *   - on failure the call prints a message to stderr and exits the process
 *     with a non-zero status, as the reference's gpuAssert does (utils.hpp:5-21).
 * Differences: the pairs are split between GPUs into contiguous ranges of
 * near-equal cells (gbsw_split_pairs), not equal pair counts; the caller's
 * current device is left as it was; ties, lengths above 1,024 and batches of
 * one pair all work;
 * nothing is printed on success unless GBSW_VERBOSE=1 is set in the
 * environment; a pair with no positive score reports 0 and -1 positions.
 */
#ifndef GPU_BSW_DRIVER_HPP
#define GPU_BSW_DRIVER_HPP

#include <cstddef>
#include <string>
#include <vector>

namespace gpu_bsw_driver {

// for storing the alignment results (driver.hpp:21-27 of the reference)
struct alignment_results {
    short* ref_begin;
    short* query_begin;
    short* ref_end;
    short* query_end;
    short* top_scores;
};

size_t get_tot_gpu_mem(int id);

void kernel_driver_dna(std::vector<std::string> reads, std::vector<std::string> contigs,
                       alignment_results* alignments, short scores[4], float factor = 1.0);

void kernel_driver_aa(std::vector<std::string> reads, std::vector<std::string> contigs,
                      alignment_results* alignments, short scoring_matrix[], short openGap,
                      short extendGap, float factor = 1.0);

}  // namespace gpu_bsw_driver

#endif
