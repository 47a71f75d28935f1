// Work schedule of the pass kernels (host interface).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsw {

struct SchedParams {
    const uint8_t* ref;
    const int64_t* ref_off;
    const uint8_t* query;
    const int64_t* query_off;
    int64_t n;
    int protein;          // 1: check protein bytes against the encoding table
    int dna_profile_ok;   // 1: DNA scores fit the int8 profile (A/C/G/T pairs can use it)
    int binned;           // 1: A/C/G/T (DNA) or profile-scored (protein) pairs go to the length-bin
                          //    classes (kClassShort, kClassLong), each with its own plan
    int match;            // reverse keys: the DNA match score and the column bound cost
    int rev_p;            //   of reverse_columns (0: no bound)
    int dual_limit;       // reverse keys: a pair of a bin whose reverse plan is dual (bit 0 of
    int rev_dual_bins;    //   rev_dual_bins: short bin, bit 1: long bin) and whose score is above
                          //   dual_limit runs its reverse pass in class 0 (int32), so that a
                          //   dual-pair reverse launch never holds one
    const int32_t* score; // reverse keys: forward results
    const int32_t* ref_end;
    const int32_t* query_end;
    uint8_t* cls;         // per pair: class of the forward pass
    int* keys;            // per pair: bucket
    int* hist;            // kBuckets counters, then exclusive offsets
    int* class_range;     // 2 * kRanges ints: [begin, end) of each class, then of the two bins
    int* order;           // n pair indices in schedule order
    int* error;
};

// Enqueues the schedule kernels of one pass on `stream`.
cudaError_t build_schedule(const SchedParams& s, bool reverse, int sms, cudaStream_t stream);

}  // namespace gbsw
