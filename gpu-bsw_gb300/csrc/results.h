// Result layout kernels shared by the host-side callers of the passes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gbsw.h"

namespace gbsw {

// The passes' results as five arrays (score, ref_begin, ref_end, query_begin,
// query_end; n each) -> one row of five per pair, rows[5 * k + f], on `stream`.
cudaError_t results_rows(const int32_t* soa, int64_t n, int32_t* rows, cudaStream_t stream);

// Shorter side from which a pair belongs to the long length bin.
int long_bin_cols();

// gbsw_align_device for a caller that already knows, on the host, how many
// pairs fall in each length bin (bin_pairs[0] short, [1] long; upper bounds
// suffice: pairs that leave the bins on the device -- raw-byte DNA -- may be
// counted).  The per-bin plan then comes from these counts, with no wait for
// the device's own counts between the schedule and the passes.
int align_device_known_bins(gbsw_context* ctx, const gbsw_scoring* scoring, const uint8_t* ref,
                            const int64_t* ref_off, const uint8_t* query, const int64_t* query_off, int64_t n,
                            int32_t max_len, int32_t* top_scores, int32_t* ref_begin, int32_t* ref_end,
                            int32_t* query_begin, int32_t* query_end, cudaStream_t stream,
                            const int64_t bin_pairs[2]);

}  // namespace gbsw
