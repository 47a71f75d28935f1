// Result layout kernels shared by the host-side callers of the passes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsw {

// The passes' results as five arrays (score, ref_begin, ref_end, query_begin,
// query_end; n each) -> one row of five per pair, rows[5 * k + f], on `stream`.
cudaError_t results_rows(const int32_t* soa, int64_t n, int32_t* rows, cudaStream_t stream);

}  // namespace gbsw
