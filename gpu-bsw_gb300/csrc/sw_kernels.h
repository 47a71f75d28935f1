// Launch interface of the Smith-Waterman pass kernels (host side).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sw_common.cuh"

namespace gbsw {

int pass_threads();
size_t pass_dynamic_smem(int score);
// `score` is one of the ScoreMode values.
cudaError_t pass_occupancy(int score, bool reverse, bool dpx, int* blocks_per_sm);
cudaError_t launch_pass(int score, bool reverse, bool dpx, const PassParams& p, int blocks,
                        cudaStream_t stream);

}  // namespace gbsw
