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
// Dual-pair int16x2 DNA passes (class kClassDual), sw_dual.cu.
cudaError_t launch_pass_dual(bool reverse, const PassParams& p, int blocks, cudaStream_t stream);
cudaError_t pass_dual_occupancy(bool reverse, int* blocks_per_sm);

}  // namespace gbsw
