// Launch interface of the Smith-Waterman pass kernels (host side).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sw_common.cuh"

namespace gbsw {

// Lanes per pair and columns per lane of the pass kernels.
constexpr int kGroupLanes = 8;
constexpr int kColsPerLane = 8;

struct PassConfig {
    bool protein = false;
    bool dpx = true;
};

int pass_threads();
int pass_group_lanes(const PassConfig& cfg);
cudaError_t pass_occupancy(const PassConfig& cfg, bool reverse, int* blocks_per_sm);
cudaError_t launch_pass(const PassConfig& cfg, bool reverse, const PassParams& p, int blocks,
                        cudaStream_t stream);

}  // namespace gbsw
