// Launch interface of the Smith-Waterman pass kernels (host side).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sw_common.cuh"

namespace gbsw {

int pass_threads();
// Strip-edge buffers a block of the int32 passes uses: one per group of
// `width` lanes, one per warp for block-per-pair teams (width kTeamLanes).
int pass_groups_per_block(int width);
// Lanes per pair ("width") of the int32 passes: 4 (kG, every variant) or 8, 16,
// 32 (DPX variants, for small batches), or kTeamLanes (block per pair, DPX).
// pass_columns gives the columns per lane of a width (0 if unsupported).
int pass_columns(int width);
size_t pass_dynamic_smem(int score, int width);
// `score` is one of the ScoreMode values.
cudaError_t pass_occupancy(int score, bool reverse, bool dpx, int width, int* blocks_per_sm);
cudaError_t launch_pass(int score, bool reverse, bool dpx, int width, const PassParams& p, int blocks,
                        cudaStream_t stream);
// Kernel of a wide variant (sw_wide.cu), nullptr if none.
const void* pick_wide(int width, int score, bool reverse);
// Dual-pair int16x2 passes (class kClassDual), sw_dual.cu: DNA at width 4,
// protein (`aa`) at widths 16 and 32.  has_dual tells whether a variant exists.
bool has_dual(bool aa, int width);
// Lanes per group of the dual variant a plan of `width` runs (sizes its scratch).
int dual_lanes(bool aa, int width);
cudaError_t launch_pass_dual(bool reverse, bool aa, int width, const PassParams& p, int blocks,
                             cudaStream_t stream);
cudaError_t pass_dual_occupancy(bool reverse, bool aa, int width, int* blocks_per_sm);

}  // namespace gbsw
