// Forward (end-position) and reverse (begin-position) Smith-Waterman passes,
// int32 scores, sm_103a: the 4-lane-group instantiations of the kernel template
// in sw_pass.cuh and the launch interface of all int32 variants.
#include "sw_pass.cuh"
#include "sw_kernels.h"

namespace gbsw {

namespace {

const void* pick4(int score, bool reverse, bool dpx) {
#define GBSW_PICK(S)                                                                       \
    if (score == S) {                                                                      \
        if (reverse) return dpx ? kernel_ptr<S, true, true, kG, kC>()                      \
                                : kernel_ptr<S, true, false, kG, kC>();                    \
        return dpx ? kernel_ptr<S, false, true, kG, kC>() : kernel_ptr<S, false, false, kG, kC>(); \
    }
    GBSW_PICK(kScoreDnaProfile)
    GBSW_PICK(kScoreDnaRaw)
    GBSW_PICK(kScoreAaProfile)
    GBSW_PICK(kScoreAaWide)
#undef GBSW_PICK
    return nullptr;
}

const void* pick(int score, bool reverse, bool dpx, int width) {
    if (width == kG) return pick4(score, reverse, dpx);
    return dpx ? pick_wide(width, score, reverse) : nullptr;
}

}  // namespace

int pass_threads() { return kThreads; }

int pass_groups_per_block(int width) { return kThreads / (width < 32 ? width : 32); }

int pass_columns(int width) {
    switch (width) {
        case 4: return kC;
        case 8: return 8;
        case 16: return 8;
        case 32: return 4;
        case kTeamLanes: return kTeamColumns;
        default: return 0;
    }
}

size_t pass_dynamic_smem(int score, int width) {
    // one kAAProfRows x (width * columns) int8 profile per group
    return score == kScoreAaProfile ? (size_t)kThreads * kAAProfRows * (size_t)pass_columns(width) : 0;
}

cudaError_t pass_occupancy(int score, bool reverse, bool dpx, int width, int* blocks_per_sm) {
    const void* fn = pick(score, reverse, dpx, width);
    if (!fn) return cudaErrorInvalidValue;
    const size_t dyn = pass_dynamic_smem(score, width);
    if (dyn > 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kThreads, dyn);
}

cudaError_t launch_pass(int score, bool reverse, bool dpx, int width, const PassParams& p, int blocks,
                        cudaStream_t stream) {
    const void* fn = pick(score, reverse, dpx, width);
    if (!fn) return cudaErrorInvalidValue;
    const size_t dyn = pass_dynamic_smem(score, width);
    if (dyn > 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    void* args[] = {(void*)&p};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(kThreads), args, dyn, stream);
}

}  // namespace gbsw
