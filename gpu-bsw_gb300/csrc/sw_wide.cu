// Wide-group instantiations of the int32 passes (sw_pass.cuh) for small batches:
// 8 lanes x 8 columns, 16 lanes x 8 columns and 32 lanes x 4 columns per pair,
// and block per pair ("128 lanes"): the block's four warps of 32 lanes x 8
// columns share one pair, a warp per column strip.  A batch too small to fill
// the GPU with 4-lane groups finishes when its longest pair does; spreading
// each pair over more lanes, each with fewer columns, shortens that serial
// time.  DPX forms only.
#include "sw_pass.cuh"
#include "sw_kernels.h"

namespace gbsw {

const void* pick_wide(int width, int score, bool reverse) {
#define GBSW_PICK_W(S, G, C)                                                                         \
    if (score == S) return reverse ? kernel_ptr<S, true, true, G, C>() : kernel_ptr<S, false, true, G, C>();
#define GBSW_PICK_ALL(G, C)               \
    GBSW_PICK_W(kScoreDnaProfile, G, C)   \
    GBSW_PICK_W(kScoreDnaRaw, G, C)       \
    GBSW_PICK_W(kScoreAaProfile, G, C)    \
    GBSW_PICK_W(kScoreAaWide, G, C)       \
    return nullptr;
#define GBSW_PICK_T(S, C)                                                                                     \
    if (score == S) return reverse ? kernel_ptr<S, true, true, 32, C, kThreads / 32>()                         \
                                   : kernel_ptr<S, false, true, 32, C, kThreads / 32>();
    switch (width) {
        case 8: { GBSW_PICK_ALL(8, 8) }
        case 16: { GBSW_PICK_ALL(16, 8) }
        case 32: { GBSW_PICK_ALL(32, 4) }
        case kTeamLanes: {
            GBSW_PICK_T(kScoreDnaProfile, kTeamColumns)
            GBSW_PICK_T(kScoreDnaRaw, kTeamColumns)
            GBSW_PICK_T(kScoreAaProfile, kTeamColumns)
            GBSW_PICK_T(kScoreAaWide, kTeamColumns)
            return nullptr;
        }
        default: return nullptr;
    }
#undef GBSW_PICK_T
#undef GBSW_PICK_ALL
#undef GBSW_PICK_W
}

}  // namespace gbsw
