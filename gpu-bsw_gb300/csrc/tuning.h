// The tuning table a context starts with: per (kind, length bin, pair-count
// bucket) the kernel variant measured fastest on GB300 (gbsw_tuning in gbsw.h).
// The entries come from gpu-bsw_gb300/tune_sweep.py, which runs gbsw_tune_device
// over synthetic batches of each bin and bucket and writes tuning_gb300.inc.
#pragma once
#include "../../include/gbsw.h"

namespace gbsw {

inline gbsw_tuning builtin_tuning() {
    gbsw_tuning t{};
#include "tuning_gb300.inc"
    return t;
}

}  // namespace gbsw
