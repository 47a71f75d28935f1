/*
 * gpu_bsw/utils.hpp -- the part of the reference's utils.hpp (utils.hpp:23-25)
 * that callers of the driver use: releasing the pinned result arrays that
 * kernel_driver_dna / kernel_driver_aa allocate.  Declared at global scope, as
 * in the reference.
 */
#ifndef GPU_BSW_UTILS_HPP
#define GPU_BSW_UTILS_HPP

#include "driver.hpp"

void free_alignments(gpu_bsw_driver::alignment_results* alignments);

#endif
