// Per-SNP scale rule shared by the decoding and NMF-fill statistics kernels.
#pragma once
#include "slfmm_internal.h"

namespace slfmm {

// compute_scale (src/bed.rs:382-395) with p = mean / 2, in the reference's
// operation order with round-to-nearest FP64 intrinsics so that no FMA
// contraction changes the bits.
__device__ __forceinline__ double scale_from_mean(double mean, int norm) {
    const double pp = __ddiv_rn(mean, 2.0);
    const double twopq = __dmul_rn(__dmul_rn(2.0, pp), __dsub_rn(1.0, pp));
    if (norm == SLFMM_NORM_CENTER_ONLY) return twopq < 1e-20 ? 0.0 : 1.0;
    const double denom = __dsqrt_rn(twopq);
    return denom > 1e-10 ? __ddiv_rn(1.0, denom) : 0.0;
}

}  // namespace slfmm
