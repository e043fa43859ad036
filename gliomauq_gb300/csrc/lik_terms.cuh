// Per-point terms of HGG_Likelihood (source/Likelihood/source/HGG_Likelihood.cpp)
// shared by the likelihood reductions (likelihood.cu) and the screening chain
// (affine_chain.cu). Both are compiled with -fmad=false.
#pragma once

namespace gbg {

__device__ __forceinline__ int sgn_d(double d) {  // HGG_Likelihood::sgn, eps = 0 (:155-160)
    if (d < -0.0) return -1;
    return d > 0.0;
}

// log Bernoulli(alpha(u)) of observation y, alpha = 0.5 + 0.5 sgn(u - uc)
// (1 - exp(-(u - uc)^2 / slope)) (:136-153); is2 = 1 / slope
__device__ __forceinline__ double log_bernoulli(double u, double y, double uc, double is2) {
    const double diff = u - uc;
    const double alpha = 0.5 + 0.5 * sgn_d(diff) * (1. - exp(-diff * diff * is2));
    return (y == 1) ? log(alpha) : log(1. - alpha);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace gbg
