// Phase rotation helpers shared by the DAS kernels.
#pragma once

#include <cuda_runtime.h>

namespace ustb {

// 2*pi split in two floats (Cody & Waite additive range reduction): C1 is
// 2*pi rounded to float, C2 the float nearest to (2*pi - C1).  With an FMA for
// each step the reduced argument carries ~1e-12 rad of error for |x| < 1e5.
constexpr double kTwoPiD = 6.283185307179586476925286766559;
constexpr float kTwoPiHi = (float)kTwoPiD;
constexpr float kTwoPiLo = (float)(kTwoPiD - (double)(float)kTwoPiD);
constexpr float kInvTwoPi = (float)(1.0 / kTwoPiD);

// exp(i*x) for |x| up to ~1e5 rad: Cody-Waite reduction of x to [-pi, pi]
// (two FMAs), then the hardware sine/cosine approximations on the reduced
// argument (absolute error below 4e-7 on [-pi, pi]).  x itself is used exactly
// as given, so callers that round x like the reference does reproduce its phase.
// The nearest integer to x / 2pi is taken by adding and subtracting 1.5 * 2^23
// (exact for |x / 2pi| < 2^22; any integer k keeps the reduction exact), which
// keeps the conversion pipe free for the sine and cosine.
__device__ __forceinline__ void expi_reduced(float x, float& c, float& s) {
    const float k = __fsub_rn(__fmaf_rn(x, kInvTwoPi, 12582912.0f), 12582912.0f);
    float r = fmaf(-k, kTwoPiHi, x);
    r = fmaf(-k, kTwoPiLo, r);
    __sincosf(r, &s, &c);
}

}  // namespace ustb
