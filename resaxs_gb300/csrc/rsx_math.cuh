// FP32 sine/cosine with explicit range reduction, written for this project.
//
// Method (published, textbook):
//  * additive range reduction of Cody & Waite (1980): n = nearest integer to
//    x * 2/pi, r = (x - n*P1) - n*P2 where P1 + P2 (+ P3) is pi/2 split into
//    FP32 numbers (P1 = fl(pi/2), P2 = fl(pi/2 - P1), P3 = fl(pi/2 - P1 - P2),
//    computed from a 60-digit value of pi); with FMA the first step is exact,
//    and the second is carried as a separate low part (see sincos_rr2);
//  * the Taylor series of sin and cos about 0 on |r| <= pi/4 (the
//    "small-argument series"): sin to r^9 (truncation < 2e-10 relative),
//    cos to r^10 (truncation < 2e-11);
//  * quadrant selection by n mod 4.
// The nearest-integer step uses the 1.5*2^23 rounding constant so that it
// stays on the FMA pipe (|x * 2/pi| < 2^22 is required; callers keep q*r far
// below that).
#pragma once
#include <cuda_runtime.h>

namespace rsx {

constexpr float kTwoOverPi = 0.636619772367581343f;
constexpr float kPio2P1 = 1.5707963705062866f;        // 0x3fc90fdb
constexpr float kPio2P2 = -4.371138828673793e-08f;     // 0xb33bbd2e
constexpr float kPio2P3 = -1.7151245100058819e-15f;    // 0xa6f72ced
constexpr float kRound = 12582912.0f;                  // 1.5 * 2^23
constexpr float kPio4 = 0.785398163397448310f;

// Taylor coefficients (-1)^k / (2k+1)!  and (-1)^k / (2k)!
constexpr float kS1 = -1.0f / 6.0f;
constexpr float kS2 = 1.0f / 120.0f;
constexpr float kS3 = -1.0f / 5040.0f;
constexpr float kS4 = 1.0f / 362880.0f;
constexpr float kC1 = -0.5f;
constexpr float kC2 = 1.0f / 24.0f;
constexpr float kC3 = -1.0f / 720.0f;
constexpr float kC4 = 1.0f / 40320.0f;
constexpr float kC5 = -1.0f / 3628800.0f;

// sin and cos of the unevaluated sum x_hi + x_lo (|x_lo| <= ulp(x_hi)),
// with the reduction split so that no FP32 rounding sees a constant offset.
// r = x - n*pi/2 is carried as r_hi = x_hi - n*P1 (exact: both terms are
// multiples of 2^-23 and the difference is below 1 in magnitude) plus
// r_lo = x_lo - n*P2 (P3 lies below FP32 resolution here).  Adding r_lo to
// r_hi directly would round every argument of a binade the same way (r_lo is
// nearly constant while r_hi sits on the FP32 grid), a bias of ~0.5 ulp that
// is invisible per term but coherent over 1e10 pair terms.  Instead r_lo
// enters through the first-order terms
//   sin(r_hi + r_lo) = sin(r_hi) + r_lo cos(r_hi),  cos(...) = cos(r_hi) - r_lo sin(r_hi),
// added to the small, continuously varying parts of the series before the
// single final addition of r_hi (resp. 1).  Callers pass the exact rounding
// error of the product that formed the argument as x_lo (x = q*r:
// x_lo = fma(q, r, -x)), which removes the phase rounding the same way.
// Accuracy about 1 ulp; mean error over uniformly distributed arguments
// indistinguishable from zero (< 1e-11).  Valid for |x * 2/pi| < 2^22.
__device__ __forceinline__ void sincos_rr2(float x, float x_lo, float &s, float &c)
{
    const float t = fmaf(x, kTwoOverPi, kRound);
    const float fn = t - kRound;
    const float rh = fmaf(-fn, kPio2P1, x);
    const float rl = fmaf(-fn, kPio2P2, x_lo);
    const float r2 = rh * rh;
    float ps = fmaf(r2, kS4, kS3);
    ps = fmaf(r2, ps, kS2);
    ps = fmaf(r2, ps, kS1);
    float pc = fmaf(r2, kC5, kC4);
    pc = fmaf(r2, pc, kC3);
    pc = fmaf(r2, pc, kC2);
    pc = fmaf(r2, pc, kC1);
    const float r3 = rh * r2;
    const float sp = fmaf(r3, ps, rh);   // sin(r_hi)
    const float cp = fmaf(r2, pc, 1.0f); // cos(r_hi)
    const float sv0 = rh + fmaf(r3, ps, rl * cp);
    const float cv0 = 1.0f + fmaf(r2, pc, -rl * sp);
    const int n = __float_as_int(t); // low bits of the rounded integer
    const bool swap = n & 1;
    const float sv = swap ? cv0 : sv0;
    const float cv = swap ? sv0 : cv0;
    // sin negated in quadrants 2,3; cos negated in quadrants 1,2
    const unsigned sgn_s = (unsigned)(n & 2) << 30;
    const unsigned sgn_c = (unsigned)((n + 1) & 2) << 30;
    s = __uint_as_float(__float_as_uint(sv) ^ sgn_s);
    c = __uint_as_float(__float_as_uint(cv) ^ sgn_c);
}

// sincos_rr2 for |x| < pi/4, where the reduction step is the identity (n = 0):
// the same operations without the reduction and quadrant logic, so the
// results are bit-identical to sincos_rr2's on that range.
__device__ __forceinline__ void sincos_small2(float x, float x_lo, float &s, float &c)
{
    const float r2 = x * x;
    float ps = fmaf(r2, kS4, kS3);
    ps = fmaf(r2, ps, kS2);
    ps = fmaf(r2, ps, kS1);
    float pc = fmaf(r2, kC5, kC4);
    pc = fmaf(r2, pc, kC3);
    pc = fmaf(r2, pc, kC2);
    pc = fmaf(r2, pc, kC1);
    const float r3 = x * r2;
    const float sp = fmaf(r3, ps, x);
    const float cp = fmaf(r2, pc, 1.0f);
    s = x + fmaf(r3, ps, x_lo * cp);
    c = 1.0f + fmaf(r2, pc, -x_lo * sp);
}

// sin and cos of the product a*b, its rounding error folded in exactly.
__device__ __forceinline__ void sincos_prod(float a, float b, float &s, float &c)
{
    const float x = a * b;
    sincos_rr2(x, fmaf(a, b, -x), s, c);
}

} // namespace rsx
