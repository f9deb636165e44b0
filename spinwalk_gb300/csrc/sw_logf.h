// Bit-exact reproduction of the host libm's logf on the domain the Gaussian generator uses.
//
// libstdc++'s normal_distribution<float> (Marsaglia polar method) calls std::log(float), i.e.
// the platform libm's logf, on r2 = x*x + y*y in [2^-48, 1] (x, y are 2u-1 for 24-bit u, so a
// nonzero x*x is >= 2^-48). Trajectories are bit-exact only if the GPU returns the same float.
//
// Method (project design):
//   1. logf_cand(): a float-float evaluation of log, accurate to ~2^-38 relative, written with
//      explicit IEEE single operations (+, -, *, fma) so that the host and the device compute
//      the SAME float for every input. It is correctly rounded except on a tiny fraction of
//      inputs.
//   2. At start-up the host evaluates its own libm logf and logf_cand on every float of the
//      domain and marks, in a bitmap (one bit per input, 50 MB), the inputs where they differ:
//      ~2e5 of 4e8 (glibc 2.39: 111k of them in [0.5, 1)). Every difference is one unit in the
//      last place towards the exact value, so the device takes the candidate's neighbour on the
//      side given by the sign of the candidate's own rounding residual. The host verifies that
//      rule on every marked input before the table is used.
//
// Reduction: x = 2^k * m with m in [0.75, 1.5); m is split into 64 buckets by its bit pattern;
// r = m*invc - 1 is formed exactly as a float pair; log(x) = k*ln2 + L_j + log1p(r) with L_j =
// log(1/invc_j) (float pair, sw_logf_table.h) and log1p(r) = r - r^2/2 + r^3*(1/3 - r/4 + r^2/5
// - r^3/6).
#pragma once
#include <stdint.h>
#include <string.h>

#include "sw_logf_table.h"

#if defined(__CUDACC__)
#define SWL_HD __host__ __device__ __forceinline__
#else
#define SWL_HD inline
#include <math.h>
#endif

namespace swlogf {

// Domain covered by the exception bitmap: [2^-48, 1].
constexpr uint32_t kDomainLo = 0x27800000u;    // bits of 2^-48
constexpr uint32_t kDomainHi = 0x3f800000u;    // bits of 1.0f (inclusive)
constexpr uint32_t kBitmapWords = ((kDomainHi - kDomainLo) >> 5) + 1;

constexpr float kLn2Hi = 0x1.62e4p-1f;          // ln2 rounded to 17 bits: k*kLn2Hi is exact
constexpr float kLn2Lo = 0x1.7f7d1cp-20f;       // ln2 - kLn2Hi rounded to float
constexpr float kC3 = 0x1.555556p-2f;           // 1/3
constexpr float kC5 = 0x1.99999ap-3f;           // 1/5
constexpr float kC6 = 0x1.555556p-3f;           // 1/6

SWL_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
SWL_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// Explicitly rounded single-precision operations, identical on host and device.
#if defined(__CUDA_ARCH__)
SWL_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
SWL_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
SWL_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
SWL_HD float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
// (host translation units are compiled with -ffp-contract=off)
SWL_HD float fmul(float a, float b) { return a * b; }
SWL_HD float fadd(float a, float b) { return a + b; }
SWL_HD float fsub(float a, float b) { return a - b; }
SWL_HD float ffma(float a, float b, float c) { return fmaf(a, b, c); }
#endif

// Two-sum: s + e == a + b exactly.
SWL_HD void two_sum(float a, float b, float &s, float &e) {
    s = fadd(a, b);
    float bb = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}

// tab: 64 x {invc, Lhi, Llo}. Valid for x in [2^-48, 1]. `above` is set when the float-float
// value the candidate rounded (an approximation of log(x) to ~2^-38) lies above the result.
SWL_HD float logf_cand(float x, const float *tab, bool &above) {
    const uint32_t ix = f2u(x);
    above = false;
    if (ix == 0x3f800000u) return 0.0f;
    const int32_t t = (int32_t)(ix - 0x3f400000u);
    const int32_t k = t >> 23;                                  // arithmetic shift
    const uint32_t im = ix - ((uint32_t)k << 23);
    const float m = u2f(im);
    const uint32_t j = (im - 0x3f400000u) >> 17;                // 0..63
    const float invc = tab[3 * j], Lhi = tab[3 * j + 1], Llo = tab[3 * j + 2];
    // r = m*invc - 1 exactly, as rh + rl
    const float p = fmul(m, invc);
    const float e = ffma(m, invc, -p);
    const float rh0 = fsub(p, 1.0f);
    const float rh = fadd(rh0, e);
    const float rl = fsub(e, fsub(rh, rh0));
    // r^2 = s_hi + s_lo
    const float s_hi = fmul(rh, rh);
    float s_lo = ffma(rh, rh, -s_hi);
    s_lo = ffma(fadd(rh, rh), rl, s_lo);
    // r^3 * (1/3 - r/4 + r^2/5 - r^3/6)
    const float q1 = ffma(ffma(ffma(rh, -kC6, kC5), rh, -0.25f), rh, kC3);
    const float t3 = fmul(fmul(s_hi, rh), q1);
    // B = rh - s_hi/2 (two-sum), A = k*ln2_hi + Lhi (two-sum)
    float B, b_err, A, a_err;
    two_sum(rh, fmul(-0.5f, s_hi), B, b_err);
    const float kf = (float)k;
    two_sum(fmul(kf, kLn2Hi), Lhi, A, a_err);
    float sm = fadd(b_err, rl);
    sm = fadd(sm, fmul(-0.5f, s_lo));
    sm = fadd(sm, t3);
    sm = fadd(sm, a_err);
    sm = fadd(sm, fadd(fmul(kf, kLn2Lo), Llo));
    float Cs, c_err;
    two_sum(A, B, Cs, c_err);
    const float lo = fadd(c_err, sm);
    const float r = fadd(Cs, lo);
    above = fadd(fsub(Cs, r), lo) > 0.0f;
    return r;
}

// The candidate's neighbour one ulp away, on the side of the exact value.
SWL_HD float neighbour(float r, bool above) {
    // r < 0 on (0, 1): a larger value has a smaller magnitude, i.e. bits - 1
    const uint32_t b = f2u(r);
    return u2f(above == (r < 0.0f) ? b - 1u : b + 1u);
}

}  // namespace swlogf
