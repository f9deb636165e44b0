// IEEE-754 double addition, round to nearest even, in 64-bit integer arithmetic.
//
// The FP64 unit of this GPU retires two lanes per clock per SM, and the position update of
// the walk (x + n * dscale per axis, src/sim/kernels.cu:132) is the only double arithmetic left
// in a step; the integer pipes retire 128 lanes per clock. dadd_int gives the bit-identical
// result with integer instructions for normal operands whose biased exponents lie in
// [64, 1984] (every position and step of the walk); anything else (zeros, subnormals,
// infinities, NaN, extreme exponents) takes the hardware addition.
//
// Method (the textbook one of guard and sticky bits): align the smaller magnitude to the larger
// with 9 guard bits and a sticky bit in bit 0, add or subtract, renormalise, round the 62-bit
// sum to 53 bits to nearest even. Bits lost in the alignment are only possible when the
// exponents differ by more than 9, and then the sticky bit makes the sum odd, so it never
// lands on a rounding boundary and its rounding equals that of the exact sum.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SW_HD __host__ __device__ __forceinline__
#else
#define SW_HD inline
#endif

namespace sw {

SW_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

SW_HD double dfrom(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

SW_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return __builtin_clzll(v);
#endif
}

// -x, exactly, on the bit pattern
SW_HD uint64_t dflip(uint64_t x) { return x ^ 0x8000000000000000ull; }

// 2 |x|, exactly, for x zero or normal with |x| < 2^1023 (a walk step)
SW_HD uint64_t dtwice_abs(uint64_t x) {
    const uint64_t m = x & 0x7fffffffffffffffull;
    return m == 0u ? 0u : m + (1ull << 52);
}

#if defined(__CUDA_ARCH__)
// The out-of-range operands go to the hardware addition through a call that is not inlined, so
// that the compiler cannot evaluate it speculatively on every call.
__device__ __noinline__ uint64_t dadd_hw(uint64_t a, uint64_t b) { return dbits(dfrom(a) + dfrom(b)); }
#else
inline uint64_t dadd_hw(uint64_t a, uint64_t b) { return dbits(dfrom(a) + dfrom(b)); }
#endif

// Operands and result are bit patterns held in integer registers: a double-typed value that
// only moves between registers is copied with an FP64 instruction by the compiler for this GPU,
// which would put the slow FP64 unit back on the walk's path.
SW_HD uint64_t dadd_bits(uint64_t ua, uint64_t ub) {
    uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
    if (ea - 64u > 1920u || eb - 64u > 1920u) return dadd_hw(ua, ub);
    constexpr uint64_t kMag = 0x7fffffffffffffffull, kFrac = 0x000fffffffffffffull;
    if ((ub & kMag) > (ua & kMag)) {                 // |a| >= |b| from here on
        const uint64_t tu = ua; ua = ub; ub = tu;
        const uint32_t te = ea; ea = eb; eb = te;
    }
    const uint64_t sign = ua & ~kMag;
    const bool sub = ((ua ^ ub) >> 63) != 0;
    const uint64_t ma = ((ua & kFrac) | (1ull << 52)) << 9;   // hidden bit at bit 61
    uint64_t mb = ((ub & kFrac) | (1ull << 52)) << 9;
    const uint32_t d = ea - eb;
    if (d >= 63u) {
        mb = 1u;                                      // only the sticky bit survives
    } else if (d != 0u) {
        const uint64_t lost = mb & ((1ull << d) - 1u);
        mb = (mb >> d) | (uint64_t)(lost != 0u);
    }
    int e = (int)ea;
    uint64_t s;
    if (!sub) {
        s = ma + mb;                                  // < 2^63
        if (s >> 62) {
            s = (s >> 1) | (s & 1u);
            e += 1;
        }
    } else {
        s = ma - mb;
        if (s == 0u) return 0u;                       // x + (-x) = +0 when rounding to nearest
        const int lz = clz64(s) - 2;                  // bring the leading one back to bit 61
        s <<= lz;
        e -= lz;
    }
    const uint64_t up = (s >> 8) & (((s & 0xffu) != 0u) | (s >> 9)) & 1u;
    s = (s >> 9) + up;
    if (s >> 53) {                                    // rounded up to 2^53
        s >>= 1;
        e += 1;
    }
    return sign | ((uint64_t)e << 52) | (s & kFrac);
}

SW_HD double dadd_int(double a, double b) { return dfrom(dadd_bits(dbits(a), dbits(b))); }

// The hardware addition on bit patterns: one FP64 instruction, with operands and result in
// integer registers (no double-typed value lives across the walk's loop). The result passes
// through an opaque integer move, so that later copies of it are integer moves too.
SW_HD uint64_t dadd_fp64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(dbits(dfrom(a) + dfrom(b))));
    return r;
#else
    return dbits(dfrom(a) + dfrom(b));
#endif
}

}  // namespace sw
