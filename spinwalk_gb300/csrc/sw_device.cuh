// Device-side building blocks of the SpinWalk `sim` hot path on GB300 (sm_103a).
//
// The translation units that include this header are compiled with -fmad=false: every float and
// double expression rounds after each operation exactly like the reference's CPU build
// (x86-64 SSE2, no contraction), so trajectories are bit-exact. The only fused multiply-adds
// are the explicit ones inside logf_cand (sw_logf.h), which the host reproduces with fmaf.
#pragma once
#include <stdint.h>

#include "sw_dadd.h"
#include "sw_logf.h"
#include "sw_types.h"

namespace sw {

// ------------------------------------------------------------------------------------------
// MT19937 (the std::mt19937 parameters of the C++ standard)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

__device__ __forceinline__ uint32_t mt_twist1(uint32_t xi, uint32_t xi1, uint32_t xm) {
    uint32_t y = (xi & 0x80000000u) | (xi1 & 0x7fffffffu);
    return xm ^ (y >> 1) ^ ((xi1 & 1u) ? 0x9908b0dfu : 0u);
}

// One full regeneration of the 624-word state held in shared memory, by one warp. Same result
// as the sequential in-place loop of mersenne_twister_engine::_M_gen_rand: words [0,227) read
// only old words; [227,454) and [454,623) read words regenerated by the previous phase; word
// 623 reads the new words 0 and 396.
__device__ __forceinline__ void mt_twist_warp(uint32_t *s, int lane) {
    uint32_t v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int i = lane + 32 * k;
        if (i < 227) v[k] = mt_twist1(s[i], s[i + 1], s[i + kMtM]);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int i = lane + 32 * k;
        if (i < 227) s[i] = v[k];
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int i = 227 + lane + 32 * k;
        if (i < 454) v[k] = mt_twist1(s[i], s[i + 1], s[i - 227]);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int i = 227 + lane + 32 * k;
        if (i < 454) s[i] = v[k];
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 6; k++) {
        int i = 454 + lane + 32 * k;
        if (i < 623) v[k] = mt_twist1(s[i], s[i + 1], s[i - 227]);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 6; k++) {
        int i = 454 + lane + 32 * k;
        if (i < 623) s[i] = v[k];
    }
    __syncwarp();
    if (lane == 0) s[623] = mt_twist1(s[623], s[0], s[396]);
    __syncwarp();
}

// One word of the regeneration, x[i] <- x[i+397] ^ (y >> 1) ^ (y odd ? 0x9908b0df : 0) with
// y = upper bit of x[i] | lower 31 bits of x[i+1], written so that the integer ALU pipe (the
// bound of seeding) carries only three instructions: the bit select and the three-way xor as
// single lop3 operations and the shift. The odd-bit mask comes from the FMA pipe as
// (y - 2 (y >> 1)) * 0x9908b0df, which is exact in 32-bit arithmetic.
__device__ __forceinline__ uint32_t mt_twist1_alu3(uint32_t xi, uint32_t xi1, uint32_t xm) {
    uint32_t y, bit, mag, r;
    asm("lop3.b32 %0, %1, %2, 0x80000000, 0xE4;" : "=r"(y) : "r"(xi), "r"(xi1));  // (a&c)|(b&~c)
    const uint32_t ysh = y >> 1;
    asm("mad.lo.u32 %0, %1, 0xFFFFFFFE, %2;" : "=r"(bit) : "r"(ysh), "r"(y));
    asm("mul.lo.u32 %0, %1, 0x9908B0DF;" : "=r"(mag) : "r"(bit));
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(r) : "r"(xm), "r"(ysh), "r"(mag));  // a^b^c
    return r;
}

// The full regeneration with the state held in the registers of a HALF warp (16 lanes): lane
// hl owns the 13 consecutive words 208k + 13 hl + j in b[k][j] (k < 3, j < 13). A row k is 208
// consecutive words, fewer than 624 - 397 = 227, so no word of a row reads a word regenerated
// in the same row, and regenerating rows 0, 1, 2 in turn reproduces the sequential in-place
// order of mersenne_twister_engine::_M_gen_rand:
//   x[i+1]   same lane (j < 12), else slot 0 of lane hl+1 in row k, or of lane 0 in row k+1
//            (lane 15; row 3 is the regenerated row 0, as x[624] is the new x[0]);
//   x[i+397] 397 = 208 + 14*13 + 7: slot j+7 of lane hl+14 (j < 6) or slot j-6 of lane hl+15
//            (j >= 6), in row k+1, or k+2 where the lane index wraps; rows k+1 and k+2 modulo
//            3 are exactly the old (not yet regenerated) or new words the sequential loop reads.
// Each row costs 14 shuffles for 13 words; every value is shuffled from the row chosen by the
// PROVIDING lane, which is fixed per lane. With PRED the new words are kept only where `live`.
template <bool PRED>
__device__ __forceinline__ void mt_twist13(uint32_t (&b)[3][13], int hl, bool live) {
    constexpr unsigned FULL = 0xffffffffu;
    const bool q0 = hl == 0, q14 = hl >= 14, q15 = hl == 15;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int r1 = (k + 1) % 3, r2 = (k + 2) % 3;
        const uint32_t n12 = __shfl_sync(FULL, q0 ? b[r1][0] : b[k][0], hl + 1, 16);
        uint32_t far[13];
#pragma unroll
        for (int j = 0; j < 6; j++)
            far[j] = __shfl_sync(FULL, q14 ? b[r1][j + 7] : b[r2][j + 7], hl + 14, 16);
#pragma unroll
        for (int j = 6; j < 13; j++)
            far[j] = __shfl_sync(FULL, q15 ? b[r1][j - 6] : b[r2][j - 6], hl + 15, 16);
#pragma unroll
        for (int j = 0; j < 13; j++) {
            const uint32_t nw = mt_twist1_alu3(b[k][j], j < 12 ? b[k][j + 1] : n12, far[j]);
            b[k][j] = PRED ? (live ? nw : b[k][j]) : nw;
        }
    }
}

// Number of regenerations that mersenne_twister_engine::discard(z) performs right after
// seeding (position 624): while (z > 624 - p) { z -= 624 - p; regenerate; p = 0; }
__host__ __device__ __forceinline__ uint32_t mt_discard_twists(uint64_t z) {
    return z == 0 ? 0u : (uint32_t)(1 + (z - 1) / kMtN);
}

// ------------------------------------------------------------------------------------------
// thrust::normal_distribution<float> under nvcc (normal_distribution_nvcc, the reference's CUDA
// build): one minstd output x -> u = x - 1 folded at the middle of the range -> erfcinv.
// ------------------------------------------------------------------------------------------
constexpr uint32_t kMsRange = 2147483647u - 2u;        // minstd max - min

// The deviate for a folded u (the branch with S3 = -sqrt 2), every float op separately rounded:
// mean + stddev * S3 * erfcinv(2 p), p = u S1 + S2 (device erfcinvf).
__device__ __forceinline__ float ms_normal_folded(uint32_t u) {
    constexpr float S1 = (float)(1. / (double)kMsRange), S2 = S1 / 2;
    const float S3 = (float)(-1.4142135623730950488016887242097);
    const float p = __fadd_rn(__fmul_rn(__uint2float_rn(u), S1), S2);
    const float e = erfcinvf(__fmul_rn(2.0f, p));
    return __fadd_rn(0.0f, __fmul_rn(__fmul_rn(1.0f, S3), e));
}

// The full deviate of engine output x; with `delta` (sw_minstd.cu) the magnitude is corrected to
// what CUDA's host erfcinvf gives (the reference build's host path).
__device__ __forceinline__ float ms_normal(uint32_t x, const uint32_t *delta) {
    uint32_t u = x - 1u;
    const bool upper = u > kMsRange / 2;
    if (upper) u = kMsRange - u;
    uint32_t b = __float_as_uint(ms_normal_folded(u));
    if (delta) {
        const uint32_t nib = (__ldg(delta + (u >> 3)) >> ((u & 7u) * 4u)) & 15u;
        b = (b & 0x80000000u) | ((b & 0x7fffffffu) + (uint32_t)((int32_t)(nib ^ 8u) - 8));
    }
    // the upper branch (S3 = +sqrt 2) is the negation, and 0 + (-0) is +0 on both
    if (upper && (b & 0x7fffffffu)) b ^= 0x80000000u;
    return __uint_as_float(b);
}

// generate_canonical<float, 24>(mt19937): float(w) / 2^32, clamped below 1
// (libstdc++ bits/random.tcc, generate_canonical).
__device__ __forceinline__ float canon24(uint32_t w) {
    float f = __fmul_rn(__uint2float_rn(w), 2.3283064365386963e-10f);  // exact: * 2^-32
    return f >= 1.0f ? 0x1.fffffep-1f : f;
}

// The host libm's logf, bit for bit, on [2^-48, 1] (sw_logf.h): the candidate, or its
// neighbour towards the exact value where the host's exception bitmap says so.
__device__ __forceinline__ float logf_libm(float x, const float *s_tab, const LogfTables &L) {
    bool above;
    const float c = swlogf::logf_cand(x, s_tab, above);
    const uint32_t k = __float_as_uint(x) - swlogf::kDomainLo;
    const uint32_t w = __ldg(L.bitmap + (k >> 5));
    return ((w >> (k & 31u)) & 1u) ? swlogf::neighbour(c, above) : c;
}

// ------------------------------------------------------------------------------------------
// Exact helpers that keep the walk off the (slow) FP64 pipe
// ------------------------------------------------------------------------------------------
// float -> double, exact, with integer operations. The Gaussian deviates are 0 or have
// magnitude >= 2^-36 (|y| >= 2^-24 times sqrt(-2 ln r2 / r2)), so they are never subnormal;
// a subnormal input still takes the exact conversion instruction.
__device__ __forceinline__ double f2d_exact(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    if (e == 0u) return m ? (double)f : __hiloint2double(b & 0x80000000u, 0);
    const uint32_t hi = (b & 0x80000000u) | ((e + (1023u - 127u)) << 20) | (m >> 3);
    return __hiloint2double((int)hi, (int)(m << 29));
}

// float(d) for a double given as its bit pattern, rounded to nearest even, with integer
// operations where the result is a normal float; zero, subnormal, overflowing and non-finite
// values take the hardware conversion (out of line, so that it is not evaluated on every call).
#if defined(__CUDA_ARCH__)
__device__ __noinline__ float d2f_hw(uint64_t b) { return (float)__longlong_as_double((long long)b); }
#else
__device__ float d2f_hw(uint64_t b);
#endif
__device__ __forceinline__ float d2f_exact(uint64_t b) {
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e - (1023u - 126u) > 253u) return d2f_hw(b);           // float exponent outside 1..254
    const uint32_t mf = ((hi & 0xfffffu) << 3) | (lo >> 29);    // top 23 significand bits
    const uint32_t rem = lo & 0x1fffffffu, half = 0x10000000u;
    const uint32_t up = (rem > half) | ((rem == half) & (mf & 1u));
    // a carry out of the significand steps the exponent, up to infinity, as rounding does
    return __uint_as_float((hi & 0x80000000u) + (((e - 1023u + 127u) << 23) | mf) + up);
}

// The reference's gradient phase in degrees (kernels.cu:181-187),
//   ((gx x + gy y + gz z) * 1e-3 * dt * 1e-6 * GAMMA * RAD2DEG),
// every operation rounded as there. A lobe along one axis has two zero coefficients: their
// products are +-0 and leave a nonzero product unchanged, so only the nonzero one is formed; a
// zero product, or more than one nonzero coefficient, takes the full sum (sign of zero included).
__device__ __forceinline__ double grad_phase_deg(float gx, float gy, float gz, const uint64_t (&x)[3],
                                                 double dt_us) {
    const bool nx = (__float_as_uint(gx) << 1) != 0u, ny = (__float_as_uint(gy) << 1) != 0u,
               nz = (__float_as_uint(gz) << 1) != 0u;
    double s = 0.;
    bool full = (int)nx + (int)ny + (int)nz != 1;
    if (!full) {
        const float g1 = nx ? gx : (ny ? gy : gz);
        const uint64_t x1 = nx ? x[0] : (ny ? x[1] : x[2]);
        s = f2d_exact(g1) * dfrom(x1);
        full = (__double_as_longlong(s) << 1) == 0;
    }
    if (full)
        s = f2d_exact(gx) * dfrom(x[0]) + f2d_exact(gy) * dfrom(x[1]) + f2d_exact(gz) * dfrom(x[2]);
    return s * 1e-3 * dt_us * 1e-6 * kGamma * kRad2Deg;
}

// v < 0 and v >= bound (bound > 0) on the bit patterns (positive doubles order as integers).
__device__ __forceinline__ bool dneg(uint64_t v) {
    return (int64_t)v < 0 && (v & 0x7fffffffffffffffull) != 0u;
}
__device__ __forceinline__ bool dge_pos(uint64_t v, double bound) {
    return (int64_t)v >= __double_as_longlong(bound);
}

// (int64_t)(v * s2g) as the reference computes it (double product, truncation), via an FP32
// estimate: v is truncated to 24 bits from its bit pattern (relative error < 2^-23), s2g_f is
// s2g rounded to float (< 2^-24), the float product adds < 2^-24, so |p - v*s2g| < 2^-22 |p|.
// When p is farther than 2^-21 |p| from an integer (all but ~1e-4 of the calls at 500 voxels)
// floor(p) is the answer; otherwise, and for v <= 0, tiny v or p >= 2^22, the exact double
// product is used. floor(p) itself is taken without the conversion units (64-bit conversions
// and rounding run on the slow FP64 pipe of this GPU): adding 1.5 * 2^23 rounds a p in
// [0, 2^22) to the nearest integer n exactly, and the sum's bit pattern is 0x4B400000 + n.
__device__ __forceinline__ int64_t voxel_coord(uint64_t vb, double s2g, float s2g_f) {
    const uint32_t hi = (uint32_t)(vb >> 32), lo = (uint32_t)vb;
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if ((int32_t)hi > 0 && e > 1023u - 120u) {
        const float vf = __uint_as_float(((e - 1023u + 127u) << 23) | ((hi & 0xfffffu) << 3) |
                                         (lo >> 29));
        const float p = __fmul_rn(vf, s2g_f);
        if (p < 4194304.0f) {                                      // 2^22
            const float t = __fadd_rn(p, 12582912.0f);             // 1.5 * 2^23
            float fl = __fsub_rn(t, 12582912.0f);
            int32_t n = __float_as_int(t) - 0x4B400000;
            if (fl > p) {
                fl = __fsub_rn(fl, 1.0f);
                n -= 1;
            }
            const float fr = __fsub_rn(p, fl);
            const float margin = __fmul_rn(p, 4.76837158203125e-07f);   // 2^-21
            if (fr > margin && __fsub_rn(1.0f, fr) > margin) return (int64_t)n;
        }
    }
    return (int64_t)(dfrom(vb) * s2g);
}

// dscale != 0 for a non-negative double, as an integer test (a double compare is an FP64-pipe
// instruction)
__device__ __forceinline__ bool dnonzero(double v) { return __double_as_longlong(v) != 0; }

// ------------------------------------------------------------------------------------------
// One attempted move of a spin (src/sim/kernels.cu:130-170), shared by the walk kernels
// ------------------------------------------------------------------------------------------
enum MoveResult { kMoveAccepted = 0, kMoveRejected = 1, kMoveLost = 2, kMoveOOB = 3 };

// One packed voxel record as {field bits, substrate label}: 8-byte records hold the float field,
// 4-byte records (SW_FIELD_BF16) the field as bfloat16 in bits 0-15 and the label in bits 16-23.
__device__ __forceinline__ uint2 voxel_record(const uint2 *__restrict__ vox, int64_t ind,
                                              int32_t bf16) {
    if (bf16) {
        const uint32_t r = __ldg(reinterpret_cast<const uint32_t *>(vox) + ind);
        return make_uint2(r << 16, r >> 16);
    }
    return __ldg(vox + ind);
}

struct WalkRegs {
    uint64_t xo[3];           // last accepted position (bit patterns of the doubles)
    int64_t ind_old;
    uint32_t ts_old;          // substrate of the last accepted voxel
    float field;              // its field (deg per step)
    double dscale;            // its step std-dev
    uint32_t itr;             // consecutive rejected moves
    uint32_t nh, nc, uh, uc;  // ring buffer heads / counts
};

// Draws three deviates (when the substrate diffuses), wraps at the FoV, looks the voxel up and
// applies the permeability test. On acceptance xn holds the new position and the voxel state in
// w is updated; w.xo is left to the caller (it commits xn after the Bloch events).
__device__ __forceinline__ int walk_move(WalkRegs &w, uint64_t (&xn)[3], const DevParams &P,
                                         const DevTables &Tb, const uint2 *__restrict__ vox,
                                         const float *nb, const float *ub) {
    xn[0] = w.xo[0];
    xn[1] = w.xo[1];
    xn[2] = w.xo[2];
    if (dnonzero(w.dscale)) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float g = nb[w.nh];
            w.nh = (w.nh + 1 == kNormBuf) ? 0 : w.nh + 1;
            const uint64_t rnd = dbits(f2d_exact(g) * w.dscale);   // hardware DMUL
            uint64_t v = dadd_fp64(w.xo[i], rnd);   // w.xo[i] + rnd
            // the wrap in integer arithmetic too: the compiler evaluates a cheap double
            // expression here on every step whatever the branch, on the slow FP64 unit
            if (dneg(v))
                v = dadd_bits(v, P.cross_fov ? dbits(P.fov[i]) : dtwice_abs(rnd));
            else if (dge_pos(v, P.fov[i]))
                v = dadd_bits(v, dflip(P.cross_fov ? dbits(P.fov[i]) : dtwice_abs(rnd)));
            xn[i] = v;
        }
        w.nc -= 3;
    }
    const int64_t ind = voxel_coord(xn[0], P.s2g[0], P.s2g_f[0]) * P.nynz +
                        voxel_coord(xn[1], P.s2g[1], P.s2g_f[1]) * P.nz +
                        voxel_coord(xn[2], P.s2g[2], P.s2g_f[2]);
    if (ind >= P.matrix_length || ind < 0) return kMoveOOB;
    if (ind != w.ind_old) {
        const uint2 v = voxel_record(vox, ind, P.field_bf16);
        const uint32_t ts = v.y;
        if (ts != w.ts_old) {
            const float u = ub[w.uh];
            w.uh = (w.uh + 1 == kUnifBuf) ? 0 : w.uh + 1;
            w.uc--;
            if (u >= __ldg(Tb.pXY + w.ts_old * P.n_substrate + ts))
                return (uint64_t)(w.itr++) > P.max_iterations ? kMoveLost : kMoveRejected;
            w.ts_old = ts;
        }
        w.ind_old = ind;
        w.field = __uint_as_float(v.x);
        w.dscale = __ldg(Tb.dscale + w.ts_old);
    }
    w.itr = 0;
    return kMoveAccepted;
}

// ------------------------------------------------------------------------------------------
// Bloch primitives, float path (src/sim/kernels.cuh:82-230, kernels.cu:45-52)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void xrot_f(float s, float c, const float *a, float *b) {
    b[0] = a[0];
    b[1] = c * a[1] - s * a[2];
    b[2] = s * a[1] + c * a[2];
}
__device__ __forceinline__ void yrot_f(float s, float c, const float *a, float *b) {
    b[0] = c * a[0] + s * a[2];
    b[1] = a[1];
    b[2] = -s * a[0] + c * a[2];
}
__device__ __forceinline__ void zrot_f(float s, float c, const float *a, float *b) {
    b[0] = c * a[0] - s * a[1];
    b[1] = s * a[0] + c * a[1];
    b[2] = a[2];
}
__device__ __forceinline__ void rf_f(const RfOp &op, const float *a, float *b) {
    switch (op.kind) {
        case 0: xrot_f(op.s, op.c, a, b); break;
        case 1: xrot_f(-op.s, op.c, a, b); break;
        case 2: yrot_f(op.s, op.c, a, b); break;
        case 3: yrot_f(-op.s, op.c, a, b); break;
        default: {
            float t[3];
            zrot_f(-op.sp, op.cp, a, b);
            xrot_f(op.s, op.c, b, t);
            zrot_f(op.sp, op.cp, t, b);
        }
    }
}
// dephase_relax: zrot by the accumulated phase (degrees), then T1/T2 relaxation with the
// double exp of the reference and relax()'s double constant 1.
__device__ __forceinline__ void dephase_relax_f(const float *a, float *b, float phase, float T1,
                                                float T2, float dt_s) {
    float ang = (float)((double)phase * kDeg2Rad);
    float s, c;
    sincosf(ang, &s, &c);
    zrot_f(s, c, a, b);
    if (T1 >= 0 && T2 >= 0) {
        float e1 = (float)exp((double)(-dt_s / T1));
        float e2 = (float)exp((double)(-dt_s / T2));
        b[0] = b[0] * e2;
        b[1] = b[1] * e2;
        b[2] = (float)(1. + (double)e1 * ((double)b[2] - 1.));
    }
}

// ---- FP64 path ----------------------------------------------------------------------------
__device__ __forceinline__ void xrot_d(double s, double c, const double *a, double *b) {
    b[0] = a[0];
    b[1] = c * a[1] - s * a[2];
    b[2] = s * a[1] + c * a[2];
}
__device__ __forceinline__ void yrot_d(double s, double c, const double *a, double *b) {
    b[0] = c * a[0] + s * a[2];
    b[1] = a[1];
    b[2] = -s * a[0] + c * a[2];
}
__device__ __forceinline__ void zrot_d(double s, double c, const double *a, double *b) {
    b[0] = c * a[0] - s * a[1];
    b[1] = s * a[0] + c * a[1];
    b[2] = a[2];
}
__device__ __forceinline__ void rf_d(const RfOp &op, const double *a, double *b) {
    switch (op.kind) {
        case 0: xrot_d(op.sd, op.cd, a, b); break;
        case 1: xrot_d(-op.sd, op.cd, a, b); break;
        case 2: yrot_d(op.sd, op.cd, a, b); break;
        case 3: yrot_d(-op.sd, op.cd, a, b); break;
        default: {
            double t[3];
            zrot_d(-op.spd, op.cpd, a, b);
            xrot_d(op.sd, op.cd, b, t);
            zrot_d(op.spd, op.cpd, t, b);
        }
    }
}
__device__ __forceinline__ void dephase_relax_d(const double *a, double *b, double phase,
                                                double T1, double T2, double dt_s) {
    double s, c;
    sincos(phase * kDeg2Rad, &s, &c);
    zrot_d(s, c, a, b);
    if (T1 >= 0 && T2 >= 0) {
        double e1 = exp(-dt_s / T1), e2 = exp(-dt_s / T2);
        b[0] *= e2;
        b[1] *= e2;
        b[2] = 1. + e1 * (b[2] - 1.);
    }
}

// Compensated float accumulation (Knuth two-sum), value = s + e.
__device__ __forceinline__ void kahan_add(float &s, float &e, float x) {
    float t = s + x;
    float bp = t - s;
    e += (s - (t - bp)) + (x - bp);
    s = t;
}

}  // namespace sw
