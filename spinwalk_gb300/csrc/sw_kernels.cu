// CUDA kernels of the SpinWalk `sim` hot path for GB300 (sm_103a).
//
// The reference runs one thread per spin that seeds two std::mt19937, draws Gaussian steps and
// walks all time points in one go (cu_sim / sim::sim, src/sim/kernels.cu:57-233). Here the
// same per-spin computation is split so that each part runs in the shape the GPU likes:
//
//   k_pack    : mask + fieldmap -> one 8-byte record per voxel (one gather per step)
//   k_seed    : one HALF warp per spin: mt19937(seed+spin) + discard(seed+spin), the 624-word
//               state held in 16 lanes' registers (13 words each), regenerated with shuffles
//   k_init    : one thread per spin: initial voxel, substrate and state (kernels.cu:90-104)
//   k_refill  : one WARP per spin: tops up the spin's ring buffers of Gaussian deviates
//               (libstdc++ polar method, 32 candidate pairs per pass, accepted pairs compacted
//               with a ballot) and crossing uniforms, twisting the state when a block runs out
//   k_walk    : one thread per spin: walk + mask/permeability + field + Bloch events until the
//               spin's buffers run low, then saves its state (kernels.cu:107-232)
//
// k_refill and k_walk alternate until every spin has finished. All kernels are compiled with
// -fmad=false (see sw_device.cuh).
#include <cuda_bf16.h>

#include <algorithm>
#include <cuda_runtime.h>

#include "sw_device.cuh"
#include "sw_kernels.h"
#include "spinwalk_gpu.h"

namespace sw {

// ------------------------------------------------------------------------------------------
// Also flags substrate labels >= n_substrate (the reference's driver refuses such a mask,
// src/sim/monte_carlo.cu:113-118); the host checks the flag before any walk reads the tables.
__global__ void k_pack(const uint8_t *__restrict__ mask, const float *__restrict__ field,
                       uint2 *__restrict__ out, int64_t n, uint32_t n_substrate,
                       uint32_t *__restrict__ bad_label, int bf16) {
    bool bad = false;
    uint32_t *out4 = reinterpret_cast<uint32_t *>(out);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float fv = field ? field[i] : 0.f;
        const uint32_t m = mask[i];
        bad |= m >= n_substrate;
        if (bf16)
            out4[i] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(fv)) | (m << 16);
        else
            out[i] = make_uint2(__float_as_uint(fv), m);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(bad_label, 1u);
}

// ------------------------------------------------------------------------------------------
// Seeding: std::mt19937 gen(seed + spin); gen.discard(seed + spin)   (kernels.cu:82-88)
// ------------------------------------------------------------------------------------------
// One HALF warp per spin (mt_twist13 layout), two spins per warp. The two spins of a warp are
// neighbours, so their discard counts differ by one and their regeneration counts by at most
// one: both halves run the common count together, then at most one regeneration whose result
// only the half that needs it keeps. Seeding (623 dependent multiply-adds) runs on one lane per
// half into shared memory. The discard work, sum over spins of seed + spin words, is what
// bounds this kernel (integer pipes), not memory.
constexpr int kSeedWarps = 4;

template <bool FAN>
__global__ void __launch_bounds__(32 * kSeedWarps)
    k_seed(DevParams P, RngState G, uint32_t spin_lo, uint32_t spin_hi, SeedCopies F) {
    __shared__ uint32_t s_mt[2 * kSeedWarps][kMtN];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, half = lane >> 4, hl = lane & 15;
    uint32_t *s = s_mt[2 * w + half];
    const uint32_t n = spin_hi - spin_lo;
    for (uint32_t pair = blockIdx.x * kSeedWarps + w; 2ull * pair < n;
         pair += gridDim.x * kSeedWarps) {
        const uint32_t idx = 2 * pair + half;
        const bool valid = idx < n;                  // an odd count leaves one half idle
        const uint32_t spin = spin_hi - 1 - (valid ? idx : n - 1);  // largest discard first
        const uint64_t sd = P.seed + spin;
        if (hl == 0) {                               // mersenne_twister_engine::seed
            uint32_t x = (uint32_t)sd;
            s[0] = x;
            for (uint32_t i = 1; i < kMtN; i++) {
                x = 1812433253u * (x ^ (x >> 30)) + i;
                s[i] = x;
            }
        }
        __syncwarp();
        uint32_t b[3][13];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int j = 0; j < 13; j++) b[k][j] = s[208 * k + 13 * hl + j];
        __syncwarp();
        const uint32_t mine = mt_discard_twists(sd);
        const uint32_t other = __shfl_xor_sync(0xffffffffu, mine, 16);
        const uint32_t common = min(mine, other);
        for (uint32_t t = 0; t < common; t++) mt_twist13<false>(b, hl, true);
        if (max(mine, other) > common) mt_twist13<true>(b, hl, mine > common);
        // discard leaves the position at z - 624 (regenerations - 1), or 624 when z == 0
        const uint32_t p = mine == 0 ? (uint32_t)kMtN : (uint32_t)(sd - (uint64_t)kMtN * (mine - 1));
        if (valid) {
            uint32_t *gr = G.mt_r + (size_t)spin * kMtN, *gu = G.mt_u + (size_t)spin * kMtN;
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int j = 0; j < 13; j++) {
                    gr[208 * k + 13 * hl + j] = b[k][j];
                    gu[208 * k + 13 * hl + j] = b[k][j];
                }
            if (hl == 0) {
                G.p_r[spin] = p;
                G.p_u[spin] = p;
                G.nhead[spin] = 0;
                G.ncnt[spin] = 0;
                G.uhead[spin] = 0;
                G.ucnt[spin] = 0;
            }
        }
        if (FAN) {              // further copies: staged in the half warp's block, stored coalesced
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int j = 0; j < 13; j++) s[208 * k + 13 * hl + j] = b[k][j];
            __syncwarp();
            if (valid)
                for (uint32_t d = 0; d < F.n; d++) {
                    const SeedCopy c = F.d[d];
                    if (spin >= c.n) continue;
                    uint32_t *dst = c.mt + (size_t)spin * kMtN;
                    for (int i = hl; i < kMtN; i += 16) dst[i] = s[i];
                    if (hl == 0) {
                        c.p[spin] = p;
                        c.c0[spin] = 0;
                        c.c1[spin] = 0;
                        c.c2[spin] = 0;
                    }
                }
            __syncwarp();       // the block is reseeded in the next pass
        }
    }
}

// ------------------------------------------------------------------------------------------
// Seeding by jump-ahead (sw_mtjump.h): the same state as k_seed for spins whose discard count
// z = seed + spin is large, in work independent of z. With J = 624 R - 1 (R regenerations of
// discard(z)) and g = x^J mod phi (host-computed, one per R), the state after J words is
// h_j = XOR over k with g_k = 1 of x[k + j], j < 624, over the spin's own output sequence x:
// a correlation of g with x, i.e. one 624 x 624 Hankel product per 624-step block of k.
//
// One level of Karatsuba splits each block product (outputs j = j' + 312 f, steps k = 624 a +
// 312 e + r, f, e in {0, 1}) into three half-size products whose sums over the blocks are again
// correlations:
//   P1_j' = XOR over k in B of (g_(k-312) ^ g_k) x[k + j']
//   P2_j' = XOR over k in A of g_k e[k + j'],   P3_j' = XOR over k in B of g_k e[k + j']
//   h_j' = P1_j' ^ P2_j',   h_(312+j') = P1_j' ^ P3_j'                            (j' < 312)
// with A, B the first and second halves of every 624-step block and e[i] = x[i] ^ x[i + 312]:
// three correlations of 312 outputs over 9984 steps each, 3/4 of the direct XOR work.
//
// A thread block of three warps takes two spins that share R (hence g): warp w computes P_(w+1)
// for both, lanes 0-15 for the first spin and 16-31 for the second, each lane the 21 outputs
// j' = 21 l + i (16 x 21 = 336 >= 312) in registers. Each spin's x and e live in 1024-word rings
// in shared memory; before block a the three warps produce x 624 words further (three rounds of
// 208, which read only older words) and then e 624 words further, with a barrier after each
// (the rings hold just the windows of one block), then run their 312 steps of the block: 15 groups of 21 steps (the last masked to 18), each group reading the
// lane's 42 sequence words at one base address (the first 64 ring slots are mirrored past the
// end) and adding windows on the polynomial's bits three at a time. The two spins' rings are 16
// words apart modulo the 32 banks, so the two half-warps' reads do not conflict. The block of
// regeneration R is then h_1 .. h_623 plus one more word.
// ------------------------------------------------------------------------------------------
constexpr int kJumpPer = 21;              // outputs per lane: 16 x 21 = 336 >= 312 per spin
constexpr int kJumpWin = 2 * kJumpPer;    // sequence words a lane reads per group of 21 steps
constexpr uint32_t kJumpRing = 1024;      // words per sequence ring
constexpr uint32_t kJumpMask = kJumpRing - 1u;
constexpr uint32_t kJumpMirror = 64;      // ring slots copied past the end
constexpr uint32_t kJumpStride = kJumpRing + kJumpMirror + 16;   // ring to ring: 16 mod 32 banks
constexpr uint32_t kJumpXAhead = 1272;    // x is generated to 624 a + 1272 before block a
constexpr uint32_t kJumpEAhead = 960;     // e to 624 a + 960 (the windows of block a reach there)
constexpr uint32_t kJumpXFrom = 312;      // block a reads x from 624 a + 312 (P1), e from 624 a
constexpr uint32_t kJumpRound = 208;      // x words per generation round (x[n] reads x[n - 227])
constexpr int kJumpBlocksPerSm = 8;
static_assert(kJumpStride % 32 == 16, "the second spin's rings must sit 16 banks over");
static_assert(kJumpWin <= (int)kJumpMirror, "mirror too short for one window");
static_assert(kJumpRound <= 227 && 3 * kJumpRound == kMtN, "three rounds per block");
// Block a reads x[624 a + 312, 624 a + 962) and e[624 a, 624 a + 960); forming e[n] needs x[n]
// and x[n + 312]. With x generated to 624 a + 1272 the ring holds x from 624 a + 248, and the
// rounds before block a + 1 overwrite only x below 624 a + 872 (read by block a alone, done).
static_assert(kJumpXAhead - kJumpRing <= kJumpXFrom, "x ring too short for block a");
static_assert(kJumpXAhead - kJumpRing <= kJumpEAhead - kMtN + 312, "e formed from overwritten x");
static_assert(kJumpEAhead <= kJumpRing, "e ring too short for block a");
static_assert(kJumpEAhead + 312 <= kJumpXAhead, "e is formed from generated x only");
// the last step of a block (624 a + 623) with the last padded output (335) reads 624 a + 958
static_assert(kMtN - 1 + 16 * kJumpPer - 1 < (int)kJumpEAhead, "windows reach unformed e");
constexpr uint32_t kJumpBlocks = (kMtDegreeDev + kMtN - 1) / kMtN;   // 32 blocks of 624 steps
constexpr size_t kJumpSmem = 4 * kJumpStride * sizeof(uint32_t);

// Bits k0 .. k0 + 20 of the jump polynomial (624 words; bits past 19936 are zero).
__device__ __forceinline__ uint32_t jump_bits(const uint32_t *__restrict__ g, uint32_t k0) {
    const uint32_t q = k0 >> 5, r = k0 & 31u;
    uint64_t v = __ldg(g + q);
    if (q + 1 < (uint32_t)kMtN) v |= (uint64_t)__ldg(g + q + 1) << 32;
    return (uint32_t)(v >> r) & ((1u << kJumpPer) - 1u);
}

__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}

// Steps T .. T + 2 of a group on their three polynomial bits: two windows are added with one
// three-input xor, so a triple costs one operation per word on average instead of 1.5.
template <int T>
__device__ __forceinline__ void jump_triple(uint32_t (&h)[kJumpPer], const uint32_t (&W)[kJumpWin],
                                            uint32_t bits) {
    switch (bits & 7u) {
    case 1:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] ^= W[T + i];
        break;
    case 2:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] ^= W[T + 1 + i];
        break;
    case 4:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] ^= W[T + 2 + i];
        break;
    case 3:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] = xor3(h[i], W[T + i], W[T + 1 + i]);
        break;
    case 5:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] = xor3(h[i], W[T + i], W[T + 2 + i]);
        break;
    case 6:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] = xor3(h[i], W[T + 1 + i], W[T + 2 + i]);
        break;
    case 7:
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] ^= xor3(W[T + i], W[T + 1 + i], W[T + 2 + i]);
        break;
    default:
        break;
    }
}

__device__ __forceinline__ void jump_put(uint32_t *ring, uint32_t n, uint32_t v) {
    const uint32_t slot = n & kJumpMask;
    ring[slot] = v;
    if (slot < kJumpMirror) ring[kJumpRing + slot] = v;
}

// Spins [lo, hi) in pairs that share R: R changes where (seed + spin) % 624 == 1, so the range
// splits into a head segment up to the first such spin and segments of 624 spins after it; each
// segment is paired from its start (an odd segment leaves its last spin alone: both halves then
// compute it and one writes). Pair p -> first spin and whether a second follows.
struct JumpPairs {
    uint32_t lo, hi, b0, head_pairs, n_pairs;
    static JumpPairs make(uint64_t seed, uint32_t lo, uint32_t hi) {
        JumpPairs q;
        q.lo = lo;
        q.hi = hi;
        const uint32_t r = (uint32_t)((seed + lo) % kMtN);      // spin lo + (1 - r) mod 624
        const uint64_t b0 = (uint64_t)lo + (r <= 1 ? 1 - r : kMtN + 1 - r);
        q.b0 = (uint32_t)std::min<uint64_t>(b0, hi);
        const uint32_t n0 = q.b0 - lo, rest = hi - q.b0;
        q.head_pairs = (n0 + 1) / 2;
        const uint32_t full = rest / kMtN, tail = rest % kMtN;
        q.n_pairs = q.head_pairs + full * (kMtN / 2) + (tail + 1) / 2;
        return q;
    }
    __device__ void pair(uint32_t p, uint32_t &s0, bool &two) const {
        uint32_t end;
        if (p < head_pairs) {
            s0 = lo + 2 * p;
            end = b0;
        } else {
            const uint32_t pp = p - head_pairs, seg = pp / (kMtN / 2);
            const uint32_t base = b0 + seg * kMtN;
            s0 = base + 2 * (pp % (kMtN / 2));
            end = (uint32_t)min((uint64_t)hi, (uint64_t)base + kMtN);
        }
        two = s0 + 1 < end;
    }
};

template <bool FAN>
__global__ void __launch_bounds__(96, kJumpBlocksPerSm)
    k_seed_jump(DevParams P, RngState G, const uint32_t *__restrict__ polys, uint64_t R_lo,
                JumpPairs pairs, SeedCopies F) {
    extern __shared__ uint32_t s_jump[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, half = lane >> 4, hl = lane & 15;
    const int t = threadIdx.x;
    // rings: x of spin 0, x of spin 1, e of spin 0, e of spin 1
    uint32_t *xr0 = s_jump, *xr1 = s_jump + kJumpStride;
    uint32_t *er0 = s_jump + 2 * kJumpStride, *er1 = s_jump + 3 * kJumpStride;
    for (uint32_t p = blockIdx.x; p < pairs.n_pairs; p += gridDim.x) {
        uint32_t s0;
        bool two;
        pairs.pair(p, s0, two);
        const uint32_t R = mt_discard_twists(P.seed + s0);
        const uint32_t *g = polys + (size_t)(R - R_lo) * kMtN;
        __syncthreads();                                 // the previous pair's reads are done
        if (lane == 0 && w < 2) {                        // mersenne_twister_engine::seed
            uint32_t *xr = w ? xr1 : xr0;
            uint32_t x = (uint32_t)(P.seed + s0 + (w && two ? 1 : 0));
            jump_put(xr, 0, x);
            for (uint32_t i = 1; i < kMtN; i++) {
                x = 1812433253u * (x ^ (x >> 30)) + i;
                jump_put(xr, i, x);
            }
        }
        // x[n] = f(x[n - 624], x[n - 623], x[n - 227]) for n in [from, to), to - from <= 227
        auto x_round = [&](uint32_t from, uint32_t to) {
            for (uint32_t i = t; i < 2 * (to - from); i += 96) {
                uint32_t *xr = i < to - from ? xr0 : xr1;
                const uint32_t n = from + (i < to - from ? i : i - (to - from));
                jump_put(xr, n, mt_twist1_alu3(xr[(n - 624u) & kJumpMask], xr[(n - 623u) & kJumpMask],
                                               xr[(n - 227u) & kJumpMask]));
            }
        };
        // e[n] = x[n] ^ x[n + 312] for n in [from, to), both halves
        auto e_form = [&](uint32_t from, uint32_t to) {
            for (uint32_t i = t; i < 2 * (to - from); i += 96) {
                const uint32_t m = to - from, n = from + (i < m ? i : i - m);
                const uint32_t *xr = i < m ? xr0 : xr1;
                jump_put(i < m ? er0 : er1, n, xr[n & kJumpMask] ^ xr[(n + 312u) & kJumpMask]);
            }
        };
        // x to 1272 before block 0, and e[0, 624) while the x it reads is still in the ring
        __syncthreads();
        e_form(0, 312);
        x_round(624, 832);
        __syncthreads();
        x_round(832, 1040);
        __syncthreads();
        e_form(312, 624);
        x_round(1040, 1248);
        __syncthreads();
        x_round(1248, kJumpXAhead);
        __syncthreads();
        uint32_t e_done = kMtN;
        uint32_t h[kJumpPer];
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) h[i] = 0;
        const uint32_t *seq = w == 0 ? (half ? xr1 : xr0) : (half ? er1 : er0);
        for (uint32_t a = 0; a < kJumpBlocks; a++) {
            const uint32_t xa = kMtN * a + kJumpXAhead - kMtN, ea = kMtN * a + kJumpEAhead;
            if (a > 0) {                                 // x to 624 a + 1272 (block 0: above)
                x_round(xa, xa + kJumpRound);
                __syncthreads();
                x_round(xa + kJumpRound, xa + 2 * kJumpRound);
                __syncthreads();
                x_round(xa + 2 * kJumpRound, xa + 3 * kJumpRound);
                __syncthreads();
            }
            e_form(e_done, ea);                          // e to 624 a + 960
            e_done = ea;
            __syncthreads();
            // this warp's 312 steps of block a: A (first half) for P2, B for P1 and P3
            const uint32_t run = kMtN * a + (w == 1 ? 0u : 312u);
            for (uint32_t u = 0; u < 312; u += kJumpPer) {
                const uint32_t k0 = run + u;
                uint32_t gb = jump_bits(g, k0);
                if (w == 0) gb ^= jump_bits(g, k0 - 312);
                if (u + kJumpPer > 312) gb &= (1u << (312 - u)) - 1u;
                if (gb == 0) continue;
                const uint32_t *wp = seq + ((k0 + kJumpPer * hl) & kJumpMask);
                uint32_t W[kJumpWin];
#pragma unroll
                for (int m = 0; m < kJumpWin; m++) W[m] = wp[m];
                jump_triple<0>(h, W, gb);
                jump_triple<3>(h, W, gb >> 3);
                jump_triple<6>(h, W, gb >> 6);
                jump_triple<9>(h, W, gb >> 9);
                jump_triple<12>(h, W, gb >> 12);
                jump_triple<15>(h, W, gb >> 15);
                jump_triple<18>(h, W, gb >> 18);
            }
            __syncthreads();                             // block a's reads are done
        }
        // P_(w+1) of spin `half` -> s_jump[(3 half + w) * 336 + j']
#pragma unroll
        for (int i = 0; i < kJumpPer; i++) s_jump[(3 * half + w) * 336 + kJumpPer * hl + i] = h[i];
        __syncthreads();
        // h_j' = P1 ^ P2, h_(312+j') = P1 ^ P3 -> state words at 2048 + 624 sp + j
        uint32_t *hs = s_jump + 2048;
        for (uint32_t i = t; i < 2 * 624; i += 96) {
            const uint32_t sp = i / 624, j = i % 624, jj = j % 312;
            const uint32_t *Ps = s_jump + 3 * sp * 336;
            hs[i] = Ps[jj] ^ Ps[(j < 312 ? 336 : 2 * 336) + jj];
        }
        __syncthreads();
        // block of regeneration R: x[624 R + q] = h_(q+1), q < 623, and one more twist word
        for (uint32_t i = t; i < 2 * 624; i += 96) {
            const uint32_t sp = i / 624, q = i % 624;
            if (sp == 1 && !two) continue;
            const uint32_t spin = s0 + sp;
            const uint32_t *hp = hs + 624 * sp;
            const uint32_t v = q < kMtN - 1 ? hp[q + 1] : mt_twist1(hp[0], hp[1], hp[397]);
            G.mt_r[(size_t)spin * kMtN + q] = v;
            G.mt_u[(size_t)spin * kMtN + q] = v;
            const uint32_t pos = (uint32_t)(P.seed + spin - (uint64_t)kMtN * (R - 1));
            if (q == 0) {
                G.p_r[spin] = pos;
                G.p_u[spin] = pos;
                G.nhead[spin] = 0;
                G.ncnt[spin] = 0;
                G.uhead[spin] = 0;
                G.ucnt[spin] = 0;
            }
            if (FAN)
                for (uint32_t d = 0; d < F.n; d++) {
                    const SeedCopy c = F.d[d];
                    if (spin >= c.n) continue;
                    c.mt[(size_t)spin * kMtN + q] = v;
                    if (q == 0) {
                        c.p[spin] = pos;
                        c.c0[spin] = 0;
                        c.c1[spin] = 0;
                        c.c2[spin] = 0;
                    }
                }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Generator flavour of the reference's CUDA build (kernels.cu:76-80): thrust::minstd_rand,
// x <- 48271 x mod (2^31 - 1), one 31-bit state per generator (kept in p_r / p_u).
// ------------------------------------------------------------------------------------------
constexpr uint32_t kMsA = 48271u, kMsM = 2147483647u;

__host__ __device__ constexpr uint32_t ms_mulmod(uint64_t x, uint64_t y) {
    // exact x*y mod (2^31 - 1) for x, y < 2^31: 2^31 = 1 (mod m), so fold the high bits twice
    const uint64_t p = x * y;
    const uint64_t r = (p & kMsM) + (p >> 31);
    const uint64_t r2 = (r & kMsM) + (r >> 31);
    return (uint32_t)(r2 >= kMsM ? r2 - kMsM : r2);
}

struct MsPow {                       // kMsA^(j+1) mod m, j < 32: lane j's jump ahead
    uint32_t v[32];
};
constexpr MsPow ms_pow_table() {
    MsPow t{};
    uint32_t a = kMsA;
    for (int j = 0; j < 32; j++) {
        t.v[j] = a;
        a = ms_mulmod(a, kMsA);
    }
    return t;
}
__constant__ MsPow c_ms_pow = ms_pow_table();

// linear_congruential_engine::seed + discard (thrust/random/detail/linear_congruential_engine
// .inl, linear_congruential_engine_discard.h): x0 = s mod m (1 if that is 0), then a^z x0.
__device__ __forceinline__ uint32_t ms_seed_discard(uint32_t s, uint64_t z) {
    uint32_t x = s % kMsM;
    if (x == 0u) x = 1u;
    uint64_t mul = kMsA, acc = 1;
    while (z) {
        if (z & 1u) acc = ms_mulmod(acc, mul);
        mul = ms_mulmod(mul, mul);
        z >>= 1;
    }
    return ms_mulmod(acc, x);
}

__global__ void k_seed_minstd(DevParams P, RngState G, uint32_t spin_lo, uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (spin >= spin_hi) return;
    const uint64_t sd = P.seed + spin;                 // kernels.cu:77-78, 87-88
    const uint32_t x = ms_seed_discard((uint32_t)sd, sd);
    G.p_r[spin] = x;
    G.p_u[spin] = x;
    G.nhead[spin] = 0;
    G.ncnt[spin] = 0;
    G.uhead[spin] = 0;
    G.ucnt[spin] = 0;
}

// thrust::uniform_real_distribution<float>(0, 1): (x - min) / (1 + (max - min)), then * 1 + 0
__device__ __forceinline__ float ms_uniform(uint32_t x) {
    const float r = __fdiv_rn(__uint2float_rn(x - 1u), __fadd_rn(1.0f, (float)(kMsM - 2u)));
    return __fadd_rn(__fmul_rn(r, 1.0f), 0.0f);
}

// One warp per spin: lane l takes the (l+1)-th next engine output, 32 per pass. Tops up the
// spin's Gaussian ring (and its uniform ring when at most half full).
// Gaussian deviates a spin can still draw: three per remaining step of its walk (all scans to
// come), plus 1/16 and 96 for rejected moves (a rejected crossing draws its step again). A
// refill stops there instead of filling the whole ring: the last round of a short walk would
// otherwise generate deviates nobody reads. A spin that draws more pauses and is topped up in
// the next round, as when its ring runs out; the sequence it reads is the same either way.
__device__ __forceinline__ uint32_t normals_left(const DevParams &P, const uint32_t *__restrict__ tp,
                                                 const uint32_t *__restrict__ ds, uint32_t spin,
                                                 uint32_t flags) {
    const uint32_t d = ds[spin], t = (flags & kFlagStarted) ? tp[spin] : 0u;
    if (d > P.n_dummy_scan) return 0u;
    const uint64_t steps = (uint64_t)(P.n_dummy_scan - d) * P.n_timepoints +
                           (t < P.n_timepoints ? P.n_timepoints - t : 0u);
    const uint64_t n = 3 * steps + ((3 * steps) >> 4) + 96;
    return n > 0xffffffffull ? 0xffffffffu : (uint32_t)n;
}

__device__ __forceinline__ void refill_spin_minstd(uint32_t spin, const RngState &G,
                                                   const uint32_t *__restrict__ ms_delta,
                                                   uint32_t cap, int lane) {
    const uint32_t nc = G.ncnt[spin], nh = G.nhead[spin], uc = G.ucnt[spin], nlen = G.nlen;
    const uint32_t fill = min(nlen, cap);
    if (nc < fill) {
        uint32_t x = G.p_r[spin];
        float *nb = G.nbuf + (size_t)spin * nlen;
        const uint32_t K = fill - nc, wpos = nh + nc;
        for (uint32_t b = 0; b < K; b += 32) {
            const uint32_t r = min(32u, K - b);
            if ((uint32_t)lane < r)
                nb[(wpos + b + lane) % nlen] =
                    ms_normal(ms_mulmod(x, c_ms_pow.v[lane]), ms_delta);
            x = ms_mulmod(x, c_ms_pow.v[r - 1]);
        }
        if (lane == 0) {
            G.p_r[spin] = x;
            G.ncnt[spin] = fill;
        }
    }
    if (uc <= kUnifBuf / 2) {
        uint32_t x = G.p_u[spin];
        float *ub = G.ubuf + (size_t)spin * kUnifBuf;
        const uint32_t K = kUnifBuf - uc, wpos = G.uhead[spin] + uc;
        for (uint32_t b = 0; b < K; b += 32) {
            const uint32_t r = min(32u, K - b);
            if ((uint32_t)lane < r)
                ub[(wpos + b + lane) % kUnifBuf] = ms_uniform(ms_mulmod(x, c_ms_pow.v[lane]));
            x = ms_mulmod(x, c_ms_pow.v[r - 1]);
        }
        if (lane == 0) {
            G.p_u[spin] = x;
            G.ucnt[spin] = kUnifBuf;
        }
    }
}

__global__ void __launch_bounds__(128)
    k_refill_minstd(DevParams P, RngState G, const uint32_t *__restrict__ flags,
                    const uint32_t *__restrict__ tp, const uint32_t *__restrict__ ds,
                    const uint32_t *__restrict__ ms_delta, uint32_t spin_lo, uint32_t spin_hi) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t spin = spin_lo + blockIdx.x * 4 + w; spin < spin_hi; spin += gridDim.x * 4) {
        const uint32_t f = flags[spin];
        if (f & kFlagDone) continue;
        refill_spin_minstd(spin, G, ms_delta, normals_left(P, tp, ds, spin, f), lane);
        __syncwarp();
    }
}

__global__ void k_debug_ms_normal(uint32_t x_lo, uint32_t n, float *y, const uint32_t *delta) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = ms_normal(x_lo + i, delta);
}

// ------------------------------------------------------------------------------------------
// Initial state (kernels.cu:90-104)
// ------------------------------------------------------------------------------------------
__global__ void k_init(DevParams P, DevTables Tb, const uint2 *__restrict__ vox,
                       const float *__restrict__ M0, const float *__restrict__ XYZ0,
                       SpinState S, Outputs O, int fp64_state, uint32_t spin_lo,
                       uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (spin >= spin_hi) return;
    float p0[3], m[3];
    for (int i = 0; i < 3; i++) {
        p0[i] = XYZ0[3 * (size_t)spin + i];
        m[i] = M0[3 * (size_t)spin + i];
    }
    if (O.XYZ1) {
        float *xyz1 = O.XYZ1 + 3 * (size_t)spin * P.traj_len;
        for (int i = 0; i < 3; i++) xyz1[i] = p0[i];               // kernels.cu:96
    }
    S.x[spin] = dbits((double)p0[0]);
    S.y[spin] = dbits((double)p0[1]);
    S.z[spin] = dbits((double)p0[2]);
    S.mx[spin] = m[0];
    S.my[spin] = m[1];
    S.mz[spin] = m[2];
    S.acc[spin] = 0.f;
    S.acc_e[spin] = 0.f;
    if (fp64_state) {
        S.accd[spin] = 0.;
        S.dmx[spin] = m[0];
        S.dmy[spin] = m[1];
        S.dmz[spin] = m[2];
    }
    S.field[spin] = 0.f;
    S.ind_old[spin] = P.matrix_length + 1;
    S.tp[spin] = 0;
    S.tp_old[spin] = 0;
    S.ds[spin] = 0;
    S.itr[spin] = 0;
    S.ctr[spin] = 1;
    S.ctr2[spin] = 0;
    const int64_t i0 = (int64_t)((double)p0[0] * P.s2g[0]) * P.nynz +
                       (int64_t)((double)p0[1] * P.s2g[1]) * P.nz +
                       (int64_t)((double)p0[2] * P.s2g[2]);
    if (i0 < 0 || i0 >= P.matrix_length) {
        S.flags[spin] = kFlagDone | ((uint32_t)SW_SPIN_START_OOB << 16);
        if (O.status) O.status[spin] = SW_SPIN_START_OOB;
        return;
    }
    S.flags[spin] = voxel_record(vox, i0, P.field_bf16).y & 0xffu;  // ts_old, not started
}

// ------------------------------------------------------------------------------------------
// Generator refill
// ------------------------------------------------------------------------------------------
constexpr int kRefillWarps = 4;
static_assert(kRefillBatchSpins == 32u * kRefillWarps, "32 spins per warp in the batch refill");

// Brings the spin's current 624-word block into shared memory (if it is not there yet),
// regenerates it, and writes it back.
__device__ __forceinline__ void twist_block(uint32_t *gst, uint32_t *s, bool &in_smem, int lane) {
    if (!in_smem)
        for (int i = lane; i < kMtN; i += 32) s[i] = gst[i];
    __syncwarp();
    mt_twist_warp(s, lane);
    for (int i = lane; i < kMtN; i += 32) gst[i] = s[i];
    in_smem = true;
    __syncwarp();
}

__device__ __forceinline__ uint32_t block_word(const uint32_t *gst, const uint32_t *s,
                                               bool in_smem, uint32_t i) {
    return in_smem ? s[i] : gst[i];
}

// Appends K polar pairs (normal_distribution<float>: y*m first, x*m saved for the next call) from
// the mt19937 state gst at position p to the ring nb of rlen deviates, from slot wpos on (wpos +
// 2 K < 3 rlen); 32 candidate pairs per pass, accepted pairs compacted with a ballot. `s` is the
// warp's 624-word shared block.
__device__ __forceinline__ uint32_t ring_slot(uint32_t x, uint32_t rlen) {   // x < 3 rlen
    x -= x >= rlen ? rlen : 0u;
    x -= x >= rlen ? rlen : 0u;
    return x;
}

__device__ __forceinline__ void refill_normals_mt(uint32_t *gst, uint32_t &p, float *nb,
                                                  uint32_t rlen, uint32_t wpos, uint32_t K,
                                                  uint32_t *s, const float *s_tab,
                                                  const LogfTables &L, int lane) {
    const unsigned lt_mask = (1u << lane) - 1u;
    uint32_t produced = 0;
    bool in_smem = false;
    while (produced < K) {
        if (p >= (uint32_t)kMtN) {
            twist_block(gst, s, in_smem, lane);
            p = 0;
        }
        uint32_t w0 = 0, w1 = 0;
        uint32_t npairs;
        bool straddle = false;
        if (kMtN - p == 1) {            // pair = last word of this block + first of next
            w0 = block_word(gst, s, in_smem, kMtN - 1);
            twist_block(gst, s, in_smem, lane);
            w1 = s[0];
            npairs = 1;
            straddle = true;
        } else {
            npairs = min(32u, (kMtN - p) / 2);
            if ((uint32_t)lane < npairs) {
                w0 = block_word(gst, s, in_smem, p + 2 * lane);
                w1 = block_word(gst, s, in_smem, p + 2 * lane + 1);
            }
        }
        const bool valid = (uint32_t)lane < npairs;
        const float u1 = canon24(mt_temper(w0)), u2 = canon24(mt_temper(w1));
        const float x = 2.0f * u1 - 1.0f, y = 2.0f * u2 - 1.0f;
        const float r2 = x * x + y * y;
        const bool ok = valid && !(r2 > 1.0f || r2 == 0.0f);
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        const uint32_t rank = __popc(bal & lt_mask);
        const uint32_t need = K - produced;
        if (ok && rank < need) {
            const float lg = logf_libm(r2, s_tab, L);
            const float mult = __fsqrt_rn(__fdiv_rn(-2.0f * lg, r2));
            const uint32_t pos = ring_slot(wpos + 2 * (produced + rank), rlen);
            nb[pos] = y * mult;                                  // returned first
            nb[pos + 1 == rlen ? 0 : pos + 1] = x * mult;        // saved for the next call
        }
        const uint32_t nacc = __popc(bal);
        if (nacc <= need) {
            produced += nacc;
            p = straddle ? 1 : p + 2 * npairs;
        } else {
            const unsigned m2 = __ballot_sync(0xffffffffu, ok && rank == need - 1);
            const uint32_t last = __ffs(m2) - 1;
            produced = K;
            p = p + 2 * (last + 1);
        }
    }
}

// Appends `need` crossing uniforms (uniform_real_distribution<float>(0,1)) from the state gst at
// position p to the ring ub of RLEN entries (a power of two), from count wpos on.
template <uint32_t RLEN>
__device__ __forceinline__ void refill_uniforms_mt(uint32_t *gst, uint32_t &p, float *ub,
                                                   uint32_t wpos, uint32_t need, uint32_t *s,
                                                   int lane) {
    uint32_t produced = 0;
    bool in_smem = false;
    while (produced < need) {
        if (p >= (uint32_t)kMtN) {
            twist_block(gst, s, in_smem, lane);
            p = 0;
        }
        const uint32_t n = min(min(32u, (uint32_t)kMtN - p), need - produced);
        if ((uint32_t)lane < n) {
            const uint32_t wv = block_word(gst, s, in_smem, p + lane);
            ub[(wpos + produced + lane) % RLEN] = canon24(mt_temper(wv));
        }
        p += n;
        produced += n;
    }
}

// One warp tops up the rings of one spin from its mt19937 states: Gaussian deviates from gen_r
// (normal_distribution<float>, polar method) and, when at most half full, crossing uniforms from
// gen_u. `s` is the warp's 624-word shared block.
__device__ __forceinline__ void refill_spin_mt(uint32_t spin, const RngState &G,
                                               const LogfTables &L, const float *s_tab,
                                               uint32_t *s, uint32_t cap, int lane) {
    const uint32_t nc = G.ncnt[spin], fill = min(G.nlen, cap);
    const uint32_t K = fill > nc ? min((fill - nc + 1) / 2, (G.nlen - nc) / 2) : 0u;  // pairs
    if (K > 0) {
        uint32_t p = G.p_r[spin];
        refill_normals_mt(G.mt_r + (size_t)spin * kMtN, p, G.nbuf + (size_t)spin * G.nlen, G.nlen,
                          G.nhead[spin] + nc, K, s, s_tab, L, lane);
        if (lane == 0) {
            G.p_r[spin] = p;
            G.ncnt[spin] = nc + 2 * K;
        }
    }
    const uint32_t uc = G.ucnt[spin];
    if (uc <= kUnifBuf / 2) {
        const uint32_t need = kUnifBuf - uc;
        uint32_t p = G.p_u[spin];
        refill_uniforms_mt<kUnifBuf>(G.mt_u + (size_t)spin * kMtN, p,
                                     G.ubuf + (size_t)spin * kUnifBuf, G.uhead[spin] + uc, need,
                                     s, lane);
        if (lane == 0) {
            G.p_u[spin] = p;
            G.ucnt[spin] = uc + need;
        }
    }
}

__global__ void __launch_bounds__(32 * kRefillWarps)
    k_refill(DevParams P, RngState G, const uint32_t *__restrict__ flags,
             const uint32_t *__restrict__ tp, const uint32_t *__restrict__ ds, LogfTables L,
             uint32_t spin_lo, uint32_t spin_hi) {
    __shared__ float s_tab[192];
    __shared__ uint32_t s_mt[kRefillWarps][kMtN];
    for (int i = threadIdx.x; i < 192; i += blockDim.x) s_tab[i] = L.tab[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t spin = spin_lo + blockIdx.x * kRefillWarps + w; spin < spin_hi;
         spin += gridDim.x * kRefillWarps) {
        const uint32_t f = flags[spin];
        if (f & kFlagDone) continue;
        refill_spin_mt(spin, G, L, s_tab, s_mt[w], normals_left(P, tp, ds, spin, f), lane);
        __syncwarp();
    }
}

// Pooled generators (PoolState): one warp per stream tops its Gaussian ring up to the lowest
// read position of the pairs that paused in the last walk plus kPoolNorm (whole pairs); streams
// no walking pair reported are skipped. The deviates of stream s are those spin s draws in every
// instance of the batch. The pair with the lowest read position then has a full ring, so the
// batch always makes progress.
__global__ void __launch_bounds__(32 * kRefillWarps)
    k_refill_pool(PoolState Q, LogfTables L, uint32_t n_streams) {
    __shared__ float s_tab[192];
    __shared__ uint32_t s_mt[kRefillWarps][kMtN];
    for (int i = threadIdx.x; i < 192; i += blockDim.x) s_tab[i] = L.tab[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t st = blockIdx.x * kRefillWarps + w; st < n_streams;
         st += gridDim.x * kRefillWarps) {
        const uint32_t nm = Q.nmin[st];
        if (nm == kPoolNone) continue;
        const uint32_t target = (nm + kPoolNorm) & ~1u, w0 = Q.nw[st];
        if (target > w0) {
            uint32_t p = Q.p_r[st];
            refill_normals_mt(Q.mt_r + (size_t)st * kMtN, p, Q.nbuf + (size_t)st * kPoolNorm,
                              kPoolNorm, w0 & (kPoolNorm - 1), (target - w0) / 2, s_mt[w], s_tab,
                              L, lane);
            if (lane == 0) {
                Q.p_r[st] = p;
                Q.nw[st] = target;
            }
        }
        if (lane == 0) Q.nmin[st] = kPoolNone;      // the next walk reports afresh
        __syncwarp();
    }
}

// Instance of work block b of a fused batch launch: the last descriptor whose first block is
// <= b (descriptors in block order), found by thread 0 and shared with the block.
template <bool WALK>
__device__ __forceinline__ uint32_t batch_instance(const BatchInst *__restrict__ D, uint32_t n_inst,
                                                   uint32_t b, uint32_t *s_k) {
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = n_inst;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint32_t b0 = WALK ? D[mid].walk_block0 : D[mid].unif_block0;
            if (b0 <= b) lo = mid; else hi = mid;
        }
        *s_k = lo;
    }
    __syncthreads();
    return *s_k;
}

// The crossing uniforms of a pooled batch, every instance in one launch (each instance spin has
// its own gen_u ring, topped up when at most half full, as k_refill does): block b covers
// 32 * kRefillWarps consecutive spins of one instance, one warp per 32 of them. The warp reads
// their counters together and tops up, one after the other, the rings of those that need it:
// after the first round only spins that crossed substrates do, so most warps only look.
__global__ void __launch_bounds__(32 * kRefillWarps)
    k_refill_uniforms_batch(const BatchInst *__restrict__ D, uint32_t n_inst) {
    __shared__ uint32_t s_mt[kRefillWarps][kMtN];
    __shared__ uint32_t s_k;
    const BatchInst &I = D[batch_instance<false>(D, n_inst, blockIdx.x, &s_k)];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t base = ((blockIdx.x - I.unif_block0) * kRefillWarps + w) * 32;
    const uint32_t mine = base + lane;
    const RngState &G = I.G;
    bool needy = false;
    uint32_t uc = 0;
    if (mine < I.n_spins && !(I.S.flags[mine] & kFlagDone)) {
        uc = G.ucnt[mine];
        needy = uc <= kUnifBuf / 2;
    }
    unsigned todo = __ballot_sync(0xffffffffu, needy);
    while (todo) {
        const int l = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t spin = base + l;
        const uint32_t c = __shfl_sync(0xffffffffu, uc, l);
        const uint32_t need = kUnifBuf - c;
        uint32_t p = G.p_u[spin];
        refill_uniforms_mt<kUnifBuf>(G.mt_u + (size_t)spin * kMtN, p,
                                     G.ubuf + (size_t)spin * kUnifBuf, G.uhead[spin] + c, need,
                                     s_mt[w], lane);
        if (lane == 0) {
            G.p_u[spin] = p;
            G.ucnt[spin] = c + need;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------------
// Signal mode: one echo's M added to its (echo, substrate) sums. The lanes of a warp that reach
// an echo together with the same key are summed by shuffles first, so that one lane per key
// does the atomic additions (the lanes of a warp are spins walking in step).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void signal_add(const Outputs &O, uint32_t key, const double (&v)[3]) {
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
    double s[3] = {v[0], v[1], v[2]};
    unsigned rest = grp & ~(1u << leader);
    while (rest) {
        const int b = __ffs(rest) - 1;
        rest &= rest - 1;
        for (int i = 0; i < 3; i++) {
            const double x = __shfl_sync(grp, v[i], b);
            if (lane == leader) s[i] += x;
        }
    }
    if (lane == leader) {
        for (int i = 0; i < 3; i++) atomicAdd(O.sig + 3 * (size_t)key + i, s[i]);
        atomicAdd(O.cnt + key, (unsigned long long)__popc(grp));
    }
}

// ------------------------------------------------------------------------------------------
// The walk (kernels.cu:107-232)
// ------------------------------------------------------------------------------------------
// POOL: the spin draws its Gaussian steps from the pooled stream of its id (PoolState Q) instead
// of its own ring, G.nhead holding its read position there (an absolute count); its crossing
// uniforms come from its own ring as usual.
template <int PREC, bool DBL, bool POOL = false>
__device__ __forceinline__ bool walk_spin(const uint32_t spin, uint32_t flags, const DevParams &P,
                                          const DevTables &Tb, const uint2 *__restrict__ vox,
                                          const SpinState &S, const RngState &G,
                                          const Outputs &O, const PoolState &Q = PoolState{}) {
    constexpr bool KAHAN = PREC == SW_PREC_KAHAN;
    uint64_t xo[3] = {S.x[spin], S.y[spin], S.z[spin]};    // bit patterns of the doubles
    float m0[3] = {S.mx[spin], S.my[spin], S.mz[spin]}, m1[3];
    float acc = S.acc[spin], acc_e = KAHAN ? S.acc_e[spin] : 0.f;
    double accd = 0., d0[3] = {0., 0., 0.}, d1[3];
    if (DBL) {
        accd = S.accd[spin];
        d0[0] = S.dmx[spin];
        d0[1] = S.dmy[spin];
        d0[2] = S.dmz[spin];
    }
    float field = S.field[spin];
    int64_t ind_old = S.ind_old[spin];
    uint32_t tp = S.tp[spin], tp_old = S.tp_old[spin], ds = S.ds[spin], itr = S.itr[spin];
    uint32_t ctr = S.ctr[spin], ctr2 = S.ctr2[spin];
    uint32_t c_rf = ctr & 0xffffu, c_te = ctr >> 16, c_dph = ctr2 & 0xffffu, c_grad = ctr2 >> 16;
    uint32_t ts_old = flags & 0xffu;
    bool started = (flags & kFlagStarted) != 0;
    double dscale = __ldg(Tb.dscale + ts_old);

    const uint32_t NLEN = POOL ? kPoolNorm : G.nlen;
    constexpr uint32_t ULEN = kUnifBuf;
    uint32_t nh, nc;
    const float *nb;
    if (POOL) {
        const uint32_t nr = G.nhead[spin];
        nc = Q.nw[spin] - nr;
        nh = nr & (kPoolNorm - 1);
        nb = Q.nbuf + (size_t)spin * kPoolNorm;
    } else {
        nh = G.nhead[spin];
        nc = G.ncnt[spin];
        nb = G.nbuf + (size_t)spin * NLEN;
    }
    uint32_t uh = G.uhead[spin], uc = G.ucnt[spin];
    const float *ub = G.ubuf + (size_t)spin * kUnifBuf;

    constexpr uint32_t NONE = 0xffffffffu;
    const bool last_scan0 = ds == P.n_dummy_scan;
    uint32_t t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
    uint32_t t_te = (last_scan0 && c_te < P.n_TE) ? (uint32_t)Tb.te_tp[c_te] : NONE;
    uint32_t t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
    uint32_t t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;
    // The earliest pending event time from `from` on: one compare per step instead of four.
    // An event whose time has passed never fires (as in the reference, whose per-step
    // comparisons never meet it again), so it is left out.
    uint32_t t_next = NONE;
    auto next_event = [&](uint32_t from) {
        uint32_t t = NONE;
        if (t_dph >= from) t = min(t, t_dph);
        if (t_grad >= from) t = min(t, t_grad);
        if (t_rf >= from) t = min(t, t_rf);
        if (t_te >= from) t = min(t, t_te);
        t_next = t;
    };
    next_event(tp);

    int status = -1;   // -1: paused (buffers ran low)
    for (;;) {
        if (!started) {
            if (ds > P.n_dummy_scan) { status = SW_SPIN_OK; break; }
            const RfOp op = Tb.scan_rf[ds];                         // kernels.cu:110-120
            rf_f(op, m0, m1);
            m0[0] = m1[0]; m0[1] = m1[1]; m0[2] = m1[2];
            if (DBL) {
                rf_d(op, d0, d1);
                d0[0] = d1[0]; d0[1] = d1[1]; d0[2] = d1[2];
            }
            ind_old = P.matrix_length + 1;                          // kernels.cu:123-126
            tp = tp_old = 0;
            c_rf = 1; c_te = 0; c_dph = 0; c_grad = 0;
            acc = 0.f; acc_e = 0.f; accd = 0.;
            started = true;
            t_rf = 1 < P.n_RF ? (uint32_t)Tb.rf[1].tp : NONE;
            t_te = (ds == P.n_dummy_scan && P.n_TE > 0) ? (uint32_t)Tb.te_tp[0] : NONE;
            t_dph = P.n_dephasing > 0 ? (uint32_t)Tb.dph_tp[0] : NONE;
            t_grad = P.n_gradient > 0 ? (uint32_t)Tb.grad_tp[0] : NONE;
            next_event(0);
        }
        if (tp >= P.n_timepoints) {                                 // kernels.cu:225-231
            const float te = (float)((double)((tp - tp_old) * (uint32_t)P.timestep_us) * 1e-6);
            dephase_relax_f(m0, m1, KAHAN ? acc + acc_e : acc, __ldg(Tb.T1f + ts_old),
                            __ldg(Tb.T2f + ts_old), te);
            m0[0] = m1[0]; m0[1] = m1[1]; m0[2] = m1[2];
            if (DBL) {
                const double ted = (double)(tp - tp_old) * (double)P.timestep_us * 1e-6;
                dephase_relax_d(d0, d1, accd, __ldg(Tb.T1d + ts_old), __ldg(Tb.T2d + ts_old), ted);
                d0[0] = d1[0]; d0[1] = d1[1]; d0[2] = d1[2];
            }
            ds++;
            started = false;
            continue;
        }
        if ((dnonzero(dscale) && nc < 3) || uc == 0) break;             // buffers low: pause

        // ---- random walk + boundary (kernels.cu:130-137) ----
        uint64_t xn[3] = {xo[0], xo[1], xo[2]};
        if (dnonzero(dscale)) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const float g = nb[nh];
                nh = (nh + 1 == NLEN) ? 0 : nh + 1;
                const uint64_t rnd = dbits(f2d_exact(g) * dscale);   // hardware DMUL
                uint64_t v = dadd_fp64(xo[i], rnd);  // xo[i] + rnd
                // the wrap in integer arithmetic too: the compiler evaluates a cheap double
                // expression here on every step whatever the branch, on the slow FP64 unit
                if (dneg(v))
                    v = dadd_bits(v, P.cross_fov ? dbits(P.fov[i]) : dtwice_abs(rnd));
                else if (dge_pos(v, P.fov[i]))
                    v = dadd_bits(v, dflip(P.cross_fov ? dbits(P.fov[i]) : dtwice_abs(rnd)));
                xn[i] = v;
            }
            nc -= 3;
        }
        // ---- voxel index (kernels.cu:140-147) ----
        const int64_t ind = voxel_coord(xn[0], P.s2g[0], P.s2g_f[0]) * P.nynz +
                            voxel_coord(xn[1], P.s2g[1], P.s2g_f[1]) * P.nz +
                            voxel_coord(xn[2], P.s2g[2], P.s2g_f[2]);
        if (ind >= P.matrix_length || ind < 0) { status = SW_SPIN_OOB; break; }
        // ---- mask, permeability, field (kernels.cu:150-170) ----
        if (ind != ind_old) {
            const uint2 v = voxel_record(vox, ind, P.field_bf16);
            const uint32_t ts = v.y;
            if (ts != ts_old) {
                const float u = ub[uh];
                uh = (uh + 1 == ULEN) ? 0 : uh + 1;
                uc--;
                if (u >= __ldg(Tb.pXY + ts_old * P.n_substrate + ts)) {
                    if ((uint64_t)(itr++) > P.max_iterations) { status = SW_SPIN_LOST; break; }
                    continue;
                }
                ts_old = ts;
            }
            ind_old = ind;
            field = __uint_as_float(v.x);
            dscale = __ldg(Tb.dscale + ts_old);
        }
        // ---- phase accumulation (kernels.cu:171-172) ----
        if (KAHAN) kahan_add(acc, acc_e, field); else acc += field;
        if (DBL) accd += (double)field;
        itr = 0;
        if (tp == t_next) {
        // ---- ideal dephasing (kernels.cu:175-178) ----
        if (tp == t_dph) {
            const float deg = __ldg(Tb.dph_deg + c_dph);
            const float inc = (float)spin * deg / (float)P.n_spins;
            if (KAHAN) kahan_add(acc, acc_e, inc); else acc += inc;
            if (DBL) accd += (double)spin * (double)deg / (double)P.n_spins;
            c_dph++;
            t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
        }
        // ---- gradient (kernels.cu:181-187) ----
        if (tp == t_grad) {
            const double g = grad_phase_deg(__ldg(Tb.gx + c_grad), __ldg(Tb.gy + c_grad),
                                            __ldg(Tb.gz + c_grad), xn, (double)P.timestep_us);
            if (KAHAN) {
                const float ghi = d2f_exact(dbits(g));
                kahan_add(acc, acc_e, ghi);
                kahan_add(acc, acc_e, d2f_exact(dadd_fp64(dbits(g), dflip(dbits(f2d_exact(ghi))))));
            } else {
                acc = d2f_exact(dadd_fp64(dbits(f2d_exact(acc)), dbits(g)));   // (float)((double)acc + g)
            }
            if (DBL) accd += g;
            c_grad++;
            t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;
        }
        // ---- RF pulse (kernels.cu:190-199) ----
        if (tp == t_rf) {
            const float te = (float)((double)((tp - tp_old) * (uint32_t)P.timestep_us) * 1e-6);
            dephase_relax_f(m0, m1, KAHAN ? acc + acc_e : acc, __ldg(Tb.T1f + ts_old),
                            __ldg(Tb.T2f + ts_old), te);
            const RfOp op = Tb.rf[c_rf];
            rf_f(op, m1, m0);
            if (DBL) {
                const double ted = (double)(tp - tp_old) * (double)P.timestep_us * 1e-6;
                dephase_relax_d(d0, d1, accd, __ldg(Tb.T1d + ts_old), __ldg(Tb.T2d + ts_old), ted);
                rf_d(op, d1, d0);
            }
            acc = 0.f; acc_e = 0.f; accd = 0.;
            tp_old = tp;
            c_rf++;
            t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
        }
        // ---- echo, last scan only (kernels.cu:202-215) ----
        if (tp == t_te) {
            const float te = (float)((double)((tp - tp_old) * (uint32_t)P.timestep_us) * 1e-6);
            dephase_relax_f(m0, m1, KAHAN ? acc + acc_e : acc, __ldg(Tb.T1f + ts_old),
                            __ldg(Tb.T2f + ts_old), te);
            if (DBL) {
                const double ted = (double)(tp - tp_old) * (double)P.timestep_us * 1e-6;
                dephase_relax_d(d0, d1, accd, __ldg(Tb.T1d + ts_old), __ldg(Tb.T2d + ts_old), ted);
                d0[0] = d1[0]; d0[1] = d1[1]; d0[2] = d1[2];
            }
            for (int i = 0; i < 3; i++) m0[i] = m1[i];
            if (O.sig) {
                double v[3];
                for (int i = 0; i < 3; i++) v[i] = (PREC == SW_PREC_FP64) ? d1[i] : (double)m1[i];
                signal_add(O, c_te * P.n_substrate + ts_old, v);
            } else {
                const size_t o = 3 * ((size_t)spin * P.n_TE + c_te);
                for (int i = 0; i < 3; i++) {
                    O.M1[o + i] = (PREC == SW_PREC_FP64) ? (float)d1[i] : m1[i];
                    if (DBL && O.M1d) O.M1d[o + i] = d1[i];
                }
                O.T[(size_t)spin * P.n_TE + c_te] = (uint8_t)ts_old;
            }
            acc = 0.f; acc_e = 0.f; accd = 0.;
            tp_old = tp;
            c_te++;
            t_te = c_te < P.n_TE ? (uint32_t)Tb.te_tp[c_te] : NONE;
        }
        next_event(tp + 1);
        }
        // ---- accept the move (kernels.cu:218-223) ----
        xo[0] = xn[0]; xo[1] = xn[1]; xo[2] = xn[2];
        if (P.record_traj && O.XYZ1) {
            float *dst = O.XYZ1 + 3 * ((size_t)spin * P.traj_len + (size_t)ds * P.n_timepoints + tp);
            dst[0] = (float)dfrom(xn[0]); dst[1] = (float)dfrom(xn[1]); dst[2] = (float)dfrom(xn[2]);
        }
        tp++;
    }

    // ---- save state ----
    S.x[spin] = xo[0]; S.y[spin] = xo[1]; S.z[spin] = xo[2];
    S.mx[spin] = m0[0]; S.my[spin] = m0[1]; S.mz[spin] = m0[2];
    S.acc[spin] = acc;
    if (KAHAN) S.acc_e[spin] = acc_e;
    if (DBL) {
        S.accd[spin] = accd;
        S.dmx[spin] = d0[0]; S.dmy[spin] = d0[1]; S.dmz[spin] = d0[2];
    }
    S.field[spin] = field;
    S.ind_old[spin] = ind_old;
    S.tp[spin] = tp; S.tp_old[spin] = tp_old; S.ds[spin] = ds; S.itr[spin] = itr;
    S.ctr[spin] = c_rf | (c_te << 16);
    S.ctr2[spin] = c_dph | (c_grad << 16);
    if (POOL) {               // read position: written count minus what is left
        const uint32_t nr = Q.nw[spin] - nc;
        G.nhead[spin] = nr;
        if (status < 0) atomicMin(Q.nmin + spin, nr);   // the next refill keeps what it needs
    } else {
        G.nhead[spin] = nh; G.ncnt[spin] = nc;
    }
    G.uhead[spin] = uh; G.ucnt[spin] = uc;
    uint32_t nf = ts_old | (started ? kFlagStarted : 0u);
    if (status >= 0) {
        nf |= kFlagDone | ((uint32_t)status << 16);
        if (!P.record_traj && O.XYZ1) {
            float *dst = O.XYZ1 + 3 * (size_t)spin * P.traj_len;
            dst[0] = (float)dfrom(xo[0]); dst[1] = (float)dfrom(xo[1]); dst[2] = (float)dfrom(xo[2]);
        }
        if (O.status) O.status[spin] = status;
    }
    S.flags[spin] = nf;
    return status < 0;
}

// 4 blocks of 256 per SM (64 registers): the walk is latency bound and its occupancy pays more
// than the registers the compiler would otherwise take (SE walk 37.7 vs 44.0 ms at 78 registers);
// a fifth block (48 registers, 76 bytes of spills) is slower again (SE 75.3 -> 83.1 ms of walk
// launch time per pass, GRE 1.11 -> 1.26 ms)
template <int PREC, bool DBL>
__global__ void __launch_bounds__(256, 4)
    k_walk(DevParams P, DevTables Tb, const uint2 *__restrict__ vox, SpinState S, RngState G,
           Outputs O, uint32_t *active, uint32_t spin_lo, uint32_t spin_hi,
           const uint32_t *__restrict__ order) {
    // grid-stride by whole warps: a grid smaller than the spins (a cap on blocks per SM) leaves
    // room on each SM for the other half's refill
    const uint32_t stride = gridDim.x * blockDim.x, lane = threadIdx.x & 31u;
    uint32_t paused = 0;
    for (uint32_t base = spin_lo + blockIdx.x * blockDim.x + (threadIdx.x - lane);
         base < spin_hi; base += stride) {
        const uint32_t i = base + lane;
        bool still = false;
        if (i < spin_hi) {
            const uint32_t spin = order ? __ldg(order + i) : i;
            const uint32_t flags = S.flags[spin];
            if (!(flags & kFlagDone)) still = walk_spin<PREC, DBL>(spin, flags, P, Tb, vox, S, G, O);
        }
        paused += __popc(__ballot_sync(0xffffffffu, still));
    }
    if (lane == 0 && paused) atomicAdd(active, paused);
}

// The walk of a pooled batch, every instance in one launch: work block b walks 256 spins of one
// instance (whose parameters, tables and state it reads from its descriptor), drawing their
// steps from the pooled streams Q (G.nhead: the instance's read positions in them). A grid
// smaller than the work blocks makes it persistent: each block strides over them.
template <int PREC, bool DBL>
__global__ void __launch_bounds__(256, 4)
    k_walk_batch(const BatchInst *__restrict__ D, uint32_t n_inst, uint32_t walk_blocks,
                 const uint2 *__restrict__ vox, PoolState Q, uint32_t *active) {
    __shared__ uint32_t s_k;
    uint32_t paused = 0;
    for (uint32_t b = blockIdx.x; b < walk_blocks; b += gridDim.x) {
        __syncthreads();                             // s_k of the previous work block is read
        const BatchInst &I = D[batch_instance<true>(D, n_inst, b, &s_k)];
        const uint32_t spin = (b - I.walk_block0) * 256 + threadIdx.x;
        bool still = false;
        if (spin < I.n_spins) {
            const uint32_t flags = I.S.flags[spin];
            if (!(flags & kFlagDone))
                still = walk_spin<PREC, DBL, true>(spin, flags, I.P, I.Tb, vox, I.S, I.G, I.O, Q);
        }
        paused += __popc(__ballot_sync(0xffffffffu, still));
    }
    if ((threadIdx.x & 31) == 0 && paused) atomicAdd(active, paused);
}

__global__ void k_debug_logf(const float *x, float *y, uint64_t n, LogfTables L) {
    __shared__ float s_tab[192];
    for (int i = threadIdx.x; i < 192; i += blockDim.x) s_tab[i] = L.tab[i];
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        y[i] = logf_libm(x[i], s_tab, L);
}

__global__ void k_debug_d2f(const double *x, float *y, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        y[i] = d2f_exact(dbits(x[i]));
}

__global__ void k_debug_dadd(const double *a, const double *b, double *y, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        y[i] = dadd_int(a[i], b[i]);
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
static int grid_for(int64_t work, int block, int max_blocks) {
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    return (int)(g < max_blocks ? g : max_blocks);
}

cudaError_t launch_pack(const uint8_t *mask, const float *field, uint2 *out, int64_t n,
                        uint32_t n_substrate, uint32_t *bad_label, cudaStream_t st, bool bf16) {
    k_pack<<<grid_for(n, 256, 152 * 32), 256, 0, st>>>(mask, field, out, n, n_substrate,
                                                        bad_label, bf16 ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_seed(const DevParams &P, const RngState &G, cudaStream_t st) {
    return launch_seed_range(P, G, 0, P.n_spins, st);
}

cudaError_t launch_seed_range(const DevParams &P, const RngState &G, uint32_t lo, uint32_t hi,
                              cudaStream_t st, const JumpTable *jt, SeedCopies fan) {
    if (hi <= lo) return cudaSuccess;
    if (P.rng == SW_RNG_MINSTD) {
        k_seed_minstd<<<grid_for(hi - lo, 256, 1 << 30), 256, 0, st>>>(P, G, lo, hi);
        return cudaGetLastError();
    }
    // spins from c on jump (z = seed + spin >= z_min), the rest discard
    uint32_t c = hi;
    if (jt && jt->polys) {
        if (jt->z_min < (uint64_t)kMtN) return cudaErrorInvalidValue;
        c = (uint32_t)std::min<uint64_t>(hi, std::max<uint64_t>(lo, P.seed >= jt->z_min ? 0 : jt->z_min - P.seed));
        if (c < hi && (mt_discard_twists(P.seed + c) < jt->R_lo ||
                       mt_discard_twists(P.seed + hi - 1) >= jt->R_hi))
            return cudaErrorInvalidValue;            // the table does not cover these spins
    }
    if (c > lo) {
        const int grid = grid_for(((int64_t)c - lo + 1) / 2, kSeedWarps, 1 << 30);
        if (fan.n)
            k_seed<true><<<grid, 32 * kSeedWarps, 0, st>>>(P, G, lo, c, fan);
        else
            k_seed<false><<<grid, 32 * kSeedWarps, 0, st>>>(P, G, lo, c, fan);
    }
    if (hi > c) {
        const JumpPairs jp = JumpPairs::make(P.seed, c, hi);
        const int grid = (int)std::min<uint32_t>(jp.n_pairs, 152 * kJumpBlocksPerSm);
        if (fan.n)
            k_seed_jump<true><<<grid, 96, kJumpSmem, st>>>(P, G, jt->polys, jt->R_lo, jp, fan);
        else
            k_seed_jump<false><<<grid, 96, kJumpSmem, st>>>(P, G, jt->polys, jt->R_lo, jp, fan);
    }
    return cudaGetLastError();
}

cudaError_t launch_init(const DevParams &P, const DevTables &Tb, const uint2 *vox,
                        const float *M0, const float *XYZ0, const SpinState &S,
                        const Outputs &O, bool fp64_state, cudaStream_t st) {
    return launch_init_range(P, Tb, vox, M0, XYZ0, S, O, fp64_state, 0, P.n_spins, st);
}

cudaError_t launch_init_range(const DevParams &P, const DevTables &Tb, const uint2 *vox,
                              const float *M0, const float *XYZ0, const SpinState &S,
                              const Outputs &O, bool fp64_state, uint32_t lo, uint32_t hi,
                              cudaStream_t st) {
    if (hi <= lo) return cudaSuccess;
    k_init<<<grid_for(hi - lo, 256, 1 << 30), 256, 0, st>>>(P, Tb, vox, M0, XYZ0, S, O,
                                                           fp64_state ? 1 : 0, lo, hi);
    return cudaGetLastError();
}

cudaError_t launch_refill(const DevParams &P, const RngState &G, const SpinState &S,
                          const LogfTables &L, cudaStream_t st) {
    return launch_refill_range(P, G, S, L, 0, P.n_spins, st);
}

cudaError_t launch_refill_range(const DevParams &P, const RngState &G, const SpinState &S,
                                const LogfTables &L, uint32_t lo, uint32_t hi, cudaStream_t st) {
    if (hi <= lo) return cudaSuccess;
    if (P.rng == SW_RNG_MINSTD) {
        k_refill_minstd<<<grid_for(hi - lo, 4, 152 * 64), 128, 0, st>>>(P, G, S.flags, S.tp, S.ds,
                                                                         L.ms_delta, lo, hi);
        return cudaGetLastError();
    }
    k_refill<<<grid_for(hi - lo, kRefillWarps, 152 * 64), 32 * kRefillWarps, 0, st>>>(
        P, G, S.flags, S.tp, S.ds, L, lo, hi);
    return cudaGetLastError();
}

cudaError_t launch_walk(int prec, bool dbl, const DevParams &P, const DevTables &Tb,
                        const uint2 *vox, const SpinState &S, const RngState &G,
                        const Outputs &O, uint32_t *active, cudaStream_t st) {
    return launch_walk_range(prec, dbl, P, Tb, vox, S, G, O, active, 0, P.n_spins, st);
}

cudaError_t launch_walk_range(int prec, bool dbl, const DevParams &P, const DevTables &Tb,
                              const uint2 *vox, const SpinState &S, const RngState &G,
                              const Outputs &O, uint32_t *active, uint32_t lo, uint32_t hi,
                              cudaStream_t st, const uint32_t *order, int block, int max_blocks) {
    if (hi <= lo) return cudaSuccess;
    if (block != 64 && block != 128 && block != 256) return cudaErrorInvalidValue;
    const int g = grid_for(hi - lo, block, max_blocks > 0 ? max_blocks : 1 << 30);
    if (prec == SW_PREC_FP64)
        k_walk<SW_PREC_FP64, true><<<g, block, 0, st>>>(P, Tb, vox, S, G, O, active, lo, hi, order);
    else if (prec == SW_PREC_KAHAN && dbl)
        k_walk<SW_PREC_KAHAN, true><<<g, block, 0, st>>>(P, Tb, vox, S, G, O, active, lo, hi, order);
    else if (prec == SW_PREC_KAHAN)
        k_walk<SW_PREC_KAHAN, false><<<g, block, 0, st>>>(P, Tb, vox, S, G, O, active, lo, hi, order);
    else if (dbl)
        k_walk<SW_PREC_FP32, true><<<g, block, 0, st>>>(P, Tb, vox, S, G, O, active, lo, hi, order);
    else
        k_walk<SW_PREC_FP32, false><<<g, block, 0, st>>>(P, Tb, vox, S, G, O, active, lo, hi, order);
    return cudaGetLastError();
}

cudaError_t launch_refill_pool(const PoolState &Q, const LogfTables &L, uint32_t n_streams,
                               cudaStream_t st) {
    if (n_streams == 0) return cudaSuccess;
    k_refill_pool<<<grid_for(n_streams, kRefillWarps, 152 * 64), 32 * kRefillWarps, 0, st>>>(
        Q, L, n_streams);
    return cudaGetLastError();
}

cudaError_t launch_refill_uniforms_batch(const BatchInst *D, uint32_t n_inst, uint32_t unif_blocks,
                                         cudaStream_t st) {
    if (!n_inst || !unif_blocks) return cudaSuccess;
    k_refill_uniforms_batch<<<unif_blocks, 32 * kRefillWarps, 0, st>>>(D, n_inst);
    return cudaGetLastError();
}

cudaError_t launch_walk_batch(int prec, bool dbl, const BatchInst *D, uint32_t n_inst,
                              uint32_t walk_blocks, const uint2 *vox, const PoolState &Q,
                              uint32_t *active, cudaStream_t st, int max_blocks) {
    if (!n_inst || !walk_blocks) return cudaSuccess;
    const uint32_t g = max_blocks > 0 ? std::min<uint32_t>(walk_blocks, (uint32_t)max_blocks)
                                      : walk_blocks;
    const uint32_t wb = walk_blocks;
    if (prec == SW_PREC_FP64)
        k_walk_batch<SW_PREC_FP64, true><<<g, 256, 0, st>>>(D, n_inst, wb, vox, Q, active);
    else if (prec == SW_PREC_KAHAN && dbl)
        k_walk_batch<SW_PREC_KAHAN, true><<<g, 256, 0, st>>>(D, n_inst, wb, vox, Q, active);
    else if (prec == SW_PREC_KAHAN)
        k_walk_batch<SW_PREC_KAHAN, false><<<g, 256, 0, st>>>(D, n_inst, wb, vox, Q, active);
    else if (dbl)
        k_walk_batch<SW_PREC_FP32, true><<<g, 256, 0, st>>>(D, n_inst, wb, vox, Q, active);
    else
        k_walk_batch<SW_PREC_FP32, false><<<g, 256, 0, st>>>(D, n_inst, wb, vox, Q, active);
    return cudaGetLastError();
}

cudaError_t launch_debug_d2f(const double *x, float *y, uint64_t n, cudaStream_t st) {
    k_debug_d2f<<<grid_for((int64_t)n, 256, 152 * 16), 256, 0, st>>>(x, y, n);
    return cudaGetLastError();
}

cudaError_t launch_debug_dadd(const double *a, const double *b, double *y, uint64_t n,
                              cudaStream_t st) {
    k_debug_dadd<<<grid_for((int64_t)n, 256, 152 * 16), 256, 0, st>>>(a, b, y, n);
    return cudaGetLastError();
}

cudaError_t launch_debug_ms_normal(uint32_t x_lo, uint32_t n, float *y, const uint32_t *delta,
                                   cudaStream_t st) {
    k_debug_ms_normal<<<grid_for((int64_t)n, 256, 152 * 16), 256, 0, st>>>(x_lo, n, y, delta);
    return cudaGetLastError();
}

cudaError_t launch_debug_logf(const float *x, float *y, uint64_t n, const LogfTables &L,
                              cudaStream_t st) {
    k_debug_logf<<<grid_for((int64_t)n, 256, 152 * 16), 256, 0, st>>>(x, y, n, L);
    return cudaGetLastError();
}

}  // namespace sw
