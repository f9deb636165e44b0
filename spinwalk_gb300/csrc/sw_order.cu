// Morton re-sort of the spins: the order in which the walk kernel's threads take spins.
//
// The walk gathers one packed voxel record per step at the spin's position. Spins that share a
// warp but sit far apart in the phantom gather from 32 different cache lines; spins taken in
// the order of their positions along a Morton (Z-order) curve share lines and L2 sets when the
// phantom holds several spins per line. The spins' results do not depend on the order (each
// spin's walk reads only its own state and generators), so re-sorting changes which thread
// walks which spin and nothing else. The reference keeps the spins in id order (one thread per
// spin, src/sim/kernels.cu:70-90); this order is an addition of this implementation.
//
// Counting sort on a Morton key of the spin's current voxel, coarsened to `bits` bits per axis:
// k_order_key (key + histogram), k_order_scan (one block, exclusive scan in place),
// k_order_scatter (positions by atomics; the order inside a bucket is arbitrary). Finished
// spins get the last bucket, so whole warps of them exit at once.
#include <cuda_runtime.h>

#include "sw_device.cuh"
#include "sw_kernels.h"

namespace sw {

namespace {

__device__ __forceinline__ uint32_t coord_bits(uint64_t xb, double s2g, int64_t n, int shift) {
    int64_t i = (int64_t)(dfrom(xb) * s2g);
    i = i < 0 ? 0 : (i >= n ? n - 1 : i);
    return (uint32_t)i >> shift;
}

__global__ void k_order_key(DevParams P, SpinState S, OrderState Q, OrderShape sh,
                            uint32_t spin_lo, uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (spin >= spin_hi) return;
    uint32_t key = sh.n_buckets - 1;
    if (!(S.flags[spin] & kFlagDone)) {
        const uint32_t cx = coord_bits(S.x[spin], P.s2g[0], sh.n[0], sh.shift[0]);
        const uint32_t cy = coord_bits(S.y[spin], P.s2g[1], sh.n[1], sh.shift[1]);
        const uint32_t cz = coord_bits(S.z[spin], P.s2g[2], sh.n[2], sh.shift[2]);
        uint32_t m = 0;
        for (int b = sh.bits - 1; b >= 0; b--)                 // x most significant
            m = (m << 3) | (((cx >> b) & 1u) << 2) | (((cy >> b) & 1u) << 1) | ((cz >> b) & 1u);
        key = min(m, sh.n_buckets - 2);
    }
    Q.key[spin] = key;
    atomicAdd(Q.hist + key, 1u);
}

// Exclusive scan of n_buckets counters by one block of 1024 threads: thread t owns a contiguous
// run of ceil(n / 1024) counters.
__global__ void __launch_bounds__(1024) k_order_scan(uint32_t *hist, uint32_t n_buckets) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x, per = (n_buckets + 1023) / 1024;
    const uint32_t b0 = min(t * per, n_buckets), b1 = min(b0 + per, n_buckets);
    uint32_t s = 0;
    for (uint32_t b = b0; b < b1; b++) s += hist[b];
    part[t] = s;
    __syncthreads();
    for (uint32_t d = 1; d < 1024; d <<= 1) {                   // Hillis-Steele, inclusive
        const uint32_t v = t >= d ? part[t - d] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t ? part[t - 1] : 0u;
    for (uint32_t b = b0; b < b1; b++) {
        const uint32_t c = hist[b];
        hist[b] = run;
        run += c;
    }
}

__global__ void k_order_scatter(OrderState Q, uint32_t spin_lo, uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (spin >= spin_hi) return;
    const uint32_t pos = atomicAdd(Q.hist + Q.key[spin], 1u);
    Q.order[spin_lo + pos] = spin;
}

int ceil_log2(int64_t v) {
    int b = 0;
    while (((int64_t)1 << b) < v) b++;
    return b;
}

}  // namespace

OrderShape order_shape(const DevParams &P, uint32_t n_spins) {
    OrderShape sh{};
    // about 8 spins per bucket, at most 6 bits (64 cells) per axis
    int bits = (ceil_log2((int64_t)n_spins / 8 + 1) + 2) / 3;
    bits = bits < 1 ? 1 : (bits > kOrderMaxBitsPerAxis ? kOrderMaxBitsPerAxis : bits);
    sh.bits = bits;
    sh.n[2] = P.nz;
    sh.n[1] = P.nynz / P.nz;
    sh.n[0] = P.matrix_length / P.nynz;
    for (int i = 0; i < 3; i++) {
        const int s = ceil_log2(sh.n[i]) - bits;
        sh.shift[i] = s > 0 ? s : 0;
    }
    sh.n_buckets = (1u << (3 * bits)) + 1;      // + the bucket of finished spins
    return sh;
}

size_t order_hist_words() { return (1u << (3 * kOrderMaxBitsPerAxis)) + 1; }

cudaError_t launch_order(const DevParams &P, const SpinState &S, const OrderState &Q,
                         uint32_t lo, uint32_t hi, cudaStream_t st) {
    if (hi <= lo) return cudaSuccess;
    const OrderShape sh = order_shape(P, hi - lo);
    cudaError_t e = cudaMemsetAsync(Q.hist, 0, sh.n_buckets * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)((hi - lo + 255) / 256);
    k_order_key<<<g, 256, 0, st>>>(P, S, Q, sh, lo, hi);
    k_order_scan<<<1, 1024, 0, st>>>(Q.hist, sh.n_buckets);
    k_order_scatter<<<g, 256, 0, st>>>(Q, lo, hi);
    return cudaGetLastError();
}

}  // namespace sw
