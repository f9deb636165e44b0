// Kernel launchers of sw_kernels.cu (host side).
#pragma once
#include <cuda_runtime.h>

#include "sw_device.cuh"

namespace sw {

// bf16: 4-byte records (bfloat16 field | label << 16) instead of 8-byte {float field, label}
cudaError_t launch_pack(const uint8_t *mask, const float *field, uint2 *out, int64_t n,
                        uint32_t n_substrate, uint32_t *bad_label, cudaStream_t st,
                        bool bf16 = false);
cudaError_t launch_seed(const DevParams &P, const RngState &G, cudaStream_t st);
// Jump polynomials on the device (sw_mtjump.h): 624 words per regeneration count R in
// [R_lo, R_hi), for the spins whose discard count seed + spin is at least z_min (>= 624).
struct JumpTable {
    const uint32_t *polys = nullptr;
    uint64_t R_lo = 0, R_hi = 0;
    uint64_t z_min = ~0ull;
};
// Further destinations of the seeded state (a pooled batch: every instance's gen_u starts from
// its stream's seeded state): spin s < n gets the 624 words in mt, its position in p and the
// three ring counters c0, c1, c2 zeroed. d is a device array of n entries.
struct SeedCopy {
    uint32_t *mt, *p;
    uint32_t *c0, *c1, *c2;
    uint32_t n;
};
struct SeedCopies {
    const SeedCopy *d = nullptr;
    uint32_t n = 0;
};
// Spins with seed + spin >= jt->z_min are seeded by jump-ahead when jt is given (it must cover
// their regeneration counts), the others by the plain discard. With `fan`, the seeding kernels
// also store the state at those destinations (an instance of the kernels of its own: the
// seeding without destinations compiles as if they did not exist).
cudaError_t launch_seed_range(const DevParams &P, const RngState &G, uint32_t lo, uint32_t hi,
                              cudaStream_t st, const JumpTable *jt = nullptr,
                              SeedCopies fan = SeedCopies{});
// Tops up the rings of the spins in [lo, hi) that are not done, each to what its remaining walk
// can draw at most (S: flags, time point and scan of every spin).
cudaError_t launch_refill_range(const DevParams &P, const RngState &G, const SpinState &S,
                                const LogfTables &L, uint32_t lo, uint32_t hi, cudaStream_t st);
// order: walk order of the spins (null = id order); block: threads per block (64..256);
// max_blocks > 0 caps the grid (the blocks then stride over the spins).
cudaError_t launch_walk_range(int prec, bool dbl, const DevParams &P, const DevTables &Tb,
                              const uint2 *vox, const SpinState &S, const RngState &G,
                              const Outputs &O, uint32_t *active, uint32_t lo, uint32_t hi,
                              cudaStream_t st, const uint32_t *order = nullptr, int block = 256,
                              int max_blocks = 0);
// Pooled Gaussian generators of a batch (PoolState): refill of streams [0, n_streams).
cudaError_t launch_refill_pool(const PoolState &Q, const LogfTables &L, uint32_t n_streams,
                               cudaStream_t st);
// Spins per block of k_refill_uniforms_batch (32 per warp).
constexpr uint32_t kRefillBatchSpins = 128;
// The crossing-uniform refill and the walk of every instance of a pooled batch, one launch each:
// D holds n_inst descriptors (device memory) whose block ranges tile [0, walk_blocks) and
// [0, unif_blocks); each instance's results equal its own sw_sim run bit for bit.
cudaError_t launch_refill_uniforms_batch(const BatchInst *D, uint32_t n_inst, uint32_t unif_blocks,
                                         cudaStream_t st);
// max_blocks > 0 caps the walk's grid (persistent blocks striding over the work blocks).
cudaError_t launch_walk_batch(int prec, bool dbl, const BatchInst *D, uint32_t n_inst,
                              uint32_t walk_blocks, const uint2 *vox, const PoolState &Q,
                              uint32_t *active, cudaStream_t st, int max_blocks = 0);
// Morton re-sort of spins [lo, hi) into Q.order (sw_order.cu).
cudaError_t launch_order(const DevParams &P, const SpinState &S, const OrderState &Q,
                         uint32_t lo, uint32_t hi, cudaStream_t st);
OrderShape order_shape(const DevParams &P, uint32_t n_spins);
size_t order_hist_words();
cudaError_t launch_init(const DevParams &P, const DevTables &Tb, const uint2 *vox,
                        const float *M0, const float *XYZ0, const SpinState &S,
                        const Outputs &O, bool fp64_state, cudaStream_t st);
cudaError_t launch_init_range(const DevParams &P, const DevTables &Tb, const uint2 *vox,
                              const float *M0, const float *XYZ0, const SpinState &S,
                              const Outputs &O, bool fp64_state, uint32_t lo, uint32_t hi,
                              cudaStream_t st);
cudaError_t launch_refill(const DevParams &P, const RngState &G, const SpinState &S,
                          const LogfTables &L, cudaStream_t st);
cudaError_t launch_walk(int prec, bool dbl, const DevParams &P, const DevTables &Tb,
                        const uint2 *vox, const SpinState &S, const RngState &G,
                        const Outputs &O, uint32_t *active, cudaStream_t st);
cudaError_t launch_debug_dadd(const double *a, const double *b, double *y, uint64_t n,
                              cudaStream_t st);
cudaError_t launch_debug_d2f(const double *x, float *y, uint64_t n, cudaStream_t st);
cudaError_t launch_debug_ms_normal(uint32_t x_lo, uint32_t n, float *y, const uint32_t *delta,
                                   cudaStream_t st);
cudaError_t launch_debug_logf(const float *x, float *y, uint64_t n, const LogfTables &L,
                              cudaStream_t st);

}  // namespace sw
