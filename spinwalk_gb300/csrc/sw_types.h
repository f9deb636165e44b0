// Plain-data types shared by the host C++ and the CUDA kernels (no CUDA types here).
#pragma once
#include <stdint.h>

namespace sw {


constexpr double kDeg2Rad = 0.0174532925199433;  // DEG2RAD, src/sim/simulation_parameters.cuh:24
constexpr double kRad2Deg = 57.2957795130823;    // RAD2DEG, simulation_parameters.cuh:25
constexpr double kGamma = 267515315.;            // GAMMA,   src/definitions.h:20

constexpr int kMtN = 624;                        // mt19937 state size (words)
constexpr int kMtM = 397;

// Ring buffers of generator output per spin (refilled between walk chunks).
constexpr uint32_t kNormBuf = 768;               // Gaussian deviates: 256 steps x 3 axes (default)
constexpr uint32_t kUnifBuf = 128;               // uniform deviates for crossing attempts
constexpr uint32_t kStepsPerRound = kNormBuf / 3;  // longest walk of one refill/walk round
// Seeding: by default, spins whose discard count seed + spin reaches this jump ahead
// (k_seed_jump) instead of regenerating seed + spin words (k_seed); sw_tuning.jump_min_kwords
// overrides it. Measured on GB300: the jump costs 0.34 us of the whole GPU per spin whatever the
// count, the discard 1 / 4.2e12 s per word, so they break even near 1.44e6 words.
constexpr uint64_t kJumpMinZ = 1408ull * 1024;
constexpr int kMtDegreeDev = 19937;               // degree of mt19937's characteristic polynomial

// Pooled Gaussian generators of a batch whose instances share the seed: one gen_r and one ring
// of deviates per spin id s (a "stream"), read by every instance's spin s at its own position.
// Counts are absolute since seeding; ring slot = count % kPoolNorm. (The crossing uniforms of
// gen_u stay with each instance's spin: with two pooled rings, a spin waiting for uniforms held
// back by a slower one could hold back that spin's Gaussians in turn.)
constexpr uint32_t kPoolNorm = 1024;             // Gaussian deviates per stream
constexpr uint32_t kPoolNone = 0xffffffffu;      // no walking pair reported a read position
struct PoolState {
    uint32_t *mt_r;           // [n_streams][624]
    uint32_t *p_r;            // next output index in the current block
    float *nbuf;              // [n_streams][kPoolNorm]
    uint32_t *nw;             // deviates written so far
    uint32_t *nmin;           // lowest read position of the pairs that paused in the last walk
};

// Spin flags word: bits 0-7 ts_old (substrate of the last accepted voxel), bit 8 "scan
// started", bit 9 done, bits 16-23 status (SW_SPIN_*).
constexpr uint32_t kFlagStarted = 1u << 8;
constexpr uint32_t kFlagDone = 1u << 9;

// One RF rotation, with the trigonometry precomputed on the host with the host libm (the values
// the reference computes inside xrot_withphase, src/sim/kernels.cuh:160-206).
//   kind 0: xrot(s,c)   1: xrot(-s,c)   2: yrot(s,c)   3: yrot(-s,c)
//   kind 4: zrot(-sp,cp) -> xrot(s,c) -> zrot(sp,cp)
struct RfOp {
    int32_t kind;
    int32_t tp;               // time point (RF events k >= 1; unused for the scan-start pulse)
    float s, c, sp, cp;       // float path
    double sd, cd, spd, cpd;  // FP64 path
};

// Device-resident copies of the scalar parameters (passed by value to every kernel).
struct DevParams {
    double fov[3];
    double s2g[3];            // phantom_size / fov  (kernels.cu:98)
    float s2g_f[3];           // s2g rounded to float (fast path of voxel_coord)
    int64_t nz, nynz;         // row-major strides (kernels.cuh:53-60)
    int64_t matrix_length;
    uint64_t seed;
    uint64_t max_iterations;
    uint32_t n_spins, n_timepoints, n_substrate, n_dummy_scan;
    uint32_t n_TE, n_RF, n_dephasing, n_gradient;
    int32_t timestep_us;
    int32_t cross_fov, record_traj, fieldmap_exist;
    uint64_t traj_len;        // XYZ1 slots per spin
    uint32_t rng;             // SW_RNG_MT19937 or SW_RNG_MINSTD (generator flavour)
    int32_t field_bf16;       // packed phantom of 4-byte records (bf16 field | label << 16)
};

// Small read-only tables (device pointers into one allocation).
struct DevTables {
    const double *dscale;     // [ns] step std-dev (m)
    const float *T1f, *T2f;   // [ns] float(T1_ms*1e-3) as the reference stores it (kernels.cu:167)
    const double *T1d, *T2d;  // [ns] T1_ms*1e-3 in double (FP64 path)
    const float *pXY;         // [ns*ns]
    const RfOp *rf;           // [n_RF]  (index 0 unused)
    const RfOp *scan_rf;      // [n_dummy_scan+1] scan-start pulse incl. phase cycling
    const int32_t *te_tp;     // [n_TE]
    const int32_t *dph_tp;    // [n_dephasing]
    const float *dph_deg;
    const int32_t *grad_tp;   // [n_gradient]
    const float *gx, *gy, *gz;
};

// Bit-exact logf tables (see sw_logf.h).
struct LogfTables {
    const float *tab;         // 64 x {invc, Lhi, Llo}
    const uint32_t *bitmap;   // bit (x_bits - 2^-48 bits): host libm differs from the candidate
    // minstd flavour: 4-bit host-minus-device ulp corrections of its Gaussian deviate
    // (sw_minstd.cu), indexed by the folded engine output
    const uint32_t *ms_delta = nullptr;
};

// Per-spin walk state between chunks (structure of arrays, one entry per spin).
struct SpinState {
    uint64_t *x, *y, *z;      // xyz_old (kernels.cu:93): bit patterns of the doubles
    float *mx, *my, *mz;      // m0
    float *acc, *acc_e;       // accumulated phase (+ two-sum error in KAHAN mode)
    double *accd;             // FP64 phase (FP64 mode / shadow)
    double *dmx, *dmy, *dmz;  // FP64 magnetisation (FP64 mode / shadow)
    float *field;             // field of the last accepted voxel (deg / step)
    int64_t *ind_old;
    uint32_t *tp, *tp_old, *ds, *itr;
    uint32_t *ctr;            // c_rf | c_te << 16
    uint32_t *ctr2;           // c_dph | c_grad << 16
    uint32_t *flags;
};

// Generator state: two mt19937 per spin (gen_r for the walk, gen_u for crossings,
// kernels.cu:82-83) and the ring buffers of their output.
struct RngState {
    uint32_t *mt_r, *mt_u;    // [n][624]
    uint32_t *p_r, *p_u;      // next output index in the current 624-word block
    float *nbuf;              // [n][nlen]
    uint32_t *nhead, *ncnt;
    float *ubuf;              // [n][kUnifBuf]
    uint32_t *uhead, *ucnt;
    uint32_t nlen = kNormBuf; // Gaussian deviates per ring: 3 x the steps of one round
};

struct Outputs {
    float *M1;                // [n][n_TE][3]
    double *M1d;              // optional FP64 shadow
    float *XYZ1;              // [n][traj_len][3] (may be null in signal mode)
    uint8_t *T;               // [n][n_TE]
    int32_t *status;          // optional
    // Signal mode (sig != null): instead of M1 / T, every echo adds the spin's M to
    // sig[te][substrate][3] and counts it in cnt[te][substrate].
    double *sig = nullptr;
    unsigned long long *cnt = nullptr;
};

// One instance of a fused batch launch (k_walk_batch, k_refill_uniforms_batch): what the
// per-instance kernels take as parameters, read by each block from device memory. Blocks are
// dealt out instance by instance: instance k owns the walk blocks [walk_block0, +ceil(n/256))
// and the uniform-refill blocks [unif_block0, +ceil(n/128)).
struct BatchInst {
    DevParams P;
    DevTables Tb;
    SpinState S;
    RngState G;
    Outputs O;
    uint32_t n_spins;
    uint32_t walk_block0, unif_block0;
};

// Walk order of the spins (Morton re-sort, sw_order.cu). order and key are indexed by global
// spin id like SpinState; hist has order_hist_words() counters.
constexpr int kOrderMaxBitsPerAxis = 6;
struct OrderState {
    uint32_t *order;          // [n]: thread lo+i walks spin order[lo+i]
    uint32_t *key;            // [n]
    uint32_t *hist;           // bucket counters, then offsets
};
struct OrderShape {
    int bits;                 // Morton bits per axis
    int shift[3];             // voxel coordinate >> shift = cell coordinate
    int64_t n[3];             // phantom size per axis
    uint32_t n_buckets;       // 2^(3 bits) cells + 1 bucket of finished spins
};

}  // namespace sw
