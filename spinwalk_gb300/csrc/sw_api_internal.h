// Internal helpers of the C ABI (sw_api.cu), shared with sw_noalloc.cu.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_kernels.h"
#include "sw_types.h"

namespace sw {
namespace api {

// Bump allocator over the workspace (256-byte aligned slices).
struct Carve {
    char *base;
    size_t off = 0;
    template <typename T>
    T *take(size_t n) {
        off = (off + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += n * sizeof(T);
        return p;
    }
};

// Host image of the small tables, laid out exactly like the device copy.
struct TableImage {
    std::vector<char> bytes;
    static constexpr size_t kUnset = ~size_t(0);
    size_t o_dscale = kUnset, o_T1f = kUnset, o_T2f = kUnset, o_T1d = kUnset,
           o_T2d = kUnset, o_pXY = kUnset, o_rf = kUnset, o_scan = kUnset, o_te = kUnset,
           o_dtp = kUnset, o_ddeg = kUnset, o_gtp = kUnset, o_gx = kUnset, o_gy = kUnset,
           o_gz = kUnset;
    bool complete() const {
        for (size_t o : {o_dscale, o_T1f, o_T2f, o_T1d, o_T2d, o_pXY, o_rf, o_scan,
                         o_te, o_dtp, o_ddeg, o_gtp, o_gx, o_gy, o_gz})
            if (o == kUnset) return false;
        return true;
    }
    template <typename T>
    size_t put(const T *src, size_t n) {
        size_t off = (bytes.size() + 15) & ~size_t(15);
        bytes.resize(off + std::max<size_t>(1, n) * sizeof(T));
        if (n) std::memcpy(bytes.data() + off, src, n * sizeof(T));
        return off;
    }
};

// Device workspace of one call, carved from one allocation.
struct Layout {
    uint2 *vox;
    char *tables;
    uint32_t *active;
    SpinState S;
    RngState G;
    OrderState Q;             // walk order (Morton re-sort)
    size_t bytes;
};

// Process-wide tuning of the walk (sw_set_tuning / sw_autotune), read at the start of a call.
sw_tuning current_tuning();
// Grid cap of the walk kernel under tuning t (0: one thread per spin, no cap).
int walk_grid_cap(const sw_tuning &t);
// Gaussian deviates per ring (3 per step of a round) under tuning t. The default for sw_sim /
// sw_sim_device is 512 steps: on GB300 it measured 0.8 % faster than 256 on the SE workload and
// 4 % on GRE (one round instead of two), for 3 KB more ring memory per spin.
constexpr uint32_t kDefaultRingSteps = 512;
inline uint32_t ring_len(const sw_tuning &t) {
    return 3u * (t.ring_steps ? t.ring_steps : kDefaultRingSteps);
}
// The discard count from which seeding jumps ahead under tuning t (at least 624).
inline uint64_t jump_min_z(const sw_tuning &t) {
    const uint64_t z = t.jump_min_kwords ? 1024ull * t.jump_min_kwords : kJumpMinZ;
    return z < 624 ? 624 : z;
}
// Device jump polynomials (sw_mtjump.h) for the spins [lo, hi) of `seed` whose discard count
// seed + spin reaches z_min, computed on the host and copied into buf (grown on demand; the
// caller makes sure no kernel still reads it). jt.polys stays null when no spin jumps.
int jump_table(uint64_t seed, uint32_t lo, uint32_t hi, uint64_t z_min, uint32_t *&buf,
               size_t &buf_words, JumpTable &jt);

// sw_sim_batch with pooled generators (sw_pool.cu): runs the batch and sets `taken`, or leaves
// `taken` false for the engine path (another generator flavour, or a pool larger than half the
// free device memory).
int run_batch_pooled(const sw_instance *items, uint32_t n_items, const float *pFieldMap,
                     const uint8_t *pMask, int precision, bool &taken);

// sw_release_workspaces, per part: the current device's batch pool (sw_pool.cu) and the engine
// of the one-call entry points (sw_engine.cu); each waits for its lock, i.e. for a running call.
void release_pool_memory(int dev);
void release_call_engine(int dev);

// Kernel timing of the last call on this thread (sw_last_timing).
extern thread_local sw_timing g_timing;
// Sets sw_last_error() for the calling thread and returns `code`.
int fail(int code, const std::string &msg);
// Parameter checks shared by every entry point.
int check_args(const sw_params *p, const sw_sequence *q);
DevParams dev_params(const sw_params *p, const sw_sequence *q);
void build_tables(const sw_params *p, const sw_sequence *q, TableImage &im);
DevTables dev_tables(const TableImage &im, const char *d);
// base == nullptr: only measures (Layout::bytes). nlen: Gaussian deviates per ring.
Layout layout(char *base, size_t n, int64_t ml, size_t table_bytes, bool dbl,
              bool mt_state = true, uint32_t nlen = kNormBuf);
// The current device's logf tables (built and uploaded on first use); {nullptr, nullptr} and
// sw_last_error() set on failure.
LogfTables device_logf_tables();
// The current device's correction table of the minstd flavour's deviates (sw_minstd.cu), built
// on first use; nullptr and sw_last_error() set on failure.
const uint32_t *minstd_delta_table();

}  // namespace api
}  // namespace sw
