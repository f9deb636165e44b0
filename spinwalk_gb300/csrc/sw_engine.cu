// sw_engine: many `sim` jobs on one GPU -- the batched scale sweeps and the serving loop.
//
// The reference runs one job at a time: monte_carlo::run packs nothing, seeds every spin of every
// scale again (src/sim/kernels.cu:82-88) and launches one cu_sim per scale with a device
// synchronisation after each (src/sim/monte_carlo.cu:310-335). The engine keeps instead
//   * phantoms resident in HBM, packed once (mask + field, 8 B per voxel), shared by jobs;
//   * one seed cache per simulation seed: the generator state of spin s depends only on seed + s,
//     so the states of spins [0, n) are computed once (k_seed) and every job with that seed copies
//     its spin range from the cache (2.5 KB per spin per generator, a device-to-device copy);
//   * a fixed set of slots, each a CUDA stream with its own workspace for `slot_spins` spins, its
//     device I/O buffer and a pinned staging buffer. A job is cut into spin-range chunks of at most
//     one slot's capacity (spins are independent); slots run chunks of different jobs at the same
//     time, so small jobs fill the GPU together and big ones never need more than a slot's memory.
// A chunk is: stage inputs (pinned) -> copy its range of the seed cache -> k_init ->
// ceil(steps / ring steps) refill/walk rounds issued without waiting (no spin can finish in
// fewer: a round advances a spin by at most the steps its Gaussian ring holds, the tuning's
// ring_steps when the engine was created) -> then one round at a time until the walk reports no
// active spin -> results back through the staging buffer. The host only polls events.
//
// Every job gives the results of its own sw_sim call, bit for bit (tests/test_engine.py).
// One host thread drives an engine (the C entry points lock it).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"
#include "sw_kernels.h"

using namespace sw::api;

namespace {

#define EN_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr size_t kTableBytes = 1 << 20;        // per slot: RF / TE / gradient tables of a job

double now_s() {
    using clk = std::chrono::steady_clock;
    return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

// Host copies into and out of the pinned staging buffers: large ones are split across host
// threads (one core copies about 10 GB/s; a 1e6-spin chunk with 8 echoes moves ~250 MB).
void par_memcpy(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPiece = 4 << 20;
    if (bytes < 2 * kPiece) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const int64_t pieces = (int64_t)((bytes + kPiece - 1) / kPiece);
#pragma omp parallel for num_threads(8) schedule(static)
    for (int64_t i = 0; i < pieces; i++) {
        const size_t o = (size_t)i * kPiece, n = std::min(kPiece, bytes - o);
        std::memcpy(static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, n);
    }
}

// p shifted down by lo elements, so that p_shifted[spin] for spin in [lo, hi) is p[spin - lo]:
// the kernels index by global spin id, the slot buffers hold one chunk.
template <typename T>
T *shift(T *p, uint64_t lo_elems) {
    if (!p) return p;
    return reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(p) - lo_elems * sizeof(T));
}

struct Phantom {
    uint2 *vox = nullptr;
    int64_t ml = 0;
    uint64_t dims[3] = {0, 0, 0};
    uint32_t n_substrate = 0;
    bool field = false;
    bool bf16 = false;              // 4-byte records (SW_FIELD_BF16)
    int jobs = 0;                   // jobs still using it
};

struct SeedCache {
    uint32_t *mt = nullptr;         // [cap][624]: spins base .. base + n - 1
    uint32_t *p = nullptr;          // [cap]
    uint32_t base = 0, n = 0, cap = 0;
    cudaEvent_t ready = nullptr;    // recorded after the last seeding on the seed stream
    uint32_t jobs = 0;              // queued or running jobs that copy from it
    uint64_t last_use = 0;          // engine tick of the last job that used it
};

struct Job {
    int64_t id = 0;
    int32_t phantom = 0;
    int precision = SW_PREC_FP32;
    sw_params p{};
    sw_sequence q{};
    // owned copies of the sequence arrays (the caller's may go away after submit)
    std::vector<double> diff;
    std::vector<float> T1, T2, pXY, FA, PH, ddeg, gx, gy, gz;
    std::vector<int32_t> RFus, TEus, dus, gus;
    TableImage im;
    char *h_tables = nullptr;       // pinned copy of im.bytes
    sw::DevParams P{};
    const float *M0 = nullptr, *XYZ0 = nullptr;
    float *M1 = nullptr, *XYZ1 = nullptr;
    uint8_t *T = nullptr;
    int32_t *status = nullptr;
    size_t nte = 0, trj = 0;
    uint32_t spin_lo = 0, spin_hi = 0;  // the job's spins; host buffers hold their rows only
    uint32_t next_lo = 0, chunk = 0;    // next spin to hand out, spins per chunk
    int running = 0;
    int rc = SW_OK;
    double t_submit = 0, t_done = 0;
    SeedCache *seed = nullptr;
    sw_tuning tuning{};                 // walk tuning at submission (sw_set_tuning)
    // signal mode: per-(echo, substrate) sums instead of per-spin M1 / T / XYZ1
    double *h_sig = nullptr, *d_sig = nullptr;
    uint64_t *h_cnt = nullptr;
    unsigned long long *d_cnt = nullptr;
    size_t n_keys = 0;
};

struct Slot {
    cudaStream_t st = nullptr;
    char *ws = nullptr;
    Layout L{};
    uint32_t cap = 0;
    char *d_io = nullptr, *h_io = nullptr;   // device I/O buffer, pinned staging
    size_t io_bytes = 0;
    uint32_t *h_active = nullptr;            // pinned
    cudaEvent_t ev = nullptr;
    enum State { FREE, RUNNING, DRAINING } state = FREE;
    Job *job = nullptr;
    uint32_t lo = 0, hi = 0;
    uint64_t rounds = 0, max_rounds = 0;
    // byte offsets of the sections of a chunk in d_io / h_io
    size_t o_M0 = 0, o_XYZ0 = 0, o_M1 = 0, o_XYZ1 = 0, o_T = 0, o_st = 0, in_bytes = 0, out_bytes = 0;
};

}  // namespace

struct sw_engine {
    std::mutex mu;
    int device = 0;
    uint32_t nlen = sw::kNormBuf;            // Gaussian deviates per ring in every slot
    uint64_t budget = 0, used = 0;
    cudaStream_t seed_st = nullptr;
    uint32_t *seed_scratch = nullptr;        // ring counters written by k_seed, not needed here
    uint32_t *d_jump = nullptr;              // jump polynomials of the last seeding's high spin ids
    size_t jump_words = 0;
    uint32_t scratch_cap = 0;
    std::vector<Slot> slots;
    std::map<int32_t, Phantom> phantoms;
    int32_t next_phantom = 1;
    std::map<uint64_t, std::unique_ptr<SeedCache>> seeds;
    std::deque<std::unique_ptr<Job>> queue;  // jobs with spins left to hand out or running
    std::vector<std::unique_ptr<Job>> finished;
    int64_t next_job = 1;
    sw::LogfTables LT{nullptr, nullptr};
    uint64_t launches = 0, rounds = 0, seedings = 0;   // kernels, refill/walk rounds, k_seed calls
    uint64_t tick = 0;                                  // seed cache use counter (LRU)
};

namespace {

// Seeds k_seed's range [a, b) into cache C (whose first spin is C.base) on the seed stream.
int seed_into(sw_engine *E, SeedCache &C, uint64_t seed, uint32_t a, uint32_t b) {
    if (b <= a) return SW_OK;
    if (E->scratch_cap < b - C.base) {
        if (E->seed_scratch) {
            EN_CUDA(cudaStreamSynchronize(E->seed_st));
            cudaFree(E->seed_scratch);
            E->seed_scratch = nullptr;
            E->scratch_cap = 0;
        }
        EN_CUDA(cudaMalloc(&E->seed_scratch, (size_t)C.cap * 4));
        E->scratch_cap = C.cap;
    }
    sw::DevParams P{};
    P.seed = seed;
    sw::RngState G{};
    G.mt_r = G.mt_u = shift(C.mt, (uint64_t)C.base * sw::kMtN);
    G.p_r = G.p_u = shift(C.p, (uint64_t)C.base);
    G.nhead = G.ncnt = G.uhead = G.ucnt = shift(E->seed_scratch, (uint64_t)C.base);
    sw::JumpTable jt;                    // high spin ids jump ahead instead of discarding
    const uint64_t zmin = jump_min_z(current_tuning());
    if (P.rng == SW_RNG_MT19937 && (uint64_t)seed + b > zmin) {
        EN_CUDA(cudaStreamSynchronize(E->seed_st));     // the last seeding may still read it
        const int rj = jump_table(seed, a, b, zmin, E->d_jump, E->jump_words, jt);
        if (rj) return rj;
    }
    EN_CUDA(sw::launch_seed_range(P, G, a, b, E->seed_st, &jt));
    E->launches++;
    E->seedings++;
    return SW_OK;
}

// Makes the seed cache of `seed` hold spins [lo, hi) (the generator state of spin s after
// mt19937(seed + s).discard(seed + s), kernels.cu:82-88); grows it when needed.
int ensure_seeded(sw_engine *E, uint64_t seed, uint32_t lo, uint32_t hi, SeedCache *&out) {
    auto &slot = E->seeds[seed];
    if (!slot) {
        slot.reset(new SeedCache());
        EN_CUDA(cudaEventCreateWithFlags(&slot->ready, cudaEventDisableTiming));
    }
    SeedCache &C = *slot;
    out = &C;
    if (C.n && lo >= C.base && hi <= C.base + C.n) return SW_OK;
    const uint32_t old_lo = C.base, old_hi = C.base + C.n;
    const uint32_t new_lo = C.n ? std::min(lo, old_lo) : lo;
    const uint32_t new_hi = C.n ? std::max(hi, old_hi) : hi;
    if (new_lo != old_lo || new_hi - new_lo > C.cap) {      // reallocate, keep what is seeded
        const uint64_t want = (uint64_t)new_hi - new_lo;
        const uint32_t cap = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(want, 2ull * C.cap), 0xffffffffu);
        const uint32_t capped = (uint32_t)std::max<uint64_t>(want, std::min<uint64_t>(cap, want + (want >> 1)));
        const size_t bytes = (size_t)capped * sw::kMtN * 4 + (size_t)capped * 4;
        if (E->used + bytes > E->budget) {   // evict caches no job uses, least recently used first
            EN_CUDA(cudaStreamSynchronize(E->seed_st));
            while (E->used + bytes > E->budget) {
                auto victim = E->seeds.end();
                for (auto it = E->seeds.begin(); it != E->seeds.end(); ++it)
                    if (it->first != seed && it->second->jobs == 0 && it->second->mt &&
                        (victim == E->seeds.end() || it->second->last_use < victim->second->last_use))
                        victim = it;
                if (victim == E->seeds.end()) break;
                SeedCache &V = *victim->second;
                cudaFree(V.mt);
                cudaFree(V.p);
                cudaEventDestroy(V.ready);
                E->used -= (size_t)V.cap * sw::kMtN * 4 + (size_t)V.cap * 4;
                E->seeds.erase(victim);
            }
        }
        if (E->used + bytes > E->budget)
            return fail(SW_ERR_NOMEM, "seed cache of " + std::to_string(capped) + " spins exceeds the HBM budget");
        uint32_t *mt = nullptr, *p = nullptr;
        EN_CUDA(cudaMalloc(&mt, (size_t)capped * sw::kMtN * 4));
        EN_CUDA(cudaMalloc(&p, (size_t)capped * 4));
        if (C.n) {
            const size_t o = (size_t)old_lo - new_lo;
            EN_CUDA(cudaMemcpyAsync(mt + o * sw::kMtN, C.mt, (size_t)C.n * sw::kMtN * 4, cudaMemcpyDeviceToDevice, E->seed_st));
            EN_CUDA(cudaMemcpyAsync(p + o, C.p, (size_t)C.n * 4, cudaMemcpyDeviceToDevice, E->seed_st));
        }
        if (C.mt) {                          // slots may still be copying from the old cache
            EN_CUDA(cudaDeviceSynchronize());
            cudaFree(C.mt);
            cudaFree(C.p);
            E->used -= (size_t)C.cap * sw::kMtN * 4 + (size_t)C.cap * 4;
        }
        C.mt = mt;
        C.p = p;
        C.cap = capped;
        E->used += bytes;
    }
    C.base = new_lo;
    int rc = SW_OK;
    if (C.n == 0) {
        rc = seed_into(E, C, seed, new_lo, new_hi);
    } else {
        if (!rc) rc = seed_into(E, C, seed, new_lo, old_lo);
        if (!rc) rc = seed_into(E, C, seed, old_hi, new_hi);
    }
    if (rc) return rc;
    EN_CUDA(cudaEventRecord(C.ready, E->seed_st));
    C.n = new_hi - new_lo;
    return SW_OK;
}

struct ChunkView {
    sw::SpinState S;
    sw::RngState G;
    sw::OrderState Q;
    sw::Outputs O;
    const float *M0, *XYZ0;
};

ChunkView view(const Slot &s) {
    const Job &j = *s.job;
    const uint64_t lo = s.lo;
    ChunkView v;
    v.S = s.L.S;
    v.G = s.L.G;
    sw::SpinState &S = v.S;
    S.x = shift(S.x, lo); S.y = shift(S.y, lo); S.z = shift(S.z, lo);
    S.mx = shift(S.mx, lo); S.my = shift(S.my, lo); S.mz = shift(S.mz, lo);
    S.acc = shift(S.acc, lo); S.acc_e = shift(S.acc_e, lo); S.accd = shift(S.accd, lo);
    S.dmx = shift(S.dmx, lo); S.dmy = shift(S.dmy, lo); S.dmz = shift(S.dmz, lo);
    S.field = shift(S.field, lo); S.ind_old = shift(S.ind_old, lo);
    S.tp = shift(S.tp, lo); S.tp_old = shift(S.tp_old, lo); S.ds = shift(S.ds, lo);
    S.itr = shift(S.itr, lo); S.ctr = shift(S.ctr, lo); S.ctr2 = shift(S.ctr2, lo);
    S.flags = shift(S.flags, lo);
    sw::RngState &G = v.G;
    G.mt_r = shift(G.mt_r, lo * sw::kMtN); G.mt_u = shift(G.mt_u, lo * sw::kMtN);
    G.p_r = shift(G.p_r, lo); G.p_u = shift(G.p_u, lo);
    G.nbuf = shift(G.nbuf, lo * G.nlen); G.nhead = shift(G.nhead, lo); G.ncnt = shift(G.ncnt, lo);
    G.ubuf = shift(G.ubuf, lo * sw::kUnifBuf); G.uhead = shift(G.uhead, lo); G.ucnt = shift(G.ucnt, lo);
    v.Q = s.L.Q;
    v.Q.order = shift(v.Q.order, lo);
    v.Q.key = shift(v.Q.key, lo);
    char *d = s.d_io;
    v.O.M1d = nullptr;
    v.O.status = shift(reinterpret_cast<int32_t *>(d + s.o_st), lo);
    if (j.d_sig) {
        v.O.M1 = nullptr;
        v.O.XYZ1 = nullptr;
        v.O.T = nullptr;
        v.O.sig = j.d_sig;
        v.O.cnt = j.d_cnt;
    } else {
        v.O.M1 = shift(reinterpret_cast<float *>(d + s.o_M1), lo * 3 * j.nte);
        v.O.XYZ1 = shift(reinterpret_cast<float *>(d + s.o_XYZ1), lo * 3 * j.trj);
        v.O.T = shift(reinterpret_cast<uint8_t *>(d + s.o_T), lo * j.nte);
    }
    v.M0 = shift(reinterpret_cast<const float *>(d + s.o_M0), lo * 3);
    v.XYZ0 = shift(reinterpret_cast<const float *>(d + s.o_XYZ0), lo * 3);
    return v;
}

// Hands the next spin range of a ready job to a free slot and issues the chunk's work.
int start_chunk(sw_engine *E, Slot &s, Job &j) {
    const uint32_t lo = j.next_lo, hi = std::min<uint32_t>(j.spin_hi, lo + j.chunk);
    j.next_lo = hi;
    j.running++;
    s.job = &j;
    s.lo = lo;
    s.hi = hi;
    const bool sig = j.d_sig != nullptr;
    const size_t c = hi - lo, nte = sig ? 0 : j.nte, trj = sig ? 0 : j.trj, r = lo - j.spin_lo;
    size_t off = 0;
    auto sec = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~size_t(255); return o; };
    s.o_M0 = sec(c * 12);
    s.o_XYZ0 = sec(c * 12);
    s.o_M1 = sec(c * nte * 12);
    s.o_T = sec(c * nte);
    s.o_XYZ1 = sec(c * trj * 12);
    s.in_bytes = off;                    // inputs and the outputs' starting contents
    s.o_st = sec(c * 4);
    s.out_bytes = off - s.o_M1;
    // stage: inputs and the caller's current output contents (slots the walk never reaches keep
    // them, as with sw_sim)
    par_memcpy(s.h_io + s.o_M0, j.M0 + 3 * r, c * 12);
    par_memcpy(s.h_io + s.o_XYZ0, j.XYZ0 + 3 * r, c * 12);
    if (nte) {
        par_memcpy(s.h_io + s.o_M1, j.M1 + 3 * nte * r, c * nte * 12);
        par_memcpy(s.h_io + s.o_T, j.T + nte * r, c * nte);
    }
    if (trj) par_memcpy(s.h_io + s.o_XYZ1, j.XYZ1 + 3 * trj * r, c * trj * 12);
    EN_CUDA(cudaMemcpyAsync(s.d_io, s.h_io, s.in_bytes, cudaMemcpyHostToDevice, s.st));
    EN_CUDA(cudaMemcpyAsync(s.L.tables, j.h_tables, j.im.bytes.size(), cudaMemcpyHostToDevice, s.st));
    const uint64_t steps = (uint64_t)j.p.n_timepoints * (uint64_t)(j.p.n_dummy_scan + 1);
    s.max_rounds = 64 + steps * (j.p.max_iterations + 2);
    s.rounds = 0;
    s.state = Slot::RUNNING;
    if (j.P.rng == SW_RNG_MINSTD) {      // thrust::minstd_rand: seeding is a modular power
        const ChunkView v = view(s);
        EN_CUDA(sw::launch_seed_range(j.P, v.G, lo, hi, s.st));
        E->launches++;
        return SW_OK;
    }
    // generator states of spins [lo, hi): the job's range of the seed cache, both generators
    EN_CUDA(cudaStreamWaitEvent(s.st, j.seed->ready, 0));
    const size_t sc = lo - j.seed->base;                 // the chunk's first spin in the cache
    EN_CUDA(cudaMemcpyAsync(s.L.G.mt_r, j.seed->mt + sc * sw::kMtN, c * sw::kMtN * 4, cudaMemcpyDeviceToDevice, s.st));
    EN_CUDA(cudaMemcpyAsync(s.L.G.mt_u, j.seed->mt + sc * sw::kMtN, c * sw::kMtN * 4, cudaMemcpyDeviceToDevice, s.st));
    EN_CUDA(cudaMemcpyAsync(s.L.G.p_r, j.seed->p + sc, c * 4, cudaMemcpyDeviceToDevice, s.st));
    EN_CUDA(cudaMemcpyAsync(s.L.G.p_u, j.seed->p + sc, c * 4, cudaMemcpyDeviceToDevice, s.st));
    EN_CUDA(cudaMemsetAsync(s.L.G.nhead, 0, c * 4, s.st));
    EN_CUDA(cudaMemsetAsync(s.L.G.ncnt, 0, c * 4, s.st));
    EN_CUDA(cudaMemsetAsync(s.L.G.uhead, 0, c * 4, s.st));
    EN_CUDA(cudaMemsetAsync(s.L.G.ucnt, 0, c * 4, s.st));
    return SW_OK;
}

// Issues `k` refill/walk rounds (after k_init when first) and the read-back of the active count.
int issue_rounds(sw_engine *E, Slot &s, uint64_t k, bool first) {
    Job &j = *s.job;
    const Phantom &ph = E->phantoms[j.phantom];
    const ChunkView v = view(s);
    const sw::DevTables Tb = dev_tables(j.im, s.L.tables);
    const bool dbl = j.precision == SW_PREC_FP64;
    if (first)
        EN_CUDA(sw::launch_init_range(j.P, Tb, ph.vox, v.M0, v.XYZ0, v.S, v.O, dbl, s.lo, s.hi, s.st));
    const uint32_t ri = j.tuning.resort_interval;
    for (uint64_t r = 0; r < k; r++) {
        if (r + 1 == k) EN_CUDA(cudaMemsetAsync(s.L.active, 0, sizeof(uint32_t), s.st));
        EN_CUDA(sw::launch_refill_range(j.P, v.G, v.S, E->LT, s.lo, s.hi, s.st));
        if (ri && (s.rounds + r) % ri == 0) {
            EN_CUDA(sw::launch_order(j.P, v.S, v.Q, s.lo, s.hi, s.st));
            E->launches += 3;
        }
        EN_CUDA(sw::launch_walk_range(j.precision, dbl, j.P, Tb, ph.vox, v.S, v.G, v.O,
                                      s.L.active, s.lo, s.hi, s.st, ri ? v.Q.order : nullptr,
                                      (int)j.tuning.walk_block));
    }
    s.rounds += k;
    E->rounds += k;
    E->launches += 2 * k + (first ? 1 : 0);
    EN_CUDA(cudaMemcpyAsync(s.h_active, s.L.active, 4, cudaMemcpyDeviceToHost, s.st));
    EN_CUDA(cudaEventRecord(s.ev, s.st));
    return SW_OK;
}

void job_done_check(sw_engine *E, Job &j) {
    if (j.running == 0 && (j.next_lo >= j.spin_hi || j.rc != SW_OK)) {
        if (j.d_sig) {                    // every chunk has drained: the sums are final
            if (j.rc == SW_OK &&
                (cudaMemcpy(j.h_sig, j.d_sig, j.n_keys * 24, cudaMemcpyDeviceToHost) != cudaSuccess ||
                 cudaMemcpy(j.h_cnt, j.d_cnt, j.n_keys * 8, cudaMemcpyDeviceToHost) != cudaSuccess))
                j.rc = fail(SW_ERR_CUDA, "signal read-back");
            cudaFree(j.d_sig);
            cudaFree(j.d_cnt);
            j.d_sig = nullptr;
            j.d_cnt = nullptr;
        }
        j.t_done = now_s();
        E->phantoms[j.phantom].jobs--;
        if (j.seed) {                      // its chunks no longer copy from the cache
            j.seed->jobs--;
            j.seed = nullptr;
        }
        if (j.h_tables) {
            cudaFreeHost(j.h_tables);
            j.h_tables = nullptr;
        }
        for (auto it = E->queue.begin(); it != E->queue.end(); ++it)
            if (it->get() == &j) {
                E->finished.push_back(std::move(*it));
                E->queue.erase(it);
                break;
            }
    }
}

// One pass over the slots: advance every chunk whose last work completed, start new chunks.
// Returns the number of slots that made progress.
int pump(sw_engine *E, int &rc) {
    rc = SW_OK;
    int progress = 0;
    for (Slot &s : E->slots) {
        if (s.state == Slot::FREE) continue;
        const cudaError_t q = cudaEventQuery(s.ev);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) {
            rc = fail(SW_ERR_CUDA, std::string("chunk: ") + cudaGetErrorString(q));
            return progress;
        }
        Job &j = *s.job;
        progress++;
        if (s.state == Slot::RUNNING) {
            if (*s.h_active != 0) {
                if (s.rounds >= s.max_rounds) {
                    j.rc = fail(SW_ERR_TIMEOUT, "walk did not finish");
                    j.running--;
                    s.state = Slot::FREE;
                    job_done_check(E, j);
                    continue;
                }
                if ((rc = issue_rounds(E, s, 1, false))) return progress;
            } else {
                if ((rc = [&]() {
                         EN_CUDA(cudaMemcpyAsync(s.h_io + s.o_M1, s.d_io + s.o_M1, s.out_bytes,
                                                 cudaMemcpyDeviceToHost, s.st));
                         EN_CUDA(cudaEventRecord(s.ev, s.st));
                         return SW_OK;
                     }()))
                    return progress;
                s.state = Slot::DRAINING;
            }
        } else {                                         // DRAINING: results are in h_io
            const bool sig = j.d_sig != nullptr;
            const size_t c = s.hi - s.lo, nte = sig ? 0 : j.nte, trj = sig ? 0 : j.trj,
                         r = s.lo - j.spin_lo;
            if (nte) {
                par_memcpy(j.M1 + 3 * nte * r, s.h_io + s.o_M1, c * nte * 12);
                par_memcpy(j.T + nte * r, s.h_io + s.o_T, c * nte);
            }
            if (trj) par_memcpy(j.XYZ1 + 3 * trj * r, s.h_io + s.o_XYZ1, c * trj * 12);
            if (j.status) par_memcpy(j.status + r, s.h_io + s.o_st, c * 4);
            j.running--;
            s.state = Slot::FREE;
            s.job = nullptr;
            job_done_check(E, j);
        }
    }
    for (Slot &s : E->slots) {
        if (s.state != Slot::FREE) continue;
        Job *pick = nullptr;
        for (auto &jp : E->queue)
            if (jp->rc == SW_OK && jp->next_lo < jp->spin_hi && jp->chunk > 0) {
                pick = jp.get();
                break;
            }
        if (!pick) break;
        if ((rc = start_chunk(E, s, *pick))) return progress;
        const uint64_t steps = (uint64_t)pick->p.n_timepoints * (uint64_t)(pick->p.n_dummy_scan + 1);
        const uint64_t per_round = s.L.G.nlen / 3;
        if ((rc = issue_rounds(E, s, (steps + per_round - 1) / per_round, true))) return progress;
        progress++;
    }
    return progress;
}

int engine_submit(sw_engine *E, int32_t phantom, const sw_params *p, const sw_sequence *q,
                  int precision, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
                  uint8_t *T, int32_t *status, int64_t *job_id, uint64_t spin_lo = 0,
                  uint64_t spin_hi = ~0ull, double *sig = nullptr, uint64_t *cnt = nullptr) {
    int rc = check_args(p, q);
    if (rc) return rc;
    auto pit = E->phantoms.find(phantom);
    if (pit == E->phantoms.end()) return fail(SW_ERR_INVALID, "unknown phantom");
    const Phantom &ph = pit->second;
    for (int i = 0; i < 3; i++)
        if (p->phantom_size[i] != ph.dims[i]) return fail(SW_ERR_INVALID, "phantom_size differs from the phantom's");
    if (p->n_substrate < ph.n_substrate)
        return fail(SW_ERR_INVALID, "the mask holds more substrate types than the config defines");
    if (p->fieldmap_exist && !ph.field) return fail(SW_ERR_INVALID, "fieldmap_exist but the phantom has no fieldmap");
    if ((precision & SW_FIELD_BF16) && !ph.bf16)
        return fail(SW_ERR_INVALID, "SW_FIELD_BF16 on a phantom of float records");
    const uint32_t rng = (uint32_t)precision & ~(uint32_t)(SW_PREC_MASK | SW_FIELD_BF16);
    precision &= SW_PREC_MASK;
    if (precision != SW_PREC_FP32 && precision != SW_PREC_FP64 && precision != SW_PREC_KAHAN)
        return fail(SW_ERR_INVALID, "precision");
    if (rng != SW_RNG_MT19937 && rng != SW_RNG_MINSTD) return fail(SW_ERR_INVALID, "generator flavour");
    if (p->n_spins > 0xffffffffull) return fail(SW_ERR_INVALID, "n_spins");
    if (spin_hi == ~0ull) spin_hi = p->n_spins;
    if (spin_lo > spin_hi || spin_hi > p->n_spins) return fail(SW_ERR_INVALID, "spin range outside [0, n_spins)");
    const size_t n = spin_hi - spin_lo, nte = q->n_TE;
    const size_t trj = p->enRecordTrajectory ? (size_t)(p->n_dummy_scan + 1) * p->n_timepoints : 1;
    const bool signal = sig != nullptr;
    if (signal && !cnt) return fail(SW_ERR_INVALID, "signal mode needs the count array");
    if (n && (!M0 || !XYZ0 || (!signal && (!XYZ1 || (nte && (!M1 || !T))))))
        return fail(SW_ERR_INVALID, "null host buffer");
    std::unique_ptr<Job> j(new Job());
    j->id = E->next_job++;
    j->phantom = phantom;
    j->precision = precision;
    j->tuning = current_tuning();
    j->p = *p;
    j->p.fieldmap_exist = p->fieldmap_exist && ph.field;
    const uint32_t ns = p->n_substrate;
    j->diff.assign(q->diffusivity, q->diffusivity + ns);
    j->T1.assign(q->T1_ms, q->T1_ms + ns);
    j->T2.assign(q->T2_ms, q->T2_ms + ns);
    j->pXY.assign(q->pXY, q->pXY + (size_t)ns * ns);
    j->FA.assign(q->RF_FA_deg, q->RF_FA_deg + q->n_RF);
    j->PH.assign(q->RF_PH_deg, q->RF_PH_deg + q->n_RF);
    j->RFus.assign(q->RF_us, q->RF_us + q->n_RF);
    if (nte) j->TEus.assign(q->TE_us, q->TE_us + nte);
    if (q->n_dephasing) {
        j->dus.assign(q->dephasing_us, q->dephasing_us + q->n_dephasing);
        j->ddeg.assign(q->dephasing_deg, q->dephasing_deg + q->n_dephasing);
    }
    if (q->n_gradient) {
        j->gus.assign(q->gradient_us, q->gradient_us + q->n_gradient);
        j->gx.assign(q->gradientX_mTm, q->gradientX_mTm + q->n_gradient);
        j->gy.assign(q->gradientY_mTm, q->gradientY_mTm + q->n_gradient);
        j->gz.assign(q->gradientZ_mTm, q->gradientZ_mTm + q->n_gradient);
    }
    sw_sequence &Q = j->q;
    Q = *q;
    Q.diffusivity = j->diff.data(); Q.T1_ms = j->T1.data(); Q.T2_ms = j->T2.data();
    Q.pXY = j->pXY.data(); Q.RF_FA_deg = j->FA.data(); Q.RF_PH_deg = j->PH.data();
    Q.RF_us = j->RFus.data(); Q.TE_us = j->TEus.data(); Q.dephasing_us = j->dus.data();
    Q.dephasing_deg = j->ddeg.data(); Q.gradient_us = j->gus.data();
    Q.gradientX_mTm = j->gx.data(); Q.gradientY_mTm = j->gy.data(); Q.gradientZ_mTm = j->gz.data();
    build_tables(&j->p, &Q, j->im);
    if (!j->im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
    if (j->im.bytes.size() > kTableBytes) return fail(SW_ERR_INVALID, "sequence tables larger than 1 MiB");
    if (rng == SW_RNG_MINSTD && !E->LT.ms_delta && !(E->LT.ms_delta = minstd_delta_table()))
        return SW_ERR_CUDA;
    EN_CUDA(cudaMallocHost(&j->h_tables, j->im.bytes.size()));
    std::memcpy(j->h_tables, j->im.bytes.data(), j->im.bytes.size());
    j->P = dev_params(&j->p, &Q);
    j->P.rng = rng;
    j->P.field_bf16 = ph.bf16 ? 1 : 0;
    j->M0 = M0; j->XYZ0 = XYZ0; j->M1 = M1; j->XYZ1 = XYZ1; j->T = T; j->status = status;
    j->nte = nte;
    j->trj = trj;
    j->spin_lo = j->next_lo = (uint32_t)spin_lo;
    j->spin_hi = (uint32_t)spin_hi;
    if (signal) {                         // zeroed device sums, shared by the job's chunks
        j->h_sig = sig;
        j->h_cnt = cnt;
        j->n_keys = std::max<size_t>(1, nte * p->n_substrate);
        EN_CUDA(cudaMalloc(&j->d_sig, j->n_keys * 24));
        EN_CUDA(cudaMalloc(&j->d_cnt, j->n_keys * 8));
        EN_CUDA(cudaMemset(j->d_sig, 0, j->n_keys * 24));
        EN_CUDA(cudaMemset(j->d_cnt, 0, j->n_keys * 8));
    }
    // chunk: a slot's spin capacity, or what its I/O buffer holds for this job
    const size_t per_spin = signal ? 24 + 4 + 5 * 256 : 24 + nte * 13 + trj * 12 + 4 + 5 * 256;
    const Slot &s0 = E->slots[0];
    j->chunk = (uint32_t)std::min<size_t>(s0.cap, s0.io_bytes / per_spin);
    if (n && j->chunk == 0) return fail(SW_ERR_NOMEM, "one spin's trajectory exceeds a slot's I/O buffer");
    if (n && rng == SW_RNG_MT19937) {   // the minstd flavour seeds per chunk (O(log) discard)
        rc = ensure_seeded(E, p->seed, (uint32_t)spin_lo, (uint32_t)spin_hi, j->seed);
        if (rc) {
            cudaFreeHost(j->h_tables);
            return rc;
        }
        j->seed->jobs++;
        j->seed->last_use = ++E->tick;
    }
    j->t_submit = now_s();
    E->phantoms[phantom].jobs++;
    *job_id = j->id;
    E->queue.push_back(std::move(j));
    if (n == 0) job_done_check(E, *E->queue.back());
    return SW_OK;
}

void engine_free(sw_engine *E) {
    cudaDeviceSynchronize();
    for (Slot &s : E->slots) {
        if (s.ws) cudaFree(s.ws);
        if (s.d_io) cudaFree(s.d_io);
        if (s.h_io) cudaFreeHost(s.h_io);
        if (s.h_active) cudaFreeHost(s.h_active);
        if (s.ev) cudaEventDestroy(s.ev);
        if (s.st) cudaStreamDestroy(s.st);
    }
    for (auto &kv : E->phantoms) cudaFree(kv.second.vox);
    for (auto &kv : E->seeds) {
        cudaFree(kv.second->mt);
        cudaFree(kv.second->p);
        if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    }
    for (auto &j : E->queue)
        if (j->h_tables) cudaFreeHost(j->h_tables);
    if (E->seed_scratch) cudaFree(E->seed_scratch);
    if (E->d_jump) cudaFree(E->d_jump);
    if (E->seed_st) cudaStreamDestroy(E->seed_st);
    delete E;
}

int engine_create(int device, uint32_t n_slots, uint32_t slot_spins, uint64_t budget,
                  sw_engine **out) {
    if (!out || n_slots == 0 || n_slots > 64 || slot_spins == 0)
        return fail(SW_ERR_INVALID, "engine: 1..64 slots of >= 1 spin");
    EN_CUDA(cudaSetDevice(device));
    sw::LogfTables LT = device_logf_tables();
    if (!LT.tab) return SW_ERR_CUDA;
    sw_engine *E = new sw_engine();
    E->device = device;
    E->LT = LT;
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    E->budget = budget ? budget : (uint64_t)(freeb * 0.85);
    E->nlen = ring_len(current_tuning());
    auto bad = [&](int code) { engine_free(E); return code; };
    if (cudaStreamCreateWithFlags(&E->seed_st, cudaStreamNonBlocking) != cudaSuccess)
        return bad(fail(SW_ERR_CUDA, "stream"));
    E->slots.resize(n_slots);
    for (Slot &s : E->slots) {
        s.cap = slot_spins;
        Layout m = layout(nullptr, slot_spins, 0, kTableBytes, true, true, E->nlen);
        s.io_bytes = (size_t)slot_spins * 256 + (16 << 20);
        if (E->used + m.bytes + s.io_bytes > E->budget)
            return bad(fail(SW_ERR_NOMEM, "slots exceed the HBM budget"));
        if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMalloc(&s.ws, m.bytes) != cudaSuccess || cudaMalloc(&s.d_io, s.io_bytes) != cudaSuccess ||
            cudaMallocHost(&s.h_io, s.io_bytes) != cudaSuccess ||
            cudaMallocHost(&s.h_active, 4) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return bad(fail(SW_ERR_NOMEM, "slot buffers"));
        }
        s.L = layout(s.ws, slot_spins, 0, kTableBytes, true, true, E->nlen);
        E->used += m.bytes + s.io_bytes;
    }
    *out = E;
    return SW_OK;
}

int engine_add_phantom(sw_engine *E, const uint8_t *mask, const float *field, const uint64_t dims[3],
                       uint32_t n_substrate, int32_t *id, int flags = 0) {
    if (!mask || !dims || !id) return fail(SW_ERR_INVALID, "null argument");
    if (flags & ~SW_FIELD_BF16) return fail(SW_ERR_INVALID, "phantom flags");
    const bool bf16 = (flags & SW_FIELD_BF16) != 0;
    const int64_t ml = (int64_t)(dims[0] * dims[1] * dims[2]);
    if (ml <= 0 || n_substrate == 0 || n_substrate > 256) return fail(SW_ERR_INVALID, "phantom size / substrates");
    const size_t bytes = (size_t)ml * (bf16 ? 4 : 8);
    if (E->used + bytes > E->budget) {        // evict idle phantoms, oldest first
        for (auto it = E->phantoms.begin(); it != E->phantoms.end() && E->used + bytes > E->budget;) {
            if (it->second.jobs == 0) {
                cudaFree(it->second.vox);
                E->used -= (size_t)it->second.ml * (it->second.bf16 ? 4 : 8);
                it = E->phantoms.erase(it);
            } else {
                ++it;
            }
        }
        if (E->used + bytes > E->budget) return fail(SW_ERR_NOMEM, "phantom exceeds the HBM budget");
    }
    Phantom ph;
    ph.ml = ml;
    for (int i = 0; i < 3; i++) ph.dims[i] = dims[i];
    ph.n_substrate = n_substrate;
    ph.field = field != nullptr;
    ph.bf16 = bf16;
    uint8_t *d_mask = nullptr;
    float *d_field = nullptr;
    uint32_t *d_bad = nullptr, h_bad = 0;
    EN_CUDA(cudaMalloc(&ph.vox, bytes));
    auto cleanup = [&](int code) {
        cudaFree(d_mask);
        cudaFree(d_field);
        cudaFree(d_bad);
        if (code) cudaFree(ph.vox);
        return code;
    };
    if (cudaMalloc(&d_mask, ml) != cudaSuccess || (field && cudaMalloc(&d_field, ml * 4) != cudaSuccess) ||
        cudaMalloc(&d_bad, 4) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(fail(SW_ERR_NOMEM, "phantom upload buffers"));
    }
    if (cudaMemcpy(d_mask, mask, ml, cudaMemcpyHostToDevice) != cudaSuccess ||
        (field && cudaMemcpy(d_field, field, ml * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemset(d_bad, 0, 4) != cudaSuccess ||
        sw::launch_pack(d_mask, d_field, ph.vox, ml, n_substrate, d_bad, E->seed_st, bf16) != cudaSuccess ||
        cudaMemcpyAsync(&h_bad, d_bad, 4, cudaMemcpyDeviceToHost, E->seed_st) != cudaSuccess ||
        cudaStreamSynchronize(E->seed_st) != cudaSuccess)
        return cleanup(fail(SW_ERR_CUDA, "phantom upload"));
    if (h_bad) return cleanup(fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate"));
    cleanup(SW_OK);
    E->launches++;
    *id = E->next_phantom++;
    E->phantoms[*id] = ph;
    E->used += bytes;
    return SW_OK;
}

}  // namespace

extern "C" {

int sw_engine_create(int device, uint32_t n_slots, uint32_t slot_spins, uint64_t hbm_budget,
                     sw_engine **out) {
    return engine_create(device, n_slots, slot_spins, hbm_budget, out);
}

int sw_engine_destroy(sw_engine *e) {
    if (!e) return SW_ERR_INVALID;
    cudaSetDevice(e->device);
    engine_free(e);
    return SW_OK;
}

int sw_engine_add_phantom(sw_engine *e, const uint8_t *mask, const float *field_deg_per_step,
                          const uint64_t dims[3], uint32_t n_substrate, int32_t *phantom_id) {
    return sw_engine_add_phantom_ex(e, mask, field_deg_per_step, dims, n_substrate, 0, phantom_id);
}

int sw_engine_add_phantom_ex(sw_engine *e, const uint8_t *mask, const float *field_deg_per_step,
                             const uint64_t dims[3], uint32_t n_substrate, int flags,
                             int32_t *phantom_id) {
    if (!e) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(SW_ERR_CUDA, "device");
    return engine_add_phantom(e, mask, field_deg_per_step, dims, n_substrate, phantom_id, flags);
}

int sw_engine_submit(sw_engine *e, int32_t phantom, const sw_params *param, const sw_sequence *seq,
                     int precision, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
                     uint8_t *T, int32_t *status, int64_t *job_id) {
    if (!e || !job_id) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(SW_ERR_CUDA, "device");
    return engine_submit(e, phantom, param, seq, precision, M0, XYZ0, M1, XYZ1, T, status, job_id);
}

int sw_engine_poll(sw_engine *e, int wait, sw_job_result *done, uint32_t max_done,
                   uint32_t *n_done) {
    if (!e || !n_done) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(SW_ERR_CUDA, "device");
    *n_done = 0;
    for (;;) {
        int rc = SW_OK;
        const int progress = pump(e, rc);
        if (rc) return rc;
        const bool idle = e->queue.empty();
        if (!e->finished.empty() && (!wait || idle || wait == 1)) break;
        if (!wait || idle) break;
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    uint32_t k = 0;
    while (k < max_done && !e->finished.empty()) {
        Job &j = *e->finished.front();
        if (done) {
            done[k].job_id = j.id;
            done[k].rc = j.rc;
            done[k].latency_s = j.t_done - j.t_submit;
        }
        k++;
        e->finished.erase(e->finished.begin());
    }
    *n_done = k;
    return SW_OK;
}

}  // extern "C"

namespace {
constexpr int kMaxBatchDevices = 64;
std::mutex g_batch_mu;
sw_engine *g_batch_engine[kMaxBatchDevices] = {};

// The engine of the one-call entry points (sw_sim_batch, sw_sim_spins) on the current device:
// its slots (workspaces, staging buffers) are kept from call to call; the caller holds
// g_batch_mu.
int acquire_call_engine(uint32_t slots, uint32_t slot_spins, sw_engine *&out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxBatchDevices)
        return fail(SW_ERR_CUDA, "no current CUDA device");
    sw_engine *&E = g_batch_engine[dev];
    if (E && (E->slots.size() < slots || E->slots[0].cap < slot_spins ||
              E->nlen != ring_len(current_tuning()))) {
        engine_free(E);
        E = nullptr;
    }
    int rc = SW_OK;
    if (!E && (rc = engine_create(dev, slots, slot_spins, 0, &E))) {
        E = nullptr;
        return rc;
    }
    E->launches = E->rounds = E->seedings = 0;
    out = E;
    return SW_OK;
}

// Runs the queued jobs to completion and drops the call's phantoms and seed caches (every call
// does its full work); after a failure the whole engine is dropped.
int finish_call_engine(sw_engine *E, int rc) {
    while (!rc && !E->queue.empty()) {
        const int progress = pump(E, rc);
        if (!progress && !rc) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    for (auto &j : E->finished)
        if (!rc && j->rc) rc = j->rc;
    const std::string err = rc ? std::string(sw_last_error()) : std::string();
    g_timing.n_launches = (uint32_t)E->launches;
    g_timing.n_chunks = (uint32_t)E->rounds;
    int dev = 0;
    cudaGetDevice(&dev);
    if (rc) {
        engine_free(E);
        g_batch_engine[dev] = nullptr;
        return fail(rc, err);
    }
    cudaDeviceSynchronize();
    for (auto &kv : E->phantoms) cudaFree(kv.second.vox);
    E->phantoms.clear();
    for (auto &kv : E->seeds) {
        cudaFree(kv.second->mt);
        cudaFree(kv.second->p);
        cudaEventDestroy(kv.second->ready);
    }
    E->seeds.clear();
    E->finished.clear();
    E->used = 0;
    for (const Slot &s : E->slots) E->used += s.L.bytes + s.io_bytes;
    return SW_OK;
}
}  // namespace

void sw::api::release_call_engine(int dev) {
    if (dev < 0 || dev >= kMaxBatchDevices) return;
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (g_batch_engine[dev]) engine_free(g_batch_engine[dev]);
    g_batch_engine[dev] = nullptr;
}

extern "C" {

int sw_sim_batch(const sw_instance *items, uint32_t n_items, const float *pFieldMap,
                 const uint8_t *pMask, int precision) {
    // checks before any CUDA call
    if (!items || n_items == 0) return fail(SW_ERR_INVALID, "no instances");
    if (!pMask) return fail(SW_ERR_INVALID, "null mask");
    const sw_params *p0 = items[0].param;
    uint64_t n_max = 0;
    for (uint32_t i = 0; i < n_items; i++) {
        const sw_instance &it = items[i];
        int rc = check_args(it.param, it.seq);
        if (rc) return fail(rc, "instance " + std::to_string(i) + ": " + sw_last_error());
        const sw_params *p = it.param;
        if (p->seed != p0->seed)
            return fail(SW_ERR_INVALID, "instances of a batch share the seed (their generator "
                                        "states are seeded once)");
        if (p->matrix_length != p0->matrix_length || p->fieldmap_exist != p0->fieldmap_exist ||
            p->n_substrate != p0->n_substrate)
            return fail(SW_ERR_INVALID, "instances of a batch share the phantom");
        for (int k = 0; k < 3; k++)
            if (p->phantom_size[k] != p0->phantom_size[k])
                return fail(SW_ERR_INVALID, "instances of a batch share the phantom");
        n_max = std::max<uint64_t>(n_max, p->n_spins);
    }
    if (p0->fieldmap_exist && !pFieldMap) return fail(SW_ERR_INVALID, "null fieldmap");
    g_timing = sw_timing{};
    const double t0 = now_s();
    {   // one generator pair per spin id for all instances (sw_pool.cu), where it applies
        bool taken = false;
        const int rp = run_batch_pooled(items, n_items, pFieldMap, pMask, precision, taken);
        if (taken || rp) {
            if (!rp) g_timing.total_ms = (float)((now_s() - t0) * 1e3);
            return rp;
        }
    }
    std::lock_guard<std::mutex> lk(g_batch_mu);
    const uint32_t slots = std::min<uint32_t>(8, n_items);
    const uint32_t slot_spins = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(n_max, 1u << 20));
    sw_engine *E = nullptr;
    int rc = acquire_call_engine(slots, slot_spins, E);
    if (rc) return rc;
    const uint64_t dims[3] = {p0->phantom_size[0], p0->phantom_size[1], p0->phantom_size[2]};
    int32_t ph = 0;
    rc = engine_add_phantom(E, pMask, p0->fieldmap_exist ? pFieldMap : nullptr, dims,
                            p0->n_substrate, &ph, precision & SW_FIELD_BF16);
    SeedCache *sc = nullptr;
    if (!rc) rc = ensure_seeded(E, p0->seed, 0, (uint32_t)n_max, sc);   // one seeding, largest n
    std::vector<uint32_t> order(n_items);
    for (uint32_t i = 0; i < n_items; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return items[a].param->n_spins > items[b].param->n_spins;      // largest first
    });
    for (uint32_t i : order) {
        if (rc) break;
        const sw_instance &it = items[i];
        int64_t jid = 0;
        rc = engine_submit(E, ph, it.param, it.seq, precision, it.M0, it.XYZ0, it.M1, it.XYZ1,
                           it.T, it.status, &jid);
    }
    const uint64_t seedings = E->seedings;
    rc = finish_call_engine(E, rc);
    if (!rc && seedings > 1) rc = fail(SW_ERR_INVALID, "internal error: batch seeded more than once");
    if (rc) return rc;
    g_timing.total_ms = (float)((now_s() - t0) * 1e3);
    return SW_OK;
}

int sw_sim_spins(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                 const uint8_t *pMask, const float *M0, const float *XYZ0, uint32_t spin_lo,
                 uint32_t spin_hi, float *M1, float *XYZ1, uint8_t *T, int32_t *status,
                 int precision) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    if (!pMask) return fail(SW_ERR_INVALID, "null mask");
    if (param->fieldmap_exist && !pFieldMap) return fail(SW_ERR_INVALID, "null fieldmap");
    if (spin_lo > spin_hi || spin_hi > param->n_spins)
        return fail(SW_ERR_INVALID, "spin range outside [0, n_spins)");
    g_timing = sw_timing{};
    if (spin_hi == spin_lo) return SW_OK;
    const double t0 = now_s();
    std::lock_guard<std::mutex> lk(g_batch_mu);
    sw_engine *E = nullptr;
    const uint32_t n = spin_hi - spin_lo;
    rc = acquire_call_engine(4, std::max<uint32_t>(1, std::min<uint32_t>((n + 3) / 4, 1u << 20)), E);
    if (rc) return rc;
    const uint64_t dims[3] = {param->phantom_size[0], param->phantom_size[1], param->phantom_size[2]};
    int32_t ph = 0;
    rc = engine_add_phantom(E, pMask, param->fieldmap_exist ? pFieldMap : nullptr, dims,
                            param->n_substrate, &ph, precision & SW_FIELD_BF16);
    int64_t jid = 0;
    if (!rc)
        rc = engine_submit(E, ph, param, seq, precision, M0, XYZ0, M1, XYZ1, T, status, &jid,
                           spin_lo, spin_hi);
    rc = finish_call_engine(E, rc);
    if (rc) return rc;
    g_timing.total_ms = (float)((now_s() - t0) * 1e3);
    return SW_OK;
}

int sw_engine_submit_signal(sw_engine *e, int32_t phantom, const sw_params *param,
                            const sw_sequence *seq, int precision, const float *M0,
                            const float *XYZ0, double *signal, uint64_t *count, int32_t *status,
                            int64_t *job_id) {
    if (!e || !job_id || !signal || !count) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(SW_ERR_CUDA, "device");
    return engine_submit(e, phantom, param, seq, precision, M0, XYZ0, nullptr, nullptr, nullptr,
                         status, job_id, 0, ~0ull, signal, count);
}

int sw_sim_signal(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                  const uint8_t *pMask, const float *M0, const float *XYZ0, double *signal,
                  uint64_t *count, int32_t *status, int precision) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    if (!pMask || !signal || !count) return fail(SW_ERR_INVALID, "null buffer");
    if (param->fieldmap_exist && !pFieldMap) return fail(SW_ERR_INVALID, "null fieldmap");
    g_timing = sw_timing{};
    const size_t keys = (size_t)seq->n_TE * param->n_substrate;
    if (param->n_spins == 0) {
        std::memset(signal, 0, keys * 24);
        std::memset(count, 0, keys * 8);
        return SW_OK;
    }
    const double t0 = now_s();
    std::lock_guard<std::mutex> lk(g_batch_mu);
    sw_engine *E = nullptr;
    const uint64_t n = param->n_spins;
    rc = acquire_call_engine(4, (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + 3) / 4, 1u << 20)), E);
    if (rc) return rc;
    const uint64_t dims[3] = {param->phantom_size[0], param->phantom_size[1], param->phantom_size[2]};
    int32_t ph = 0;
    rc = engine_add_phantom(E, pMask, param->fieldmap_exist ? pFieldMap : nullptr, dims,
                            param->n_substrate, &ph, precision & SW_FIELD_BF16);
    int64_t jid = 0;
    if (!rc)
        rc = engine_submit(E, ph, param, seq, precision, M0, XYZ0, nullptr, nullptr, nullptr,
                           status, &jid, 0, ~0ull, signal, count);
    rc = finish_call_engine(E, rc);
    if (rc) return rc;
    g_timing.total_ms = (float)((now_s() - t0) * 1e3);
    return SW_OK;
}

int sw_engine_pending(sw_engine *e, uint32_t *n_pending) {
    if (!e || !n_pending) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    *n_pending = (uint32_t)e->queue.size();
    return SW_OK;
}

int sw_engine_get_stats(sw_engine *e, sw_engine_stats *out) {
    if (!e || !out) return SW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    out->launches = e->launches;
    out->rounds = e->rounds;
    out->seedings = e->seedings;
    out->hbm_used = e->used;
    out->hbm_budget = e->budget;
    out->seed_caches = e->seeds.size();
    return SW_OK;
}

}  // extern "C"
