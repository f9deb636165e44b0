// Batches with pooled Gaussian generators: sw_sim_batch when every instance shares the seed
// (which the batch requires) and draws from std::mt19937.
//
// The reference's scale loop runs one simulation per instance (src/sim/monte_carlo.cu:273-337)
// and seeds every spin's generators anew each time: mt19937(seed + spin), discard(seed + spin)
// (src/sim/kernels.cu:82-88). So spin s of every instance draws the SAME sequence of Gaussian
// steps; instances differ only in how fast they consume it (rejected crossings redraw, and the
// sequences differ). Here each spin id s is one "stream": one gen_r and one ring of deviates
// (PoolState), seeded once and refilled once per round for all instances together; every
// instance keeps only its read positions. The Gaussian work of a batch -- three deviates per
// step, most of a round's refill -- is then that of its largest instance instead of the sum over
// instances. Each instance's spins keep their own gen_u (crossing uniforms, drawn only at
// substrate changes), copied from the stream's seeded state: pooling both kinds could deadlock
// (one spin waiting for uniforms a slower spin holds back, that one waiting for Gaussians the
// first holds back), while with one pooled kind the slowest reader always gets a full ring.
//
// A round: k_refill_pool over the streams, then the crossing uniforms and the walks of all
// instances, one launch each over every instance (k_refill_uniforms_batch, k_walk_batch: blocks
// dealt out instance by instance, per-instance descriptors in the workspace); the round is
// captured once per call as a CUDA graph and launched once per round. A stream's ring is topped
// up to the lowest read position of the pairs that paused in the previous walk plus the ring
// length, so nothing unread is overwritten. Results equal one sw_sim call per instance bit for
// bit (tests/test_batch.py).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <omp.h>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"
#include "sw_kernels.h"

namespace {

using namespace sw::api;

constexpr int kMaxDevices = 64;
struct PoolCtx {
    std::mutex mu;
    char *d = nullptr;                   // device workspace
    size_t d_bytes = 0;
    char *h = nullptr;                   // pinned staging of the instances' inputs and outputs
    size_t h_bytes = 0;
    uint32_t *d_jump = nullptr;          // jump polynomials of the high spin ids
    size_t jump_words = 0;
    cudaStream_t main = nullptr;         // pack, seeding, rounds, copies
    cudaStream_t side = nullptr;         // instance inputs and k_init, beside the seeding
    cudaEvent_t side_done = nullptr;
    cudaEvent_t stage[4] = {};           // timing: the seeding, then the rounds
    cudaEvent_t piece[8] = {};           // output read-back in pieces
    uint32_t *h_active = nullptr;        // pinned
    bool ready = false;
};
PoolCtx g_pool[kMaxDevices];

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

#define PL_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
        }                                                                                  \
    } while (0)

int ensure_ctx(PoolCtx &c) {
    if (c.ready) return SW_OK;
    int lo = 0, hi = 0;
    PL_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PL_CUDA(cudaStreamCreateWithPriority(&c.main, cudaStreamNonBlocking, hi));
    PL_CUDA(cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, hi));
    PL_CUDA(cudaEventCreateWithFlags(&c.side_done, cudaEventDisableTiming));
    for (auto &e : c.stage) PL_CUDA(cudaEventCreate(&e));
    for (auto &e : c.piece) PL_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PL_CUDA(cudaMallocHost(&c.h_active, sizeof(uint32_t)));
    c.ready = true;
    return SW_OK;
}

// Host copies between the caller's buffers and the pinned staging, all of a call's arrays at
// once: cut into pieces of 2 MiB and spread over every core (one core copies about 10 GB/s,
// and most instances' arrays are too small to split on their own).
struct CopyJob {
    void *dst;
    const void *src;
    size_t bytes;
};

void par_copy_all(const std::vector<CopyJob> &jobs) {
    constexpr size_t kPiece = 2 << 20;
    std::vector<CopyJob> pieces;
    for (const CopyJob &j : jobs)
        for (size_t o = 0; o < j.bytes; o += kPiece)
            pieces.push_back(CopyJob{static_cast<char *>(j.dst) + o,
                                     static_cast<const char *>(j.src) + o,
                                     std::min(kPiece, j.bytes - o)});
    const int64_t np = (int64_t)pieces.size();
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(np, std::min(omp_get_num_procs(), 32)));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int64_t i = 0; i < np; i++) std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes);
}

struct Inst {
    const sw_instance *it;
    size_t n, nte, trj;
    bool dbl;
    TableImage im;
    sw::DevParams P;
    sw::SpinState S;
    sw::RngState G;                      // nhead: read positions in the streams; own gen_u
    char *tables;
    // device I/O (offsets into the I/O region, same offsets in the pinned staging): the inputs
    // of all instances first, then their outputs
    size_t o_M0, o_XYZ0, o_M1, o_T, o_XYZ1, o_st;
};

}  // namespace

void sw::api::release_pool_memory(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return;
    PoolCtx &X = g_pool[dev];
    std::lock_guard<std::mutex> lk(X.mu);
    if (X.d) cudaFree(X.d);
    if (X.h) cudaFreeHost(X.h);
    if (X.d_jump) cudaFree(X.d_jump);
    X.d = nullptr;
    X.h = nullptr;
    X.d_jump = nullptr;
    X.d_bytes = X.h_bytes = X.jump_words = 0;
}

int sw::api::run_batch_pooled(const sw_instance *items, uint32_t n_items, const float *pFieldMap,
                              const uint8_t *pMask, int precision, bool &taken) {
    taken = false;
    const bool bf16 = (precision & SW_FIELD_BF16) != 0;
    const uint32_t rng = (uint32_t)precision & ~(uint32_t)(SW_PREC_MASK | SW_FIELD_BF16);
    const int prec = precision & SW_PREC_MASK;
    if (rng != SW_RNG_MT19937) return SW_OK;                 // minstd: the engine path
    if (prec != SW_PREC_FP32 && prec != SW_PREC_FP64 && prec != SW_PREC_KAHAN)
        return fail(SW_ERR_INVALID, "precision");
    const sw_params *p0 = items[0].param;
    const size_t ml = (size_t)p0->matrix_length;
    uint64_t n_max = 0;
    for (uint32_t i = 0; i < n_items; i++) n_max = std::max<uint64_t>(n_max, items[i].param->n_spins);
    if (n_max == 0) {
        taken = true;
        return SW_OK;
    }

    // ---- layout: phantom, pool, per-instance state, then the I/O region ----
    std::vector<Inst> in(n_items);
    Carve c{nullptr};
    auto plan = [&](char *base) {
        c = Carve{base};
        uint2 *vox = c.take<uint2>(bf16 ? (ml + 1) / 2 : ml);
        (void)vox;
        c.take<uint32_t>(4);                                  // active counter, bad-label flag
        c.take<uint32_t>(n_max * sw::kMtN);                  // mt_r
        for (int k = 0; k < 3; k++) c.take<uint32_t>(n_max);  // p_r nw nmin
        c.take<float>(n_max * sw::kPoolNorm);
        c.take<sw::BatchInst>(n_items);                      // descriptors of the fused launches
        c.take<sw::SeedCopy>(n_items);                       // gen_u of every instance
        for (Inst &I : in) {
            const size_t n = I.n;
            I.tables = c.take<char>(I.im.bytes.size());
            sw::SpinState &S = I.S;
            S.x = c.take<uint64_t>(n);
            S.y = c.take<uint64_t>(n);
            S.z = c.take<uint64_t>(n);
            S.mx = c.take<float>(n);
            S.my = c.take<float>(n);
            S.mz = c.take<float>(n);
            S.acc = c.take<float>(n);
            S.acc_e = c.take<float>(n);
            S.accd = c.take<double>(I.dbl ? n : 1);
            S.dmx = c.take<double>(I.dbl ? n : 1);
            S.dmy = c.take<double>(I.dbl ? n : 1);
            S.dmz = c.take<double>(I.dbl ? n : 1);
            S.field = c.take<float>(n);
            S.ind_old = c.take<int64_t>(n);
            S.tp = c.take<uint32_t>(n);
            S.tp_old = c.take<uint32_t>(n);
            S.ds = c.take<uint32_t>(n);
            S.itr = c.take<uint32_t>(n);
            S.ctr = c.take<uint32_t>(n);
            S.ctr2 = c.take<uint32_t>(n);
            S.flags = c.take<uint32_t>(n);
            I.G = sw::RngState{};
            I.G.nhead = c.take<uint32_t>(n);
            I.G.mt_u = c.take<uint32_t>(n * sw::kMtN);
            I.G.p_u = c.take<uint32_t>(n);
            I.G.ubuf = c.take<float>(n * sw::kUnifBuf);
            I.G.uhead = c.take<uint32_t>(n);
            I.G.ucnt = c.take<uint32_t>(n);
        }
    };
    size_t io = 0;
    for (uint32_t i = 0; i < n_items; i++) {
        Inst &I = in[i];
        I.it = &items[i];
        const sw_params *p = I.it->param;
        I.n = p->n_spins;
        I.nte = I.it->seq->n_TE;
        I.trj = p->enRecordTrajectory ? (size_t)(p->n_dummy_scan + 1) * p->n_timepoints : 1;
        I.dbl = prec == SW_PREC_FP64;
        build_tables(p, I.it->seq, I.im);
        if (!I.im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
        I.P = dev_params(p, I.it->seq);
        I.P.rng = SW_RNG_MT19937;
        I.P.field_bf16 = bf16 ? 1 : 0;
    }
    auto sec = [&](size_t bytes) { size_t o = io; io = (io + bytes + 255) & ~size_t(255); return o; };
    for (Inst &I : in) {
        I.o_M0 = sec(I.n * 12);
        I.o_XYZ0 = sec(I.n * 12);
    }
    const size_t out_begin = io;          // outputs: uploaded with their contents, read back
    for (Inst &I : in) {
        I.o_M1 = sec(I.n * I.nte * 12);
        I.o_T = sec(I.n * I.nte);
        I.o_XYZ1 = sec(I.n * I.trj * 12);
        I.o_st = sec(I.n * 4);
    }
    plan(nullptr);
    const size_t state_bytes = (c.off + 255) & ~size_t(255);
    const size_t need = state_bytes + io + 256;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return SW_OK;                                        // let the engine path report it
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(SW_ERR_CUDA, "no current CUDA device");
    }
    PoolCtx &X = g_pool[dev];
    std::lock_guard<std::mutex> lk(X.mu);
    // the pool holds every instance at once: above half the free memory, run instances as
    // engine jobs instead (bounded slots)
    if (need > X.d_bytes && need - X.d_bytes > free_b / 2) return SW_OK;
    taken = true;
    int rc = ensure_ctx(X);
    if (rc) return rc;
    // whichever way the call returns, nothing of it is left running on the context's streams
    // (the next call reuses the workspace)
    struct Drain {
        PoolCtx &X;
        ~Drain() {
            cudaStreamSynchronize(X.main);
            cudaStreamSynchronize(X.side);
        }
    } drain{X};
    const LogfTables LT = device_logf_tables();
    if (!LT.tab) return SW_ERR_CUDA;
    if (need > X.d_bytes) {
        if (X.d) cudaFree(X.d);
        X.d = nullptr;
        X.d_bytes = 0;
        cudaError_t e = cudaMalloc(&X.d, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, "batch workspace of " + std::to_string(need >> 20) +
                                          " MiB: " + cudaGetErrorString(e));
        }
        X.d_bytes = need;
    }
    if (io > X.h_bytes) {
        if (X.h) cudaFreeHost(X.h);
        X.h = nullptr;
        X.h_bytes = 0;
        cudaError_t e = cudaMallocHost(&X.h, io);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, "batch staging of " + std::to_string(io >> 20) +
                                          " MiB: " + cudaGetErrorString(e));
        }
        X.h_bytes = io;
    }
    plan(X.d);
    Carve c2{X.d};
    uint2 *vox = c2.take<uint2>(bf16 ? (ml + 1) / 2 : ml);
    uint32_t *cnt = c2.take<uint32_t>(4);
    sw::PoolState Q;
    Q.mt_r = c2.take<uint32_t>(n_max * sw::kMtN);
    Q.p_r = c2.take<uint32_t>(n_max);
    Q.nw = c2.take<uint32_t>(n_max);
    Q.nmin = c2.take<uint32_t>(n_max);
    Q.nbuf = c2.take<float>(n_max * sw::kPoolNorm);
    sw::BatchInst *d_inst = c2.take<sw::BatchInst>(n_items);
    sw::SeedCopy *d_fan = c2.take<sw::SeedCopy>(n_items);
    char *d_io = X.d + state_bytes;
    cudaStream_t ms = X.main;
    uint32_t launches = 0;

    // ---- generator streams first (they read nothing of the call's inputs), then the phantom
    // (mask + field -> records) beside them on the side stream ----
    PL_CUDA(cudaEventRecord(X.stage[0], ms));
    sw::JumpTable jt;
    rc = jump_table(p0->seed, 0, (uint32_t)n_max, jump_min_z(current_tuning()), X.d_jump,
                    X.jump_words, jt);
    if (rc) return rc;
    {
        sw::DevParams Ps{};
        Ps.seed = p0->seed;
        Ps.rng = SW_RNG_MT19937;
        // k_seed writes the state twice (gen_r and gen_u start alike) and zeroes four ring
        // counters per spin: here the stream's state, its written count and its lowest read
        // position, which is where every stream starts
        sw::RngState Gs{};
        Gs.mt_r = Gs.mt_u = Q.mt_r;
        Gs.p_r = Gs.p_u = Q.p_r;
        Gs.nhead = Gs.uhead = Q.nw;
        Gs.ncnt = Gs.ucnt = Q.nmin;
        // each instance's gen_u starts from the same seeded state: the seeding kernels store it
        // there as well, with the instance's read positions and uniform counters zeroed (their
        // stores hide under the integer work of the seeding; 64 device copies afterwards would
        // put ~10 ms of copying between the seeding and the first round)
        std::vector<sw::SeedCopy> fan;
        for (Inst &I : in)
            if (I.n) fan.push_back({I.G.mt_u, I.G.p_u, I.G.nhead, I.G.uhead, I.G.ucnt, (uint32_t)I.n});
        PL_CUDA(cudaMemcpyAsync(d_fan, fan.data(), fan.size() * sizeof(sw::SeedCopy),
                                cudaMemcpyHostToDevice, ms));
        PL_CUDA(sw::launch_seed_range(Ps, Gs, 0, (uint32_t)n_max, ms, &jt,
                                      sw::SeedCopies{d_fan, (uint32_t)fan.size()}));
        PL_CUDA(cudaEventRecord(X.stage[1], ms));
        launches++;
    }
    cudaStream_t w0 = X.side;
    {
        uint8_t *d_mask = nullptr;
        float *d_field = nullptr;
        // the I/O region is free until the instances' inputs are staged (uploaded later on the
        // same stream): use it for the phantom upload when it is large enough, else a temporary
        // allocation
        const size_t ph_bytes = ml + (p0->fieldmap_exist ? ml * 4 : 0) + 512;
        char *tmp = nullptr;
        char *up = d_io;
        auto bail = [&](int code) {          // the seeding is in flight on the main stream
            cudaStreamSynchronize(ms);
            cudaStreamSynchronize(w0);
            if (tmp) cudaFree(tmp);
            return code;
        };
        if (ph_bytes > io) {
            const cudaError_t e = cudaMalloc(&tmp, ph_bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                tmp = nullptr;
                return bail(fail(SW_ERR_NOMEM, std::string("phantom upload: ") + cudaGetErrorString(e)));
            }
            up = tmp;
        }
        d_mask = reinterpret_cast<uint8_t *>(up);
        if (p0->fieldmap_exist) d_field = reinterpret_cast<float *>(up + ((ml + 255) & ~size_t(255)));
        cudaError_t e = cudaMemcpyAsync(d_mask, pMask, ml, cudaMemcpyHostToDevice, w0);
        if (e == cudaSuccess && d_field)
            e = cudaMemcpyAsync(d_field, pFieldMap, ml * 4, cudaMemcpyHostToDevice, w0);
        if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, 4 * sizeof(uint32_t), w0);
        if (e == cudaSuccess)
            e = sw::launch_pack(d_mask, d_field, vox, (int64_t)ml, p0->n_substrate, cnt + 1, w0, bf16);
        uint32_t bad = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, cnt + 1, 4, cudaMemcpyDeviceToHost, w0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(w0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return bail(fail(SW_ERR_CUDA, std::string("phantom: ") + cudaGetErrorString(e)));
        }
        launches++;
        if (bad) return bail(fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate"));
        if (tmp) {
            cudaFree(tmp);
            tmp = nullptr;
        }
    }

    // ---- instances: inputs (and the outputs' current contents) staged, uploaded, k_init ----
    {
        std::vector<CopyJob> jobs;
        for (Inst &I : in) {
            const sw_instance &it = *I.it;
            jobs.push_back({X.h + I.o_M0, it.M0, I.n * 12});
            jobs.push_back({X.h + I.o_XYZ0, it.XYZ0, I.n * 12});
            if (I.nte) {
                jobs.push_back({X.h + I.o_M1, it.M1, I.n * I.nte * 12});
                jobs.push_back({X.h + I.o_T, it.T, I.n * I.nte});
            }
            jobs.push_back({X.h + I.o_XYZ1, it.XYZ1, I.n * I.trj * 12});
        }
        par_copy_all(jobs);
    }
    PL_CUDA(cudaMemcpyAsync(d_io, X.h, io, cudaMemcpyHostToDevice, w0));
    std::vector<sw::DevTables> Tb(n_items);
    std::vector<sw::Outputs> O(n_items);
    for (uint32_t i = 0; i < n_items; i++) {
        Inst &I = in[i];
        PL_CUDA(cudaMemcpyAsync(I.tables, I.im.bytes.data(), I.im.bytes.size(), cudaMemcpyHostToDevice, w0));
        Tb[i] = dev_tables(I.im, I.tables);
        O[i] = sw::Outputs{I.nte ? reinterpret_cast<float *>(d_io + I.o_M1) : nullptr, nullptr,
                           reinterpret_cast<float *>(d_io + I.o_XYZ1),
                           I.nte ? reinterpret_cast<uint8_t *>(d_io + I.o_T) : nullptr,
                           reinterpret_cast<int32_t *>(d_io + I.o_st)};
        if (!I.n) continue;
        PL_CUDA(sw::launch_init_range(I.P, Tb[i], vox, reinterpret_cast<const float *>(d_io + I.o_M0),
                                      reinterpret_cast<const float *>(d_io + I.o_XYZ0), I.S, O[i],
                                      I.dbl, 0, (uint32_t)I.n, w0));
        launches++;
    }
    PL_CUDA(cudaEventRecord(X.side_done, w0));
    PL_CUDA(cudaStreamWaitEvent(ms, X.side_done, 0));

    // ---- rounds ----
    uint64_t steps_max = 0, max_rounds = 64;
    for (const Inst &I : in) {
        const sw_params *p = I.it->param;
        const uint64_t st = (uint64_t)p->n_timepoints * (uint64_t)(p->n_dummy_scan + 1);
        steps_max = std::max(steps_max, st);
        max_rounds = std::max<uint64_t>(max_rounds, 64 + st * (p->max_iterations + 2));
    }
    // Descriptors of the walking instances for the fused launches, in block order.
    std::vector<sw::BatchInst> desc;
    uint32_t walk_blocks = 0, unif_blocks = 0;
    for (uint32_t i = 0; i < n_items; i++) {
        const Inst &I = in[i];
        if (!I.n) continue;
        sw::BatchInst b{};
        b.P = I.P;
        b.Tb = Tb[i];
        b.S = I.S;
        b.G = I.G;
        b.O = O[i];
        b.n_spins = (uint32_t)I.n;
        b.walk_block0 = walk_blocks;
        b.unif_block0 = unif_blocks;
        walk_blocks += (uint32_t)((I.n + 255) / 256);
        unif_blocks += (uint32_t)((I.n + sw::kRefillBatchSpins - 1) / sw::kRefillBatchSpins);
        desc.push_back(b);
    }
    const uint32_t n_desc = (uint32_t)desc.size();
    PL_CUDA(cudaMemcpyAsync(d_inst, desc.data(), n_desc * sizeof(sw::BatchInst),
                            cudaMemcpyHostToDevice, ms));
    // One round as a CUDA graph, captured once per call and launched once per round: the pooled
    // refill of the Gaussian streams, then the crossing uniforms and the walk of every instance,
    // each as one launch over all instances (blocks dealt out instance by instance). Every
    // kernel reads its state from the workspace, so the same graph serves every round; results
    // equal one sw_sim call per instance bit for bit.
    struct RoundGraph {                      // destroyed on every way out of the call
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        void drop() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = nullptr;
            graph = nullptr;
        }
        ~RoundGraph() { drop(); }
    } rg;
    cudaGraph_t &graph = rg.graph;
    cudaGraphExec_t &exec = rg.exec;
    const uint32_t round_kernels = 3;
    auto drop_graph = [&]() { rg.drop(); };
    auto capture_round = [&]() -> int {
        PL_CUDA(cudaStreamBeginCapture(ms, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
        ok(cudaMemsetAsync(cnt, 0, sizeof(uint32_t), ms));
        ok(sw::launch_refill_pool(Q, LT, (uint32_t)n_max, ms));
        ok(sw::launch_refill_uniforms_batch(d_inst, n_desc, unif_blocks, ms));
        ok(sw::launch_walk_batch(prec, prec == SW_PREC_FP64, d_inst, n_desc, walk_blocks, vox, Q,
                                 cnt, ms, walk_grid_cap(current_tuning())));
        const cudaError_t ec = cudaStreamEndCapture(ms, &graph);
        if (e == cudaSuccess) e = ec;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            drop_graph();
            return fail(SW_ERR_CUDA, std::string("round graph: ") + cudaGetErrorString(e));
        }
        return SW_OK;
    };
    rc = capture_round();
    if (rc) return rc;
    PL_CUDA(cudaEventRecord(X.stage[2], ms));
    // every pair needs 3 deviates per step and a round gives at most kPoolNorm: no pair can
    // finish sooner than r0 rounds, which are issued without waiting
    const uint64_t r0 = std::max<uint64_t>(1, (3 * steps_max + sw::kPoolNorm - 1) / sw::kPoolNorm);
    uint64_t rounds = 0;
    for (;; rounds++) {
        if (rounds >= max_rounds) {
            cudaStreamSynchronize(ms);
            drop_graph();
            return fail(SW_ERR_TIMEOUT, "walk did not finish");
        }
        cudaError_t e = cudaGraphLaunch(exec, ms);
        if (e == cudaSuccess && rounds + 1 >= r0) {
            e = cudaMemcpyAsync(X.h_active, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, ms);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ms);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaStreamSynchronize(ms);
            drop_graph();
            return fail(SW_ERR_CUDA, std::string("round: ") + cudaGetErrorString(e));
        }
        if (rounds + 1 >= r0 && *X.h_active == 0) break;
    }
    drop_graph();
    launches += round_kernels * (uint32_t)(rounds + 1);
    PL_CUDA(cudaEventRecord(X.stage[3], ms));

    // ---- outputs: read back in pieces of whole instances (their output sections are
    // contiguous, in instance order); the host copies a piece into the caller's arrays while the
    // next one is still on its way ----
    {
        constexpr uint32_t kPieces = sizeof(X.piece) / sizeof(X.piece[0]);
        const size_t out_bytes = io - out_begin;
        std::vector<uint32_t> first(1, 0u);              // first instance of every piece
        for (uint32_t i = 0; i < n_items && first.size() < kPieces; i++) {
            const size_t end = in[i].o_st + in[i].n * 4;
            if ((end - out_begin) * kPieces >= out_bytes * first.size() && i + 1 < n_items)
                first.push_back(i + 1);
        }
        first.push_back(n_items);
        const uint32_t np = (uint32_t)first.size() - 1;
        for (uint32_t k = 0; k < np; k++) {
            const size_t a = in[first[k]].o_M1;
            const size_t b = k + 1 < np ? in[first[k + 1]].o_M1 : io;
            if (b > a)
                PL_CUDA(cudaMemcpyAsync(X.h + a, d_io + a, b - a, cudaMemcpyDeviceToHost, ms));
            PL_CUDA(cudaEventRecord(X.piece[k], ms));
        }
        for (uint32_t k = 0; k < np; k++) {
            PL_CUDA(cudaEventSynchronize(X.piece[k]));
            std::vector<CopyJob> jobs;
            for (uint32_t i = first[k]; i < first[k + 1]; i++) {
                const Inst &I = in[i];
                const sw_instance &it = *I.it;
                if (I.nte) {
                    jobs.push_back({it.M1, X.h + I.o_M1, I.n * I.nte * 12});
                    jobs.push_back({it.T, X.h + I.o_T, I.n * I.nte});
                }
                jobs.push_back({it.XYZ1, X.h + I.o_XYZ1, I.n * I.trj * 12});
                if (it.status) jobs.push_back({it.status, X.h + I.o_st, I.n * 4});
            }
            par_copy_all(jobs);
        }
    }
    g_timing.n_chunks = (uint32_t)(rounds + 1);          // refill/walk rounds
    g_timing.n_launches = launches;
    // stage times (CUDA events on the main stream): the seeding; the rounds (the pooled
    // refills, uniforms and walks together); the call's wall time is set by the caller
    cudaEventElapsedTime(&g_timing.seed_ms, X.stage[0], X.stage[1]);
    cudaEventElapsedTime(&g_timing.walk_ms, X.stage[2], X.stage[3]);
    return SW_OK;
}
