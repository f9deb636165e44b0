// C ABI of libspinwalk_gpu (include/spinwalk_gpu.h): argument checks, device workspace,
// parameter-table upload and the seed -> (refill, walk)* launch sequence.
//
// The workspace (packed phantom, per-spin walk state, generator state and buffers) is owned by
// a per-device context, grown on demand and reused across calls; calls on the same device are
// serialised by a mutex. Nothing here exits or traps: failures come back as SW_ERR_* codes
// with a message in sw_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_host.h"
#include "sw_kernels.h"
#include "sw_mtjump.h"
#include "sw_api_internal.h"

namespace sw {
namespace api {


thread_local std::string g_err;
thread_local sw_timing g_timing{};

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define SW_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)


int check_args(const sw_params *p, const sw_sequence *q) {
    if (!p || !q) return fail(SW_ERR_INVALID, "null params or sequence");
    if (p->n_substrate == 0 || p->n_substrate > 256) return fail(SW_ERR_INVALID, "n_substrate");
    if (!q->diffusivity || !q->T1_ms || !q->T2_ms || !q->pXY)
        return fail(SW_ERR_INVALID, "tissue tables missing");
    if (q->n_RF == 0 || !q->RF_FA_deg || !q->RF_PH_deg || !q->RF_us)
        return fail(SW_ERR_INVALID, "at least one RF pulse (RF_T = 0) is required");
    if (q->n_TE > 0xffff || q->n_RF > 0xffff || q->n_dephasing > 0xffff || q->n_gradient > 0xffff)
        return fail(SW_ERR_INVALID, "event tables longer than the 16-bit counters of the reference");
    if (q->n_TE && !q->TE_us) return fail(SW_ERR_INVALID, "TE table");
    if (q->n_dephasing && (!q->dephasing_us || !q->dephasing_deg))
        return fail(SW_ERR_INVALID, "dephasing table");
    if (q->n_gradient &&
        (!q->gradient_us || !q->gradientX_mTm || !q->gradientY_mTm || !q->gradientZ_mTm))
        return fail(SW_ERR_INVALID, "gradient table");
    if (p->n_dummy_scan < 0) return fail(SW_ERR_INVALID, "n_dummy_scan < 0 (call sw_prepare_params)");
    if (p->timestep_us <= 0) return fail(SW_ERR_INVALID, "timestep_us");
    const int64_t ml = (int64_t)(p->phantom_size[0] * p->phantom_size[1] * p->phantom_size[2]);
    if (ml <= 0 || ml != p->matrix_length) return fail(SW_ERR_INVALID, "matrix_length != Nx*Ny*Nz");
    for (int i = 0; i < 3; i++)
        if (!(p->fov[i] > 0)) return fail(SW_ERR_INVALID, "fov must be positive");
    return SW_OK;
}

sw::DevParams dev_params(const sw_params *p, const sw_sequence *q) {
    sw::DevParams d{};
    for (int i = 0; i < 3; i++) {
        d.fov[i] = p->fov[i];
        d.s2g[i] = (double)p->phantom_size[i] / p->fov[i];       // kernels.cu:98
        d.s2g_f[i] = (float)d.s2g[i];
    }
    d.nz = (int64_t)p->phantom_size[2];
    d.nynz = (int64_t)p->phantom_size[1] * (int64_t)p->phantom_size[2];
    d.matrix_length = p->matrix_length;
    d.seed = p->seed;
    d.max_iterations = p->max_iterations;
    d.n_spins = p->n_spins;
    d.n_timepoints = p->n_timepoints;
    d.n_substrate = p->n_substrate;
    d.n_dummy_scan = (uint32_t)p->n_dummy_scan;
    d.n_TE = q->n_TE;
    d.n_RF = q->n_RF;
    d.n_dephasing = q->n_dephasing;
    d.n_gradient = q->n_gradient;
    d.timestep_us = p->timestep_us;
    d.cross_fov = p->enCrossFOV ? 1 : 0;
    d.record_traj = p->enRecordTrajectory ? 1 : 0;
    d.fieldmap_exist = p->fieldmap_exist ? 1 : 0;
    d.traj_len = p->enRecordTrajectory
                     ? (uint64_t)(p->n_dummy_scan + 1) * (uint64_t)p->n_timepoints : 1;
    return d;
}


void build_tables(const sw_params *p, const sw_sequence *q, TableImage &im) {
    const uint32_t ns = p->n_substrate;
    std::vector<float> T1f(ns), T2f(ns);
    std::vector<double> T1d(ns), T2d(ns);
    for (uint32_t i = 0; i < ns; i++) {
        T1f[i] = q->T1_ms[i] * 1e-3;          // kernels.cu:167-168 (float * double -> float)
        T2f[i] = q->T2_ms[i] * 1e-3;
        T1d[i] = q->T1_ms[i] * 1e-3;
        T2d[i] = q->T2_ms[i] * 1e-3;
    }
    std::vector<sw::RfOp> rf, scan;
    sw::build_rf(p, q, rf);
    sw::build_scan_rf(p, q, scan);
    im.o_dscale = im.put(q->diffusivity, ns);
    im.o_T1f = im.put(T1f.data(), ns);
    im.o_T2f = im.put(T2f.data(), ns);
    im.o_T1d = im.put(T1d.data(), ns);
    im.o_T2d = im.put(T2d.data(), ns);
    im.o_pXY = im.put(q->pXY, (size_t)ns * ns);
    im.o_rf = im.put(rf.data(), rf.size());
    im.o_scan = im.put(scan.data(), scan.size());
    im.o_te = im.put(q->TE_us, q->n_TE);
    im.o_dtp = im.put(q->dephasing_us, q->n_dephasing);
    im.o_ddeg = im.put(q->dephasing_deg, q->n_dephasing);
    im.o_gtp = im.put(q->gradient_us, q->n_gradient);
    im.o_gx = im.put(q->gradientX_mTm, q->n_gradient);
    im.o_gy = im.put(q->gradientY_mTm, q->n_gradient);
    im.o_gz = im.put(q->gradientZ_mTm, q->n_gradient);
}

sw::DevTables dev_tables(const TableImage &im, const char *d) {
    sw::DevTables t{};
    t.dscale = reinterpret_cast<const double *>(d + im.o_dscale);
    t.T1f = reinterpret_cast<const float *>(d + im.o_T1f);
    t.T2f = reinterpret_cast<const float *>(d + im.o_T2f);
    t.T1d = reinterpret_cast<const double *>(d + im.o_T1d);
    t.T2d = reinterpret_cast<const double *>(d + im.o_T2d);
    t.pXY = reinterpret_cast<const float *>(d + im.o_pXY);
    t.rf = reinterpret_cast<const sw::RfOp *>(d + im.o_rf);
    t.scan_rf = reinterpret_cast<const sw::RfOp *>(d + im.o_scan);
    t.te_tp = reinterpret_cast<const int32_t *>(d + im.o_te);
    t.dph_tp = reinterpret_cast<const int32_t *>(d + im.o_dtp);
    t.dph_deg = reinterpret_cast<const float *>(d + im.o_ddeg);
    t.grad_tp = reinterpret_cast<const int32_t *>(d + im.o_gtp);
    t.gx = reinterpret_cast<const float *>(d + im.o_gx);
    t.gy = reinterpret_cast<const float *>(d + im.o_gy);
    t.gz = reinterpret_cast<const float *>(d + im.o_gz);
    return t;
}


// Lays out the whole workspace; with base == nullptr it only measures.
Layout layout(char *base, size_t n, int64_t ml, size_t table_bytes, bool dbl, bool mt_state,
              uint32_t nlen) {
    Carve c{base};
    Layout L{};
    L.vox = c.take<uint2>(ml);
    L.tables = c.take<char>(table_bytes);
    L.active = c.take<uint32_t>(4);
    sw::SpinState &S = L.S;
    S.x = c.take<uint64_t>(n);
    S.y = c.take<uint64_t>(n);
    S.z = c.take<uint64_t>(n);
    S.mx = c.take<float>(n);
    S.my = c.take<float>(n);
    S.mz = c.take<float>(n);
    S.acc = c.take<float>(n);
    S.acc_e = c.take<float>(n);
    S.accd = c.take<double>(dbl ? n : 1);
    S.dmx = c.take<double>(dbl ? n : 1);
    S.dmy = c.take<double>(dbl ? n : 1);
    S.dmz = c.take<double>(dbl ? n : 1);
    S.field = c.take<float>(n);
    S.ind_old = c.take<int64_t>(n);
    S.tp = c.take<uint32_t>(n);
    S.tp_old = c.take<uint32_t>(n);
    S.ds = c.take<uint32_t>(n);
    S.itr = c.take<uint32_t>(n);
    S.ctr = c.take<uint32_t>(n);
    S.ctr2 = c.take<uint32_t>(n);
    S.flags = c.take<uint32_t>(n);
    sw::RngState &G = L.G;
    G.mt_r = c.take<uint32_t>(mt_state ? n * sw::kMtN : 1);      // minstd: state in p_r / p_u
    G.mt_u = c.take<uint32_t>(mt_state ? n * sw::kMtN : 1);
    G.p_r = c.take<uint32_t>(n);
    G.p_u = c.take<uint32_t>(n);
    G.nlen = nlen;
    G.nbuf = c.take<float>(n * nlen);
    G.nhead = c.take<uint32_t>(n);
    G.ncnt = c.take<uint32_t>(n);
    G.ubuf = c.take<float>(n * sw::kUnifBuf);
    G.uhead = c.take<uint32_t>(n);
    G.ucnt = c.take<uint32_t>(n);
    L.Q.order = c.take<uint32_t>(n);
    L.Q.key = c.take<uint32_t>(n);
    L.Q.hist = c.take<uint32_t>(2 * sw::order_hist_words());   // one histogram per half of the rounds
    L.bytes = c.off + 256;
    return L;
}

}  // namespace api
}  // namespace sw

using namespace sw::api;

namespace {

constexpr int kMaxDevices = 64;
constexpr int kMaxTimedChunks = 4096;
constexpr uint32_t kMaxSeedChunks = 64;

struct DeviceCtx {
    std::mutex mu;
    bool logf_ready = false;
    float *d_logf_tab = nullptr;
    uint32_t *d_logf_bitmap = nullptr;
    char *ws = nullptr;
    size_t ws_size = 0;
    char *io = nullptr;                    // sw_sim: device copies of the caller's host buffers
    size_t io_size = 0;
    uint32_t *h_active = nullptr;          // pinned
    std::vector<cudaEvent_t> ev;           // timing events: 4 call-level, then 3 per round
    cudaStream_t seed_st = nullptr;        // lowest priority: seeding of the chunks
    cudaStream_t walk_st = nullptr;        // highest priority: pack, init, refill, walk
    cudaStream_t walk_st2 = nullptr;       // highest priority: the second half's rounds
    std::vector<cudaEvent_t> pev;          // pipeline: start, done, seed chunk c done / timed
    uint32_t *d_jump = nullptr;            // jump polynomials of the call's high spin ids
    size_t jump_words = 0;
};
DeviceCtx g_ctx[kMaxDevices];

int ensure_logf(DeviceCtx &c) {
    if (c.logf_ready) return SW_OK;
    const sw::LogfExceptions &ex = sw::logf_exceptions();
    if (ex.wide != 0)
        return fail(SW_ERR_INVALID, "the host logf differs from the device candidate by more "
                                    "than one ulp towards the exact value on " +
                                        std::to_string(ex.wide) + " inputs");
    SW_CUDA(cudaMalloc(&c.d_logf_tab, 192 * sizeof(float)));
    SW_CUDA(cudaMalloc(&c.d_logf_bitmap, ex.bitmap.size() * sizeof(uint32_t)));
    SW_CUDA(cudaMemcpy(c.d_logf_tab, sw::logf_reduction_table(), 192 * sizeof(float),
                       cudaMemcpyHostToDevice));
    SW_CUDA(cudaMemcpy(c.d_logf_bitmap, ex.bitmap.data(), ex.bitmap.size() * sizeof(uint32_t),
                       cudaMemcpyHostToDevice));
    SW_CUDA(cudaMallocHost(&c.h_active, 2 * sizeof(uint32_t)));
    c.ev.resize(3 * kMaxTimedChunks + 4);
    for (auto &e : c.ev) SW_CUDA(cudaEventCreate(&e));
    int lo_prio = 0, hi_prio = 0;
    SW_CUDA(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    SW_CUDA(cudaStreamCreateWithPriority(&c.seed_st, cudaStreamNonBlocking, lo_prio));
    SW_CUDA(cudaStreamCreateWithPriority(&c.walk_st, cudaStreamNonBlocking, hi_prio));
    SW_CUDA(cudaStreamCreateWithPriority(&c.walk_st2, cudaStreamNonBlocking, hi_prio));
    c.pev.resize(4 + 2 * kMaxSeedChunks);
    for (auto &e : c.pev) SW_CUDA(cudaEventCreate(&e));
    c.logf_ready = true;
    return SW_OK;
}

sw::LogfTables logf_tables(const DeviceCtx &c) {
    return sw::LogfTables{c.d_logf_tab, c.d_logf_bitmap};
}

// Boundaries of `C` spin chunks of equal seeding cost: spin s costs its seeding, discard(seed+s)
// words plus about one block (624 words) of seeding and first twist.
std::vector<uint32_t> seed_chunks(const sw::DevParams &P, uint32_t C) {
    const double n = P.n_spins, a = (double)P.seed + 624.0;
    auto F = [&](double x) { return x * a + 0.5 * x * (x - 1.0); };   // cost of spins [0, x)
    std::vector<uint32_t> b(C + 1, 0);
    b[C] = P.n_spins;
    const double total = F(n);
    for (uint32_t c = 1; c < C; c++) {
        const double t = total * c / C;
        double lo = 0, hi = n;
        for (int it = 0; it < 64; it++) {
            const double mid = 0.5 * (lo + hi);
            (F(mid) < t ? lo : hi) = mid;
        }
        b[c] = std::max(b[c - 1], std::min(P.n_spins, (uint32_t)hi));
    }
    return b;
}

// One call between its set-up and its walk: workspace laid out, parameter tables uploaded on
// the caller's stream, seeding launched on the context's seed stream.
struct Call {
    Layout L{};
    sw::DevParams P{};
    sw::DevTables Tb{};
    sw::LogfTables LT{};
    int precision = SW_PREC_FP32;          // SW_PREC_* alone
    bool dbl = false;                      // FP64 state (FP64 arithmetic or the FP64 shadow)
    uint32_t C = 1;                        // seed chunks
    std::vector<uint32_t> b;               // their spin boundaries
    uint32_t launches = 0;
};

// Waits for everything a call may have left on the context's streams (error paths).
void drain(DeviceCtx &ctx) {
    if (!ctx.logf_ready) return;           // the streams are created with the tables
    cudaStreamSynchronize(ctx.seed_st);
    cudaStreamSynchronize(ctx.walk_st);
    cudaStreamSynchronize(ctx.walk_st2);
}

// Set-up of a call and the launch of its seeding. The seeding reads nothing of the caller's
// (generators depend only on seed + spin id) and writes only the context's workspace, so it is
// not ordered after `st`: it runs while the caller's stream still produces the inputs, and while
// sw_sim copies them from the host. Every call waits for its own work before it returns, so the
// workspace is idle here.
int begin_call(DeviceCtx &ctx, const sw_params *p, const sw_sequence *q, int precision,
               bool fp64_shadow, cudaStream_t st, Call &c) {
    g_timing = sw_timing{};
    const size_t n = p->n_spins;
    const bool bf16 = (precision & SW_FIELD_BF16) != 0;
    const uint32_t rng = (uint32_t)precision & ~(uint32_t)(SW_PREC_MASK | SW_FIELD_BF16);
    precision &= SW_PREC_MASK;
    if (precision != SW_PREC_FP32 && precision != SW_PREC_FP64 && precision != SW_PREC_KAHAN)
        return fail(SW_ERR_INVALID, "precision");
    if (rng != SW_RNG_MT19937 && rng != SW_RNG_MINSTD) return fail(SW_ERR_INVALID, "generator flavour");
    int rc = ensure_logf(ctx);
    if (rc) return rc;
    c.precision = precision;
    c.dbl = precision == SW_PREC_FP64 || fp64_shadow;

    TableImage im;
    build_tables(p, q, im);
    if (!im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
    const uint32_t nlen = ring_len(current_tuning());
    Layout &L = c.L;
    L = layout(nullptr, n, p->matrix_length, im.bytes.size(), c.dbl, rng == SW_RNG_MT19937, nlen);
    if (L.bytes > ctx.ws_size) {
        if (ctx.ws) {
            SW_CUDA(cudaStreamSynchronize(st));
            cudaFree(ctx.ws);
            ctx.ws = nullptr;
            ctx.ws_size = 0;
        }
        cudaError_t e = cudaMalloc(&ctx.ws, L.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, "workspace of " + std::to_string(L.bytes >> 20) +
                                          " MiB: " + cudaGetErrorString(e));
        }
        ctx.ws_size = L.bytes;
    }
    L = layout(ctx.ws, n, p->matrix_length, im.bytes.size(), c.dbl, rng == SW_RNG_MT19937, nlen);
    // a pageable source: the copy has taken `im` by the time it returns
    SW_CUDA(cudaMemcpyAsync(L.tables, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st));

    c.P = dev_params(p, q);
    c.P.rng = rng;
    c.P.field_bf16 = bf16 ? 1 : 0;
    c.Tb = dev_tables(im, L.tables);
    c.LT = logf_tables(ctx);
    if (rng == SW_RNG_MINSTD && !(c.LT.ms_delta = minstd_delta_table())) return SW_ERR_CUDA;

    const sw_tuning tu = current_tuning();
    // 0 = 1. With the rounds as two halves, a seeded chunk's walk beside the next chunk's seeding
    // gains only where the walk is a sizeable share of the discards (SE, 1e6 spins, 2001 steps:
    // 187.3 -> 184.7 ms per call with 8 chunks, 191.0 with 12), and loses elsewhere (2e6 spins of
    // 801 steps: 495.9 -> 498.2 ms; 2e5 spins: 7.72 -> 8.81 ms; 1e5 spins, 401 steps: 3.50 ->
    // 5.78 ms with 4); callers with SE-like shapes can ask for 8.
    const uint32_t C = tu.seed_chunks ? tu.seed_chunks : 1u;
    c.C = std::min<uint32_t>(std::min<uint32_t>(C, kMaxSeedChunks), (uint32_t)n);
    c.b = seed_chunks(c.P, c.C);
    // high spin ids jump ahead instead of discarding (the previous call has finished with the
    // table: every call waits for its work before it returns)
    sw::JumpTable jt;
    if (c.P.rng == SW_RNG_MT19937) {
        const int rj = jump_table(c.P.seed, 0, c.P.n_spins, jump_min_z(tu), ctx.d_jump,
                                  ctx.jump_words, jt);
        if (rj) return rj;
    }
    cudaStream_t ss = ctx.seed_st;
    SW_CUDA(cudaEventRecord(ctx.ev[0], ss));              // the call's first GPU work
    // seeding of every chunk, each chunk bracketed by events (start, done)
    for (uint32_t k = 0; k < c.C; k++) {
        SW_CUDA(cudaEventRecord(ctx.pev[4 + 2 * k], ss));
        SW_CUDA(sw::launch_seed_range(c.P, L.G, c.b[k], c.b[k + 1], ss, &jt));
        SW_CUDA(cudaEventRecord(ctx.pev[5 + 2 * k], ss));
        c.launches++;
    }
    return SW_OK;
}

// The walk of one call: the reference's per-spin loop over time points (kernels.cu:107-232) cut
// into rounds of refill + walk, at which the generator rings are topped up.
//
// Pipeline: the spins were seeded in chunks of equal seeding cost on a low-priority stream
// (begin_call); on a high-priority stream each chunk, once seeded, is initialised and given the
// rounds that no spin can finish sooner than (ceil(steps / ring steps)), so the walk of chunk c
// runs beside the seeding of chunk c + 1 (the seed is integer-issue bound, the walk latency
// bound). Then rounds over all spins until none is active. Adds kernel times and rounds to
// g_timing.
int walk_pipeline(DeviceCtx &ctx, const sw_params *p, Call &c, const sw::Outputs &O,
                  const float *d_M0, const float *d_XYZ0) {
    cudaEvent_t *ev = ctx.ev.data();
    const sw::DevParams &P = c.P;
    const Layout &L = c.L;
    const uint32_t C = c.C;
    const std::vector<uint32_t> &b = c.b;
    uint32_t &launches = c.launches;
    const sw_tuning tu = current_tuning();
    const uint64_t steps = (uint64_t)p->n_timepoints * (uint64_t)(p->n_dummy_scan + 1);
    const uint64_t per_round = L.G.nlen / 3;      // steps a full ring lasts
    const uint64_t r0 = (steps + per_round - 1) / per_round;
    const uint64_t max_rounds = 64 + steps * (p->max_iterations + 2);
    // the rounds run as H independent halves of the spins, half h on stream ws[h] with its own
    // active counter (L.active[0] / [2])
    // 0 = auto: two halves from 2^17 spins on (SE 1e6 spins: 192.1 -> 189.0 ms per call, the
    // refill of one half overlapping the walk of the other)
    const uint32_t want = tu.round_streams ? tu.round_streams : (P.n_spins >= (1u << 17) ? 2u : 1u);
    const uint32_t H = (want == 2 && P.n_spins >= 2) ? 2u : 1u;
    const cudaStream_t ws[2] = {ctx.walk_st, ctx.walk_st2};
    const uint32_t hb[3] = {0u, H == 2 ? P.n_spins / 2 : P.n_spins, P.n_spins};
    uint32_t timed = 0;
    // one refill + (re-sort) + walk round over spins [lo, hi) of half h
    auto round = [&](uint32_t h, uint32_t lo, uint32_t hi, uint64_t r) -> int {
        cudaStream_t st = ws[h];
        const bool t = timed < kMaxTimedChunks;
        cudaEvent_t *e = ev + 4 + 3 * timed;
        if (t) SW_CUDA(cudaEventRecord(e[0], st));
        SW_CUDA(sw::launch_refill_range(P, L.G, L.S, c.LT, lo, hi, st));
        if (t) SW_CUDA(cudaEventRecord(e[1], st));
        if (tu.resort_interval && r % tu.resort_interval == 0) {
            sw::OrderState Qh = L.Q;                    // each half sorts with its own histogram
            Qh.hist = L.Q.hist + h * sw::order_hist_words();
            SW_CUDA(sw::launch_order(P, L.S, Qh, lo, hi, st));
            launches += 3;
        }
        SW_CUDA(sw::launch_walk_range(c.precision, c.dbl, P, c.Tb, L.vox, L.S, L.G, O,
                                      L.active + 2 * h, lo, hi, st,
                                      tu.resort_interval ? L.Q.order : nullptr,
                                      (int)tu.walk_block, walk_grid_cap(tu)));
        if (t) SW_CUDA(cudaEventRecord(e[2], st));
        if (t) timed++;
        launches += 2;
        return SW_OK;
    };
    if (H == 2) {                          // the second stream starts after the call's pack
        SW_CUDA(cudaEventRecord(ctx.pev[2], ws[0]));
        SW_CUDA(cudaStreamWaitEvent(ws[1], ctx.pev[2], 0));
    }
    int rc;
    // the first r0 rounds (no spin can finish sooner) of each seeded piece, without waiting
    for (uint32_t h = 0; h < H; h++)
        for (uint32_t k = 0; k < C; k++) {
            const uint32_t lo = std::max(b[k], hb[h]), hi = std::min(b[k + 1], hb[h + 1]);
            if (hi <= lo) continue;
            SW_CUDA(cudaStreamWaitEvent(ws[h], ctx.pev[5 + 2 * k], 0));
            SW_CUDA(sw::launch_init_range(P, c.Tb, L.vox, d_M0, d_XYZ0, L.S, O, c.dbl, lo, hi,
                                          ws[h]));
            launches++;
            for (uint64_t r = 0; r < r0; r++)
                if ((rc = round(h, lo, hi, r))) return rc;
        }
    uint64_t rounds = r0;
    for (;; rounds++) {
        if (rounds >= max_rounds) return fail(SW_ERR_TIMEOUT, "walk did not finish");
        for (uint32_t h = 0; h < H; h++) {
            SW_CUDA(cudaMemsetAsync(L.active + 2 * h, 0, sizeof(uint32_t), ws[h]));
            if ((rc = round(h, hb[h], hb[h + 1], rounds))) return rc;
            SW_CUDA(cudaMemcpyAsync(ctx.h_active + h, L.active + 2 * h, sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, ws[h]));
        }
        uint32_t act = 0;
        for (uint32_t h = 0; h < H; h++) {
            SW_CUDA(cudaStreamSynchronize(ws[h]));
            act += ctx.h_active[h];
        }
        if (act == 0) break;
    }
    if (H == 2) {                          // join: the call continues on the first stream
        SW_CUDA(cudaEventRecord(ctx.pev[3], ws[1]));
        SW_CUDA(cudaStreamWaitEvent(ws[0], ctx.pev[3], 0));
    }
    for (uint32_t i = 0; i < timed; i++) {
        float a = 0.f, w = 0.f;
        cudaEvent_t *e = ev + 4 + 3 * i;
        cudaEventElapsedTime(&a, e[0], e[1]);
        cudaEventElapsedTime(&w, e[1], e[2]);
        g_timing.refill_ms += a;
        g_timing.walk_ms += w;
    }
    for (uint32_t k = 0; k < C; k++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ctx.pev[4 + 2 * k], ctx.pev[5 + 2 * k]);
        g_timing.seed_ms += t;
    }
    g_timing.n_chunks += (uint32_t)(rounds + 1);
    return SW_OK;
}

// The rest of a begun call, once its inputs are (or will be, in `st`'s order) on the device:
// pack, label check, initial state and the rounds; joined back into `st`, waited for.
int finish_call(DeviceCtx &ctx, Call &c, const sw_params *p, const float *d_field,
                const uint8_t *d_mask, const float *d_M0, const float *d_XYZ0, float *d_M1,
                float *d_XYZ1, uint8_t *d_T, int32_t *d_status, double *d_M1d, cudaStream_t st) {
    const Layout &L = c.L;
    sw::Outputs O{d_M1, d_M1d, d_XYZ1, d_T, d_status};
    cudaEvent_t *ev = ctx.ev.data();
    auto bail = [&](int code) { drain(ctx); return code; };
#define SW_CUDA_B(call)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return bail(fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_))); \
    } while (0)
    // the walk streams are ordered after the caller's stream (inputs, tables)
    SW_CUDA_B(cudaEventRecord(ctx.pev[0], st));
    SW_CUDA_B(cudaStreamWaitEvent(ctx.walk_st, ctx.pev[0], 0));
    cudaStream_t ws = ctx.walk_st;
    SW_CUDA_B(cudaMemsetAsync(L.active, 0, 2 * sizeof(uint32_t), ws));
    SW_CUDA_B(sw::launch_pack(d_mask, p->fieldmap_exist ? d_field : nullptr, L.vox,
                              p->matrix_length, p->n_substrate, L.active + 1, ws,
                              c.P.field_bf16 != 0));
    c.launches++;
    SW_CUDA_B(cudaMemcpyAsync(ctx.h_active, L.active + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, ws));
    SW_CUDA_B(cudaStreamSynchronize(ws));
    if (*ctx.h_active != 0)
        return bail(fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate"));
    const int rc = walk_pipeline(ctx, p, c, O, d_M0, d_XYZ0);
    if (rc) return bail(rc);
    SW_CUDA_B(cudaEventRecord(ctx.pev[1], ws));
    SW_CUDA_B(cudaStreamWaitEvent(st, ctx.pev[1], 0));
    SW_CUDA_B(cudaEventRecord(ev[3], st));
    SW_CUDA_B(cudaEventSynchronize(ev[3]));
#undef SW_CUDA_B
    cudaEventElapsedTime(&g_timing.total_ms, ev[0], ev[3]);
    g_timing.n_launches = c.launches;
    return SW_OK;
}

int run_device(DeviceCtx &ctx, const sw_params *p, const sw_sequence *q, const float *d_field,
               const uint8_t *d_mask, const float *d_M0, const float *d_XYZ0, float *d_M1,
               float *d_XYZ1, uint8_t *d_T, int32_t *d_status, int precision, double *d_M1d,
               cudaStream_t st) {
    if (p->n_spins == 0) {
        g_timing = sw_timing{};
        return SW_OK;
    }
    Call c;
    const int rc = begin_call(ctx, p, q, precision, d_M1d != nullptr, st, c);
    if (rc) {
        drain(ctx);
        return rc;
    }
    return finish_call(ctx, c, p, d_field, d_mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T, d_status,
                       d_M1d, st);
}

DeviceCtx *current_ctx(int *dev_out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    if (dev_out) *dev_out = dev;
    return &g_ctx[dev];
}

}  // namespace

sw::LogfTables sw::api::device_logf_tables() {
    DeviceCtx *ctx = current_ctx(nullptr);
    if (!ctx) {
        fail(SW_ERR_CUDA, "no current CUDA device");
        return sw::LogfTables{nullptr, nullptr};
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ensure_logf(*ctx) != SW_OK) return sw::LogfTables{nullptr, nullptr};
    return logf_tables(*ctx);
}

namespace {
std::mutex g_tune_mu;
sw_tuning g_tune{0u, 256u, 0u, 0u, 0u, 0u, 0u, {0u}};
}  // namespace

int sw::api::walk_grid_cap(const sw_tuning &t) {
    if (!t.walk_blocks_per_sm) return 0;
    static int sms = [] {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return 152;
        }
        return n;
    }();
    return (int)t.walk_blocks_per_sm * sms;
}

int sw::api::jump_table(uint64_t seed, uint32_t lo, uint32_t hi, uint64_t z_min, uint32_t *&buf,
                        size_t &buf_words, sw::JumpTable &jt) {
    jt = sw::JumpTable{};
    const uint64_t c = std::max<uint64_t>(lo, seed >= z_min ? 0 : z_min - seed);
    if (c >= hi) return SW_OK;                      // every spin discards
    const uint64_t R_lo = sw::mt_regenerations(seed + c), R_hi = sw::mt_regenerations(seed + hi - 1) + 1;
    const size_t words = (size_t)(R_hi - R_lo) * sw::kJumpPolyWords;
    std::vector<uint32_t> host(words);
    try {
        sw::mt_jump_polys(R_lo, (uint32_t)(R_hi - R_lo), host.data());
    } catch (const std::exception &e) {
        return fail(SW_ERR_INVALID, std::string("jump polynomials: ") + e.what());
    }
    if (words > buf_words) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        buf_words = 0;
        cudaError_t e = cudaMalloc(&buf, words * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, std::string("jump polynomials: ") + cudaGetErrorString(e));
        }
        buf_words = words;
    }
    cudaError_t e = cudaMemcpy(buf, host.data(), words * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SW_ERR_CUDA, std::string("jump polynomials: ") + cudaGetErrorString(e));
    }
    jt.polys = buf;
    jt.R_lo = R_lo;
    jt.R_hi = R_hi;
    jt.z_min = z_min;
    return SW_OK;
}

sw_tuning sw::api::current_tuning() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune;
}

extern "C" {

int sw_set_tuning(const sw_tuning *t) {
    if (!t) return fail(SW_ERR_INVALID, "null tuning");
    if (t->walk_block != 64 && t->walk_block != 128 && t->walk_block != 256)
        return fail(SW_ERR_INVALID, "walk_block must be 64, 128 or 256");
    if (t->resort_interval > 1u << 20) return fail(SW_ERR_INVALID, "resort_interval too large");
    if (t->seed_chunks > kMaxSeedChunks) return fail(SW_ERR_INVALID, "seed_chunks > 64");
    if (t->round_streams > 2) return fail(SW_ERR_INVALID, "round_streams must be 0, 1 or 2");
    if (t->walk_blocks_per_sm > 16) return fail(SW_ERR_INVALID, "walk_blocks_per_sm must be 0 .. 16");
    if (t->ring_steps != 0 && (t->ring_steps < 32 || t->ring_steps > 4096))
        return fail(SW_ERR_INVALID, "ring_steps must be 0 (default) or 32 .. 4096");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune = *t;
    return SW_OK;
}

int sw_get_tuning(sw_tuning *t) {
    if (!t) return fail(SW_ERR_INVALID, "null tuning");
    *t = current_tuning();
    return SW_OK;
}

int sw_abi_version(void) { return SW_ABI_VERSION; }

const char *sw_last_error(void) { return g_err.c_str(); }

int sw_device_count(int *count) {
    if (!count) return SW_ERR_INVALID;
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        cudaGetLastError();
        return fail(SW_ERR_CUDA, cudaGetErrorString(e));
    }
    return SW_OK;
}

int sw_release_workspaces(void) {
    int dev = 0;
    DeviceCtx *ctx = current_ctx(&dev);
    if (!ctx) return fail(SW_ERR_CUDA, "no current CUDA device");
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (ctx->ws) cudaFree(ctx->ws);
        if (ctx->io) cudaFree(ctx->io);
        if (ctx->d_jump) cudaFree(ctx->d_jump);
        ctx->ws = ctx->io = nullptr;
        ctx->d_jump = nullptr;
        ctx->ws_size = ctx->io_size = ctx->jump_words = 0;
    }
    release_pool_memory(dev);
    release_call_engine(dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SW_ERR_CUDA, std::string("release: ") + cudaGetErrorString(e));
    return SW_OK;
}

int sw_sync(void *stream) {
    SW_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return SW_OK;
}

int sw_last_timing(sw_timing *out) {
    if (!out) return SW_ERR_INVALID;
    *out = g_timing;
    return SW_OK;
}

int sw_sim_device(const sw_params *param, const sw_sequence *seq, const float *d_FieldMap,
                  const uint8_t *d_Mask, const float *d_M0, const float *d_XYZ0, float *d_M1,
                  float *d_XYZ1, uint8_t *d_T, int32_t *d_status, int precision,
                  double *d_M1_fp64, void *stream) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    if (param->n_spins && (!d_Mask || !d_M0 || !d_XYZ0 || !d_XYZ1 || (seq->n_TE && (!d_M1 || !d_T))))
        return fail(SW_ERR_INVALID, "null device buffer");
    DeviceCtx *ctx = current_ctx(nullptr);
    if (!ctx) return fail(SW_ERR_CUDA, "no current CUDA device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return run_device(*ctx, param, seq, d_FieldMap, d_Mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T,
                      d_status, precision, d_M1_fp64, (cudaStream_t)stream);
}

int sw_sim(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
           const uint8_t *pMask, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
           uint8_t *T, int32_t *status, int precision, double *M1_fp64) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    const size_t n = param->n_spins;
    if (n == 0) return SW_OK;
    if (!pMask || !M0 || !XYZ0 || !XYZ1 || (seq->n_TE && (!M1 || !T)))
        return fail(SW_ERR_INVALID, "null host buffer");
    const size_t ml = (size_t)param->matrix_length, nte = seq->n_TE;
    const size_t trj = param->enRecordTrajectory
                           ? (size_t)(param->n_dummy_scan + 1) * param->n_timepoints : 1;
    const bool has_field = param->fieldmap_exist && pFieldMap;
    // one device allocation for all user-visible buffers
    size_t off = 0;
    auto slot = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~size_t(255); return o; };
    const size_t o_mask = slot(ml), o_field = slot(has_field ? ml * 4 : 0), o_M0 = slot(n * 12),
                 o_XYZ0 = slot(n * 12), o_M1 = slot(n * nte * 12), o_XYZ1 = slot(n * trj * 12),
                 o_T = slot(n * nte), o_st = slot(status ? n * 4 : 0),
                 o_M1d = slot(M1_fp64 ? n * nte * 24 : 0);
    DeviceCtx *ctx = current_ctx(nullptr);
    if (!ctx) return fail(SW_ERR_CUDA, "no current CUDA device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    // the device copies of the caller's buffers live in the context's I/O region, grown on
    // demand and kept for the next call like the workspace
    if (off + 256 > ctx->io_size) {
        if (ctx->io) cudaFree(ctx->io);
        ctx->io = nullptr;
        ctx->io_size = 0;
        cudaError_t e = cudaMalloc(&ctx->io, off + 256);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, std::string("buffers: ") + cudaGetErrorString(e));
        }
        ctx->io_size = off + 256;
    }
    char *d = ctx->io;
    cudaStream_t st = nullptr;
    // the seeding starts first: it needs none of the inputs, so the host-to-device copies below
    // (the phantom above all) run while the GPU seeds
    Call c;
    bool begun = false;
    auto done = [&](int code) {
        if (begun) drain(*ctx);
        return code;
    };
#define SW_TRY(call)                                                                       \
    do {                                                                                   \
        cudaError_t e2 = (call);                                                           \
        if (e2 != cudaSuccess)                                                             \
            return done(fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e2))); \
    } while (0)
    begun = true;                          // from here an error return waits for the GPU
    if (int rc0 = begin_call(*ctx, param, seq, precision, M1_fp64 != nullptr, st, c))
        return done(rc0);
    SW_TRY(cudaMemcpyAsync(d + o_mask, pMask, ml, cudaMemcpyHostToDevice, st));
    if (has_field) SW_TRY(cudaMemcpyAsync(d + o_field, pFieldMap, ml * 4, cudaMemcpyHostToDevice, st));
    SW_TRY(cudaMemcpyAsync(d + o_M0, M0, n * 12, cudaMemcpyHostToDevice, st));
    SW_TRY(cudaMemcpyAsync(d + o_XYZ0, XYZ0, n * 12, cudaMemcpyHostToDevice, st));
    // outputs start from the caller's contents: slots the walk never reaches keep them, as in
    // the reference (whose GPU path uploads M1/XYZ1/T too, monte_carlo.cu:256-260)
    if (nte) {
        SW_TRY(cudaMemcpyAsync(d + o_M1, M1, n * nte * 12, cudaMemcpyHostToDevice, st));
        SW_TRY(cudaMemcpyAsync(d + o_T, T, n * nte, cudaMemcpyHostToDevice, st));
    }
    SW_TRY(cudaMemcpyAsync(d + o_XYZ1, XYZ1, n * trj * 12, cudaMemcpyHostToDevice, st));
    if (M1_fp64) SW_TRY(cudaMemcpyAsync(d + o_M1d, M1_fp64, n * nte * 24, cudaMemcpyHostToDevice, st));
    {
        const int rc2 = finish_call(*ctx, c, param, has_field ? (float *)(d + o_field) : nullptr,
                                    (uint8_t *)(d + o_mask), (float *)(d + o_M0),
                                    (float *)(d + o_XYZ0), (float *)(d + o_M1),
                                    (float *)(d + o_XYZ1), (uint8_t *)(d + o_T),
                                    status ? (int32_t *)(d + o_st) : nullptr,
                                    M1_fp64 ? (double *)(d + o_M1d) : nullptr, st);
        begun = false;                     // finish_call drained on its own errors
        if (rc2) return done(rc2);
    }
    if (nte) {
        SW_TRY(cudaMemcpyAsync(M1, d + o_M1, n * nte * 12, cudaMemcpyDeviceToHost, st));
        SW_TRY(cudaMemcpyAsync(T, d + o_T, n * nte, cudaMemcpyDeviceToHost, st));
    }
    SW_TRY(cudaMemcpyAsync(XYZ1, d + o_XYZ1, n * trj * 12, cudaMemcpyDeviceToHost, st));
    if (status) SW_TRY(cudaMemcpyAsync(status, d + o_st, n * 4, cudaMemcpyDeviceToHost, st));
    if (M1_fp64) SW_TRY(cudaMemcpyAsync(M1_fp64, d + o_M1d, n * nte * 24, cudaMemcpyDeviceToHost, st));
    SW_TRY(cudaStreamSynchronize(st));
#undef SW_TRY
    return done(SW_OK);
}

int sw_debug_dadd(const double *d_a, const double *d_b, double *d_y, uint64_t n, void *stream) {
    if (!d_a || !d_b || !d_y) return fail(SW_ERR_INVALID, "null device buffer");
    SW_CUDA(sw::launch_debug_dadd(d_a, d_b, d_y, n, (cudaStream_t)stream));
    return SW_OK;
}

int sw_debug_d2f(const double *d_x, float *d_y, uint64_t n, void *stream) {
    if (!d_x || !d_y) return fail(SW_ERR_INVALID, "null device buffer");
    SW_CUDA(sw::launch_debug_d2f(d_x, d_y, n, (cudaStream_t)stream));
    return SW_OK;
}

int sw_debug_ms_normal(uint32_t x_lo, uint32_t n, float *d_y, void *stream) {
    if (!d_y) return fail(SW_ERR_INVALID, "null device buffer");
    const uint32_t *delta = minstd_delta_table();
    if (!delta) return SW_ERR_CUDA;
    SW_CUDA(sw::launch_debug_ms_normal(x_lo, n, d_y, delta, (cudaStream_t)stream));
    return SW_OK;
}

int sw_debug_logf(const float *d_x, float *d_y, uint64_t n, void *stream) {
    DeviceCtx *ctx = current_ctx(nullptr);
    if (!ctx) return fail(SW_ERR_CUDA, "no current CUDA device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    int rc = ensure_logf(*ctx);
    if (rc) return rc;
    SW_CUDA(sw::launch_debug_logf(d_x, d_y, n, logf_tables(*ctx), (cudaStream_t)stream));
    return SW_OK;
}

}  // extern "C"
