// sw_autotune: picks the walk tuning (Morton re-sort interval, walk block size, steps per
// refill/walk round) for a problem by timing its refill and walk kernels on the device under each
// candidate.
//
// The probe walks the problem's own phantom, spins and start positions, so the spin density per
// voxel and cache line -- what decides whether sorted warps share gathers -- is the real one.
// Only the generator flavour differs (SW_RNG_MINSTD: O(log) seeding per spin instead of the
// sum over spins of seed + spin mt19937 words); the walk kernel and its ring buffers are the same.
// Schedule (one stream, CUDA events around every kernel of interest):
//   rings of 256 steps: warm-up round; then per block size: kProbeUnsorted rounds in id order,
//   one re-sort, then kProbeAges rounds in that order (ages 0 .. kProbeAges-1 after the sort);
//   then for every other ring length: seeding and start again, a warm-up round and
//   kProbeUnsorted rounds in id order at block 256.
// A candidate's cost is device time per 256 walk steps: (refill + walk) of a round scaled by
// 256 / its ring's steps; a re-sort interval I adds its sort: (sort + sum_{a < I} round(age a)) / I,
// ages beyond the probe taking the last measured age.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"
#include "sw_kernels.h"

using namespace sw::api;

namespace {

constexpr uint32_t kProbeUnsorted = 2;
constexpr uint32_t kProbeAges = 8;
constexpr uint32_t kIntervals[] = {1, 2, 4, 8};
constexpr uint32_t kBlocks[] = {256, 128};
constexpr uint32_t kRingSteps[] = {128, 512};     // besides the default 256
constexpr uint32_t kMaxRingSteps = 512;

struct DevMem {
    char *p = nullptr;
    ~DevMem() {
        if (p) cudaFree(p);
    }
};
struct Stream {
    cudaStream_t s = nullptr;
    std::vector<cudaEvent_t> ev;
    ~Stream() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace

extern "C" int sw_autotune(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                           const uint8_t *pMask, const float *XYZ0, int apply, sw_tuning *best,
                           sw_tune_entry *table, uint32_t table_len, uint32_t *n_entries) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    if (!best) return fail(SW_ERR_INVALID, "null best");
    if (n_entries) *n_entries = 0;
    *best = current_tuning();
    const size_t n = param->n_spins, ml = (size_t)param->matrix_length;
    if (n == 0) return SW_OK;
    if (!pMask || !XYZ0) return fail(SW_ERR_INVALID, "null host buffer");
    const bool has_field = param->fieldmap_exist && pFieldMap;

    TableImage im;
    build_tables(param, seq, im);
    if (!im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
    const size_t n_keys = (size_t)std::max<uint32_t>(1, seq->n_TE) * param->n_substrate;
    size_t off = 0;
    auto slot = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) & ~size_t(255);
        return o;
    };
    const Layout Lm = layout(nullptr, n, param->matrix_length, im.bytes.size(), false, false,
                             3 * kMaxRingSteps);
    const size_t o_ws = slot(Lm.bytes), o_mask = slot(ml), o_field = slot(has_field ? ml * 4 : 0),
                 o_xyz = slot(n * 12), o_m0 = slot(n * 12), o_sig = slot(n_keys * 32);
    const size_t total = off;

    const sw::LogfTables LT0 = device_logf_tables();
    if (!LT0.bitmap) return SW_ERR_CUDA;
    sw::LogfTables LT = LT0;
    if (!(LT.ms_delta = minstd_delta_table())) return SW_ERR_CUDA;

#define TU_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
        }                                                                                  \
    } while (0)
    DevMem mem;
    {
        cudaError_t e = cudaMalloc(&mem.p, total);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, "autotune probe of " + std::to_string(total >> 20) +
                                          " MiB: " + cudaGetErrorString(e));
        }
    }
    Stream S;
    TU_CUDA(cudaStreamCreateWithFlags(&S.s, cudaStreamNonBlocking));
    const uint32_t n_ev = 4 * (1 + 2 * (kProbeUnsorted + kProbeAges) +
                               2 * (1 + kProbeUnsorted));
    S.ev.resize(n_ev, nullptr);
    for (auto &e : S.ev) TU_CUDA(cudaEventCreate(&e));
    cudaStream_t st = S.s;
    char *d = mem.p;
    Layout L = layout(d + o_ws, n, param->matrix_length, im.bytes.size(), false, false);
    TU_CUDA(cudaMemcpyAsync(d + o_mask, pMask, ml, cudaMemcpyHostToDevice, st));
    if (has_field) TU_CUDA(cudaMemcpyAsync(d + o_field, pFieldMap, ml * 4, cudaMemcpyHostToDevice, st));
    TU_CUDA(cudaMemcpyAsync(d + o_xyz, XYZ0, n * 12, cudaMemcpyHostToDevice, st));
    TU_CUDA(cudaMemsetAsync(d + o_m0, 0, n * 12, st));
    TU_CUDA(cudaMemsetAsync(d + o_sig, 0, n_keys * 32, st));
    TU_CUDA(cudaMemcpyAsync(L.tables, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st));

    sw::DevParams P = dev_params(param, seq);
    P.rng = SW_RNG_MINSTD;
    P.n_dummy_scan = 0;
    P.record_traj = 0;
    P.traj_len = 1;
    const uint32_t probe_rounds = 1 + 2 * (kProbeUnsorted + kProbeAges);
    P.n_timepoints = std::max<uint32_t>(P.n_timepoints, (probe_rounds + 2) * kMaxRingSteps);
    const sw::DevTables Tb = dev_tables(im, L.tables);
    sw::Outputs O{nullptr, nullptr, nullptr, nullptr, nullptr};
    O.sig = reinterpret_cast<double *>(d + o_sig);
    O.cnt = reinterpret_cast<unsigned long long *>(d + o_sig + n_keys * 24);

    // seeding and start of every spin with rings of nlen deviates (the layout for that length)
    auto start = [&](uint32_t nlen) -> int {
        L = layout(d + o_ws, n, param->matrix_length, im.bytes.size(), false, false, nlen);
        TU_CUDA(cudaMemsetAsync(L.active, 0, 2 * sizeof(uint32_t), st));
        TU_CUDA(sw::launch_seed(P, L.G, st));
        TU_CUDA(sw::launch_init(P, Tb, L.vox, reinterpret_cast<const float *>(d + o_m0),
                                reinterpret_cast<const float *>(d + o_xyz), L.S, O, false, st));
        return SW_OK;
    };
    TU_CUDA(cudaMemsetAsync(L.active, 0, 2 * sizeof(uint32_t), st));
    TU_CUDA(sw::launch_pack(reinterpret_cast<const uint8_t *>(d + o_mask),
                            has_field ? reinterpret_cast<const float *>(d + o_field) : nullptr,
                            L.vox, param->matrix_length, param->n_substrate, L.active + 1, st));
    uint32_t bad = 0;
    TU_CUDA(cudaMemcpyAsync(&bad, L.active + 1, 4, cudaMemcpyDeviceToHost, st));
    TU_CUDA(cudaStreamSynchronize(st));
    if (bad) return fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate");
    if ((rc = start(sw::kNormBuf))) return rc;

    // one round: refill, optional re-sort, walk; events er (before the refill), e0 (before the
    // sort), e1 (after it), e2 (after the walk)
    uint32_t evi = 0;
    struct RoundEv { uint32_t er, e0, e1, e2; };
    auto round = [&](bool sort, const uint32_t *order, int block, RoundEv &r) -> int {
        r = RoundEv{evi, evi + 1, evi + 2, evi + 3};
        evi += 4;
        TU_CUDA(cudaEventRecord(S.ev[r.er], st));
        TU_CUDA(sw::launch_refill(P, L.G, L.S, LT, st));
        TU_CUDA(cudaEventRecord(S.ev[r.e0], st));
        if (sort) TU_CUDA(sw::launch_order(P, L.S, L.Q, 0, P.n_spins, st));
        TU_CUDA(cudaEventRecord(S.ev[r.e1], st));
        TU_CUDA(sw::launch_walk_range(SW_PREC_FP32, false, P, Tb, L.vox, L.S, L.G, O, L.active, 0,
                                      P.n_spins, st, order, block));
        TU_CUDA(cudaEventRecord(S.ev[r.e2], st));
        return SW_OK;
    };
    RoundEv warm{};
    if ((rc = round(false, nullptr, 256, warm))) return rc;
    std::vector<RoundEv> unsorted[2], aged[2];
    for (int b = 0; b < 2; b++) {
        unsorted[b].resize(kProbeUnsorted);
        aged[b].resize(kProbeAges);
        for (uint32_t k = 0; k < kProbeUnsorted; k++)
            if ((rc = round(false, nullptr, (int)kBlocks[b], unsorted[b][k]))) return rc;
        for (uint32_t a = 0; a < kProbeAges; a++)
            if ((rc = round(a == 0, L.Q.order, (int)kBlocks[b], aged[b][a]))) return rc;
    }
    std::vector<RoundEv> ring_runs[2];
    for (int q = 0; q < 2; q++) {
        if ((rc = start(3 * kRingSteps[q]))) return rc;
        ring_runs[q].resize(kProbeUnsorted);
        if ((rc = round(false, nullptr, 256, warm))) return rc;
        for (uint32_t k = 0; k < kProbeUnsorted; k++)
            if ((rc = round(false, nullptr, 256, ring_runs[q][k]))) return rc;
    }
    TU_CUDA(cudaStreamSynchronize(st));
    auto ms = [&](uint32_t a, uint32_t b) {
        float t = 0.f;
        cudaEventElapsedTime(&t, S.ev[a], S.ev[b]);
        return t;
    };
    // refill + walk of a round (the sort excluded)
    auto round_ms = [&](const RoundEv &r) { return ms(r.er, r.e0) + ms(r.e1, r.e2); };
    const uint32_t def_steps = sw::kNormBuf / 3;
    std::vector<sw_tune_entry> cand;
    for (int b = 0; b < 2; b++) {
        float u = 0.f;
        for (const RoundEv &r : unsorted[b]) u += round_ms(r);
        cand.push_back(sw_tune_entry{0u, kBlocks[b], u / kProbeUnsorted, 0.f, def_steps});
        const float sort_ms = ms(aged[b][0].e0, aged[b][0].e1);
        for (uint32_t I : kIntervals) {
            float t = sort_ms;
            for (uint32_t a = 0; a < I; a++) t += round_ms(aged[b][std::min(a, kProbeAges - 1)]);
            cand.push_back(sw_tune_entry{I, kBlocks[b], t / (float)I, sort_ms, def_steps});
        }
    }
    for (int q = 0; q < 2; q++) {
        float u = 0.f;
        for (const RoundEv &r : ring_runs[q]) u += round_ms(r);
        const float per_def_round = u / kProbeUnsorted * (float)def_steps / (float)kRingSteps[q];
        cand.push_back(sw_tune_entry{0u, 256u, per_def_round, 0.f, kRingSteps[q]});
    }
#undef TU_CUDA
    size_t bi = 0;
    for (size_t i = 1; i < cand.size(); i++)
        if (cand[i].ms_per_round < cand[bi].ms_per_round) bi = i;
    sw_tuning t = current_tuning();
    t.resort_interval = cand[bi].resort_interval;
    t.walk_block = cand[bi].walk_block;
    t.ring_steps = cand[bi].ring_steps;
    *best = t;
    if (table)
        for (uint32_t i = 0; i < std::min<size_t>(table_len, cand.size()); i++) table[i] = cand[i];
    if (n_entries) *n_entries = (uint32_t)cand.size();
    if (apply) return sw_set_tuning(&t);
    return SW_OK;
}
