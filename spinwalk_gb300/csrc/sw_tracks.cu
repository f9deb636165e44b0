// sw_sim_tracks: one walk, many Bloch tracks.
//
// The reference re-runs the complete walk for every scale of a config (src/sim/monte_carlo.cu:
// 273-337) even when only the RF phase changes (phase-cycling scales) and for every DUMMY_SCAN
// setting. The trajectory (positions, voxels, substrates, rejected moves) depends only on the
// seeds, XYZ0, the phantom and the tissue tables -- not on RF phases, flip angles or the number
// of scans (the forced voxel reload at a scan start never draws a uniform: the spin is still in a
// voxel of its own substrate). So every such instance ("track") can ride on ONE walk.
//
// Tracks are grouped by RF configuration (scan-start phase cycling, per-pulse flip angles and
// phases). Per spin and group only the magnetisation m_g is stored; the walk kernel logs the Bloch
// events of each spin and a second kernel applies them with one thread per (group, spin). Within a scan, all groups
// share the accumulated phase (`acc`) and its event times, because dephasing, gradients and the
// RF/echo times are common. A track = (group, recording scan d): before scan d it is m_g; in
// scan d it records echoes; from its first echo on, its magnetisation (m_rec) and phase
// (acc_rec, reset at each echo) diverge from the group's -- one extra state per group in a
// recording scan. A track ends with its recording scan. Every float operation is the one the
// plain kernel performs for that instance, so each track is bit-identical to sw_sim on it.
//
// Gradient scales (the reference's gradient scale loop) change the phase, not the trajectory:
// tracks with distinct scales fall into gradient classes, and k_walk_cls keeps the phase sums
// per class (each event logs one pair of relaxation operators per class). The rounds run as two
// halves of the spins on two streams, so one half's refill and Bloch update overlap the other
// half's walk.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"
#include "sw_device.cuh"
#include "sw_host.h"
#include "sw_kernels.h"

namespace sw {

struct GroupTables {
    uint32_t n_groups, n_tracks, max_ds, n_rf;
    const RfOp *scan_rf;      // [n_groups][max_ds + 1]
    const RfOp *rf;           // [n_groups][n_rf]
    const int32_t *rec;       // [n_groups][max_ds + 1]: track recording in that scan, or -1
    const uint32_t *last_ds;  // [n_groups]
    const uint32_t *rec_any;  // [max_ds + 1]: some track records in that scan
    const int32_t *track_nd;  // [n_tracks]
    float *const *M1;         // [n_tracks] -> [n][n_TE][3]
    double *const *M1d;       // [n_tracks] -> [n][n_TE][3] FP64 shadow, entries may be null
    // gradient classes (tracks with distinct gradient scales): each keeps its own phase sums
    uint32_t n_cls;           // 1: one shared phase (the kernels without classes)
    const uint32_t *cls;      // [n_groups]: the group's class
    const float *gscale;      // [n_cls]: the class's gradient scale
    float *const *XYZ1;       // [n_tracks] -> [n][3]
    uint8_t *const *T;        // [n_tracks] -> [n][n_TE]
    int32_t *const *status;   // [n_tracks] -> [n]
};

struct GroupState {
    float *mg;                // [3][n_groups][n]
    float *mr;                // [3][n_groups][n]
    float *acc_rec;           // [n]
    float *acc_rec_e;         // [n] compensation term of acc_rec (Kahan)
    uint32_t *tp_old_rec;     // [n]
    uint32_t *rec_started;    // [n]
    double *mg64, *mr64;      // FP64 shadow of mg / mr, or null
    double *accd_rec;         // [n] FP64 shadow of acc_rec
    float *acc_c, *acc_rec_c; // [n_cls][n]: acc and acc_rec per gradient class
};

// dephase_relax_f split in two: the trigonometry and exponentials depend only on the shared
// phase, substrate and interval, so they are computed once and applied to every group.
struct RelaxOp {
    float s, c, e1, e2;
    bool relax;
};
__device__ __forceinline__ RelaxOp make_relax(float phase, float T1, float T2, float dt_s) {
    RelaxOp r;
    const float ang = (float)((double)phase * kDeg2Rad);
    sincosf(ang, &r.s, &r.c);
    r.relax = T1 >= 0 && T2 >= 0;
    r.e1 = r.relax ? (float)exp((double)(-dt_s / T1)) : 0.f;
    r.e2 = r.relax ? (float)exp((double)(-dt_s / T2)) : 0.f;
    return r;
}
__device__ __forceinline__ void apply_relax(const RelaxOp &r, const float *a, float *b) {
    zrot_f(r.s, r.c, a, b);
    if (r.relax) {
        b[0] = b[0] * r.e2;
        b[1] = b[1] * r.e2;
        b[2] = (float)(1. + (double)r.e1 * ((double)b[2] - 1.));
    }
}

// The same split of dephase_relax_d (the FP64 shadow): operands and operation order as there.
struct RelaxOpD {
    double s, c, e1, e2;
};
__device__ __forceinline__ RelaxOpD make_relax_d(double phase, double T1, double T2, double dt_s,
                                                 bool &relax) {
    RelaxOpD r;
    sincos(phase * kDeg2Rad, &r.s, &r.c);
    relax = T1 >= 0 && T2 >= 0;
    r.e1 = relax ? exp(-dt_s / T1) : 0.;
    r.e2 = relax ? exp(-dt_s / T2) : 0.;
    return r;
}
__device__ __forceinline__ void apply_relax_d(const double *r, bool relax, const double *a,
                                              double *b) {
    zrot_d(r[0], r[1], a, b);
    if (relax) {
        b[0] *= r[3];
        b[1] *= r[3];
        b[2] = 1. + r[2] * (b[2] - 1.);
    }
}

__device__ __forceinline__ void load_m(const float *base, size_t plane, size_t idx, float *m) {
    m[0] = base[idx];
    m[1] = base[plane + idx];
    m[2] = base[2 * plane + idx];
}
__device__ __forceinline__ void store_m(float *base, size_t plane, size_t idx, const float *m) {
    base[idx] = m[0];
    base[plane + idx] = m[1];
    base[2 * plane + idx] = m[2];
}
__device__ __forceinline__ void load_md(const double *base, size_t plane, size_t idx, double *m) {
    m[0] = base[idx];
    m[1] = base[plane + idx];
    m[2] = base[2 * plane + idx];
}
__device__ __forceinline__ void store_md(double *base, size_t plane, size_t idx, const double *m) {
    base[idx] = m[0];
    base[plane + idx] = m[1];
    base[2 * plane + idx] = m[2];
}

__global__ void k_groups_init(DevParams P, GroupTables GT, GroupState GS, const SpinState S,
                              const float *__restrict__ M0, const float *__restrict__ XYZ0) {
    const uint32_t spin = blockIdx.x * blockDim.x + threadIdx.x;
    if (spin >= P.n_spins) return;
    const size_t n = P.n_spins, plane = (size_t)GT.n_groups * n;
    const float m[3] = {M0[3 * (size_t)spin], M0[3 * (size_t)spin + 1], M0[3 * (size_t)spin + 2]};
    for (uint32_t g = 0; g < GT.n_groups; g++) store_m(GS.mg, plane, (size_t)g * n + spin, m);
    if (GS.mg64) {
        const double md[3] = {m[0], m[1], m[2]};
        for (uint32_t g = 0; g < GT.n_groups; g++) store_md(GS.mg64, plane, (size_t)g * n + spin, md);
        GS.accd_rec[spin] = 0.;
    }
    GS.acc_rec[spin] = 0.f;
    GS.acc_rec_e[spin] = 0.f;
    GS.tp_old_rec[spin] = 0;
    GS.rec_started[spin] = 0;
    // a start outside the phantom ends every track at once (status set by k_init)
    const uint32_t fl = S.flags[spin];
    if (fl & kFlagDone) {
        for (uint32_t t = 0; t < GT.n_tracks; t++) {
            float *x = GT.XYZ1[t] + 3 * (size_t)spin;
            x[0] = XYZ0[3 * (size_t)spin];
            x[1] = XYZ0[3 * (size_t)spin + 1];
            x[2] = XYZ0[3 * (size_t)spin + 2];
            if (GT.status[t]) GT.status[t][spin] = (int32_t)((fl >> 16) & 0xffu);
        }
    }
}

// ---- per-spin Bloch event log ----------------------------------------------------------------
// The walk kernel records, per spin and round, what the Bloch part has to do (scan starts, RF
// pulses, echoes, scan ends) together with the shared trigonometry/relaxation factors; the Bloch
// kernel then applies the log with one thread per (group, spin), so the per-group work is
// coalesced and never diverges with the spins' individual progress.
enum : uint32_t { kEvScanStart = 1, kEvRf = 2, kEvTe = 3, kEvScanEnd = 4 };
constexpr uint32_t kLogCap = 8;           // events per spin per round

// The log is kept slot-major: every field is an array [slot][spin] (spin fastest; [slot][2][spin]
// for the FP64 pairs, [slot][class][spin] for the class operators), so the walk's writes of
// slot k and the Bloch kernel's reads of slot k by 32 consecutive spins are 512-byte coalesced
// accesses, and a field an event does not use is never read.
struct EventLog {
    uint4 *head;              // x: type | idx << 8 | ts_old << 24 (idx: ds, pulse or echo index),
                              // y: scan, z: flags (bit0 r.relax, bit1 rr.relax, bit2 echo phase
                              // already started)
    float4 *r;                // s, c, e1, e2 of the shared phase
    float4 *rr;               // the same for the recording tracks' phase (after their 1st echo)
    float4 *xo;               // scan end: position
    double2 *r64, *rr64;      // FP64 shadow of r / rr: (s, c), (e1, e2)
    float4 *rc, *rrc;         // r / rr per gradient class
    size_t n;                 // spins (the stride of a slot)

    __device__ __forceinline__ size_t at(uint32_t k, uint32_t spin) const {
        return (size_t)k * n + spin;
    }
    __device__ __forceinline__ void put_head(uint32_t k, uint32_t spin, uint32_t h, uint32_t ds,
                                             uint32_t flags) const {
        head[at(k, spin)] = make_uint4(h, ds, flags, 0u);
    }
};

__device__ __forceinline__ float4 relax4(const RelaxOp &r) { return make_float4(r.s, r.c, r.e1, r.e2); }
__device__ __forceinline__ RelaxOp get_relax(const float4 v, bool relax) {
    RelaxOp r;
    r.s = v.x; r.c = v.y; r.e1 = v.z; r.e2 = v.w;
    r.relax = relax;
    return r;
}
// FP64 operator pair of slot k: a[(2k) n + spin] = (s, c), a[(2k+1) n + spin] = (e1, e2)
__device__ __forceinline__ void put_relax64(double2 *a, const EventLog &L, uint32_t k,
                                            uint32_t spin, const double *o) {
    a[(size_t)(2 * k) * L.n + spin] = make_double2(o[0], o[1]);
    a[(size_t)(2 * k + 1) * L.n + spin] = make_double2(o[2], o[3]);
}
__device__ __forceinline__ void get_relax64(const double2 *a, const EventLog &L, uint32_t k,
                                            uint32_t spin, double *o) {
    const double2 p = a[(size_t)(2 * k) * L.n + spin], q = a[(size_t)(2 * k + 1) * L.n + spin];
    o[0] = p.x; o[1] = p.y; o[2] = q.x; o[3] = q.y;
}

// KAHAN: compensated float phase sums (acc, acc_rec), as the plain kernel's SW_PREC_KAHAN.
// SHADOW: FP64 phase sums beside them and FP64 relaxation operators in log64, as the plain
// kernel's FP64 shadow (DBL) computes them.
template <bool KAHAN, bool SHADOW>
__device__ __forceinline__ bool walk_logged_spin(const uint32_t spin, uint32_t flags,
                                                 const DevParams &P, const DevTables &Tb,
                                                 const GroupTables &GT, const GroupState &GS,
                                                 const uint2 *__restrict__ vox,
                                                 const SpinState &S, const RngState &G,
                                                 uint32_t *log_count, const EventLog &L) {
    WalkRegs w;
    w.xo[0] = S.x[spin]; w.xo[1] = S.y[spin]; w.xo[2] = S.z[spin];
    w.ind_old = S.ind_old[spin];
    w.ts_old = flags & 0xffu;
    w.field = S.field[spin];
    w.dscale = __ldg(Tb.dscale + w.ts_old);
    w.itr = S.itr[spin];
    w.nh = G.nhead[spin]; w.nc = G.ncnt[spin]; w.uh = G.uhead[spin]; w.uc = G.ucnt[spin];
    const float *nb = G.nbuf + (size_t)spin * kNormBuf;
    const float *ub = G.ubuf + (size_t)spin * kUnifBuf;
    uint32_t ne = 0;

    float acc = S.acc[spin], acc_rec = GS.acc_rec[spin];
    float acc_e = KAHAN ? S.acc_e[spin] : 0.f, acc_rec_e = KAHAN ? GS.acc_rec_e[spin] : 0.f;
    double accd = SHADOW ? S.accd[spin] : 0., accd_rec = SHADOW ? GS.accd_rec[spin] : 0.;
    uint32_t tp = S.tp[spin], tp_old = S.tp_old[spin], tp_old_rec = GS.tp_old_rec[spin];
    uint32_t ds = S.ds[spin];
    bool rec_started = GS.rec_started[spin] != 0;
    uint32_t ctr = S.ctr[spin], ctr2 = S.ctr2[spin];
    uint32_t c_rf = ctr & 0xffffu, c_te = ctr >> 16, c_dph = ctr2 & 0xffffu, c_grad = ctr2 >> 16;
    bool started = (flags & kFlagStarted) != 0;

    auto fadd = [&](float &s_, float &e_, float x) {
        if (KAHAN) kahan_add(s_, e_, x); else s_ += x;
    };
    // relaxation operator of a phase sum over (tp - t0) time points, float and FP64
    auto relax_f = [&](float a, float e, uint32_t t0) {
        const float te = (float)((double)((tp - t0) * (uint32_t)P.timestep_us) * 1e-6);
        return make_relax(KAHAN ? a + e : a, __ldg(Tb.T1f + w.ts_old), __ldg(Tb.T2f + w.ts_old), te);
    };
    auto relax_d = [&](double a, uint32_t t0, double *dst, bool &relax) {
        const double ted = (double)(tp - t0) * (double)P.timestep_us * 1e-6;
        const RelaxOpD r = make_relax_d(a, __ldg(Tb.T1d + w.ts_old), __ldg(Tb.T2d + w.ts_old), ted,
                                        relax);
        dst[0] = r.s; dst[1] = r.c; dst[2] = r.e1; dst[3] = r.e2;
    };

    constexpr uint32_t NONE = 0xffffffffu;
    bool rec_scan = ds <= GT.max_ds && GT.rec_any[ds] != 0;
    uint32_t t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
    uint32_t t_te = (rec_scan && c_te < P.n_TE) ? (uint32_t)Tb.te_tp[c_te] : NONE;
    uint32_t t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
    uint32_t t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;

    int status = -1;
    for (;;) {
        if (ne + 4 > kLogCap) break;                                // log full: pause
        if (!started) {
            if (ds > GT.max_ds) { status = SW_SPIN_OK; break; }
            L.put_head(ne++, spin, kEvScanStart | (ds << 8), ds, 0u);  // kernels.cu:110-120
            w.ind_old = P.matrix_length + 1;
            tp = tp_old = 0;
            c_rf = 1; c_te = 0; c_dph = 0; c_grad = 0;
            acc = 0.f; acc_e = 0.f;
            acc_rec = 0.f; acc_rec_e = 0.f;
            accd = 0.; accd_rec = 0.;
            tp_old_rec = 0;
            rec_started = false;
            rec_scan = GT.rec_any[ds] != 0;
            started = true;
            t_rf = 1 < P.n_RF ? (uint32_t)Tb.rf[1].tp : NONE;
            t_te = (rec_scan && P.n_TE > 0) ? (uint32_t)Tb.te_tp[0] : NONE;
            t_dph = P.n_dephasing > 0 ? (uint32_t)Tb.dph_tp[0] : NONE;
            t_grad = P.n_gradient > 0 ? (uint32_t)Tb.grad_tp[0] : NONE;
            continue;
        }
        if (tp >= P.n_timepoints) {                                 // kernels.cu:225-231
            const RelaxOp r = relax_f(acc, acc_e, tp_old);
            L.put_head(ne, spin, kEvScanEnd | (ds << 8), ds, r.relax ? 1u : 0u);
            L.r[L.at(ne, spin)] = relax4(r);
            L.xo[L.at(ne, spin)] = make_float4((float)dfrom(w.xo[0]), (float)dfrom(w.xo[1]),
                                               (float)dfrom(w.xo[2]), 0.f);
            if (SHADOW) {
                bool rl;
                double o[4];
                relax_d(accd, tp_old, o, rl);
                put_relax64(L.r64, L, ne, spin, o);
            }
            ne++;
            ds++;
            started = false;
            continue;
        }
        if ((dnonzero(w.dscale) && w.nc < 3) || w.uc == 0) break;      // buffers low: pause

        uint64_t xn[3];
        const int mv = walk_move(w, xn, P, Tb, vox, nb, ub);
        if (mv == kMoveRejected) continue;
        if (mv == kMoveLost) { status = SW_SPIN_LOST; break; }
        if (mv == kMoveOOB) { status = SW_SPIN_OOB; break; }

        fadd(acc, acc_e, w.field);                                  // kernels.cu:171
        if (rec_started) fadd(acc_rec, acc_rec_e, w.field);
        if (SHADOW) {
            accd += (double)w.field;
            if (rec_started) accd_rec += (double)w.field;
        }
        if (tp == t_dph) {                                          // kernels.cu:175-178
            const float deg = __ldg(Tb.dph_deg + c_dph);
            const float inc = (float)spin * deg / (float)P.n_spins;
            fadd(acc, acc_e, inc);
            if (rec_started) fadd(acc_rec, acc_rec_e, inc);
            if (SHADOW) {
                const double incd = (double)spin * (double)deg / (double)P.n_spins;
                accd += incd;
                if (rec_started) accd_rec += incd;
            }
            c_dph++;
            t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
        }
        if (tp == t_grad) {                                         // kernels.cu:181-187
            const double g = grad_phase_deg(__ldg(Tb.gx + c_grad), __ldg(Tb.gy + c_grad),
                                            __ldg(Tb.gz + c_grad), xn, (double)P.timestep_us);
            if (KAHAN) {
                const float ghi = d2f_exact(dbits(g));
                const float glo = d2f_exact(dadd_fp64(dbits(g), dflip(dbits(f2d_exact(ghi)))));
                kahan_add(acc, acc_e, ghi);
                kahan_add(acc, acc_e, glo);
                if (rec_started) {
                    kahan_add(acc_rec, acc_rec_e, ghi);
                    kahan_add(acc_rec, acc_rec_e, glo);
                }
            } else {
                acc = d2f_exact(dadd_fp64(dbits(f2d_exact(acc)), dbits(g)));
                if (rec_started) acc_rec = d2f_exact(dadd_fp64(dbits(f2d_exact(acc_rec)), dbits(g)));
            }
            if (SHADOW) {
                accd += g;
                if (rec_started) accd_rec += g;
            }
            c_grad++;
            t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;
        }
        if (tp == t_rf) {                                           // kernels.cu:190-199
            const RelaxOp r = relax_f(acc, acc_e, tp_old);
            uint32_t fl = (r.relax ? 1u : 0u) | (rec_started ? 4u : 0u);
            L.r[L.at(ne, spin)] = relax4(r);
            if (SHADOW) {
                bool rl;
                double o[4];
                relax_d(accd, tp_old, o, rl);
                put_relax64(L.r64, L, ne, spin, o);
            }
            if (rec_started) {
                const RelaxOp rr = relax_f(acc_rec, acc_rec_e, tp_old_rec);
                fl |= rr.relax ? 2u : 0u;
                L.rr[L.at(ne, spin)] = relax4(rr);
                if (SHADOW) {
                    bool rl;
                    double o[4];
                    relax_d(accd_rec, tp_old_rec, o, rl);
                    put_relax64(L.rr64, L, ne, spin, o);
                }
                acc_rec = 0.f; acc_rec_e = 0.f; accd_rec = 0.;
                tp_old_rec = tp;
            }
            L.put_head(ne, spin, kEvRf | (c_rf << 8), ds, fl);
            ne++;
            acc = 0.f; acc_e = 0.f; accd = 0.;
            tp_old = tp;
            c_rf++;
            t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
        }
        if (tp == t_te) {                                           // kernels.cu:202-215
            const uint32_t t0 = rec_started ? tp_old_rec : tp_old;
            const RelaxOp r = rec_started ? relax_f(acc_rec, acc_rec_e, t0) : relax_f(acc, acc_e, t0);
            L.put_head(ne, spin, kEvTe | (c_te << 8) | (w.ts_old << 24), ds,
                       (r.relax ? 1u : 0u) | (rec_started ? 4u : 0u));
            L.r[L.at(ne, spin)] = relax4(r);
            if (SHADOW) {
                bool rl;
                double o[4];
                relax_d(rec_started ? accd_rec : accd, t0, o, rl);
                put_relax64(L.r64, L, ne, spin, o);
            }
            ne++;
            acc_rec = 0.f; acc_rec_e = 0.f; accd_rec = 0.;
            tp_old_rec = tp;
            rec_started = true;
            c_te++;
            t_te = c_te < P.n_TE ? (uint32_t)Tb.te_tp[c_te] : NONE;
        }
        w.xo[0] = xn[0]; w.xo[1] = xn[1]; w.xo[2] = xn[2];
        tp++;
    }
    log_count[spin] = ne;
    if (status > 0) {            // lost / out of bounds: every track still running ends here
        for (uint32_t t = 0; t < GT.n_tracks; t++) {
            if ((uint32_t)GT.track_nd[t] < ds) continue;
            float *x = GT.XYZ1[t] + 3 * (size_t)spin;
            x[0] = (float)dfrom(w.xo[0]); x[1] = (float)dfrom(w.xo[1]); x[2] = (float)dfrom(w.xo[2]);
            if (GT.status[t]) GT.status[t][spin] = status;
        }
    }
    S.x[spin] = w.xo[0]; S.y[spin] = w.xo[1]; S.z[spin] = w.xo[2];
    S.acc[spin] = acc;
    GS.acc_rec[spin] = acc_rec;
    if (KAHAN) {
        S.acc_e[spin] = acc_e;
        GS.acc_rec_e[spin] = acc_rec_e;
    }
    if (SHADOW) {
        S.accd[spin] = accd;
        GS.accd_rec[spin] = accd_rec;
    }
    GS.tp_old_rec[spin] = tp_old_rec;
    GS.rec_started[spin] = rec_started ? 1u : 0u;
    S.field[spin] = w.field;
    S.ind_old[spin] = w.ind_old;
    S.tp[spin] = tp; S.tp_old[spin] = tp_old; S.ds[spin] = ds; S.itr[spin] = w.itr;
    S.ctr[spin] = c_rf | (c_te << 16);
    S.ctr2[spin] = c_dph | (c_grad << 16);
    G.nhead[spin] = w.nh; G.ncnt[spin] = w.nc; G.uhead[spin] = w.uh; G.ucnt[spin] = w.uc;
    uint32_t nf = w.ts_old | (started ? kFlagStarted : 0u);
    if (status >= 0) nf |= kFlagDone | ((uint32_t)status << 16);
    S.flags[spin] = nf;
    return status < 0;
}

template <bool KAHAN, bool SHADOW>
__global__ void __launch_bounds__(256)
    k_walk_logged(DevParams P, DevTables Tb, GroupTables GT, GroupState GS,
                  const uint2 *__restrict__ vox, SpinState S, RngState G, uint32_t *active,
                  uint32_t *log_count, EventLog L, uint32_t spin_lo, uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    bool still = false;
    if (spin < spin_hi) {
        const uint32_t flags = S.flags[spin];
        if (!(flags & kFlagDone))
            still = walk_logged_spin<KAHAN, SHADOW>(spin, flags, P, Tb, GT, GS, vox, S, G,
                                                    log_count, L);
        else
            log_count[spin] = 0;
    }
    const unsigned b = __ballot_sync(0xffffffffu, still);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(active, (uint32_t)__popc(b));
}

// The logged walk with NC gradient classes (FP32 arithmetic): the trajectory and events are
// shared, the phase sums acc / acc_rec are kept per class, the gradient term of class c uses the
// sequence's gradients times gscale[c] (float multiply, as the reference's gradient scale loop,
// monte_carlo.cu:287-290), and each event logs one pair of relaxation operators per class.
// Every other operation is the one walk_logged_spin performs.
template <int NC, bool KAHAN>
__device__ __forceinline__ bool walk_cls_spin(const uint32_t spin, uint32_t flags,
                                              const DevParams &P, const DevTables &Tb,
                                              const GroupTables &GT, const GroupState &GS,
                                              const uint2 *__restrict__ vox, const SpinState &S,
                                              const RngState &G, uint32_t *log_count,
                                              const EventLog &L) {
    WalkRegs w;
    w.xo[0] = S.x[spin]; w.xo[1] = S.y[spin]; w.xo[2] = S.z[spin];
    w.ind_old = S.ind_old[spin];
    w.ts_old = flags & 0xffu;
    w.field = S.field[spin];
    w.dscale = __ldg(Tb.dscale + w.ts_old);
    w.itr = S.itr[spin];
    w.nh = G.nhead[spin]; w.nc = G.ncnt[spin]; w.uh = G.uhead[spin]; w.uc = G.ucnt[spin];
    const float *nb = G.nbuf + (size_t)spin * kNormBuf;
    const float *ub = G.ubuf + (size_t)spin * kUnifBuf;
    uint32_t ne = 0;
    const size_t n = P.n_spins;
    auto cls_at = [&](uint32_t k, int c) { return ((size_t)k * NC + c) * n + spin; };

    // per class: phase sums, their compensation terms (KAHAN), gradient scale
    float acc[NC], acc_rec[NC], acc_e[NC], acc_rec_e[NC], gs[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        acc[c] = GS.acc_c[(size_t)c * n + spin];
        acc_rec[c] = GS.acc_rec_c[(size_t)c * n + spin];
        acc_e[c] = KAHAN ? GS.acc_c[(size_t)(2 * NC + c) * n + spin] : 0.f;
        acc_rec_e[c] = KAHAN ? GS.acc_c[(size_t)(3 * NC + c) * n + spin] : 0.f;
        gs[c] = __ldg(GT.gscale + c);
    }
    auto fadd = [&](float &s_, float &e_, float x) {
        if (KAHAN) kahan_add(s_, e_, x); else s_ += x;
    };
    uint32_t tp = S.tp[spin], tp_old = S.tp_old[spin], tp_old_rec = GS.tp_old_rec[spin];
    uint32_t ds = S.ds[spin];
    bool rec_started = GS.rec_started[spin] != 0;
    uint32_t ctr = S.ctr[spin], ctr2 = S.ctr2[spin];
    uint32_t c_rf = ctr & 0xffffu, c_te = ctr >> 16, c_dph = ctr2 & 0xffffu, c_grad = ctr2 >> 16;
    bool started = (flags & kFlagStarted) != 0;

    auto relax_f = [&](float a, float e, uint32_t t0) {
        const float te = (float)((double)((tp - t0) * (uint32_t)P.timestep_us) * 1e-6);
        return make_relax(KAHAN ? a + e : a, __ldg(Tb.T1f + w.ts_old), __ldg(Tb.T2f + w.ts_old), te);
    };

    constexpr uint32_t NONE = 0xffffffffu;
    bool rec_scan = ds <= GT.max_ds && GT.rec_any[ds] != 0;
    uint32_t t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
    uint32_t t_te = (rec_scan && c_te < P.n_TE) ? (uint32_t)Tb.te_tp[c_te] : NONE;
    uint32_t t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
    uint32_t t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;

    int status = -1;
    for (;;) {
        if (ne + 4 > kLogCap) break;                                // log full: pause
        if (!started) {
            if (ds > GT.max_ds) { status = SW_SPIN_OK; break; }
            L.put_head(ne++, spin, kEvScanStart | (ds << 8), ds, 0u);  // kernels.cu:110-120
            w.ind_old = P.matrix_length + 1;
            tp = tp_old = 0;
            c_rf = 1; c_te = 0; c_dph = 0; c_grad = 0;
#pragma unroll
            for (int c = 0; c < NC; c++) { acc[c] = acc_e[c] = acc_rec[c] = acc_rec_e[c] = 0.f; }
            tp_old_rec = 0;
            rec_started = false;
            rec_scan = GT.rec_any[ds] != 0;
            started = true;
            t_rf = 1 < P.n_RF ? (uint32_t)Tb.rf[1].tp : NONE;
            t_te = (rec_scan && P.n_TE > 0) ? (uint32_t)Tb.te_tp[0] : NONE;
            t_dph = P.n_dephasing > 0 ? (uint32_t)Tb.dph_tp[0] : NONE;
            t_grad = P.n_gradient > 0 ? (uint32_t)Tb.grad_tp[0] : NONE;
            continue;
        }
        if (tp >= P.n_timepoints) {                                 // kernels.cu:225-231
            bool rl = false;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const RelaxOp r = relax_f(acc[c], acc_e[c], tp_old);
                L.rc[cls_at(ne, c)] = relax4(r);
                rl = r.relax;
            }
            L.put_head(ne, spin, kEvScanEnd | (ds << 8), ds, rl ? 1u : 0u);
            L.xo[L.at(ne, spin)] = make_float4((float)dfrom(w.xo[0]), (float)dfrom(w.xo[1]),
                                               (float)dfrom(w.xo[2]), 0.f);
            ne++;
            ds++;
            started = false;
            continue;
        }
        if ((dnonzero(w.dscale) && w.nc < 3) || w.uc == 0) break;      // buffers low: pause

        uint64_t xn[3];
        const int mv = walk_move(w, xn, P, Tb, vox, nb, ub);
        if (mv == kMoveRejected) continue;
        if (mv == kMoveLost) { status = SW_SPIN_LOST; break; }
        if (mv == kMoveOOB) { status = SW_SPIN_OOB; break; }

#pragma unroll
        for (int c = 0; c < NC; c++) {                              // kernels.cu:171
            fadd(acc[c], acc_e[c], w.field);
            if (rec_started) fadd(acc_rec[c], acc_rec_e[c], w.field);
        }
        if (tp == t_dph) {                                          // kernels.cu:175-178
            const float inc = (float)spin * __ldg(Tb.dph_deg + c_dph) / (float)P.n_spins;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                fadd(acc[c], acc_e[c], inc);
                if (rec_started) fadd(acc_rec[c], acc_rec_e[c], inc);
            }
            c_dph++;
            t_dph = c_dph < P.n_dephasing ? (uint32_t)Tb.dph_tp[c_dph] : NONE;
        }
        if (tp == t_grad) {                                         // kernels.cu:181-187
            const float gx = __ldg(Tb.gx + c_grad), gy = __ldg(Tb.gy + c_grad),
                        gz = __ldg(Tb.gz + c_grad);
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const double g = grad_phase_deg(gx * gs[c], gy * gs[c], gz * gs[c], xn,
                                                (double)P.timestep_us);
                if (KAHAN) {
                    const float ghi = d2f_exact(dbits(g));
                    const float glo = d2f_exact(dadd_fp64(dbits(g), dflip(dbits(f2d_exact(ghi)))));
                    kahan_add(acc[c], acc_e[c], ghi);
                    kahan_add(acc[c], acc_e[c], glo);
                    if (rec_started) {
                        kahan_add(acc_rec[c], acc_rec_e[c], ghi);
                        kahan_add(acc_rec[c], acc_rec_e[c], glo);
                    }
                } else {
                    acc[c] = d2f_exact(dadd_fp64(dbits(f2d_exact(acc[c])), dbits(g)));
                    if (rec_started)
                        acc_rec[c] = d2f_exact(dadd_fp64(dbits(f2d_exact(acc_rec[c])), dbits(g)));
                }
            }
            c_grad++;
            t_grad = c_grad < P.n_gradient ? (uint32_t)Tb.grad_tp[c_grad] : NONE;
        }
        if (tp == t_rf) {                                           // kernels.cu:190-199
            bool rl = false, rrl = false;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const RelaxOp r = relax_f(acc[c], acc_e[c], tp_old);
                L.rc[cls_at(ne, c)] = relax4(r);
                rl = r.relax;
                if (rec_started) {
                    const RelaxOp rr = relax_f(acc_rec[c], acc_rec_e[c], tp_old_rec);
                    L.rrc[cls_at(ne, c)] = relax4(rr);
                    rrl = rr.relax;
                    acc_rec[c] = acc_rec_e[c] = 0.f;
                }
                acc[c] = acc_e[c] = 0.f;
            }
            L.put_head(ne, spin, kEvRf | (c_rf << 8), ds,
                       (rl ? 1u : 0u) | (rrl ? 2u : 0u) | (rec_started ? 4u : 0u));
            if (rec_started) tp_old_rec = tp;
            ne++;
            tp_old = tp;
            c_rf++;
            t_rf = c_rf < P.n_RF ? (uint32_t)Tb.rf[c_rf].tp : NONE;
        }
        if (tp == t_te) {                                           // kernels.cu:202-215
            const uint32_t t0 = rec_started ? tp_old_rec : tp_old;
            bool rl = false;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const RelaxOp r = rec_started ? relax_f(acc_rec[c], acc_rec_e[c], t0)
                                              : relax_f(acc[c], acc_e[c], t0);
                L.rc[cls_at(ne, c)] = relax4(r);
                rl = r.relax;
                acc_rec[c] = acc_rec_e[c] = 0.f;
            }
            L.put_head(ne, spin, kEvTe | (c_te << 8) | (w.ts_old << 24), ds,
                       (rl ? 1u : 0u) | (rec_started ? 4u : 0u));
            ne++;
            tp_old_rec = tp;
            rec_started = true;
            c_te++;
            t_te = c_te < P.n_TE ? (uint32_t)Tb.te_tp[c_te] : NONE;
        }
        w.xo[0] = xn[0]; w.xo[1] = xn[1]; w.xo[2] = xn[2];
        tp++;
    }
    log_count[spin] = ne;
    if (status > 0) {            // lost / out of bounds: every track still running ends here
        for (uint32_t t = 0; t < GT.n_tracks; t++) {
            if ((uint32_t)GT.track_nd[t] < ds) continue;
            float *x = GT.XYZ1[t] + 3 * (size_t)spin;
            x[0] = (float)dfrom(w.xo[0]); x[1] = (float)dfrom(w.xo[1]); x[2] = (float)dfrom(w.xo[2]);
            if (GT.status[t]) GT.status[t][spin] = status;
        }
    }
    S.x[spin] = w.xo[0]; S.y[spin] = w.xo[1]; S.z[spin] = w.xo[2];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        GS.acc_c[(size_t)c * n + spin] = acc[c];
        GS.acc_rec_c[(size_t)c * n + spin] = acc_rec[c];
        if (KAHAN) {
            GS.acc_c[(size_t)(2 * NC + c) * n + spin] = acc_e[c];
            GS.acc_c[(size_t)(3 * NC + c) * n + spin] = acc_rec_e[c];
        }
    }
    GS.tp_old_rec[spin] = tp_old_rec;
    GS.rec_started[spin] = rec_started ? 1u : 0u;
    S.field[spin] = w.field;
    S.ind_old[spin] = w.ind_old;
    S.tp[spin] = tp; S.tp_old[spin] = tp_old; S.ds[spin] = ds; S.itr[spin] = w.itr;
    S.ctr[spin] = c_rf | (c_te << 16);
    S.ctr2[spin] = c_dph | (c_grad << 16);
    G.nhead[spin] = w.nh; G.ncnt[spin] = w.nc; G.uhead[spin] = w.uh; G.ucnt[spin] = w.uc;
    uint32_t nf = w.ts_old | (started ? kFlagStarted : 0u);
    if (status >= 0) nf |= kFlagDone | ((uint32_t)status << 16);
    S.flags[spin] = nf;
    return status < 0;
}

template <int NC, bool KAHAN>
__global__ void __launch_bounds__(256)
    k_walk_cls(DevParams P, DevTables Tb, GroupTables GT, GroupState GS,
               const uint2 *__restrict__ vox, SpinState S, RngState G, uint32_t *active,
               uint32_t *log_count, EventLog L, uint32_t spin_lo, uint32_t spin_hi) {
    const uint32_t spin = spin_lo + blockIdx.x * blockDim.x + threadIdx.x;
    bool still = false;
    if (spin < spin_hi) {
        const uint32_t flags = S.flags[spin];
        if (!(flags & kFlagDone))
            still = walk_cls_spin<NC, KAHAN>(spin, flags, P, Tb, GT, GS, vox, S, G, log_count, L);
        else
            log_count[spin] = 0;
    }
    const unsigned b = __ballot_sync(0xffffffffu, still);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(active, (uint32_t)__popc(b));
}

// Applies each spin's logged events to every group (thread per (group, spin), spin fastest).
// SHADOW: the same events in FP64 on mg64 / mr64 (the plain kernel's FP64 shadow, per group);
// OUT64: the float outputs are the FP64 values rounded (the plain kernel's SW_PREC_FP64).
// CLS: the relaxation operators come from the group's gradient class (logc).
template <bool SHADOW, bool OUT64, bool CLS>
__global__ void __launch_bounds__(256)
    k_bloch_groups(DevParams P, GroupTables GT, GroupState GS,
                   const uint32_t *__restrict__ log_count, const EventLog L, uint32_t spin_lo,
                   uint32_t spin_hi) {
    const size_t n = P.n_spins, plane = (size_t)GT.n_groups * n, n_half = spin_hi - spin_lo;
    const size_t th = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (th >= (size_t)GT.n_groups * n_half) return;
    const uint32_t g = (uint32_t)(th / n_half);
    const uint32_t spin = spin_lo + (uint32_t)(th - (size_t)g * n_half);
    const size_t idx = (size_t)g * n + spin;                 // index in a [n_groups][n] plane
    const uint32_t cnt = log_count[spin];
    if (cnt == 0) return;
    const uint32_t span = GT.max_ds + 1, last = GT.last_ds[g];
    float m[3], mr[3], t3[3];
    double md[3], mrd[3], u3[3];
    load_m(GS.mg, plane, idx, m);
    if (SHADOW) load_md(GS.mg64, plane, idx, md);
    bool mr_loaded = false, mr_dirty = false;
    auto load_mr = [&]() {
        if (mr_loaded) return;
        load_m(GS.mr, plane, idx, mr);
        if (SHADOW) load_md(GS.mr64, plane, idx, mrd);
        mr_loaded = true;
    };
    const uint32_t ncls = CLS ? GT.n_cls : 1u, cl = CLS ? GT.cls[g] : 0u;
    // the event's operators: shared, or the group's class's
    auto op_r = [&](uint32_t k) {
        return __ldg(CLS ? L.rc + ((size_t)k * ncls + cl) * n + spin : L.r + L.at(k, spin));
    };
    auto op_rr = [&](uint32_t k) {
        return __ldg(CLS ? L.rrc + ((size_t)k * ncls + cl) * n + spin : L.rr + L.at(k, spin));
    };
    double o64[4];
    for (uint32_t k = 0; k < cnt; k++) {
        const uint4 hd = __ldg(L.head + L.at(k, spin));
        const uint32_t type = hd.x & 0xffu, id = (hd.x >> 8) & 0xffffu, ds = hd.y, flags = hd.z;
        if (ds > last) continue;                                    // group finished earlier
        const int32_t t = GT.rec[(size_t)g * span + ds];
        if (type == kEvScanStart) {
            const RfOp op = GT.scan_rf[(size_t)g * span + ds];
            rf_f(op, m, t3);
            m[0] = t3[0]; m[1] = t3[1]; m[2] = t3[2];
            if (SHADOW) {
                rf_d(op, md, u3);
                md[0] = u3[0]; md[1] = u3[1]; md[2] = u3[2];
            }
        } else if (type == kEvRf) {
            const RfOp op = GT.rf[(size_t)g * P.n_RF + id];
            apply_relax(get_relax(op_r(k), flags & 1u), m, t3);
            rf_f(op, t3, m);
            if (SHADOW) {
                get_relax64(L.r64, L, k, spin, o64);
                apply_relax_d(o64, flags & 1u, md, u3);
                rf_d(op, u3, md);
            }
            if ((flags & 4u) && t >= 0) {
                load_mr();
                apply_relax(get_relax(op_rr(k), flags & 2u), mr, t3);
                rf_f(op, t3, mr);
                if (SHADOW) {
                    get_relax64(L.rr64, L, k, spin, o64);
                    apply_relax_d(o64, flags & 2u, mrd, u3);
                    rf_d(op, u3, mrd);
                }
                mr_dirty = true;
            }
        } else if (type == kEvTe) {
            if (t < 0) continue;
            const bool from_rec = (flags & 4u) != 0;
            if (from_rec) load_mr();
            apply_relax(get_relax(op_r(k), flags & 1u), from_rec ? mr : m, t3);
            if (SHADOW) {
                get_relax64(L.r64, L, k, spin, o64);
                apply_relax_d(o64, flags & 1u, from_rec ? mrd : md, u3);
            }
            float *o = GT.M1[t] + 3 * ((size_t)spin * P.n_TE + id);
            if (OUT64) {
                o[0] = (float)u3[0]; o[1] = (float)u3[1]; o[2] = (float)u3[2];
            } else {
                o[0] = t3[0]; o[1] = t3[1]; o[2] = t3[2];
            }
            if (SHADOW && GT.M1d[t]) {
                double *od = GT.M1d[t] + 3 * ((size_t)spin * P.n_TE + id);
                od[0] = u3[0]; od[1] = u3[1]; od[2] = u3[2];
            }
            GT.T[t][(size_t)spin * P.n_TE + id] = (uint8_t)(hd.x >> 24);
            mr[0] = t3[0]; mr[1] = t3[1]; mr[2] = t3[2];
            if (SHADOW) { mrd[0] = u3[0]; mrd[1] = u3[1]; mrd[2] = u3[2]; }
            mr_loaded = mr_dirty = true;
        } else {                                                    // scan end
            apply_relax(get_relax(op_r(k), flags & 1u), m, t3);
            m[0] = t3[0]; m[1] = t3[1]; m[2] = t3[2];
            if (SHADOW) {
                get_relax64(L.r64, L, k, spin, o64);
                apply_relax_d(o64, flags & 1u, md, u3);
                md[0] = u3[0]; md[1] = u3[1]; md[2] = u3[2];
            }
            if (t >= 0) {                                           // track t ends here
                float *x = GT.XYZ1[t] + 3 * (size_t)spin;
                const float4 xo = __ldg(L.xo + L.at(k, spin));
                x[0] = xo.x; x[1] = xo.y; x[2] = xo.z;
                if (GT.status[t]) GT.status[t][spin] = SW_SPIN_OK;
            }
        }
    }
    store_m(GS.mg, plane, idx, m);
    if (SHADOW) store_md(GS.mg64, plane, idx, md);
    if (mr_dirty) {
        store_m(GS.mr, plane, idx, mr);
        if (SHADOW) store_md(GS.mr64, plane, idx, mrd);
    }
}

}  // namespace sw

namespace {

using namespace sw::api;

struct TracksCtx {
    std::mutex mu;
    char *buf = nullptr;
    size_t size = 0;
    cudaStream_t st[2] = {nullptr, nullptr};  // the two halves of the rounds
    uint32_t *h_active = nullptr;             // pinned, one counter per half
};
TracksCtx g_tctx[64];

std::vector<float> rf_array(const float *override_, const float *base, uint32_t n) {
    const float *src = override_ ? override_ : base;
    return std::vector<float>(src, src + n);
}

}  // namespace

extern "C" int sw_sim_tracks(const sw_params *param, const sw_sequence *seq,
                             const sw_track *tracks, uint32_t n_tracks, const float *pFieldMap,
                             const uint8_t *pMask, const float *M0, const float *XYZ0,
                             int precision) {
    int rc = check_args(param, seq);
    if (rc) return rc;
    const bool bf16 = (precision & SW_FIELD_BF16) != 0;
    const uint32_t rng = (uint32_t)precision & ~(uint32_t)(SW_PREC_MASK | SW_FIELD_BF16);
    precision &= SW_PREC_MASK;
    if (precision != SW_PREC_FP32 && precision != SW_PREC_KAHAN && precision != SW_PREC_FP64)
        return fail(SW_ERR_INVALID, "tracks: precision must be SW_PREC_FP32, _KAHAN or _FP64");
    if (rng != SW_RNG_MT19937 && rng != SW_RNG_MINSTD) return fail(SW_ERR_INVALID, "generator flavour");
    const bool mt = rng == SW_RNG_MT19937;
    if (!tracks || n_tracks == 0) return fail(SW_ERR_INVALID, "no tracks");
    if (param->enRecordTrajectory) return fail(SW_ERR_INVALID, "tracks do not record trajectories");
    const size_t n = param->n_spins, nte = seq->n_TE, ml = (size_t)param->matrix_length;
    if (n == 0) return SW_OK;
    if (!pMask || !M0 || !XYZ0) return fail(SW_ERR_INVALID, "null host buffer");
    for (uint32_t t = 0; t < n_tracks; t++) {
        if (tracks[t].n_dummy_scan < 0) return fail(SW_ERR_INVALID, "track n_dummy_scan < 0");
        if (!tracks[t].XYZ1 || (nte && (!tracks[t].M1 || !tracks[t].T)))
            return fail(SW_ERR_INVALID, "track output buffer missing");
    }
    bool shadow = precision == SW_PREC_FP64;
    for (uint32_t t = 0; t < n_tracks; t++) shadow = shadow || (nte && tracks[t].M1_fp64);
    // ---- group tracks by RF configuration and gradient scale ----
    using Key = std::tuple<float, float, std::vector<float>, std::vector<float>, float>;
    std::map<Key, uint32_t> gid;
    std::vector<Key> groups;
    std::vector<uint32_t> tgroup(n_tracks);
    uint32_t max_ds = 0;
    for (uint32_t t = 0; t < n_tracks; t++) {
        if (tracks[t].options & ~SW_TRACK_GRADIENT_SCALE) return fail(SW_ERR_INVALID, "track options");
        const float gsc = (tracks[t].options & SW_TRACK_GRADIENT_SCALE) ? tracks[t].gradient_scale : 1.0f;
        Key k{tracks[t].linear_phase_cycling, tracks[t].quadratic_phase_cycling,
              rf_array(tracks[t].RF_FA_deg, seq->RF_FA_deg, seq->n_RF),
              rf_array(tracks[t].RF_PH_deg, seq->RF_PH_deg, seq->n_RF), gsc};
        auto it = gid.find(k);
        if (it == gid.end()) {
            it = gid.emplace(k, (uint32_t)groups.size()).first;
            groups.push_back(k);
        }
        tgroup[t] = it->second;
        max_ds = std::max(max_ds, (uint32_t)tracks[t].n_dummy_scan);
    }
    const uint32_t ng = (uint32_t)groups.size(), span = max_ds + 1;
    std::vector<int32_t> rec((size_t)ng * span, -1), track_nd(n_tracks);
    std::vector<uint32_t> last_ds(ng, 0), rec_any(span, 0);
    for (uint32_t t = 0; t < n_tracks; t++) {
        const uint32_t d = (uint32_t)tracks[t].n_dummy_scan, g = tgroup[t];
        if (rec[(size_t)g * span + d] >= 0)
            return fail(SW_ERR_INVALID,
                        "two tracks with the same RF configuration, gradient scale and DUMMY_SCAN");
        rec[(size_t)g * span + d] = (int32_t)t;
        last_ds[g] = std::max(last_ds[g], d);
        rec_any[d] = 1;
        track_nd[t] = (int32_t)d;
    }
    // per-group RF operations: parameters::prepare's c/s and the scan-start phases of each group
    std::vector<sw::RfOp> scan_rf((size_t)ng * span), rfops((size_t)ng * seq->n_RF);
    for (uint32_t g = 0; g < ng; g++) {
        const auto &[lin, quad, fa, ph, gsc] = groups[g];
        (void)gsc;
        sw_params pg = *param;
        pg.linear_phase_cycling = lin;
        pg.quadratic_phase_cycling = quad;
        pg.n_dummy_scan = (int32_t)max_ds;
        pg.c = cosf(fa[0] * sw::kDeg2Rad);
        pg.s = sinf(fa[0] * sw::kDeg2Rad);
        sw_sequence qg = *seq;
        qg.RF_FA_deg = fa.data();
        qg.RF_PH_deg = ph.data();
        std::vector<sw::RfOp> a, b;
        sw::build_scan_rf(&pg, &qg, a);
        sw::build_rf(&pg, &qg, b);
        std::copy(a.begin(), a.end(), scan_rf.begin() + (size_t)g * span);
        std::copy(b.begin(), b.end(), rfops.begin() + (size_t)g * seq->n_RF);
    }
    sw_params pw = *param;            // the walk: the longest track
    pw.n_dummy_scan = (int32_t)max_ds;

    // gradient classes: the distinct gradient scales. One scale scales the walk's gradient table
    // (the same float multiply); several keep a phase per class in the walk (k_walk_cls).
    std::vector<float> cls_scale;
    std::vector<uint32_t> gcls(ng);
    for (uint32_t g = 0; g < ng; g++) {
        const float gsc = std::get<4>(groups[g]);
        uint32_t c = 0;
        while (c < cls_scale.size() && std::memcmp(&cls_scale[c], &gsc, 4) != 0) c++;
        if (c == cls_scale.size()) cls_scale.push_back(gsc);
        gcls[g] = c;
    }
    const uint32_t n_cls = (uint32_t)cls_scale.size();
    if (n_cls > 8) return fail(SW_ERR_INVALID, "tracks: at most 8 distinct gradient scales per call");
    if (n_cls > 1 && (precision == SW_PREC_FP64 || shadow))
        return fail(SW_ERR_INVALID, "tracks: several gradient scales need SW_PREC_FP32 or _KAHAN "
                                    "without the FP64 shadow");
    const uint32_t NC = n_cls <= 1 ? 1u : (n_cls <= 2 ? 2u : (n_cls <= 4 ? 4u : 8u));
    std::vector<float> gsx, gsy, gsz;   // the one scale applied to the sequence's gradients
    sw_sequence qw = *seq;
    if (n_cls == 1 && cls_scale[0] != 1.0f) {
        const float sc = cls_scale[0];
        for (uint32_t k = 0; k < seq->n_gradient; k++) {
            gsx.push_back(seq->gradientX_mTm[k] * sc);
            gsy.push_back(seq->gradientY_mTm[k] * sc);
            gsz.push_back(seq->gradientZ_mTm[k] * sc);
        }
        qw.gradientX_mTm = gsx.data();
        qw.gradientY_mTm = gsy.data();
        qw.gradientZ_mTm = gsz.data();
    }
    std::vector<float> gscale_pad(NC);
    for (uint32_t c = 0; c < NC; c++) gscale_pad[c] = cls_scale[std::min(c, n_cls - 1)];

    TableImage im;
    build_tables(&pw, &qw, im);
    if (!im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
    TableImage gi;                    // group tables
    const size_t o_scan = gi.put(scan_rf.data(), scan_rf.size());
    const size_t o_rf = gi.put(rfops.data(), rfops.size());
    const size_t o_rec = gi.put(rec.data(), rec.size());
    const size_t o_last = gi.put(last_ds.data(), last_ds.size());
    const size_t o_any = gi.put(rec_any.data(), rec_any.size());
    const size_t o_nd = gi.put(track_nd.data(), track_nd.size());
    const size_t o_gcls = gi.put(gcls.data(), gcls.size());
    const size_t o_gsc = gi.put(gscale_pad.data(), gscale_pad.size());

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return fail(SW_ERR_CUDA, "no current CUDA device");
    }
    TracksCtx &C = g_tctx[dev];
    std::lock_guard<std::mutex> lk(C.mu);

    // ---- one device allocation: inputs, per-track outputs, pointer arrays, walk workspace ----
    size_t off = 0;
    auto slot = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) & ~size_t(255);
        return o;
    };
    const bool has_field = param->fieldmap_exist && pFieldMap;
    const size_t o_mask = slot(ml), o_field = slot(has_field ? ml * 4 : 0), o_M0 = slot(n * 12),
                 o_XYZ0 = slot(n * 12), o_scratch_xyz = slot(n * 12), o_scratch_st = slot(n * 4),
                 o_tab = slot(im.bytes.size()), o_gtab = slot(gi.bytes.size()),
                 o_ptrs = slot(5 * sizeof(void *) * n_tracks),
                 o_mg = slot(2 * 3 * sizeof(float) * (size_t)ng * n),
                 o_gs = slot(16 * n), o_lcnt = slot(4 * n),
                 o_log = slot(4 * 16 * sw::kLogCap * n);       // head, r, rr, xo
    const size_t o_accc = slot(NC > 1 ? 4 * sizeof(float) * NC * n : 0),   // acc, acc_rec (+ compensations)
                 o_logc = slot(NC > 1 ? 2 * 16 * sw::kLogCap * NC * n : 0);   // rc, rrc
    const size_t o_mg64 = slot(shadow ? 2 * 3 * sizeof(double) * (size_t)ng * n : 0),
                 o_accd = slot(shadow ? 8 * n : 0),
                 o_log64 = slot(shadow ? 2 * 32 * sw::kLogCap * n : 0);   // r64, rr64
    std::vector<size_t> o_M1(n_tracks), o_X(n_tracks), o_T(n_tracks), o_S(n_tracks),
        o_M1d(n_tracks);
    for (uint32_t t = 0; t < n_tracks; t++) {
        o_M1[t] = slot(n * nte * 12);
        o_X[t] = slot(n * 12);
        o_T[t] = slot(n * nte);
        o_S[t] = slot(n * 4);
        o_M1d[t] = slot(tracks[t].M1_fp64 ? n * nte * 24 : 0);
    }
    const Layout Lm = layout(nullptr, n, param->matrix_length, 0, shadow, mt);
    const size_t o_ws = slot(Lm.bytes);
    if (off > C.size) {
        if (C.buf) cudaFree(C.buf);
        C.buf = nullptr;
        C.size = 0;
        cudaError_t e = cudaMalloc(&C.buf, off);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_NOMEM, "tracks buffers of " + std::to_string(off >> 20) + " MiB: " +
                                          cudaGetErrorString(e));
        }
        C.size = off;
    }
    char *d = C.buf;
    if (!C.st[0]) {
        for (int i = 0; i < 2; i++)
            if (cudaStreamCreateWithFlags(&C.st[i], cudaStreamNonBlocking) != cudaSuccess) {
                cudaGetLastError();
                return fail(SW_ERR_CUDA, "tracks streams");
            }
        if (cudaMallocHost(&C.h_active, 2 * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            return fail(SW_ERR_CUDA, "tracks pinned counters");
        }
    }
    cudaStream_t st = C.st[0];
#define TR_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
        }                                                                                  \
    } while (0)
    TR_CUDA(cudaMemcpyAsync(d + o_mask, pMask, ml, cudaMemcpyHostToDevice, st));
    if (has_field) TR_CUDA(cudaMemcpyAsync(d + o_field, pFieldMap, ml * 4, cudaMemcpyHostToDevice, st));
    TR_CUDA(cudaMemcpyAsync(d + o_M0, M0, n * 12, cudaMemcpyHostToDevice, st));
    TR_CUDA(cudaMemcpyAsync(d + o_XYZ0, XYZ0, n * 12, cudaMemcpyHostToDevice, st));
    TR_CUDA(cudaMemcpyAsync(d + o_tab, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st));
    TR_CUDA(cudaMemcpyAsync(d + o_gtab, gi.bytes.data(), gi.bytes.size(), cudaMemcpyHostToDevice, st));
    std::vector<void *> ptrs(5 * (size_t)n_tracks);
    for (uint32_t t = 0; t < n_tracks; t++) {
        const bool t64 = nte && tracks[t].M1_fp64;
        ptrs[t] = d + o_M1[t];
        ptrs[n_tracks + t] = d + o_X[t];
        ptrs[2 * n_tracks + t] = d + o_T[t];
        ptrs[3 * n_tracks + t] = tracks[t].status ? (void *)(d + o_S[t]) : nullptr;
        ptrs[4 * n_tracks + t] = t64 ? (void *)(d + o_M1d[t]) : nullptr;
        if (nte) {     // unreached echoes keep the caller's contents, as in the reference
            TR_CUDA(cudaMemcpyAsync(d + o_M1[t], tracks[t].M1, n * nte * 12, cudaMemcpyHostToDevice, st));
            TR_CUDA(cudaMemcpyAsync(d + o_T[t], tracks[t].T, n * nte, cudaMemcpyHostToDevice, st));
            if (t64)
                TR_CUDA(cudaMemcpyAsync(d + o_M1d[t], tracks[t].M1_fp64, n * nte * 24,
                                        cudaMemcpyHostToDevice, st));
        }
    }
    TR_CUDA(cudaMemcpyAsync(d + o_ptrs, ptrs.data(), ptrs.size() * sizeof(void *), cudaMemcpyHostToDevice, st));

    const Layout L = layout(d + o_ws, n, param->matrix_length, 0, shadow, mt);
    sw::DevParams P = dev_params(&pw, seq);
    P.rng = rng;
    P.field_bf16 = bf16 ? 1 : 0;
    const sw::DevTables Tb = dev_tables(im, d + o_tab);
    sw::GroupTables GT;
    GT.n_groups = ng;
    GT.n_tracks = n_tracks;
    GT.max_ds = max_ds;
    GT.n_rf = seq->n_RF;
    GT.scan_rf = reinterpret_cast<const sw::RfOp *>(d + o_gtab + o_scan);
    GT.rf = reinterpret_cast<const sw::RfOp *>(d + o_gtab + o_rf);
    GT.rec = reinterpret_cast<const int32_t *>(d + o_gtab + o_rec);
    GT.last_ds = reinterpret_cast<const uint32_t *>(d + o_gtab + o_last);
    GT.rec_any = reinterpret_cast<const uint32_t *>(d + o_gtab + o_any);
    GT.track_nd = reinterpret_cast<const int32_t *>(d + o_gtab + o_nd);
    void **dp = reinterpret_cast<void **>(d + o_ptrs);
    GT.M1 = reinterpret_cast<float *const *>(dp);
    GT.XYZ1 = reinterpret_cast<float *const *>(dp + n_tracks);
    GT.T = reinterpret_cast<uint8_t *const *>(dp + 2 * (size_t)n_tracks);
    GT.status = reinterpret_cast<int32_t *const *>(dp + 3 * (size_t)n_tracks);
    GT.M1d = reinterpret_cast<double *const *>(dp + 4 * (size_t)n_tracks);
    GT.n_cls = NC;
    GT.cls = reinterpret_cast<const uint32_t *>(d + o_gtab + o_gcls);
    GT.gscale = reinterpret_cast<const float *>(d + o_gtab + o_gsc);
    sw::GroupState GS;
    GS.mg = reinterpret_cast<float *>(d + o_mg);
    GS.mr = GS.mg + 3 * (size_t)ng * n;
    GS.acc_rec = reinterpret_cast<float *>(d + o_gs);
    GS.tp_old_rec = reinterpret_cast<uint32_t *>(d + o_gs + 4 * n);
    GS.rec_started = reinterpret_cast<uint32_t *>(d + o_gs + 8 * n);
    GS.acc_rec_e = reinterpret_cast<float *>(d + o_gs + 12 * n);
    GS.mg64 = shadow ? reinterpret_cast<double *>(d + o_mg64) : nullptr;
    GS.mr64 = shadow ? GS.mg64 + 3 * (size_t)ng * n : nullptr;
    GS.accd_rec = shadow ? reinterpret_cast<double *>(d + o_accd) : nullptr;
    GS.acc_c = NC > 1 ? reinterpret_cast<float *>(d + o_accc) : nullptr;
    GS.acc_rec_c = NC > 1 ? GS.acc_c + (size_t)NC * n : nullptr;
    if (NC > 1) TR_CUDA(cudaMemsetAsync(GS.acc_c, 0, 4 * sizeof(float) * NC * n, st));

    uint32_t *lcnt = reinterpret_cast<uint32_t *>(d + o_lcnt);
    // the event log, slot-major ([slot][spin] per field)
    sw::EventLog elog{};
    elog.n = n;
    const size_t slot_n = (size_t)sw::kLogCap * n;
    elog.head = reinterpret_cast<uint4 *>(d + o_log);
    elog.r = reinterpret_cast<float4 *>(d + o_log + 16 * slot_n);
    elog.rr = reinterpret_cast<float4 *>(d + o_log + 32 * slot_n);
    elog.xo = reinterpret_cast<float4 *>(d + o_log + 48 * slot_n);
    if (shadow) {
        elog.r64 = reinterpret_cast<double2 *>(d + o_log64);
        elog.rr64 = reinterpret_cast<double2 *>(d + o_log64 + 32 * slot_n);
    }
    if (NC > 1) {
        elog.rc = reinterpret_cast<float4 *>(d + o_logc);
        elog.rrc = reinterpret_cast<float4 *>(d + o_logc + 16 * slot_n * NC);
    }
    sw::LogfTables LT = sw::api::device_logf_tables();
    if (!LT.bitmap) return fail(SW_ERR_CUDA, "logf tables unavailable");
    if (!mt && !(LT.ms_delta = sw::api::minstd_delta_table())) return SW_ERR_CUDA;
    sw::Outputs O{nullptr, nullptr, reinterpret_cast<float *>(d + o_scratch_xyz), nullptr,
                  reinterpret_cast<int32_t *>(d + o_scratch_st)};
    g_timing = sw_timing{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    TR_CUDA(cudaEventCreate(&ev0));
    TR_CUDA(cudaEventCreate(&ev1));
    TR_CUDA(cudaEventRecord(ev0, st));
    TR_CUDA(cudaMemsetAsync(L.active, 0, 2 * sizeof(uint32_t), st));
    TR_CUDA(sw::launch_pack(reinterpret_cast<const uint8_t *>(d + o_mask),
                            has_field ? reinterpret_cast<const float *>(d + o_field) : nullptr,
                            L.vox, param->matrix_length, param->n_substrate, L.active + 1, st,
                            bf16));
    TR_CUDA(sw::launch_seed(P, L.G, st));
    TR_CUDA(sw::launch_init(P, Tb, L.vox, reinterpret_cast<const float *>(d + o_M0),
                            reinterpret_cast<const float *>(d + o_XYZ0), L.S, O, shadow, st));
    sw::k_groups_init<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        P, GT, GS, L.S, reinterpret_cast<const float *>(d + o_M0),
        reinterpret_cast<const float *>(d + o_XYZ0));
    TR_CUDA(cudaGetLastError());
    uint32_t h = 0;
    TR_CUDA(cudaMemcpyAsync(&h, L.active + 1, 4, cudaMemcpyDeviceToHost, st));
    TR_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate");
    const uint64_t steps = (uint64_t)pw.n_timepoints * (uint64_t)(max_ds + 1);
    const uint64_t max_rounds = 64 + steps * (param->max_iterations + 2);
    // the rounds as two independent halves of the spins on two streams (from 2^16 spins on):
    // one half's refill and Bloch update overlap the other half's walk
    const uint32_t H = n >= (1u << 16) ? 2u : 1u;
    const uint32_t hb[3] = {0u, H == 2 ? (uint32_t)(n / 2) : (uint32_t)n, (uint32_t)n};
    cudaEvent_t evh = nullptr;
    TR_CUDA(cudaEventCreateWithFlags(&evh, cudaEventDisableTiming));
    if (H == 2) {                                  // the second half starts after the set-up
        TR_CUDA(cudaEventRecord(evh, C.st[0]));
        TR_CUDA(cudaStreamWaitEvent(C.st[1], evh, 0));
    }
    auto issue_round = [&](uint32_t hh) -> int {
        const uint32_t lo = hb[hh], hi = hb[hh + 1];
        cudaStream_t s = C.st[hh];
        uint32_t *act = L.active + 2 * hh;
        TR_CUDA(sw::launch_refill_range(P, L.G, L.S, LT, lo, hi, s));
        const unsigned gw = (hi - lo + 255) / 256, gb = (unsigned)(((size_t)ng * (hi - lo) + 255) / 256);
        if (NC > 1) {                              // gradient classes (FP32, no shadow)
            const bool kh = precision == SW_PREC_KAHAN;
            if (NC == 2 && kh)
                sw::k_walk_cls<2, true><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            else if (NC == 2)
                sw::k_walk_cls<2, false><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            else if (NC == 4 && kh)
                sw::k_walk_cls<4, true><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            else if (NC == 4)
                sw::k_walk_cls<4, false><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            else if (kh)
                sw::k_walk_cls<8, true><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            else
                sw::k_walk_cls<8, false><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
            TR_CUDA(cudaGetLastError());
            sw::k_bloch_groups<false, false, true><<<gb, 256, 0, s>>>(P, GT, GS, lcnt, elog, lo, hi);
            TR_CUDA(cudaGetLastError());
            return SW_OK;
        }
        if (precision == SW_PREC_KAHAN && shadow)
            sw::k_walk_logged<true, true><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
        else if (precision == SW_PREC_KAHAN)
            sw::k_walk_logged<true, false><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
        else if (shadow)
            sw::k_walk_logged<false, true><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
        else
            sw::k_walk_logged<false, false><<<gw, 256, 0, s>>>(P, Tb, GT, GS, L.vox, L.S, L.G, act, lcnt, elog, lo, hi);
        TR_CUDA(cudaGetLastError());
        if (precision == SW_PREC_FP64)
            sw::k_bloch_groups<true, true, false><<<gb, 256, 0, s>>>(P, GT, GS, lcnt, elog, lo, hi);
        else if (shadow)
            sw::k_bloch_groups<true, false, false><<<gb, 256, 0, s>>>(P, GT, GS, lcnt, elog, lo, hi);
        else
            sw::k_bloch_groups<false, false, false><<<gb, 256, 0, s>>>(P, GT, GS, lcnt, elog, lo, hi);
        TR_CUDA(cudaGetLastError());
        return SW_OK;
    };
    // rounds that no spin can finish sooner (each advances a spin by at most kStepsPerRound
    // time points), issued without waiting; then rounds until no spin is active
    const uint64_t r0 = (steps + sw::kStepsPerRound - 1) / sw::kStepsPerRound;
    uint64_t round = 0;
    for (; round < r0; round++)
        for (uint32_t hh = 0; hh < H; hh++)
            if ((rc = issue_round(hh))) return rc;
    for (;; round++) {
        if (round >= max_rounds) return fail(SW_ERR_TIMEOUT, "walk did not finish");
        for (uint32_t hh = 0; hh < H; hh++) {
            TR_CUDA(cudaMemsetAsync(L.active + 2 * hh, 0, 4, C.st[hh]));
            if ((rc = issue_round(hh))) return rc;
            TR_CUDA(cudaMemcpyAsync(C.h_active + hh, L.active + 2 * hh, 4, cudaMemcpyDeviceToHost,
                                    C.st[hh]));
        }
        uint32_t live = 0;
        for (uint32_t hh = 0; hh < H; hh++) {
            TR_CUDA(cudaStreamSynchronize(C.st[hh]));
            live += C.h_active[hh];
        }
        if (live == 0) break;
    }
    if (H == 2) {                                  // join the halves on the first stream
        TR_CUDA(cudaEventRecord(evh, C.st[1]));
        TR_CUDA(cudaStreamWaitEvent(C.st[0], evh, 0));
    }
    cudaEventDestroy(evh);
    TR_CUDA(cudaEventRecord(ev1, st));
    TR_CUDA(cudaEventSynchronize(ev1));
    cudaEventElapsedTime(&g_timing.total_ms, ev0, ev1);
    g_timing.walk_ms = g_timing.total_ms;
    g_timing.n_chunks = (uint32_t)(round + 1);
    g_timing.n_launches = (uint32_t)(4 + 3 * H * (round + 1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    for (uint32_t t = 0; t < n_tracks; t++) {
        if (nte) {
            TR_CUDA(cudaMemcpyAsync(tracks[t].M1, d + o_M1[t], n * nte * 12, cudaMemcpyDeviceToHost, st));
            TR_CUDA(cudaMemcpyAsync(tracks[t].T, d + o_T[t], n * nte, cudaMemcpyDeviceToHost, st));
            if (tracks[t].M1_fp64)
                TR_CUDA(cudaMemcpyAsync(tracks[t].M1_fp64, d + o_M1d[t], n * nte * 24,
                                        cudaMemcpyDeviceToHost, st));
        }
        TR_CUDA(cudaMemcpyAsync(tracks[t].XYZ1, d + o_X[t], n * 12, cudaMemcpyDeviceToHost, st));
        if (tracks[t].status)
            TR_CUDA(cudaMemcpyAsync(tracks[t].status, d + o_S[t], n * 4, cudaMemcpyDeviceToHost, st));
    }
    TR_CUDA(cudaStreamSynchronize(st));
#undef TR_CUDA
    return SW_OK;
}
