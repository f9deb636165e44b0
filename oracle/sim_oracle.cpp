// TEST INFRASTRUCTURE ONLY: the oracle. Imported by tests/, by __graft_entry__.smoke() and by
// bench.py's CPU-baseline leg as the checker; never part of the product library.
//
// A CPU restatement, written for this project, of SpinWalk's per-spin hot path
// sim::sim (src/sim/kernels.cu:72-233, SpinWalk 1.21.0) in its CPU-only "Flavour A" form:
// std::mt19937 + std::normal_distribution<float> + std::uniform_real_distribution<float>
// (kernels.cu:82-88), i.e. the libstdc++ generators the reference links against. Every
// expression keeps the reference's operand types so float/double rounding matches; the file
// must be compiled with -ffp-contract=off (oracle/Makefile).
//
// The generator flavour of the reference's CUDA build (SW_RNG_MINSTD, kernels.cu:76-80) is
// restated too: thrust::minstd_rand, thrust::normal_distribution<float> (normal_distribution_nvcc:
// one draw, inverse erfc) and thrust::uniform_real_distribution<float>, calling CUDA's own
// host erfcinvf (this file is compiled by nvcc's host pass for that reason).
//
// On top of the reference semantics it reports a per-spin status (SW_SPIN_*), and offers the
// two extra Bloch precisions of the GPU library along the SAME walk:
//   SW_PREC_FP64  : phase sum, rotations and relaxation in double;
//   SW_PREC_KAHAN : the float phase sum replaced by a compensated (two-sum) float sum.
// Pinned against the reference itself (oracle/_ref, tests/golden/*) by tests/test_oracle.py.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <sstream>
#include <omp.h>

#include "spinwalk_gpu.h"

namespace {

constexpr double kDeg2Rad = 0.0174532925199433;   // DEG2RAD, simulation_parameters.cuh:24
constexpr double kRad2Deg = 57.2957795130823;     // RAD2DEG, simulation_parameters.cuh:25
constexpr double kGamma = 267515315.;             // GAMMA,   definitions.h:20

// ---- generators ----------------------------------------------------------------------------
struct StdGen {           // the CPU build (kernels.cu:82-88)
    std::mt19937 gen_r, gen_u;
    std::normal_distribution<float> nrm{0.f, 1.0f};
    std::uniform_real_distribution<float> uni{0.f, 1.f};
    explicit StdGen(uint64_t sd) : gen_r(sd), gen_u(sd) {
        gen_r.discard(sd);
        gen_u.discard(sd);
    }
    float normal() { return nrm(gen_r); }
    float uniform() { return uni(gen_u); }
};

struct MinstdGen {        // the CUDA build: thrust::minstd_rand (kernels.cu:77-80, 87-88)
    static constexpr uint64_t A = 48271, M = 2147483647;
    uint32_t xr, xu;
    static uint32_t seed_discard(uint64_t sd) {
        uint64_t x = (uint32_t)sd % M;              // linear_congruential_engine::seed
        if (x == 0) x = 1;
        uint64_t mul = A, acc = 1;                  // ::discard(z): a^z x mod m
        for (uint64_t z = sd; z; z >>= 1) {
            if (z & 1) acc = acc * mul % M;
            mul = mul * mul % M;
        }
        return (uint32_t)(acc * x % M);
    }
    explicit MinstdGen(uint64_t sd) : xr(seed_discard(sd)), xu(xr) {}
    static uint32_t next(uint32_t &x) { return x = (uint32_t)((uint64_t)x * A % M); }
    static float normal_of(uint32_t x) {            // normal_distribution_nvcc::sample(0, 1)
        const uint32_t range = (uint32_t)(M - 2);
        const float S1 = static_cast<float>(1. / static_cast<double>(range));
        const float S2 = S1 / 2;
        float S3 = static_cast<float>(-1.4142135623730950488016887242097);
        uint32_t u = x - 1;
        if (u > range / 2) {
            u = range - u;
            S3 = -S3;
        }
        const float p = u * S1 + S2;
        const float mean = 0.f, stddev = 1.0f;
        return mean + stddev * S3 * erfcinvf(2 * p);
    }
    float normal() { return normal_of(next(xr)); }
    float uniform() {                               // uniform_real_distribution<float>(0, 1)
        float r = static_cast<float>(next(xu) - 1);
        r /= (1.0f + static_cast<float>((uint32_t)(M - 2)));
        return (r * (1.f - 0.f)) + 0.f;
    }
};

// ---- float Bloch primitives with the reference's operand types (kernels.cuh:82-230) ------
inline void xrot_f(float s, float c, const float *a, float *b) {
    b[0] = a[0];
    b[1] = c * a[1] - s * a[2];
    b[2] = s * a[1] + c * a[2];
}
inline void yrot_f(float s, float c, const float *a, float *b) {
    b[0] = c * a[0] + s * a[2];
    b[1] = a[1];
    b[2] = -s * a[0] + c * a[2];
}
inline void zrot_f(float s, float c, const float *a, float *b) {
    b[0] = c * a[0] - s * a[1];
    b[1] = s * a[0] + c * a[1];
    b[2] = a[2];
}
// xrot_withphase(sin, cos, phase, m0, m1): kernels.cuh:160-195
inline void rf_f(float s, float c, float ph, const float *a, float *b) {
    if (ph == 0.0f) { xrot_f(s, c, a, b); return; }
    if (ph == 180.0) { xrot_f(-s, c, a, b); return; }
    if (ph == 90.0) { yrot_f(s, c, a, b); return; }
    if (ph == -90.0 || ph == 270.0) { yrot_f(-s, c, a, b); return; }
    float t[3];
    float sp = sinf((float)(ph * kDeg2Rad)), cp = cosf((float)(ph * kDeg2Rad));
    zrot_f(-sp, cp, a, b);
    xrot_f(s, c, b, t);
    zrot_f(sp, cp, t, b);
}
// dephase_relax: kernels.cu:45-52 (zrot(float theta) = kernels.cuh:147-152; exp is the
// double ::exp, relax(e1,e2) = kernels.cuh:214-219 with its double constant 1.)
inline void dephase_relax_f(const float *a, float *b, float phase, float T1, float T2,
                            float dt_s) {
    float s = sinf((float)(phase * kDeg2Rad)), c = cosf((float)(phase * kDeg2Rad));
    zrot_f(s, c, a, b);
    if (T1 >= 0 && T2 >= 0) {
        float e1 = (float)std::exp((double)(-dt_s / T1));
        float e2 = (float)std::exp((double)(-dt_s / T2));
        b[0] = b[0] * e2;
        b[1] = b[1] * e2;
        b[2] = (float)(1. + e1 * (b[2] - 1.));
    }
}

// ---- double Bloch primitives (FP64 mode) --------------------------------------------------
inline void xrot_d(double s, double c, const double *a, double *b) {
    b[0] = a[0]; b[1] = c * a[1] - s * a[2]; b[2] = s * a[1] + c * a[2];
}
inline void yrot_d(double s, double c, const double *a, double *b) {
    b[0] = c * a[0] + s * a[2]; b[1] = a[1]; b[2] = -s * a[0] + c * a[2];
}
inline void zrot_d(double s, double c, const double *a, double *b) {
    b[0] = c * a[0] - s * a[1]; b[1] = s * a[0] + c * a[1]; b[2] = a[2];
}
inline void rf_d(double fa_deg, float ph, const double *a, double *b) {
    double s = std::sin(fa_deg * kDeg2Rad), c = std::cos(fa_deg * kDeg2Rad);
    if (ph == 0.0f) { xrot_d(s, c, a, b); return; }
    if (ph == 180.0) { xrot_d(-s, c, a, b); return; }
    if (ph == 90.0) { yrot_d(s, c, a, b); return; }
    if (ph == -90.0 || ph == 270.0) { yrot_d(-s, c, a, b); return; }
    double t[3], sp = std::sin(ph * kDeg2Rad), cp = std::cos(ph * kDeg2Rad);
    zrot_d(-sp, cp, a, b);
    xrot_d(s, c, b, t);
    zrot_d(sp, cp, t, b);
}
inline void dephase_relax_d(const double *a, double *b, double phase, double T1, double T2,
                            double dt_s) {
    zrot_d(std::sin(phase * kDeg2Rad), std::cos(phase * kDeg2Rad), a, b);
    if (T1 >= 0 && T2 >= 0) {
        double e1 = std::exp(-dt_s / T1), e2 = std::exp(-dt_s / T2);
        b[0] *= e2; b[1] *= e2; b[2] = 1. + e1 * (b[2] - 1.);
    }
}

// Compensated float sum (Knuth two-sum): value() = s + e.
struct KahanF {
    float s = 0.f, e = 0.f;
    void add(float x) {
        float t = s + x;
        float bp = t - s;
        e += (s - (t - bp)) + (x - bp);
        s = t;
    }
    float value() const { return s + e; }
    void reset() { s = e = 0.f; }
};

// Row-major linear index, truncating double -> int64 (kernels.cuh:53-60).
inline int64_t sub2ind(double x, double y, double z, const sw_params *p) {
    int64_t ix = (int64_t)x, iy = (int64_t)y, iz = (int64_t)z;
    int64_t ny = (int64_t)p->phantom_size[1], nz = (int64_t)p->phantom_size[2];
    return ix * nz * ny + iy * nz + iz;
}

// One spin, following kernels.cu:72-233 statement by statement.
template <typename Gen>
void sim_spin(const sw_params *P, const sw_sequence *Q, const float *fieldmap,
              const uint8_t *mask, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
              uint8_t *T, int32_t *status, uint32_t spin, int precision, double *M1d) {
    const uint64_t trj = P->enRecordTrajectory
                             ? (uint64_t)(P->n_dummy_scan + 1) * P->n_timepoints : 1;
    float *xyz1 = XYZ1 + 3ull * spin * trj;                        // kernels.cu:75
    Gen gen(P->seed + spin);                                       // :76-88

    const bool fp64 = precision == SW_PREC_FP64;
    const bool kahan = precision == SW_PREC_KAHAN;
    const bool shadow = M1d != nullptr || fp64;

    uint32_t itr = 0;
    float field = 0., T1 = 0., T2 = 0., rf_phase = Q->RF_PH_deg[0];  // :91
    float m0[3], m1[3];
    double xyz_old[3], xyz_new[3], s2g[3];
    double d0[3], d1[3];                                            // FP64 shadow state
    for (int i = 0; i < 3; i++) {                                   // :95-99
        xyz_old[i] = xyz_new[i] = xyz1[i] = XYZ0[3ull * spin + i];
        m0[i] = M0[3ull * spin + i];
        d0[i] = m0[i];
        s2g[i] = (double)P->phantom_size[i] / P->fov[i];
    }
    const int64_t ML = P->matrix_length;
    int64_t i0 = sub2ind(xyz1[0] * s2g[0], xyz1[1] * s2g[1], xyz1[2] * s2g[2], P);  // :102
    if (i0 < 0 || i0 >= ML) {            // the reference reads mask[] out of bounds here
        if (status) status[spin] = SW_SPIN_START_OOB;
        return;
    }
    uint8_t ts, ts_old;
    ts = ts_old = mask[i0];                                          // :103
    double dscale = Q->diffusivity[ts_old];                          // :104

    const uint32_t n_te = Q->n_TE;
    for (uint32_t ds = 0; ds < (uint32_t)(P->n_dummy_scan + 1); ds++) {   // :107
        const bool last = ds == (uint32_t)P->n_dummy_scan;
        float ph = (float)((double)(rf_phase + ds * P->linear_phase_cycling) +
                           ds * (ds + 1) / 2.0 * P->quadratic_phase_cycling);  // :110
        while (ph > 360.0) ph = (float)(ph - 360.0);                 // :111-114
        while (ph < 0) ph = (float)(ph + 360.0);
        rf_f(P->s, P->c, ph, m0, m1);                                // :117
        for (int i = 0; i < 3; i++) m0[i] = m1[i];                   // :119-120
        if (shadow) {
            rf_d(Q->RF_FA_deg[0], ph, d0, d1);
            for (int i = 0; i < 3; i++) d0[i] = d1[i];
        }
        int64_t ind = 0, ind_old = ML + 1;                           // :123-126
        uint32_t tp = 0, tp_old = 0;
        uint16_t c_rf = 1, c_te = 0, c_dph = 0, c_grad = 0;
        float acc = 0.f;
        KahanF acck;
        double accd = 0.;
        while (tp < P->n_timepoints) {                               // :128
            for (int i = 0; i < 3 && dscale != 0.; i++) {            // :130-137
                double rnd = gen.normal() * dscale;
                xyz_new[i] = xyz_old[i] + rnd;
                if (xyz_new[i] < 0)
                    xyz_new[i] += (P->enCrossFOV ? P->fov[i] : 2 * std::abs(rnd));
                else if (xyz_new[i] >= P->fov[i])
                    xyz_new[i] -= (P->enCrossFOV ? P->fov[i] : 2 * std::abs(rnd));
            }
            ind = sub2ind(xyz_new[0] * s2g[0], xyz_new[1] * s2g[1], xyz_new[2] * s2g[2], P);
            if (ind >= ML || ind < 0) {                              // :141-147
                if (status) status[spin] = SW_SPIN_OOB;
                return;
            }
            if (ind != ind_old) {                                    // :150-170
                ts = mask[ind];
                if (ts != ts_old) {
                    if (gen.uniform() >= Q->pXY[ts_old * P->n_substrate + ts]) {
                        if (itr++ > P->max_iterations) {
                            if (status) status[spin] = SW_SPIN_LOST;
                            return;
                        }
                        continue;
                    }
                    ts_old = ts;
                }
                ind_old = ind;
                field = fieldmap != nullptr ? fieldmap[ind] : 0.f;
                T1 = Q->T1_ms[ts_old] * 1e-3;
                T2 = Q->T2_ms[ts_old] * 1e-3;
                dscale = Q->diffusivity[ts_old];
            }
            acc += field;                                            // :171-172
            if (kahan) acck.add(field);
            if (shadow) accd += (double)field;
            itr = 0;
            if (c_dph < Q->n_dephasing && (uint32_t)Q->dephasing_us[c_dph] == tp) {   // :175
                acc += (float)spin * Q->dephasing_deg[c_dph] / (float)P->n_spins;
                if (kahan) acck.add((float)spin * Q->dephasing_deg[c_dph] / (float)P->n_spins);
                if (shadow) accd += (double)spin * Q->dephasing_deg[c_dph] / (double)P->n_spins;
                c_dph++;
            }
            if (c_grad < Q->n_gradient && (uint32_t)Q->gradient_us[c_grad] == tp) {  // :181
                const float Gx = Q->gradientX_mTm[c_grad], Gy = Q->gradientY_mTm[c_grad],
                            Gz = Q->gradientZ_mTm[c_grad];
                double g = (Gx * xyz_new[0] + Gy * xyz_new[1] + Gz * xyz_new[2]) * 1e-3 *
                           P->timestep_us * 1e-6 * kGamma * kRad2Deg;
                acc += g;
                if (kahan) {
                    float ghi = (float)g;
                    acck.add(ghi);
                    acck.add((float)(g - (double)ghi));
                }
                if (shadow) accd += g;
                c_grad++;
            }
            if (c_rf < Q->n_RF && (uint32_t)Q->RF_us[c_rf] == tp) {  // :190-199
                float te = (tp - tp_old) * P->timestep_us * 1e-6;
                dephase_relax_f(m0, m1, kahan ? acck.value() : acc, T1, T2, te);
                float fa = Q->RF_FA_deg[c_rf];
                rf_f((float)std::sin(fa * kDeg2Rad), (float)std::cos(fa * kDeg2Rad),
                     Q->RF_PH_deg[c_rf], m1, m0);
                if (shadow) {
                    double ted = (double)(tp - tp_old) * P->timestep_us * 1e-6;
                    dephase_relax_d(d0, d1, accd, Q->T1_ms[ts_old] * 1e-3,
                                    Q->T2_ms[ts_old] * 1e-3, ted);
                    rf_d(fa, Q->RF_PH_deg[c_rf], d1, d0);
                }
                acc = 0; acck.reset(); accd = 0;
                tp_old = tp;
                c_rf++;
            }
            if (last && c_te < n_te && (uint32_t)Q->TE_us[c_te] == tp) {   // :202-215
                float te = (tp - tp_old) * P->timestep_us * 1e-6;
                dephase_relax_f(m0, m1, kahan ? acck.value() : acc, T1, T2, te);
                if (shadow) {
                    double ted = (double)(tp - tp_old) * P->timestep_us * 1e-6;
                    dephase_relax_d(d0, d1, accd, Q->T1_ms[ts_old] * 1e-3,
                                    Q->T2_ms[ts_old] * 1e-3, ted);
                    for (int i = 0; i < 3; i++) d0[i] = d1[i];
                }
                for (uint32_t i = 0; i < 3; i++) {
                    uint64_t o = 3ull * n_te * spin + 3ull * c_te + i;
                    m0[i] = m1[i];
                    M1[o] = fp64 ? (float)d1[i] : m1[i];
                    if (M1d) M1d[o] = d1[i];
                }
                T[(uint64_t)spin * n_te + c_te] = ts_old;
                acc = 0; acck.reset(); accd = 0;
                tp_old = tp;
                c_te++;
            }
            if (P->enRecordTrajectory && (tp != 0 || ds != 0)) xyz1 += 3;   // :218-221
            for (int i = 0; i < 3; i++) xyz1[i] = (float)(xyz_old[i] = xyz_new[i]);
            tp++;
        }
        float te = (tp - tp_old) * P->timestep_us * 1e-6;            // :226-231
        dephase_relax_f(m0, m1, kahan ? acck.value() : acc, T1, T2, te);
        for (int i = 0; i < 3; i++) m0[i] = m1[i];
        if (shadow) {
            double ted = (double)(tp - tp_old) * P->timestep_us * 1e-6;
            dephase_relax_d(d0, d1, accd, Q->T1_ms[ts_old] * 1e-3, Q->T2_ms[ts_old] * 1e-3,
                            ted);
            for (int i = 0; i < 3; i++) d0[i] = d1[i];
        }
    }
    if (status) status[spin] = SW_SPIN_OK;
}

}  // namespace

extern "C" {

// All spins (spin_ids == NULL) or the listed spin ids; OpenMP dynamic over n_threads
// (<= 0: all). Outputs at the reference's per-spin offsets. Returns 0.
int oracle_sim(const sw_params *P, const sw_sequence *Q, const float *fieldmap,
               const uint8_t *mask, const float *M0, const float *XYZ0, float *M1,
               float *XYZ1, uint8_t *T, int32_t *status, const uint32_t *spin_ids,
               uint32_t n_ids, int n_threads, int precision, double *M1_fp64) {
    const int64_t n = spin_ids ? (int64_t)n_ids : (int64_t)P->n_spins;
    if (n_threads <= 0) n_threads = omp_get_max_threads();
    const float *fm = P->fieldmap_exist ? fieldmap : nullptr;
    const bool minstd = (precision & ~SW_PREC_MASK) == SW_RNG_MINSTD;
    precision &= SW_PREC_MASK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
    for (int64_t i = 0; i < n; i++) {
        uint32_t spin = spin_ids ? spin_ids[i] : (uint32_t)i;
        if (minstd)
            sim_spin<MinstdGen>(P, Q, fm, mask, M0, XYZ0, M1, XYZ1, T, status, spin, precision, M1_fp64);
        else
            sim_spin<StdGen>(P, Q, fm, mask, M0, XYZ0, M1, XYZ1, T, status, spin, precision, M1_fp64);
    }
    return 0;
}

// The driver-side initial positions of monte_carlo::initialize_position
// (src/sim/monte_carlo.cu:141-151): std::mt19937(seed), uniform_real_distribution<float> over
// [0.01*fov, 0.99*fov) per axis, drawn x,y,z per spin in spin order.
int oracle_initial_positions(const float fov[3], uint64_t seed, uint32_t n_spins, float *XYZ0) {
    std::mt19937 gen(seed);
    std::uniform_real_distribution<float> dx(0.01 * fov[0], 0.99 * fov[0]);
    std::uniform_real_distribution<float> dy(0.01 * fov[1], 0.99 * fov[1]);
    std::uniform_real_distribution<float> dz(0.01 * fov[2], 0.99 * fov[2]);
    for (uint64_t i = 0; i < n_spins; i++) {
        XYZ0[3 * i + 0] = dx(gen);
        XYZ0[3 * i + 1] = dy(gen);
        XYZ0[3 * i + 2] = dz(gen);
    }
    return 0;
}

// The state of std::mt19937(z) after discard(z), as kernels.cu:82-88 leaves each generator: the
// engine's 624-word buffer and position, read back through its stream output (libstdc++ writes
// the buffer then the position). Tests check the library's jump-ahead against it.
void oracle_mt_discard(uint64_t z, uint32_t *block, uint32_t *pos) {
    std::mt19937 gen((uint32_t)z);
    gen.discard(z);
    std::stringstream ss;
    ss << gen;
    for (int i = 0; i < 624; i++) ss >> block[i];
    ss >> *pos;
}

// glibc logf over a float array (the host libm the reference links): used by tests to check
// the GPU's bit-exact logf on the GPU host's own libm.
void oracle_logf(const float *x, float *y, uint64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) y[i] = logf(x[i]);
}

// The minstd flavour's Gaussian deviate of engine outputs x_lo .. x_lo + n - 1, with CUDA's host
// erfcinvf: the tests compare it with the device's on every engine output.
void oracle_ms_normal(uint32_t x_lo, uint32_t n, float *y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) y[i] = MinstdGen::normal_of(x_lo + (uint32_t)i);
}

}  // extern "C"
