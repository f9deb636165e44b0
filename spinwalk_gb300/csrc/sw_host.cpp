// Host-side C++ of libspinwalk_gpu: parameter preparation with the reference's arithmetic, RF
// rotation tables computed with the host libm, the driver's initial spin positions, and the
// exception list that makes the device logf equal to the host libm's logf.
//
// Compiled with -ffp-contract=off so every float/double expression rounds like the reference's
// CPU build.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include <omp.h>

#include "spinwalk_gpu.h"
#include "sw_host.h"
#include "sw_logf.h"

namespace sw {

static const float kLogfTab[192] = SW_LOGF_TABLE_INIT;

const float *logf_reduction_table() { return kLogfTab; }

// Marks every float x in [2^-48, 1] where the host logf differs from logf_cand, and checks that
// the candidate's neighbour towards the exact value (swlogf::neighbour) is the libm result
// there. Built once per process (~4e8 evaluations, about a second on all cores).
const LogfExceptions &logf_exceptions() {
    static LogfExceptions ex;
    static std::once_flag once;
    std::call_once(once, [] {
        const uint32_t nw = swlogf::kBitmapWords;
        ex.bitmap.assign(nw, 0u);
        uint64_t count = 0, wide = 0;
#pragma omp parallel for schedule(static) reduction(+ : count, wide)
        for (int64_t w = 0; w < (int64_t)nw; w++) {
            uint32_t word = 0;
            for (uint32_t b = 0; b < 32; b++) {
                const uint32_t bits = swlogf::kDomainLo + ((uint32_t)w << 5) + b;
                if (bits > swlogf::kDomainHi) break;
                const float x = swlogf::u2f(bits);
                const float g = logf(x);
                bool above;
                const float c = swlogf::logf_cand(x, kLogfTab, above);
                if (swlogf::f2u(g) != swlogf::f2u(c)) {
                    word |= 1u << b;
                    count++;
                    if (swlogf::f2u(swlogf::neighbour(c, above)) != swlogf::f2u(g)) wide++;
                }
            }
            ex.bitmap[w] = word;
        }
        ex.count = count;
        ex.wide = wide;
    });
    return ex;
}

// xrot_withphase(sin, cos, phase, ...) branch selection and trigonometry
// (src/sim/kernels.cuh:160-195): the float path uses sinf/cosf of float(phase*DEG2RAD); the
// FP64 path uses the double sin/cos of the same phase.
RfOp make_rf_op(float s, float c, double fa_deg, float ph, int32_t tp) {
    RfOp op{};
    op.tp = tp;
    op.s = s;
    op.c = c;
    op.sd = std::sin(fa_deg * kDeg2Rad);
    op.cd = std::cos(fa_deg * kDeg2Rad);
    if (ph == 0.0f) op.kind = 0;
    else if (ph == 180.0) op.kind = 1;
    else if (ph == 90.0) op.kind = 2;
    else if (ph == -90.0 || ph == 270.0) op.kind = 3;
    else op.kind = 4;
    const float a = (float)(ph * kDeg2Rad);
    op.sp = sinf(a);
    op.cp = cosf(a);
    op.spd = std::sin((double)ph * kDeg2Rad);
    op.cpd = std::cos((double)ph * kDeg2Rad);
    return op;
}

// The scan-start pulse of every dummy scan, with phase cycling (kernels.cu:110-117).
void build_scan_rf(const sw_params *p, const sw_sequence *q, std::vector<RfOp> &out) {
    const uint32_t n = (uint32_t)(p->n_dummy_scan + 1);
    out.resize(n);
    const float rf_phase = q->RF_PH_deg[0];
    for (uint32_t ds = 0; ds < n; ds++) {
        float ph = (float)((double)(rf_phase + ds * p->linear_phase_cycling) +
                           ds * (ds + 1) / 2.0 * p->quadratic_phase_cycling);
        while (ph > 360.0) ph = (float)(ph - 360.0);
        while (ph < 0) ph = (float)(ph + 360.0);
        out[ds] = make_rf_op(p->s, p->c, (double)q->RF_FA_deg[0], ph, 0);
    }
}

// RF pulses k >= 1 (kernels.cu:190-199 -> kernels.cuh:203-206: sin/cos of theta*DEG2RAD in
// double, passed on as float).
void build_rf(const sw_params *, const sw_sequence *q, std::vector<RfOp> &out) {
    out.resize(q->n_RF);
    for (uint32_t k = 0; k < q->n_RF; k++) {
        const float fa = q->RF_FA_deg[k];
        const float s = (float)std::sin(fa * kDeg2Rad), c = (float)std::cos(fa * kDeg2Rad);
        out[k] = make_rf_op(s, c, (double)fa, q->RF_PH_deg[k], q->RF_us[k]);
    }
}

}  // namespace sw

namespace sw {
namespace api {
int fail(int code, const std::string &msg);   // sets sw_last_error() (sw_api.cu)
}  // namespace api
}  // namespace sw

extern "C" {

float sw_fieldmap_scale(float B0, int32_t timestep_us) {
    // src/sim/monte_carlo.cu:241: float * int32 -> float, then double factors
    return B0 * timestep_us * 1e-6 * sw::kGamma * sw::kRad2Deg;
}

int sw_prepare_params(sw_params *p, double *diffusivity, const float *RF_FA_deg,
                      const float *T1_ms) {
    if (!p || !RF_FA_deg || !T1_ms || !diffusivity)
        return sw::api::fail(SW_ERR_INVALID, "sw_prepare_params: null argument");
    if (p->timestep_us <= 0)
        return sw::api::fail(SW_ERR_INVALID, "sw_prepare_params: TIME_STEP must be positive");
    p->c = cosf(RF_FA_deg[0] * sw::kDeg2Rad);              // simulation_parameters.cuh:229-230
    p->s = sinf(RF_FA_deg[0] * sw::kDeg2Rad);
    p->n_timepoints = p->TR_us / p->timestep_us;           // :231
    if (p->seed == 0) p->seed = std::random_device{}();    // :233-234
    for (uint32_t i = 0; i < p->n_substrate; i++)          // :236-237
        diffusivity[i] = 1e-3 * std::sqrt(2. * diffusivity[i] * p->timestep_us);
    if (p->n_dummy_scan < 0)                               // :239-242
        p->n_dummy_scan = 5.0 * T1_ms[0] / float(p->TR_us * 1e-3);
    return SW_OK;
}

// monte_carlo::initialize_position without a file (src/sim/monte_carlo.cu:141-151).
int sw_initial_positions(const float fov[3], uint64_t seed, uint32_t n_spins, float *XYZ0) {
    if (!fov || !XYZ0) return sw::api::fail(SW_ERR_INVALID, "sw_initial_positions: null argument");
    std::mt19937 gen(seed);
    std::uniform_real_distribution<float> dx(0.01 * fov[0], 0.99 * fov[0]);
    std::uniform_real_distribution<float> dy(0.01 * fov[1], 0.99 * fov[1]);
    std::uniform_real_distribution<float> dz(0.01 * fov[2], 0.99 * fov[2]);
    for (uint64_t i = 0; i < n_spins; i++) {
        XYZ0[3 * i + 0] = dx(gen);
        XYZ0[3 * i + 1] = dy(gen);
        XYZ0[3 * i + 2] = dz(gen);
    }
    return SW_OK;
}

int sw_logf_exception_count(uint64_t *count, uint64_t *wide) {
    const sw::LogfExceptions &ex = sw::logf_exceptions();
    if (count) *count = ex.count;
    if (wide) *wide = ex.wide;
    return SW_OK;
}

}  // extern "C"
