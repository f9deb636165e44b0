// TEST INFRASTRUCTURE ONLY -- never linked into or called by the product library.
//
// ctypes-callable harness around the REFERENCE's own per-spin function sim::sim
// (src/sim/kernels.cu:72-233 of SpinWalk 1.21.0), compiled as C++ from the read-only source
// tree by oracle/Makefile (the CPU-only "Flavour A" build: std::mt19937 + libstdc++
// normal_distribution<float>, exactly as CMakeLists.txt:57-70 builds it without CUDA).
// Output goes to oracle/_ref/libref_sim.so. Used to generate the golden fixtures under
// tests/golden/ and to pin the restatement in oracle/sim_oracle.cpp.
//
// This file is project-written: it converts the flat C-ABI structs (include/spinwalk_gpu.h)
// into the reference's own `parameters` / `parameters_uvec` and calls sim::sim per spin,
// replicating the per-scale loop of monte_carlo::run (src/sim/monte_carlo.cu:313-321).
// It also exposes the reference's config_reader (src/sim/config_reader.cpp) so the INI
// semantics of the product host can be checked against it.

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <omp.h>

#include "kernels.cuh"          // reference: src/sim/kernels.cuh
#include "config_reader.h"      // reference: src/sim/config_reader.h
#include "spinwalk_gpu.h"       // project: include/spinwalk_gpu.h (struct layouts only)

namespace {

void to_reference(const sw_params *p, const sw_sequence *q, parameters &param,
                  parameters_uvec &u) {
    for (int i = 0; i < 3; i++) {
        param.fov[i] = p->fov[i];
        param.phantom_size[i] = (size_t)p->phantom_size[i];
    }
    param.B0 = p->B0;
    param.c = p->c;
    param.s = p->s;
    param.linear_phase_cycling = p->linear_phase_cycling;
    param.quadratic_phase_cycling = p->quadratic_phase_cycling;
    param.timestep_us = p->timestep_us;
    param.TR_us = p->TR_us;
    param.n_dummy_scan = p->n_dummy_scan;
    param.n_spins = p->n_spins;
    param.n_timepoints = p->n_timepoints;
    param.n_substrate = p->n_substrate;
    param.n_scales = p->n_scales;
    param.seed = (size_t)p->seed;
    param.max_iterations = (size_t)p->max_iterations;
    param.matrix_length = p->matrix_length;
    param.enCrossFOV = p->enCrossFOV != 0;
    param.enRecordTrajectory = p->enRecordTrajectory != 0;
    param.fieldmap_exist = p->fieldmap_exist != 0;

    u.diffusivity = {q->diffusivity, p->n_substrate};
    u.T1_ms = {q->T1_ms, p->n_substrate};
    u.T2_ms = {q->T2_ms, p->n_substrate};
    u.pXY = {q->pXY, (size_t)p->n_substrate * p->n_substrate};
    u.RF_FA_deg = {q->RF_FA_deg, q->n_RF};
    u.RF_PH_deg = {q->RF_PH_deg, q->n_RF};
    u.RF_us = {q->RF_us, q->n_RF};
    u.TE_us = {q->TE_us, q->n_TE};
    u.dephasing_deg = {q->dephasing_deg, q->n_dephasing};
    u.dephasing_us = {q->dephasing_us, q->n_dephasing};
    u.gradientX_mTm = {q->gradientX_mTm, q->n_gradient};
    u.gradientY_mTm = {q->gradientY_mTm, q->n_gradient};
    u.gradientZ_mTm = {q->gradientZ_mTm, q->n_gradient};
    u.gradient_us = {q->gradient_us, q->n_gradient};
}

}  // namespace

extern "C" {

// Runs the reference sim::sim for the listed spin ids (all spins when spin_ids == NULL),
// OpenMP dynamic schedule over n_threads (<=0: all cores). Output slicing as in the reference:
// spin s writes M1[3*nTE*s..], XYZ1[3*s*trj..], T[nTE*s..].
int ref_sim(const sw_params *p, const sw_sequence *q, const float *pFieldMap,
            const uint8_t *pMask, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
            uint8_t *T, const uint32_t *spin_ids, uint32_t n_ids, int n_threads) {
    parameters param;
    parameters_uvec u;
    to_reference(p, q, param, u);
    const int64_t n = spin_ids ? (int64_t)n_ids : (int64_t)p->n_spins;
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
    for (int64_t i = 0; i < n; i++) {
        uint32_t spin = spin_ids ? spin_ids[i] : (uint32_t)i;
        sim::sim(param, u, p->fieldmap_exist ? pFieldMap : nullptr, pMask, M0, XYZ0, M1, XYZ1,
                 T, spin);
    }
    return 0;
}

// Reads an INI file with the reference config_reader (prepare = read + check + timing_scale,
// src/sim/config_reader.cpp:25-37) and writes a flat text dump of the resulting parameters to
// out_path, one `key value...` line per field. Returns 1 on success, 0 when the reader
// rejects the file.
int ref_config_dump(const char *ini_path, const char *out_path) {
    sim::config_reader cfg;
    parameters param;
    parameters_hvec hv;
    bool ok = cfg.prepare(ini_path, &param, &hv);
    FILE *f = std::fopen(out_path, "w");
    if (!f) return -1;
    std::fprintf(f, "ok %d\n", ok ? 1 : 0);
    if (ok) {
        std::fprintf(f, "TR_us %d\ntimestep_us %d\nn_dummy_scan %d\n", param.TR_us,
                     param.timestep_us, param.n_dummy_scan);
        std::fprintf(f, "linear_phase_cycling %.9g\nquadratic_phase_cycling %.9g\n",
                     param.linear_phase_cycling, param.quadratic_phase_cycling);
        std::fprintf(f, "B0 %.9g\nseed %zu\nn_spins %u\nenCrossFOV %d\n", param.B0,
                     param.seed, param.n_spins, (int)param.enCrossFOV);
        std::fprintf(f, "enRecordTrajectory %d\nmax_iterations %zu\nn_substrate %u\n",
                     (int)param.enRecordTrajectory, param.max_iterations, param.n_substrate);
        std::fprintf(f, "n_scales %u\nscale_type %d\n", param.n_scales,
                     (int)cfg.get_scale_type());
        auto dumpf = [f](const char *k, const std::vector<float> &v) {
            std::fprintf(f, "%s", k);
            for (float x : v) std::fprintf(f, " %.9g", x);
            std::fprintf(f, "\n");
        };
        auto dumpi = [f](const char *k, const std::vector<int32_t> &v) {
            std::fprintf(f, "%s", k);
            for (int32_t x : v) std::fprintf(f, " %d", x);
            std::fprintf(f, "\n");
        };
        std::fprintf(f, "diffusivity");
        for (double x : hv.diffusivity) std::fprintf(f, " %.17g", x);
        std::fprintf(f, "\n");
        dumpf("scales", cfg.get_scales());
        dumpf("T1_ms", hv.T1_ms);
        dumpf("T2_ms", hv.T2_ms);
        dumpf("pXY", hv.pXY);
        dumpf("RF_FA_deg", hv.RF_FA_deg);
        dumpf("RF_PH_deg", hv.RF_PH_deg);
        dumpi("RF_us", hv.RF_us);
        dumpi("TE_us", hv.TE_us);
        dumpf("dephasing_deg", hv.dephasing_deg);
        dumpi("dephasing_us", hv.dephasing_us);
        dumpf("gradientX_mTm", hv.gradientX_mTm);
        dumpf("gradientY_mTm", hv.gradientY_mTm);
        dumpf("gradientZ_mTm", hv.gradientZ_mTm);
        dumpi("gradient_us", hv.gradient_us);
        for (const char *key : {"PHANTOM", "XYZ0", "M0"}) {
            auto v = cfg.get_filename(key);
            std::fprintf(f, "%s %zu\n", key, v.size());
            for (auto &s : v) std::fprintf(f, "  %s\n", s.c_str());
        }
        for (size_t i = 0; i < cfg.get_filename("PHANTOM").size(); i++)
            std::fprintf(f, "output %s\n", cfg.get_output_filename(i).c_str());
    }
    std::fclose(f);
    return ok ? 1 : 0;
}

}  // extern "C"
