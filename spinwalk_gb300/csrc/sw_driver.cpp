// sw_run_config: the reference's sim::monte_carlo::run (src/sim/monte_carlo.cu:199-355) on top
// of the GPU entry points -- config, phantoms, initial positions, fieldmap scaling, the scale
// loop and the HDF5 outputs -- plus the HDF5 helpers of the C ABI.
//
// Phase-cycling scales (WHAT_TO_SCALE = 2) and gradient scales (up to 8 distinct ones) walk
// identically, so they run as tracks of one walk (sw_sim_tracks, bit-identical to one run per
// scale; gradient scales keep one phase per scale); FoV scales, and repeated or more gradient
// scales, run as one sw_sim_batch (one walk per scale, one seeding for all), also bit-identical.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <filesystem>
#include <limits>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "spinwalk_gpu.h"
#include "sw_config.h"
#include "sw_h5.h"

namespace sw {
namespace api {
int fail(int code, const std::string &msg);   // sets sw_last_error() (sw_api.cu)
}  // namespace api
}  // namespace sw

namespace {

// Reports on stderr, as the reference's driver logs, and sets sw_last_error().
int drv_fail(int rc, const std::string &m) {
    std::fprintf(stderr, "spinwalk: %s\n", m.c_str());
    return sw::api::fail(rc, m);
}



template <typename T>
sw::h5::Dataset make_ds(const std::vector<uint64_t> &dims, const std::vector<T> &v, sw::h5::Type t) {
    sw::h5::Dataset d;
    d.dims = dims;
    d.type = t;
    d.data.resize(v.size() * sizeof(T));
    std::memcpy(d.data.data(), v.data(), d.data.size());
    return d;
}

}  // namespace

static int run_config_impl(const char *ini_path, int device) {
    using clock = std::chrono::steady_clock;
    const auto t_run = clock::now();
    if (!ini_path) return drv_fail(SW_ERR_INVALID, "no config file");
    bool device_set = false;        // selected before the first simulation, after the inputs
    sw::Config c;
    std::string err;
    int rc = sw::config_read(ini_path, c, err);
    if (rc) return drv_fail(rc, err);
    sw_params p = c.p;
    std::vector<double> dscale = c.diffusivity;
    rc = sw_prepare_params(&p, dscale.data(), c.RF_FA_deg.data(), c.T1_ms.data());  // :205
    if (rc) return drv_fail(rc, "parameters::prepare failed");

    const size_t n = p.n_spins, nte = c.TE_us.size(), ns = c.scales.size();
    const size_t trj = p.enRecordTrajectory ? (size_t)p.n_timepoints * (p.n_dummy_scan + 1) : 1;
    // allocate_memory (monte_carlo.cu:61-70): once per run, NOT cleared between phantoms
    std::vector<float> XYZ0(n * 3), XYZ0s(n * 3), XYZ1(trj * ns * n * 3), M0(n * 3),
        M1(ns * nte * n * 3);
    std::vector<uint8_t> T(ns * nte * n);
    const std::vector<float> gx0 = c.gradientX_mTm, gy0 = c.gradientY_mTm, gz0 = c.gradientZ_mTm;
    const float lin0 = p.linear_phase_cycling, quad0 = p.quadratic_phase_cycling;

    const auto &phantoms = c.files["PHANTOM"];
    for (size_t ip = 0; ip < phantoms.size(); ip++) {
        const std::string &ph = phantoms[ip];
        std::fprintf(stderr, "spinwalk: simulating phantom %s\n", ph.c_str());
        // read_phantom (monte_carlo.cu:98-123)
        std::vector<float> field, fov;
        std::vector<uint8_t> mask;
        std::vector<uint64_t> dims;
        // the fieldmap is optional: absent means none, present but unreadable is an error
        if (!sw::h5::exists(ph, "fieldmap")) field.clear();
        else if (!sw::h5::read_as(ph, "fieldmap", field, nullptr, err)) return drv_fail(SW_ERR_IO, err);
        if (!sw::h5::read_as(ph, "mask", mask, &dims, err)) return drv_fail(SW_ERR_IO, err);
        if (!sw::h5::read_as(ph, "fov", fov, nullptr, err)) return drv_fail(SW_ERR_IO, err);
        // h5_helper::read without resizing (h5_helper.h:59-66): fov holds exactly 3 values
        if (fov.size() != 3)
            return drv_fail(SW_ERR_IO, ph + ": dataset \"fov\" has different size " +
                                           std::to_string(fov.size()) + " vs 3");
        if (dims.size() != 3) return drv_fail(SW_ERR_IO, ph + ": mask must be 3-D");
        // the reference indexes the fieldmap with the mask's voxel index and never checks
        // their sizes; a shorter fieldmap would be read past its end, so it is refused
        if (!field.empty() && field.size() != mask.size())
            return drv_fail(SW_ERR_INVALID, ph + ": fieldmap has " + std::to_string(field.size()) +
                                                " voxels, mask " + std::to_string(mask.size()));
        for (int i = 0; i < 3; i++) p.phantom_size[i] = dims[i];
        const uint32_t nsub = mask.empty() ? 0 : (uint32_t)*std::max_element(mask.begin(), mask.end()) + 1;
        if (nsub > p.n_substrate)
            return drv_fail(SW_ERR_INVALID, "the mask holds more substrate types than the config defines");
        // initialize_position (monte_carlo.cu:125-153)
        const std::string &xf = c.files["XYZ0"][ip];
        if (!xf.empty()) {
            std::vector<float> x;
            if (!sw::h5::read_as(xf, "XYZ", x, nullptr, err)) return drv_fail(SW_ERR_IO, err);
            if (x.size() != XYZ0.size())           // h5_helper::read without resizing
                return drv_fail(SW_ERR_IO, xf + ": dataset \"XYZ\" has different size " +
                                               std::to_string(x.size()) + " vs " +
                                               std::to_string(XYZ0.size()));
            std::copy(x.begin(), x.end(), XYZ0.begin());
            for (size_t i = 0; i < XYZ0.size(); i++)
                if (XYZ0[i] < 0 || XYZ0[i] > fov[i % 3])
                    return drv_fail(SW_ERR_INVALID, "Initial positions are outside the FoV.");
        } else {
            sw_initial_positions(fov.data(), p.seed, p.n_spins, XYZ0.data());
        }
        // initialize_magnetization (monte_carlo.cu:155-166): the file is read, then every M0 is
        // set to (0, 0, 1) regardless -- kept as the reference does it
        const std::string &mf = c.files["M0"][ip];
        if (!mf.empty()) {
            std::vector<float> m;
            if (!sw::h5::read_as(mf, "M", m, nullptr, err)) return drv_fail(SW_ERR_IO, err);
            if (m.size() != M0.size())              // h5_helper::read without resizing
                return drv_fail(SW_ERR_IO, mf + ": dataset \"M\" has different size " +
                                               std::to_string(m.size()) + " vs " +
                                               std::to_string(M0.size()));
        }
        for (size_t i = 0; i < M0.size(); i++) M0[i] = (i % 3 == 2) ? 1.f : 0.f;
        if (!device_set) {
            if (cudaSetDevice(device) != cudaSuccess) {
                cudaGetLastError();
                return drv_fail(SW_ERR_CUDA, "device " + std::to_string(device) + " is not available");
            }
            device_set = true;
        }
        XYZ0s = XYZ0;
        p.matrix_length = (int64_t)mask.size();
        p.fieldmap_exist = field.empty() ? 0 : 1;
        const float t2d = sw_fieldmap_scale(p.B0, p.timestep_us);          // :241-244
        for (auto &v : field) v = v * t2d;
        for (int i = 0; i < 3; i++) p.fov[i] = fov[i];

        sw_sequence q{};
        q.diffusivity = dscale.data();
        q.T1_ms = c.T1_ms.data();
        q.T2_ms = c.T2_ms.data();
        q.pXY = c.pXY.data();
        q.RF_FA_deg = c.RF_FA_deg.data();
        q.RF_PH_deg = c.RF_PH_deg.data();
        q.RF_us = c.RF_us.data();
        q.n_RF = (uint32_t)c.RF_us.size();
        q.TE_us = c.TE_us.data();
        q.n_TE = (uint32_t)nte;
        q.dephasing_deg = c.dephasing_deg.data();
        q.dephasing_us = c.dephasing_us.data();
        q.n_dephasing = (uint32_t)c.dephasing_us.size();
        q.gradient_us = c.gradient_us.data();
        q.n_gradient = (uint32_t)c.gradient_us.size();
        std::vector<float> gx = gx0, gy = gy0, gz = gz0;
        q.gradientX_mTm = gx.data();
        q.gradientY_mTm = gy.data();
        q.gradientZ_mTm = gz.data();

        const auto t_sim = clock::now();
        // phase-cycling scales, and up to 8 distinct gradient scales, share one walk (tracks);
        // repeated scales would be duplicate tracks, so they take the batch below
        std::vector<float> sorted_scales(c.scales.begin(), c.scales.end());
        std::sort(sorted_scales.begin(), sorted_scales.end());
        const bool distinct = std::adjacent_find(sorted_scales.begin(), sorted_scales.end()) ==
                              sorted_scales.end();
        const bool share = (c.scale_type == 2 || (c.scale_type == 1 && ns <= 8)) && distinct;
        if (share && !p.enRecordTrajectory && ns > 1) {
            // one walk, one track per scale
            std::vector<sw_track> tracks(ns);
            std::vector<std::vector<float>> xyz(ns, std::vector<float>(n * 3));
            for (size_t k = 0; k < ns; k++) {
                sw_track &t = tracks[k];
                t = sw_track{};
                t.linear_phase_cycling = c.scale_type == 2 ? lin0 * c.scales[k] : lin0;
                t.quadratic_phase_cycling = quad0;
                if (c.scale_type == 1) {
                    t.gradient_scale = c.scales[k];
                    t.options = SW_TRACK_GRADIENT_SCALE;
                }
                t.n_dummy_scan = p.n_dummy_scan;
                t.M1 = M1.data() + 3 * nte * n * k;
                t.T = T.data() + nte * n * k;
                t.XYZ1 = xyz[k].data();
            }
            rc = sw_sim_tracks(&p, &q, tracks.data(), (uint32_t)ns, field.empty() ? nullptr : field.data(),
                               mask.data(), M0.data(), XYZ0s.data(), SW_PREC_FP32);
            if (rc) return drv_fail(rc, sw_last_error());
            for (size_t k = 0; k < ns; k++)
                std::copy(xyz[k].begin(), xyz[k].end(), XYZ1.begin() + 3 * n * trj * k);
        } else {
            // the scale loop (:273-337) as one batch: every scale is its own walk, but the
            // phantom is packed and the generators seeded once for all scales
            std::vector<sw_params> ps(ns, p);
            std::vector<sw_sequence> qs(ns, q);
            std::vector<std::vector<float>> xyz(ns), gxs(ns), gys(ns), gzs(ns);
            std::vector<sw_instance> items(ns);
            for (size_t k = 0; k < ns; k++) {
                const float scale = c.scales[k];
                xyz[k] = XYZ0;
                if (c.scale_type == 0) {
                    for (size_t i = 0; i < XYZ0.size(); i++) xyz[k][i] = XYZ0[i] * scale;
                    for (int i = 0; i < 3; i++) ps[k].fov[i] = scale * fov[i];
                } else if (c.scale_type == 1) {
                    gxs[k] = gx0;
                    gys[k] = gy0;
                    gzs[k] = gz0;
                    for (size_t i = 0; i < gx0.size(); i++) {
                        gxs[k][i] = gx0[i] * scale;
                        gys[k][i] = gy0[i] * scale;
                        gzs[k][i] = gz0[i] * scale;
                    }
                    qs[k].gradientX_mTm = gxs[k].data();
                    qs[k].gradientY_mTm = gys[k].data();
                    qs[k].gradientZ_mTm = gzs[k].data();
                } else {
                    ps[k].linear_phase_cycling = lin0 * scale;
                    ps[k].quadratic_phase_cycling = quad0;
                }
                sw_instance &it = items[k];
                it.param = &ps[k];
                it.seq = &qs[k];
                it.M0 = M0.data();
                it.XYZ0 = xyz[k].data();
                it.M1 = M1.data() + 3 * nte * n * k;
                it.XYZ1 = XYZ1.data() + 3 * n * trj * k;
                it.T = T.data() + nte * n * k;
                it.status = nullptr;
            }
            rc = sw_sim_batch(items.data(), (uint32_t)ns, field.empty() ? nullptr : field.data(),
                              mask.data(), SW_PREC_FP32);
            if (rc) return drv_fail(rc, sw_last_error());
        }
        const double sim_s = std::chrono::duration<double>(clock::now() - t_sim).count();
        std::fprintf(stderr, "spinwalk: simulation took %.3f s\n", sim_s);

        // save (monte_carlo.cu:168-197)
        std::vector<float> te_s;
        for (size_t i = 0; i < nte; i++) te_s.push_back(c.TE_us[i] * p.timestep_us * 1e-6);
        std::vector<std::pair<std::string, sw::h5::Dataset>> sets;
        sets.push_back({"M", make_ds({ns, n, nte, 3}, M1, sw::h5::kF32)});
        sets.push_back({"XYZ", make_ds({ns, n, trj, 3}, XYZ1, sw::h5::kF32)});
        sets.push_back({"T", make_ds({ns, n, nte, 1}, T, sw::h5::kU8)});
        sets.push_back({"scales", make_ds({ns, 1, 1, 1}, c.scales, sw::h5::kF32)});
        sets.push_back({"TE", make_ds({nte, 1, 1, 1}, te_s, sw::h5::kF32)});
        const std::string &out = c.outputs[ip];
        std::error_code ec;
        std::filesystem::remove(out, ec);
        if (!sw::h5::write(out, sets, err)) return drv_fail(SW_ERR_IO, err);
        std::fprintf(stderr, "spinwalk: wrote %s\n", out.c_str());
    }
    std::fprintf(stderr, "spinwalk: entire run took %.3f s\n",
                 std::chrono::duration<double>(clock::now() - t_run).count());
    return SW_OK;
}

static int h5_write_impl(const char *path, int n, const char *const *names, const int *types,
                           const int *ranks, const uint64_t *dims, const void *const *data) {
    if (!path || n < 0) return drv_fail(SW_ERR_INVALID, "sw_h5_write: null path or negative count");
    std::vector<std::pair<std::string, sw::h5::Dataset>> sets;
    size_t dpos = 0;
    for (int i = 0; i < n; i++) {
        sw::h5::Dataset d;
        if (!sw::h5::valid_type(types[i]))
            return drv_fail(SW_ERR_INVALID, std::string("dataset ") + names[i] + ": unknown type code");
        d.type = (sw::h5::Type)types[i];
        uint64_t cnt = 1;
        for (int r = 0; r < ranks[i]; r++) {
            d.dims.push_back(dims[dpos + r]);
            cnt *= dims[dpos + r];
        }
        dpos += ranks[i];
        const size_t esz = sw::h5::type_size(d.type);
        d.data.resize(cnt * esz);
        if (cnt) std::memcpy(d.data.data(), data[i], cnt * esz);
        sets.push_back({names[i], std::move(d)});
    }
    std::string err;
    if (!sw::h5::write(path, sets, err)) return drv_fail(SW_ERR_IO, err);
    return SW_OK;
}

static int h5_read_impl(const char *path, const char *name, int *type, int *rank,
                          uint64_t dims[8], void *out, uint64_t out_bytes) {
    sw::h5::Dataset d;
    std::string err;
    if (!path || !name) return drv_fail(SW_ERR_INVALID, "sw_h5_read: null path or name");
    if (!sw::h5::read(path, name, d, err, out != nullptr)) return drv_fail(SW_ERR_IO, err);
    if (d.dims.size() > 8) return drv_fail(SW_ERR_IO, "rank > 8");
    if (type) *type = (int)d.type;
    if (rank) *rank = (int)d.dims.size();
    if (dims)
        for (size_t i = 0; i < d.dims.size(); i++) dims[i] = d.dims[i];
    if (out) {
        if (out_bytes < d.data.size()) return drv_fail(SW_ERR_INVALID, "output buffer too small");
        std::memcpy(out, d.data.data(), d.data.size());
    }
    return SW_OK;
}

// The C ABI never lets an exception out (an allocation that fails for a huge NUMBER_OF_SPINS,
// for instance): it becomes an error code and a message.
template <typename F>
static int guarded(const char *what, F &&f) {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        return drv_fail(SW_ERR_NOMEM, std::string(what) + ": out of host memory");
    } catch (const std::exception &e) {
        return drv_fail(SW_ERR_IO, std::string(what) + ": " + e.what());
    }
}

extern "C" int sw_run_config(const char *ini_path, int device) {
    return guarded("sw_run_config", [&] { return run_config_impl(ini_path, device); });
}

extern "C" int sw_h5_write(const char *path, int n, const char *const *names, const int *types,
                           const int *ranks, const uint64_t *dims, const void *const *data) {
    return guarded("sw_h5_write", [&] { return h5_write_impl(path, n, names, types, ranks, dims, data); });
}

extern "C" int sw_h5_read(const char *path, const char *name, int *type, int *rank,
                          uint64_t dims[8], void *out, uint64_t out_bytes) {
    return guarded("sw_h5_read", [&] { return h5_read_impl(path, name, type, rank, dims, out, out_bytes); });
}

extern "C" int sw_device_info(int device, char *buf, uint64_t len) {
    if (!buf || len == 0) return drv_fail(SW_ERR_INVALID, "sw_device_info: no buffer");
    auto ver = [](int v) { return std::to_string(v / 1000) + "." + std::to_string((v % 1000) / 10); };
    int rt = 0, drv = 0, n = 0;
    cudaRuntimeGetVersion(&rt);
    cudaDriverGetVersion(&drv);
    std::string t = "The latest version of CUDA supported by the driver: " + ver(drv) +
                    ", current CUDA version: " + ver(rt) + "\n";
    int rc = SW_OK;
    if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
    cudaGetLastError();
    t += "Number of devices: " + std::to_string(n) + "\n";
    cudaDeviceProp prop;
    size_t free_b = 0, total_b = 0;
    int prev = -1;                           // the caller's current device, restored below
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaGetLastError();
    if (device < 0 || device >= n) {
        rc = SW_ERR_CUDA;
        t += "device " + std::to_string(device) + " is not available\n";
    } else if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || cudaSetDevice(device) != cudaSuccess ||
               cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        rc = SW_ERR_CUDA;
        t += "device " + std::to_string(device) + ": properties not available\n";
    } else {
        t += std::string(prop.name) + "\n-Compute Capability: " + std::to_string(prop.major) + "." +
             std::to_string(prop.minor) + "\n-Free GPU Memory: " + std::to_string(free_b >> 20) +
             " MB (out of " + std::to_string(total_b >> 20) + " MB)\n";
    }
    if (prev >= 0 && prev != device) {
        cudaSetDevice(prev);
        cudaGetLastError();
    }
    std::snprintf(buf, (size_t)len, "%s", t.c_str());
    if (rc) return sw::api::fail(rc, "device " + std::to_string(device) + " is not available");
    return SW_OK;
}
