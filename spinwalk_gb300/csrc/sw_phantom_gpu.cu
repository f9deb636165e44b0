// The reference's phantom generators (src/phantom/phantom_cylinder.cpp, phantom_sphere.cpp,
// phantom_base.cpp) with the mask and field computed on the GPU.
//
// Shape placement stays on the host, as the reference does it: the same engine and
// distribution (std::mt19937 / std::minstd_rand, uniform_real_distribution<float>), the same
// rejection of overlapping shapes and, for cylinders, the same voxel-counted volumes; it is
// sequential, cheap, and decides the shapes. (With random radii the reference adjusts a radius
// inside an OpenMP loop whose outcome depends on thread timing; the sequential order here is
// the reference run on one thread.)
//
// The mask and field are then one GPU thread per voxel that visits the shapes in the
// reference's order and adds each contribution with the reference's operation sequence: float
// vector arithmetic, then the double-precision field expression, then the float accumulation
// `field += double` (phantom_cylinder.cpp:241-260, phantom_sphere.cpp:177-187). Every operation
// is a separately rounded IEEE operation (-fmad=false) and the only irrational ones are square
// roots (correctly rounded on both sides) and cos(theta), computed on the host, so mask and
// field are bit-identical to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"

using sw::api::fail;

namespace {

#define PH_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr double kPi = 3.14159265358979323846;   // M_PI of the reference (phantom_base.h:17)
constexpr uint64_t kMaxAttempts = 200000000ull;   // the reference loops forever; we give up

// phantom_base::create_grid (phantom_base.cpp:100-132): voxel centre coordinates along a side.
std::vector<float> grid_base(float fov, uint64_t res) {
    const double start = fov / res / 2.0;
    const double end = fov - fov / res / 2.0;
    const double step = (end - start) / (res - 1.0);
    std::vector<float> g(res);
    for (uint64_t i = 0; i < res; i++) g[i] = static_cast<float>(start + i * step);
    return g;
}

struct Shape {            // one cylinder (axis along z) or sphere, with its voxel box
    float c[3];
    float r, r2;
    int32_t x0, x1, y0, y1, z0, z1;
};

// cylinder::calculate_volume (phantom_cylinder.cpp:126-171)
float cylinder_volume(const float *pnt, float rad, float fov, uint64_t res, const std::vector<float> &g) {
    bool intersect = false;
    for (int i = 0; i < 2; i++)
        if (pnt[i] + rad < 0 || pnt[i] - rad > fov) return -1.f;
    for (int i = 0; i < 2; i++)
        if (pnt[i] < rad - 1.5 || pnt[i] > fov - rad + 1.5) intersect = true;
    if (!intersect) return kPi * rad * rad * fov;
    const float v_size = fov / res, rad2 = rad * rad;
    const int32_t cv[2] = {int32_t(pnt[0] / v_size), int32_t(pnt[1] / v_size)};
    const int32_t rv = std::ceil(rad / fov * res) + 1;
    const int32_t x_min = std::max(0, cv[0] - rv), x_max = std::min((int32_t)res, cv[0] + rv + 2);
    const int32_t y_min = std::max(0, cv[1] - rv), y_max = std::min((int32_t)res, cv[1] + rv + 2);
    int64_t counter = 0;
    for (int32_t py = y_min; py < y_max; py++)
        for (int32_t px = x_min; px < x_max; px++) {
            const float d0 = g[px] - pnt[0], d1 = g[py] - pnt[1];
            const float d2 = d0 * d0 + d1 * d1;
            if (d2 <= rad2) counter += (int64_t)res;   // every z of the column
        }
    return (int32_t)counter * v_size * v_size * v_size;
}

// cylinder::generate_shapes (phantom_cylinder.cpp:85-123) with check_cylinder_overlap (:23-52)
int cylinder_shapes(float fov, uint64_t res, float radius, float bvf, int32_t seed,
                    const std::vector<float> &g, std::vector<Shape> &out) {
    if (2 * radius >= fov) return fail(SW_ERR_INVALID, "the radius of the cylinder is too large for the FoV");
    const bool random_radius = radius < 0;
    const float max_radius = radius > 0 ? radius : -radius;
    std::vector<float> px, py, pz, rr;
    std::mt19937 gen((size_t)seed);
    std::uniform_real_distribution<float> dist(0.f, 1.f);
    float vol_total = 0, vol_tol = fov * fov * fov;
    int32_t progress = 0;
    uint64_t attempts = 0;
    while (progress < 100) {
        if (++attempts > kMaxAttempts) return fail(SW_ERR_INVALID, "volume fraction not reached");
        float rad = random_radius ? dist(gen) * max_radius : max_radius;
        float pnt[3];
        for (int i = 0; i < 3; i++) pnt[i] = dist(gen) * (fov + 2 * rad) - rad;
        bool stop = false;
        for (size_t c = 0; c < rr.size() && !stop; c++) {
            const float d0 = pnt[0] - px[c], d1 = pnt[1] - py[c];
            const float distance = sqrtf(d0 * d0 + d1 * d1);
            if (distance <= rr[c] || distance <= rad)
                stop = true;
            else if (distance < rr[c] + rad) {
                if (!random_radius) stop = true;
                else rad = distance - rr[c];
            }
        }
        if (stop) continue;
        const float vol = cylinder_volume(pnt, rad, fov, res, g);
        if (100 * (vol + vol_total) / vol_tol > 1.02 * bvf || vol < 0) continue;
        vol_total += vol;
        progress = 100 * (100. * vol_total / vol_tol / bvf);
        px.push_back(pnt[0]);
        py.push_back(pnt[1]);
        pz.push_back(pnt[2]);
        rr.push_back(rad);
    }
    out.clear();
    for (size_t c = 0; c < rr.size(); c++) {
        Shape s{};
        s.c[0] = px[c]; s.c[1] = py[c]; s.c[2] = pz[c];
        s.r = rr[c];
        s.r2 = s.r * s.r;
        out.push_back(s);
    }
    return SW_OK;
}

// sphere::generate_shapes (phantom_sphere.cpp:80-117) with check_sphere_overlap (:22-51)
int sphere_shapes(float fov, float radius, float bvf, int32_t seed, std::vector<Shape> &out) {
    if (2 * radius >= fov) return fail(SW_ERR_INVALID, "the radius of the sphere is too large for the FoV");
    const bool random_radius = radius < 0;
    const float max_radius = radius > 0 ? radius : -radius;
    std::vector<float> px, py, pz, rr;
    std::minstd_rand gen((size_t)seed);
    std::uniform_real_distribution<float> dist(0.f, 1.f);
    float vol_sph = 0, vol_tol = fov * fov * fov;
    int32_t progress = 0;
    uint64_t attempts = 0;
    while (progress < 100) {
        if (++attempts > kMaxAttempts) return fail(SW_ERR_INVALID, "volume fraction not reached");
        float rad = random_radius ? dist(gen) * max_radius : max_radius;
        float pnt[3];
        for (int i = 0; i < 3; i++) pnt[i] = dist(gen) * fov;
        bool stop = false;
        for (size_t c = 0; c < rr.size() && !stop; c++) {
            const float d0 = pnt[0] - px[c], d1 = pnt[1] - py[c], d2 = pnt[2] - pz[c];
            const float distance = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
            if (distance <= rr[c] || distance <= rad)
                stop = true;
            else if (distance < rr[c] + rad) {
                if (!random_radius) stop = true;
                else rad = distance - rr[c];
            }
        }
        if (stop) continue;
        vol_sph += 4 * kPi / 3 * rad * rad * rad;
        px.push_back(pnt[0]);
        py.push_back(pnt[1]);
        pz.push_back(pnt[2]);
        rr.push_back(rad);
        progress = 0.95 * 100 * (100. * vol_sph / vol_tol / bvf);
    }
    out.clear();
    for (size_t c = 0; c < rr.size(); c++) {
        Shape s{};
        s.c[0] = px[c]; s.c[1] = py[c]; s.c[2] = pz[c];
        s.r = rr[c];
        s.r2 = s.r * s.r;
        out.push_back(s);
    }
    return SW_OK;
}

// Voxel boxes of generate_mask_fieldmap: +-20 voxel radii with a field, +-1 (+2) without.
void boxes(std::vector<Shape> &sh, float fov, uint64_t res, bool field, bool sphere) {
    const float v_size = fov / res;
    const int32_t R = (int32_t)res;
    for (Shape &s : sh) {
        const int32_t rv = std::ceil(s.r / v_size) + 1;
        int32_t cv[3];
        for (int i = 0; i < 3; i++) cv[i] = int32_t(s.c[i] / v_size);
        const int32_t lo = field ? 20 * rv : rv, hi = field ? 20 * rv : rv + 2;
        s.x0 = std::max(0, cv[0] - lo); s.x1 = std::min(R, cv[0] + hi);
        s.y0 = std::max(0, cv[1] - lo); s.y1 = std::min(R, cv[1] + hi);
        if (sphere) {
            s.z0 = std::max(0, cv[2] - lo); s.z1 = std::min(R, cv[2] + hi);
        } else {
            s.z0 = 0; s.z1 = R;
        }
    }
}

struct FieldConsts {
    double k;             // 2 pi (1 - Y) dChi (cylinders) or 4 pi (1 - Y) dChi (spheres)
    double k_in;          // cylinder: k (cos^2 theta - 1/3), the field inside
    float theta_s2;       // cylinder: sin^2 theta
    float b0p[3];         // cylinder: B0 projected on the plane normal to the axis, normalised
    float b0[3];          // sphere: B0
};

__global__ void k_phantom(const Shape *__restrict__ sh, uint32_t n_shapes, const float *__restrict__ g,
                          uint32_t res, int sphere, int with_field, FieldConsts K,
                          uint8_t *__restrict__ mask, float *__restrict__ field) {
    const uint64_t n = (uint64_t)res * res * res;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t pz = (uint32_t)(p % res), py = (uint32_t)((p / res) % res),
                       px = (uint32_t)(p / ((uint64_t)res * res));
        const float gx = g[px], gy = g[py], gz = g[pz];
        uint8_t m = 0;
        float f = 0.f;
        for (uint32_t c = 0; c < n_shapes; c++) {
            const Shape s = sh[c];
            if ((int32_t)px < s.x0 || (int32_t)px >= s.x1 || (int32_t)py < s.y0 ||
                (int32_t)py >= s.y1 || (int32_t)pz < s.z0 || (int32_t)pz >= s.z1)
                continue;
            const float d0 = gx - s.c[0], d1 = gy - s.c[1], d2 = gz - s.c[2];
            if (!sphere) {
                const float dist2 = d0 * d0 + d1 * d1;
                if (dist2 <= s.r2) m = 1;
                if (with_field) {
                    // projection of the voxel on the axis (0, 0, 1), as the reference forms it
                    const float dot = 0.f * d0 + 0.f * d1 + 1.f * d2;
                    const float t0 = dot * 0.f + s.c[0], t1 = dot * 0.f + s.c[1], t2 = dot * 1.f + s.c[2];
                    const float q0 = gx - t0, q1 = gy - t1, q2 = gz - t2;
                    const float phi_c = (q0 * K.b0p[0] + q1 * K.b0p[1] + q2 * K.b0p[2]) /
                                        sqrtf(q0 * q0 + q1 * q1 + q2 * q2);
                    const float phi_2c2_1 = 2 * phi_c * phi_c - 1;
                    const double add = dist2 > s.r2
                                           ? K.k * (double)(s.r2 / dist2) * (double)phi_2c2_1 * (double)K.theta_s2
                                           : K.k_in;
                    f = (float)((double)f + add);
                }
            } else {
                const float dist2 = d0 * d0 + d1 * d1 + d2 * d2;
                if (dist2 <= s.r2) m = 1;
                if (with_field) {
                    const float dp = d0 * K.b0[0] + d1 * K.b0[1] + d2 * K.b0[2];
                    const float phi_c2 = dp * dp / dist2;
                    const double add = dist2 > s.r2
                                           ? K.k * (double)s.r2 * (double)s.r / (double)dist2 /
                                                 (double)sqrtf(dist2) * ((double)phi_c2 - 1. / 3.)
                                           : 0.0;
                    f = (float)((double)f + add);
                }
            }
        }
        mask[p] = m;
        if (with_field) field[p] = f;
    }
}

int generate(bool sphere, float fov, uint64_t res, float dchi, float Y, float radius, float bvf,
             float orientation, int32_t seed, uint8_t *mask, float *field, float *bvf_out,
             bool device_out) {
    if (!mask || res < 2 || res > 4096 || !(fov > 0)) return fail(SW_ERR_INVALID, "phantom size");
    if (!(bvf > 0)) return fail(SW_ERR_INVALID, "volume fraction must be positive (percent)");
    const bool with_field = Y >= 0 && field != nullptr;
    const std::vector<float> g = grid_base(fov, res);
    std::vector<Shape> sh;
    int rc = sphere ? sphere_shapes(fov, radius, bvf, seed, sh)
                    : cylinder_shapes(fov, res, radius, bvf, seed, g, sh);
    if (rc) return rc;
    boxes(sh, fov, res, Y >= 0, sphere);
    FieldConsts K{};
    if (sphere) {
        K.k = 4 * kPi * (1 - Y) * dchi;
        K.b0[0] = 0.f; K.b0[1] = 0.f; K.b0[2] = 1.f;       // phantom_base.h:43
    } else {
        // cylinder::set_cylinder_parameters (phantom_cylinder.cpp:75-83): B0 = roty((0,0,1));
        // its projection on the xy plane, normalised, is (+-1, 0, 0) or (0, 0, 0)
        const float deg2rad = 0.0174532925199433f;
        const float s = sinf(orientation * deg2rad);
        const float b0x = s * 1.f;
        float b[3] = {b0x, 0.f, 0.f};
        const float nb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        if (nb != 0) for (int i = 0; i < 3; i++) b[i] /= nb;
        for (int i = 0; i < 3; i++) K.b0p[i] = b[i];
        const float theta_c = cos(orientation * kPi / 180);       // phantom_cylinder.cpp:200-202
        const float theta_c2 = theta_c * theta_c;
        K.theta_s2 = 1. - theta_c2;
        K.k = 2 * kPi * (1 - Y) * dchi;
        K.k_in = K.k * (theta_c2 - 1.0 / 3.0);
    }
    const uint64_t n = res * res * res;
    Shape *d_sh = nullptr;
    float *d_g = nullptr, *d_field = nullptr;
    uint8_t *d_mask = nullptr;
    auto done = [&](int code) {
        if (d_sh) cudaFree(d_sh);
        if (d_g) cudaFree(d_g);
        if (!device_out) {
            if (d_mask) cudaFree(d_mask);
            if (d_field) cudaFree(d_field);
        }
        return code;
    };
#define PH_TRY(call)                                                                      \
    do {                                                                                  \
        cudaError_t e2 = (call);                                                          \
        if (e2 != cudaSuccess)                                                            \
            return done(fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e2))); \
    } while (0)
    PH_TRY(cudaMalloc(&d_sh, std::max<size_t>(1, sh.size()) * sizeof(Shape)));
    PH_TRY(cudaMalloc(&d_g, res * sizeof(float)));
    if (device_out) {
        d_mask = mask;
        d_field = with_field ? field : nullptr;
    } else {
        PH_TRY(cudaMalloc(&d_mask, n));
        if (with_field) PH_TRY(cudaMalloc(&d_field, n * 4));
    }
    if (!sh.empty()) PH_TRY(cudaMemcpy(d_sh, sh.data(), sh.size() * sizeof(Shape), cudaMemcpyHostToDevice));
    PH_TRY(cudaMemcpy(d_g, g.data(), res * sizeof(float), cudaMemcpyHostToDevice));
    const int blocks = (int)std::min<uint64_t>((n + 255) / 256, 152ull * 64);
    k_phantom<<<blocks, 256>>>(d_sh, (uint32_t)sh.size(), d_g, (uint32_t)res, sphere ? 1 : 0,
                               with_field ? 1 : 0, K, d_mask, d_field);
    PH_TRY(cudaGetLastError());
    PH_TRY(cudaDeviceSynchronize());
    std::vector<uint8_t> hm;
    const uint8_t *mh = mask;
    if (device_out) {
        hm.resize(n);
        PH_TRY(cudaMemcpy(hm.data(), d_mask, n, cudaMemcpyDeviceToHost));
        mh = hm.data();
    } else {
        PH_TRY(cudaMemcpy(mask, d_mask, n, cudaMemcpyDeviceToHost));
        if (with_field) PH_TRY(cudaMemcpy(field, d_field, n * 4, cudaMemcpyDeviceToHost));
    }
    if (bvf_out) {       // generate_mask_fieldmap: actual volume fraction in percent
        int64_t cnt = 0;
        for (uint64_t i = 0; i < n; i++) cnt += mh[i];
        *bvf_out = (int32_t)cnt * 100.0 / n;
    }
#undef PH_TRY
    return done(SW_OK);
}

}  // namespace

extern "C" {

int sw_phantom_cylinder(float fov_um, uint64_t resolution, float dchi, float Y, float radius_um,
                        float volume_fraction, float orientation_deg, int32_t seed, uint8_t *mask,
                        float *field, float *bvf_out) {
    return generate(false, fov_um, resolution, dchi, Y, radius_um, volume_fraction,
                    orientation_deg, seed, mask, field, bvf_out, false);
}

int sw_phantom_sphere(float fov_um, uint64_t resolution, float dchi, float Y, float radius_um,
                      float volume_fraction, int32_t seed, uint8_t *mask, float *field,
                      float *bvf_out) {
    return generate(true, fov_um, resolution, dchi, Y, radius_um, volume_fraction, 0.f, seed,
                    mask, field, bvf_out, false);
}

int sw_phantom_cylinder_device(float fov_um, uint64_t resolution, float dchi, float Y,
                               float radius_um, float volume_fraction, float orientation_deg,
                               int32_t seed, uint8_t *d_mask, float *d_field, float *bvf_out) {
    return generate(false, fov_um, resolution, dchi, Y, radius_um, volume_fraction,
                    orientation_deg, seed, d_mask, d_field, bvf_out, true);
}

int sw_phantom_sphere_device(float fov_um, uint64_t resolution, float dchi, float Y,
                             float radius_um, float volume_fraction, int32_t seed,
                             uint8_t *d_mask, float *d_field, float *bvf_out) {
    return generate(true, fov_um, resolution, dchi, Y, radius_um, volume_fraction, 0.f, seed,
                    d_mask, d_field, bvf_out, true);
}

}  // extern "C"
