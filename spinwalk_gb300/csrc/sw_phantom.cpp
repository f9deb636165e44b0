// Synthetic phantoms: uint8 substrate mask + off-resonance field (Tesla at B0 = 1 T), for the
// benchmark configurations and tests. Host C++ with OpenMP; deterministic for a given seed
// (shapes are placed by one std::mt19937_64, and every voxel sums its contributions in shape
// order, each thread owning whole x-slabs).
//
// Field models follow the reference's generators:
//   infinite cylinder (src/phantom/phantom_cylinder.cpp:255-265), axis d, angle theta to B0:
//     outside  2*pi*dchi*(1-Y) * (r^2/rho^2) * cos(2*phi) * sin^2(theta)
//     inside   2*pi*dchi*(1-Y) * (cos^2(theta) - 1/3)
//   sphere (src/phantom/phantom_sphere.cpp:180-187):
//     outside  4*pi*(1-Y)*dchi * r^3/d^3 * (cos^2(phi) - 1/3),  0 inside that sphere
// Differences by design: cylinders may take random orientations (the reference's are parallel
// to z with B0 tilted), shapes may overlap, and a sphere's field is summed over a cube of
// +-window*r around it (the reference uses +-20 voxel radii); cylinders contribute everywhere.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <omp.h>

#include "spinwalk_gpu.h"

namespace {

struct Cyl {
    double c[3], d[3], r, ct, st2, bp[3];
    bool has_bp;
};

}  // namespace

namespace sw {
namespace api {
int fail(int code, const std::string &msg);   // sets sw_last_error() (sw_api.cu)
}  // namespace api
}  // namespace sw

// Upper bound on the shapes one synthetic phantom may hold (the voxel loop visits every shape).
constexpr double kMaxShapes = 1e6;

extern "C" {

int sw_phantom_cylinders(const uint32_t dims[3], const double fov[3], double radius,
                         double volume_fraction, uint64_t seed, int random_orientation,
                         double dchi, double Y, const double B0_dir[3], uint8_t *mask,
                         float *field) {
    if (!dims || !fov || !mask || radius <= 0 || volume_fraction < 0)
        return sw::api::fail(SW_ERR_INVALID, "sw_phantom_cylinders: null buffer, radius <= 0 or "
                                             "negative volume fraction");
    const uint64_t nx = dims[0], ny = dims[1], nz = dims[2];
    double b0[3] = {0, 0, 1};
    if (B0_dir) {
        double n = std::sqrt(B0_dir[0] * B0_dir[0] + B0_dir[1] * B0_dir[1] + B0_dir[2] * B0_dir[2]);
        if (n <= 0) return sw::api::fail(SW_ERR_INVALID, "B0 direction has zero length");
        for (int i = 0; i < 3; i++) b0[i] = B0_dir[i] / n;
    }
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::normal_distribution<double> N(0.0, 1.0);
    std::vector<Cyl> cyl;
    const double target = volume_fraction * fov[0] * fov[1] * fov[2];
    const double L = std::cbrt(fov[0] * fov[1] * fov[2]);
    if (target / (M_PI * radius * radius * L) > kMaxShapes)
        return sw::api::fail(SW_ERR_INVALID, "sw_phantom_cylinders: the volume fraction needs more "
                                             "than " + std::to_string((long)kMaxShapes) +
                                             " cylinders of this radius");
    double vol = 0;
    while (vol < target) {
        Cyl c{};
        for (int i = 0; i < 3; i++) c.c[i] = U(rng) * fov[i];
        if (random_orientation) {
            double n = 0;
            while (n < 1e-12) {
                for (int i = 0; i < 3; i++) c.d[i] = N(rng);
                n = std::sqrt(c.d[0] * c.d[0] + c.d[1] * c.d[1] + c.d[2] * c.d[2]);
            }
            for (int i = 0; i < 3; i++) c.d[i] /= n;
        } else {
            c.d[0] = 0; c.d[1] = 0; c.d[2] = 1;
        }
        c.r = radius;
        c.ct = c.d[0] * b0[0] + c.d[1] * b0[1] + c.d[2] * b0[2];
        c.st2 = 1 - c.ct * c.ct;
        double nb = 0;
        for (int i = 0; i < 3; i++) {
            c.bp[i] = b0[i] - c.ct * c.d[i];
            nb += c.bp[i] * c.bp[i];
        }
        nb = std::sqrt(nb);
        c.has_bp = nb > 1e-12;
        if (c.has_bp)
            for (int i = 0; i < 3; i++) c.bp[i] /= nb;
        cyl.push_back(c);
        vol += M_PI * radius * radius * L;
    }
    const double k = 2 * M_PI * dchi * (1 - Y);
    const double vx = fov[0] / nx, vy = fov[1] / ny, vz = fov[2] / nz;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ix = 0; ix < (int64_t)nx; ix++) {
        for (uint64_t iy = 0; iy < ny; iy++) {
            for (uint64_t iz = 0; iz < nz; iz++) {
                const double p[3] = {(ix + 0.5) * vx, (iy + 0.5) * vy, (iz + 0.5) * vz};
                double f = 0;
                uint8_t m = 0;
                for (const Cyl &c : cyl) {
                    double rel[3] = {p[0] - c.c[0], p[1] - c.c[1], p[2] - c.c[2]};
                    double a = rel[0] * c.d[0] + rel[1] * c.d[1] + rel[2] * c.d[2];
                    double q[3] = {rel[0] - a * c.d[0], rel[1] - a * c.d[1], rel[2] - a * c.d[2]};
                    double rho2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
                    if (rho2 <= c.r * c.r) {
                        m = 1;
                        f += k * (c.ct * c.ct - 1.0 / 3.0);
                    } else {
                        double cphi = c.has_bp ? (q[0] * c.bp[0] + q[1] * c.bp[1] + q[2] * c.bp[2]) /
                                                     std::sqrt(rho2)
                                               : 0.0;
                        f += k * (c.r * c.r / rho2) * (2 * cphi * cphi - 1) * c.st2;
                    }
                }
                const uint64_t v = ((uint64_t)ix * ny + iy) * nz + iz;
                mask[v] = m;
                if (field) field[v] = (float)f;
            }
        }
    }
    return SW_OK;
}

int sw_phantom_spheres(const uint32_t dims[3], const double fov[3], double rmin, double rmax,
                       double volume_fraction, uint64_t seed, double dchi, double Y,
                       const double B0_dir[3], double window, uint8_t *mask, float *field) {
    if (!dims || !fov || !mask || rmin <= 0 || rmax < rmin || window < 1)
        return sw::api::fail(SW_ERR_INVALID, "sw_phantom_spheres: null buffer, radii not "
                                             "0 < rmin <= rmax, or window < 1");
    const int64_t nx = dims[0], ny = dims[1], nz = dims[2];
    double b0[3] = {0, 0, 1};
    if (B0_dir) {
        double n = std::sqrt(B0_dir[0] * B0_dir[0] + B0_dir[1] * B0_dir[1] + B0_dir[2] * B0_dir[2]);
        if (n <= 0) return sw::api::fail(SW_ERR_INVALID, "B0 direction has zero length");
        for (int i = 0; i < 3; i++) b0[i] = B0_dir[i] / n;
    }
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    struct Sph { double c[3], r; };
    std::vector<Sph> sph;
    const double target = volume_fraction * fov[0] * fov[1] * fov[2];
    if (target / (4.0 / 3.0 * M_PI * rmin * rmin * rmin) > kMaxShapes)
        return sw::api::fail(SW_ERR_INVALID, "sw_phantom_spheres: the volume fraction may need more "
                                             "than " + std::to_string((long)kMaxShapes) +
                                             " spheres of these radii");
    double vol = 0;
    while (vol < target) {
        Sph s;
        s.r = rmin + (rmax - rmin) * U(rng);
        for (int i = 0; i < 3; i++) s.c[i] = U(rng) * fov[i];
        sph.push_back(s);
        vol += 4.0 / 3.0 * M_PI * s.r * s.r * s.r;
    }
    const double k = 4 * M_PI * (1 - Y) * dchi;
    const double vs[3] = {fov[0] / nx, fov[1] / ny, fov[2] / nz};
    std::memset(mask, 0, (size_t)nx * ny * nz);
    if (field) std::memset(field, 0, sizeof(float) * (size_t)nx * ny * nz);
    const int nt = omp_get_max_threads();
    // each thread owns contiguous x-slabs; shapes are visited in order -> deterministic sums
#pragma omp parallel num_threads(nt)
    {
        const int t = omp_get_thread_num();
        const int64_t x0 = nx * t / nt, x1 = nx * (t + 1) / nt;
        std::vector<double> f((size_t)(x1 - x0) * ny * nz, 0.0);
        for (const Sph &s : sph) {
            int64_t lo[3], hi[3];
            const double reach = window * s.r;
            for (int i = 0; i < 3; i++) {
                const int64_t n = i == 0 ? nx : (i == 1 ? ny : nz);
                lo[i] = std::max<int64_t>(0, (int64_t)std::floor((s.c[i] - reach) / vs[i]));
                hi[i] = std::min<int64_t>(n, (int64_t)std::ceil((s.c[i] + reach) / vs[i]) + 1);
            }
            const int64_t a0 = std::max(lo[0], x0), a1 = std::min(hi[0], x1);
            for (int64_t ix = a0; ix < a1; ix++)
                for (int64_t iy = lo[1]; iy < hi[1]; iy++)
                    for (int64_t iz = lo[2]; iz < hi[2]; iz++) {
                        const double d[3] = {(ix + 0.5) * vs[0] - s.c[0],
                                             (iy + 0.5) * vs[1] - s.c[1],
                                             (iz + 0.5) * vs[2] - s.c[2]};
                        const double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                        const uint64_t v = ((uint64_t)ix * ny + iy) * nz + iz;
                        if (d2 <= s.r * s.r) {
                            mask[v] = 1;
                        } else if (d2 <= reach * reach) {
                            const double dp = d[0] * b0[0] + d[1] * b0[1] + d[2] * b0[2];
                            const double c2 = dp * dp / d2;
                            f[(size_t)((ix - x0) * ny + iy) * nz + iz] +=
                                k * s.r * s.r * s.r / (d2 * std::sqrt(d2)) * (c2 - 1.0 / 3.0);
                        }
                    }
        }
        if (field)
            for (int64_t ix = x0; ix < x1; ix++)
                for (int64_t iy = 0; iy < ny; iy++)
                    for (int64_t iz = 0; iz < nz; iz++) {
                        const uint64_t v = ((uint64_t)ix * ny + iy) * nz + iz;
                        field[v] = (float)f[(size_t)((ix - x0) * ny + iy) * nz + iz];
                    }
    }
    return SW_OK;
}

}  // extern "C"
