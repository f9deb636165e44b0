// TEST INFRASTRUCTURE ONLY: runs the reference's own phantom generators
// (src/phantom/phantom_cylinder.cpp, phantom_sphere.cpp, built from the read-only tree by
// oracle/Makefile) and returns their mask and field from memory.
#include <cstdint>
#include <cstring>
#include <vector>

#include "phantom_cylinder.h"
#include "phantom_sphere.h"

namespace {

template <typename Shape>
struct Exposed : Shape {
    using Shape::Shape;
    const std::vector<int8_t> &mask() const { return this->m_mask; }
    const std::vector<float> &field() const { return this->m_fieldmap; }
};

template <typename S>
int copy_out(const S &ph, uint8_t *mask, float *field, float *bvf) {
    std::memcpy(mask, ph.mask().data(), ph.mask().size());
    if (field && !ph.field().empty()) std::memcpy(field, ph.field().data(), ph.field().size() * 4);
    if (bvf) *bvf = ph.get_actual_volume_fraction();
    return 1;
}

}  // namespace

extern "C" {

// phantom::cylinder(fov_um, resolution, dChi, Y, radius_um, volume_fraction, orientation,
// seed).run(false) -- src/phantom/phantom_cylinder.cpp:61-65, 288-302
int ref_phantom_cylinder(float fov_um, uint64_t res, float dchi, float Y, float radius_um,
                         float bvf, float orientation, int32_t seed, uint8_t *mask, float *field,
                         float *bvf_out) {
    Exposed<phantom::cylinder> ph(fov_um, res, dchi, Y, radius_um, bvf, orientation, seed, "");
    if (!ph.run(false)) return 0;
    return copy_out(ph, mask, field, bvf_out);
}

// phantom::sphere(fov_um, resolution, dChi, Y, radius_um, volume_fraction, seed).run(false)
// -- src/phantom/phantom_sphere.cpp:62-66, 211-225
int ref_phantom_sphere(float fov_um, uint64_t res, float dchi, float Y, float radius_um,
                       float bvf, int32_t seed, uint8_t *mask, float *field, float *bvf_out) {
    Exposed<phantom::sphere> ph(fov_um, res, dchi, Y, radius_um, bvf, seed, "");
    if (!ph.run(false)) return 0;
    return copy_out(ph, mask, field, bvf_out);
}

}  // extern "C"
