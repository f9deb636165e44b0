"""Fixtures of the reference's phantom generators (src/phantom/phantom_cylinder.cpp,
phantom_sphere.cpp), built from the read-only source tree into oracle/_ref/libref_phantom.so
(`make -C oracle ref`). Run on one OpenMP thread: with random radii the reference's placement
depends on thread timing. Writes tests/golden/phantom_*.npz.

    OMP_NUM_THREADS=1 python tests/golden/make_golden_phantoms.py
"""
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "..", "oracle", "_ref", "libref_phantom.so")

# name: (kind, fov_um, res, dchi, Y, radius_um, bvf_percent, orientation_deg, seed)
CASES = {
    "phantom_cyl_o90": ("cyl", 100.0, 40, 0.11e-6 * 0.4, 0.75, 5.0, 3.0, 90.0, 1),
    "phantom_cyl_o30_random_r": ("cyl", 80.0, 36, 0.11e-6 * 0.4, 0.6, -6.0, 4.0, 30.0, 7),
    "phantom_cyl_mask_only": ("cyl", 60.0, 32, 0.11e-6, -1.0, 4.0, 5.0, 0.0, 3),
    "phantom_sph": ("sph", 60.0, 32, 0.11e-6 * 0.4, 0.75, 4.0, 2.0, 0.0, 2),
    "phantom_sph_random_r": ("sph", 50.0, 30, 0.11e-6 * 0.4, 0.7, -5.0, 3.0, 0.0, 9),
}


def generate(name):
    kind, fov, res, dchi, Y, r, bvf, orient, seed = CASES[name]
    L = C.CDLL(LIB)
    n = res ** 3
    mask = np.zeros(n, np.uint8)
    field = np.zeros(n, np.float32)
    out = C.c_float()
    F, U = C.c_float, C.c_uint64
    if kind == "cyl":
        L.ref_phantom_cylinder.argtypes = [F, U, F, F, F, F, F, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        ok = L.ref_phantom_cylinder(fov, res, dchi, Y, r, bvf, orient, seed, mask.ctypes.data,
                                    field.ctypes.data, C.byref(out))
    else:
        L.ref_phantom_sphere.argtypes = [F, U, F, F, F, F, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        ok = L.ref_phantom_sphere(fov, res, dchi, Y, r, bvf, seed, mask.ctypes.data,
                                  field.ctypes.data, C.byref(out))
    assert ok == 1, name
    return mask, (field if Y >= 0 else None), out.value


if __name__ == "__main__":
    assert os.environ.get("OMP_NUM_THREADS") == "1", "run with OMP_NUM_THREADS=1"
    for name, args in CASES.items():
        mask, field, bvf = generate(name)
        d = dict(mask=mask, bvf=np.float32(bvf), args=json.dumps(args))
        if field is not None:
            d["field"] = field
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, mask.mean(), bvf)
