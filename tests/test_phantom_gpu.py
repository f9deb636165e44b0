"""The reference's phantom generators (src/phantom/phantom_cylinder.cpp, phantom_sphere.cpp) on
the GPU: mask, field and actual volume fraction must equal the reference build's bit for bit
(fixtures made by tests/golden/make_golden_phantoms.py)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests import oracle_lib
from tests.helpers import GOLDEN_DIR

CASES = sorted(f[:-4] for f in os.listdir(GOLDEN_DIR) if f.startswith("phantom_") and f.endswith(".npz"))


def _fixture(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    return z, json.loads(str(z["args"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_phantom_equals_reference(name):
    from spinwalk_gb300 import _lib
    z, (kind, fov, res, dchi, Y, r, bvf, orient, seed) = _fixture(name)
    if kind == "cyl":
        mask, field, got_bvf = _lib.phantom_cylinder(fov, res, dchi, Y, r, bvf, orient, seed)
    else:
        mask, field, got_bvf = _lib.phantom_sphere(fov, res, dchi, Y, r, bvf, seed)
    assert np.array_equal(mask.ravel(), z["mask"])
    if "field" in z:
        assert np.array_equal(field.ravel().view(np.uint32), z["field"].view(np.uint32))
    else:
        assert field is None
    assert np.float32(got_bvf) == z["bvf"]


@pytest.mark.skipif(not oracle_lib.ref_available(), reason="reference source tree not present")
def test_reference_build_reproduces_fixtures():
    """The oracle: the reference's generators built from source, on one thread, still give the
    committed fixtures."""
    code = ("import sys, json, numpy as np; sys.path.insert(0, %r); import make_golden_phantoms as m;"
            "out = {n: m.generate(n) for n in m.CASES};"
            "np.savez(sys.argv[1], **{n + '_mask': v[0] for n, v in out.items()},"
            " **{n + '_field': v[1] for n, v in out.items() if v[1] is not None})") % GOLDEN_DIR
    tmp = os.path.join(GOLDEN_DIR, "..", "..", "_pytest_phantoms.npz")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    try:
        subprocess.run([sys.executable, "-c", code, tmp], check=True, env=env,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        got = np.load(tmp)
        for name in CASES:
            z, _ = _fixture(name)
            assert np.array_equal(got[name + "_mask"], z["mask"])
            if "field" in z:
                assert np.array_equal(got[name + "_field"].view(np.uint32), z["field"].view(np.uint32))
    finally:
        if os.path.exists(tmp):
            os.remove(tmp)
