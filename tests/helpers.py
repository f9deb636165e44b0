"""Shared helpers of the test suite: golden fixtures and comparison tolerances."""
import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN_DIR)
                      if f.endswith(".npz") and not f.startswith(("phantom_", "minstd_")))


def load_golden(name):
    """(Problem, reference outputs) of one golden fixture."""
    from spinwalk_gb300.problem import Problem
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    kw = json.loads(str(z["kwargs"]))
    for k in ("TE_us", "RF_FA", "RF_PH", "RF_us", "dephasing_deg", "dephasing_us", "gradient_us",
              "diffusivity", "T1_ms", "T2_ms"):
        if k in kw:
            kw[k] = tuple(kw[k])
    field = z["field_T"] if z["field_T"].size else None
    fov = float(z["fov"])
    pr = Problem(z["mask"], [fov] * 3, field, XYZ0=z["XYZ0"], **kw)
    ref = dict(M1=z["M1"], XYZ1=z["XYZ1"], T=z["T"])
    return pr, ref


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return np.array_equal(a.view(np.uint8), b.view(np.uint8))
    return np.array_equal(a, b)


# Magnetisation tolerance of the FP32 path against the reference: 1e-5 relative to the spin's
# |M| (the reference's own rotations use libm sinf/cosf, the GPU its own), plus 1e-7 absolute.
M_RTOL = 1e-5
M_ATOL = 1e-7


def m_close(got, ref, rtol=M_RTOL, atol=M_ATOL):
    """Unreached echoes (NaN in the fixture) must stay NaN; the rest within tolerance."""
    nan_ref = np.isnan(ref)
    if not np.array_equal(nan_ref, np.isnan(got)):
        return False, float("inf")
    g = np.where(nan_ref, 0, got).astype(np.float64)
    r = np.where(nan_ref, 0, ref).astype(np.float64)
    scale = np.linalg.norm(r, axis=-1, keepdims=True)
    err = np.abs(g - r)
    ok = bool(np.all(err <= rtol * scale + atol))
    rel = float(np.max(err / (scale + 1e-30))) if err.size else 0.0
    return ok, rel
