"""CPU tests: the oracle is pinned to the reference, and the host-side logic of the library
(parameter preparation, initial positions, the logf exception table, the exported C ABI) is
checked without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.helpers import GOLDEN_CASES, ROOT, bits_equal, load_golden
from spinwalk_gb300 import _lib, abi
from spinwalk_gb300.problem import Problem, cylinder_phantom, fieldmap_scale
from tests import oracle_lib


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_reference_golden(case):
    """oracle/sim_oracle.cpp reproduces the reference's sim::sim outputs bit for bit."""
    pr, ref = load_golden(case)
    out = oracle_lib.run(pr, fill=np.nan)
    for k in ("M1", "XYZ1", "T"):
        assert bits_equal(out[k], ref[k]), f"{case}: {k}"


def test_golden_cases_cover_edge_statuses():
    _, lost = load_golden("lost_spins")
    assert np.isnan(lost["M1"]).any()
    pr, _ = load_golden("lost_spins")
    st = oracle_lib.run(pr)["status"]
    assert (st == abi.SW_SPIN_LOST).any() and (st == abi.SW_SPIN_OK).any()
    for case in ("out_of_bounds_periodic", "out_of_bounds_reflect"):
        pr, _ = load_golden(case)
        assert (oracle_lib.run(pr)["status"] == abi.SW_SPIN_OOB).any()


@pytest.mark.skipif(not oracle_lib.ref_available(), reason="reference source tree not present")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_live(seed):
    """Randomised configurations, oracle vs the reference built from its own sources."""
    rng = np.random.default_rng(seed)
    n = 20
    mask, field = cylinder_phantom(n, 20e-6, float(rng.uniform(2e-6, 4e-6)), 0.1, seed=seed)
    kw = dict(n_spins=100, seed=int(rng.integers(1, 1000)), TR_us=3050, TE_us=(1000, 3000),
              RF_FA=(90.0, float(rng.uniform(90, 180))), RF_PH=(0.0, float(rng.uniform(0, 360))),
              RF_us=(0, 1500), pXY=rng.uniform(0, 1, (2, 2)),
              n_dummy_scan=int(rng.integers(0, 3)),
              linear_phase_cycling=float(rng.uniform(0, 90)),
              cross_fov=bool(rng.integers(0, 2)))
    pr = Problem(mask, [20e-6] * 3, field, **kw)
    a = oracle_lib.run(pr)
    b = oracle_lib.run_ref(pr)
    for k in ("M1", "XYZ1", "T"):
        assert bits_equal(a[k], b[k]), k


@pytest.mark.skipif(not oracle_lib.ref_available(), reason="reference source tree not present")
@pytest.mark.parametrize("seed,trials", [(7, 20), (8, 20), (2024, 60)])
def test_oracle_matches_reference_on_random_configs(seed, trials):
    """The randomised configurations of the GPU parity test (tests/fuzz_configs.py, same seeds):
    several RF pulses and echoes, dephasing and gradient events, dummy scans with phase cycling,
    two or three substrates, both boundaries, trajectories, seeds up to 2^31 (and 60 more of the
    longer campaign's seed). The oracle's FP32
    run equals the reference's own sim::sim built from its sources, bit for bit, so the oracle
    the GPU is checked against is pinned on exactly these inputs."""
    from tests import fuzz_configs
    rng = np.random.default_rng(seed)
    for trial in range(trials):
        pr = fuzz_configs.random_case(rng)[0]
        a = oracle_lib.run(pr, fill=np.nan)
        b = oracle_lib.run_ref(pr, fill=np.nan)
        for k in ("M1", "XYZ1", "T"):
            assert bits_equal(a[k], b[k]), (trial, k)


def test_oracle_spin_subset_is_independent():
    """Spins are independent: a subset run writes the same values at the same slots."""
    pr, _ = load_golden("permeable")
    full = oracle_lib.run(pr)
    ids = np.array([3, 17, 100, 255], np.uint32)
    sub = oracle_lib.run(pr, spin_ids=ids)
    for k in ("M1", "XYZ1", "T"):
        assert bits_equal(full[k][ids], sub[k][ids])


def test_fieldmap_scale_matches_reference_arithmetic():
    for B0, dt in ((9.4, 50), (3.0, 25), (7.0, 20), (1.5, 10)):
        assert _lib.fieldmap_scale(B0, dt) == fieldmap_scale(B0, dt)


def test_initial_positions_match_reference_driver():
    for seed, n in ((10, 1000), (3, 17)):
        fov = [200e-6, 150e-6, 100e-6]
        assert bits_equal(_lib.initial_positions(fov, seed, n),
                          oracle_lib.initial_positions(fov, seed, n))


def test_prepare_params_matches_python_and_reference():
    L = _lib.lib()
    p = abi.SwParams()
    p.timestep_us, p.TR_us, p.n_dummy_scan, p.n_substrate, p.seed = 50, 20050, -1, 2, 0
    diff = np.array([1e-9, 2e-9])
    fa = np.array([30.0], np.float32)
    t1 = np.array([2000.0, 1500.0], np.float32)
    assert L.sw_prepare_params(C.byref(p), diff.ctypes.data_as(C.POINTER(C.c_double)),
                               fa.ctypes.data_as(C.POINTER(C.c_float)),
                               t1.ctypes.data_as(C.POINTER(C.c_float))) == 0
    assert p.n_timepoints == 401
    assert p.n_dummy_scan == int(5.0 * 2000.0 / np.float32(20050 * 1e-3))
    assert p.seed != 0
    assert diff[0] == 1e-3 * np.sqrt(2 * 1e-9 * 50)
    pr = Problem(np.zeros((2, 2, 2), np.uint8), [1e-5] * 3, RF_FA=(30.0,), n_spins=1,
                 XYZ0=np.zeros((1, 3), np.float32))
    assert np.float32(p.s) == np.float32(pr.params.s) and np.float32(p.c) == np.float32(pr.params.c)


def test_logf_exception_table():
    """The device logf = candidate + exceptions; every libm difference must be one ulp."""
    count, wide = _lib.logf_exception_count()
    assert wide == 0
    assert 0 < count < 2_000_000


def test_logf_table_header_is_reproducible(tmp_path):
    import shutil
    import subprocess
    import sys
    src = os.path.join(ROOT, "spinwalk_gb300", "csrc")
    shutil.copy(os.path.join(src, "gen_logf_table.py"), tmp_path)
    subprocess.run([sys.executable, str(tmp_path / "gen_logf_table.py")], check=True)
    assert open(tmp_path / "sw_logf_table.h").read() == \
        open(os.path.join(src, "sw_logf_table.h")).read()


def _declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(sw_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = _declared_functions()
    assert "sw_sim" in names and "sw_sim_device" in names
    for n in names:
        assert hasattr(L, n), n


def test_gpu_entry_points_fail_cleanly_without_gpu():
    if _lib.device_count() > 0:
        pytest.skip("a GPU is present")
    pr, _ = load_golden("gre")
    with pytest.raises(_lib.SpinWalkError):
        _lib.run(pr)


def test_integer_double_add_matches_ieee_on_host(tmp_path):
    """The walk's position update (sw_dadd.h, integer arithmetic) built for the host equals the
    host's IEEE double addition on 8e6 operand pairs."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "dadd_check"
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "spinwalk_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{csrc}",
                    os.path.join(here, "dadd_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    n, bad = map(int, r.stdout.split()[-2:])
    assert n > 8_000_000 and bad == 0


def test_host_entry_points_report_errors():
    """The host-only entry points return an error code and say why in sw_last_error()."""
    L = _lib.lib()
    p = abi.SwParams()
    assert L.sw_prepare_params(C.byref(p), None, None, None) == abi.SW_ERR_INVALID
    assert b"null argument" in L.sw_last_error()
    d = (C.c_double * 2)(1e-9, 1e-9)
    fa, t1 = (C.c_float * 1)(90.0), (C.c_float * 1)(1000.0)
    p.timestep_us = 0
    assert L.sw_prepare_params(C.byref(p), d, fa, t1) == abi.SW_ERR_INVALID
    assert b"TIME_STEP" in L.sw_last_error()
    assert L.sw_initial_positions(None, 1, 4, None) == abi.SW_ERR_INVALID
    assert b"sw_initial_positions" in L.sw_last_error()
    with pytest.raises(_lib.SpinWalkError, match="radius"):
        _lib.phantom_cylinders(8, 8e-6, -1e-6, 0.1, seed=1)
    with pytest.raises(_lib.SpinWalkError, match="zero length"):
        _lib.phantom_spheres(8, 8e-6, 1e-6, 2e-6, 0.1, seed=1, B0_dir=(0.0, 0.0, 0.0))
    with pytest.raises(_lib.SpinWalkError, match="more than 1000000 cylinders"):
        _lib.phantom_cylinders(8, 8e-6, 1e-12, 0.5, seed=1)
    with pytest.raises(_lib.SpinWalkError, match="more than 1000000 spheres"):
        _lib.phantom_spheres(8, 8e-6, 1e-12, 2e-6, 0.5, seed=1)
    assert _lib.config_dump("/nonexistent/x.ini", os.devnull) != 0
    assert L.sw_last_error()


def test_device_info_text():
    """sw_device_info (the CLI's -g/--gpu_info): on a machine without a GPU it says so and
    returns an error; with one it names the device and its compute capability."""
    rc, text = _lib.device_info(0)
    assert "current CUDA version" in text and "Number of devices" in text
    if _lib.device_count() == 0:
        assert rc == abi.SW_ERR_CUDA and "not available" in text
    else:
        assert rc == abi.SW_OK and "Compute Capability:" in text
