"""The benchmark's two arms (CPU, no GPU needed): the CPU reference arm makes the same inputs as
the GPU arm without loading the CUDA library, and both arms describe the workload with the same
`config` object, so that their values compare like for like."""
import json
import os
import subprocess
import sys

import numpy as np

from spinwalk_gb300 import _lib
from tests import oracle_lib
from tests.helpers import ROOT, bits_equal


def test_standalone_phantom_generator_matches_library():
    L = oracle_lib.synth()
    m1, f1 = _lib.phantom_spheres(40, 40e-6, 2e-6, 8e-6, 0.05, seed=2)
    m2, f2 = _lib.phantom_spheres(40, 40e-6, 2e-6, 8e-6, 0.05, seed=2, L=L)
    assert bits_equal(m1, m2) and bits_equal(f1, f2)
    m1, f1 = _lib.phantom_cylinders(36, 36e-6, 5e-6, 0.03, seed=1)
    m2, f2 = _lib.phantom_cylinders(36, 36e-6, 5e-6, 0.03, seed=1, L=L)
    assert bits_equal(m1, m2) and bits_equal(f1, f2)
    assert m1.any() and np.abs(f1).max() > 0


def test_oracle_side_inputs_match_library_inputs():
    sys.path.insert(0, ROOT)
    import bench
    ours = bench.Inputs()
    ref = bench.Inputs(oracle_side=True)
    assert bits_equal(ours.positions([30e-6] * 3, 10, 500), ref.positions([30e-6] * 3, 10, 500))
    assert bits_equal(ours.cylinders(30, 30e-6, 5e-6, 0.03, 4)[1],
                      ref.cylinders(30, 30e-6, 5e-6, 0.03, 4)[1])


_MAPS = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "gre", "--steps", "1",
            "--warmup", "1", "--ref-sample", "64"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("LOADED", sorted({l.split()[-1] for l in maps.splitlines() if l.endswith(".so")}))
"""


def test_reference_arm_never_loads_the_cuda_library():
    r = subprocess.run([sys.executable, "-c", _MAPS], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[0])
    loaded = lines[1]
    assert "libspinwalk_gpu" not in loaded, loaded
    assert "liboracle.so" in loaded and "libsynth.so" in loaded
    assert line["impl"] == "reference" and line["value"] > 0
    # the GPU arm's config for the same workload and flags is the same object
    sys.path.insert(0, ROOT)
    import bench
    args = bench.argparse.Namespace(field_bf16=False, rng="mt19937")
    _, desc = bench.workload("gre", inputs=bench.Inputs(oracle_side=True))
    assert line["config"] == json.loads(json.dumps(bench.bench_config(args, desc)))
    assert line["metric"] == bench.METRIC
