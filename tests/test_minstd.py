"""The generator flavour of the reference's CUDA build (SW_RNG_MINSTD: thrust::minstd_rand +
thrust::normal_distribution<float> + uniform_real_distribution<float>, src/sim/kernels.cu:76-80)
against the reference's own sim::sim as its nvcc host path builds it (fixtures from
tests/golden/make_golden_minstd.py)."""
import os

import numpy as np
import pytest

from spinwalk_gb300 import abi
from tests import oracle_lib
from tests.helpers import GOLDEN_CASES, GOLDEN_DIR, bits_equal, load_golden, m_close

FIX = os.path.join(GOLDEN_DIR, "minstd_outputs.npz")
MINSTD = abi.SW_PREC_FP32 | abi.SW_RNG_MINSTD


def _fixture(case):
    z = np.load(FIX)
    return {k: z[case + "/" + k] for k in ("M1", "XYZ1", "T")}


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_minstd_matches_reference_fixture(case):
    pr, _ = load_golden(case)
    o = oracle_lib.run(pr, precision=MINSTD)
    ref = _fixture(case)
    for k in ("M1", "XYZ1", "T"):
        assert bits_equal(o[k], ref[k]), k


@pytest.mark.skipif(not oracle_lib.ref_nvcc_available(),
                    reason="reference source tree not present (its nvcc host build)")
@pytest.mark.parametrize("seed", [7, 8])
def test_oracle_minstd_matches_reference_on_random_configs(seed):
    """The randomised configurations of the GPU parity test (tests/fuzz_configs.py, same seeds)
    in this flavour: the oracle equals the reference's nvcc host build bit for bit."""
    from tests import fuzz_configs
    rng = np.random.default_rng(seed)
    for trial in range(20):
        pr = fuzz_configs.random_case(rng)[0]
        a = oracle_lib.run(pr, precision=MINSTD, fill=np.nan)
        b = oracle_lib.run_ref_nvcc(pr, fill=np.nan)
        for k in ("M1", "XYZ1", "T"):
            assert bits_equal(a[k], b[k]), (trial, k)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_minstd_matches_reference_fixture(case):
    from spinwalk_gb300 import _lib
    pr, _ = load_golden(case)
    g = _lib.run(pr, precision=MINSTD)
    ref = _fixture(case)
    assert bits_equal(g["XYZ1"], ref["XYZ1"])
    assert bits_equal(g["T"], ref["T"])
    ok, rel = m_close(g["M1"], ref["M1"])
    assert ok, rel


@pytest.mark.gpu
def test_gpu_minstd_engine_and_batch():
    from spinwalk_gb300 import _lib
    pr, _ = load_golden("permeable")
    one = _lib.run(pr, precision=MINSTD)
    eng = _lib.Engine(n_slots=2, slot_spins=37)
    _, o = eng.submit(pr, eng.add_phantom(pr), precision=MINSTD)
    eng.run_all()
    eng.close()
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(o[k], one[k]), k


@pytest.mark.gpu
def test_gpu_minstd_deviate_equals_host_on_every_engine_output():
    """Device erfcinvf-based deviate == the oracle's (CUDA's host erfcinvf) for every engine
    output up to the fold (the deviates above it are the same magnitudes, negated), and on a
    sample above it."""
    torch = pytest.importorskip("torch")
    from spinwalk_gb300 import _lib
    chunk = 1 << 26
    top = (2147483647 - 2) // 2 + 1                 # u = x - 1 <= range / 2
    rng = np.random.default_rng(1)
    starts = list(range(1, top + 1, chunk)) + [int(v) for v in rng.integers(top, 2147483647 - chunk, 2)]
    d = torch.empty(chunk, dtype=torch.float32, device="cuda")
    for x0 in starts:
        n = min(chunk, 2147483647 - x0)
        _lib.debug_ms_normal(x0, n, d.data_ptr())
        torch.cuda.synchronize()
        got = d[:n].cpu().numpy()
        want = oracle_lib.host_ms_normal(x0, n)
        bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, f"{bad.size} mismatches from x={x0}, first x={x0 + bad[0]}"
