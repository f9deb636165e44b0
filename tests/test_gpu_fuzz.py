"""Seeded randomised configurations (tests/fuzz_configs.py) on the GPU against the oracle:
trajectories, substrates and status bit for bit, M within the FP32 bar, the FP64 shadow within
1e-12, across precisions, generator flavours, BF16 records, walk tunings and the batch path."""
import pytest

from tests import fuzz_configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [7, 8])
def test_gpu_random_configurations_match_oracle(seed):
    assert fuzz_configs.main(20, seed=seed) == 0
