"""sw_sim_batch: several instances on one phantom with one seeding of the generators (the scale
loop of src/sim/monte_carlo.cu:273-337 and mixed sweeps). Every instance must equal its own
sw_sim run bit for bit."""
import numpy as np
import pytest

from spinwalk_gb300 import _lib
from spinwalk_gb300.problem import Problem, cylinder_phantom
from tests.helpers import bits_equal

FOV = 40e-6


def _phantom():
    return cylinder_phantom(24, FOV, 4e-6, 0.12, seed=5)


def _instances():
    mask, field = _phantom()
    xyz0 = _lib.initial_positions([FOV] * 3, 10, 1200)
    gre = dict(TR_us=10050, TE_us=(4000, 10000), timestep_us=50)
    se = dict(TR_us=10050, TE_us=(10000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
              RF_us=(0, 5000), timestep_us=50, pXY=[[1, 0.3], [0.2, 1]])
    pgse = dict(TR_us=10050, TE_us=(10000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                RF_us=(0, 5000), timestep_us=50, gradient_us=(1000, 3000, 6000, 8000),
                gradient_xyz=[[40, 0, 0], [0, 0, 0], [40, 0, 0], [0, 0, 0]])
    out = []
    for s, n, kw in ((1.0, 1200, gre), (0.5, 700, se), (2.0, 1200, se), (1.5, 333, gre),
                     (1.0, 1200, pgse), (1.0, 0, gre)):
        s32 = np.float32(s)
        fov = float(s32 * np.float32(FOV))
        out.append(Problem(mask, [fov] * 3, field, n_spins=n, seed=10,
                           XYZ0=(xyz0[:n] * s32).astype(np.float32), **kw))
    g = Problem(mask, [FOV] * 3, field, n_spins=900, seed=10, XYZ0=xyz0[:900],
                **dict(pgse, gradient_xyz=np.asarray(pgse["gradient_xyz"]) * np.float32(2.5)))
    out.append(g)
    return out


@pytest.mark.gpu
def test_batch_equals_one_run_per_instance():
    probs = _instances()
    batch = _lib.run_batch(probs)
    for k, (pr, b) in enumerate(zip(probs, batch)):
        if pr.params.n_spins == 0:
            continue
        one = _lib.run(pr)
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(b[key], one[key]), (k, key)


@pytest.mark.gpu
def test_batch_counts_its_work():
    """One pack + one seeding, then per instance k_init and its refill / walk rounds (two
    launches each); every instance needs at least one round."""
    probs = _instances()
    _lib.run_batch(probs)
    t = _lib.last_timing()
    busy = sum(1 for pr in probs if pr.params.n_spins)
    assert t["n_chunks"] >= busy
    assert t["n_launches"] >= 2 + 2 * t["n_chunks"] + busy


def test_batch_rejects_mixed_seeds_and_phantoms():
    probs = _instances()[:2]
    probs[1].params.seed = 11
    with pytest.raises(_lib.SpinWalkError, match="seed"):
        _lib.run_batch(probs)
    probs = _instances()[:2]
    probs[1].params.phantom_size[0] = 23
    probs[1].params.matrix_length = 23 * 24 * 24
    with pytest.raises(_lib.SpinWalkError, match="phantom"):
        _lib.run_batch(probs)
