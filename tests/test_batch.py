"""sw_sim_batch: several instances on one phantom with one seeding of the generators (the scale
loop of src/sim/monte_carlo.cu:273-337 and mixed sweeps). Every instance must equal its own
sw_sim run bit for bit."""
import copy

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
    """One pack + one seeding of the pooled generator streams, k_init per instance, then rounds
    of three launches whatever the number of instances: the refill of the streams, the crossing
    uniforms of every instance and the walk of every instance; at least one round."""
    probs = _instances()
    _lib.run_batch(probs)
    t = _lib.last_timing()
    busy = sum(1 for pr in probs if pr.params.n_spins)
    assert busy > 1
    assert t["n_chunks"] >= 1
    assert t["n_launches"] == 2 + busy + 3 * t["n_chunks"]


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


def _rejecting_instances(n_inst=12, n=900, seed=31):
    """Instances that draw at different paces from the same generator streams: a three-substrate
    random mask (a crossing attempt on most steps) with partial permeabilities, reflecting and
    periodic boundaries, different FoV scales and sequences."""
    rng = np.random.default_rng(2)
    mask = rng.integers(0, 3, (16, 16, 16)).astype(np.uint8)
    field = rng.normal(0, 1e-7, (16, 16, 16)).astype(np.float32)
    fov = 16e-6
    xyz0 = _lib.initial_positions([fov] * 3, seed, n)
    out = []
    for i in range(n_inst):
        s32 = np.float32(0.6 + 0.1 * i)
        f = float(s32 * np.float32(fov))
        kw = dict(TR_us=8050, TE_us=(3000, 8000), timestep_us=50,
                  diffusivity=(1e-9, 2e-9, 0.5e-9), T1_ms=(1000.0, 1500.0, 2000.0),
                  T2_ms=(40.0, 30.0, 20.0),
                  pXY=[[1, .5 - .03 * i, .1], [.4, 1, .2], [.3, .6, 1]], cross_fov=i % 3 != 0)
        if i % 2:
            kw.update(RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0), RF_us=(0, 4000))
        out.append(Problem(mask, [f] * 3, field, n_spins=n - 37 * i, seed=seed,
                           XYZ0=(xyz0[:n - 37 * i] * s32).astype(np.float32), **kw))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_pooled_streams_with_uneven_consumption_equal_one_run_per_instance(precision):
    """The pooled generator streams serve instances that reject crossings at different rates
    (so their read positions drift apart within a round, further than a ring holds) and finish
    at different times."""
    probs = _rejecting_instances()
    batch = _lib.run_batch(probs, precision=precision, fill=np.nan)
    assert batch[0]["timing"]["n_chunks"] >= 2
    for k, (pr, b) in enumerate(zip(probs, batch)):
        one = _lib.run(pr, precision=precision, fill=np.nan)
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(b[key], one[key]), (k, key)


@pytest.mark.gpu
def test_pooled_batch_with_jump_ahead_seeds_and_the_minstd_flavour():
    """A large seed (the streams seeded by jump-ahead) and, through the engine path, the
    generator flavour of the reference's CUDA build."""
    probs = _rejecting_instances(n_inst=4, n=400, seed=2 ** 29 + 11)
    batch = _lib.run_batch(probs, fill=np.nan)
    for k, (pr, b) in enumerate(zip(probs, batch)):
        one = _lib.run(pr, fill=np.nan)
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(b[key], one[key]), (k, key)
    probs = _instances()
    batch = _lib.run_batch(probs, precision=0x100)
    for k, (pr, b) in enumerate(zip(probs, batch)):
        if pr.params.n_spins:
            one = _lib.run(pr, precision=0x100)
            for key in ("M1", "XYZ1", "T", "status"):
                assert bits_equal(b[key], one[key]), (k, key)


@pytest.mark.gpu
def test_batch_refused_mask_then_batch_matches():
    """The pooled batch seeds its generator streams before it uploads the phantom. A batch refused
    afterwards (a mask label >= n_substrate, found by the pack) waits for that seeding, and the
    next batch equals one run per instance bit for bit."""
    probs = _instances()
    bad = [copy.copy(pr) for pr in probs]
    mask = probs[0].mask.copy()
    mask.flat[0] = 9
    for pr in bad:
        pr.mask = mask
    with pytest.raises(_lib.SpinWalkError, match="substrate labels"):
        _lib.run_batch(bad)
    batch = _lib.run_batch(probs)
    for k, (pr, b) in enumerate(zip(probs, batch)):
        if pr.params.n_spins:
            one = _lib.run(pr)
            for key in ("M1", "XYZ1", "T", "status"):
                assert bits_equal(b[key], one[key]), (k, key)


@pytest.mark.gpu
def test_release_workspaces_frees_device_memory_and_calls_still_match():
    """sw_release_workspaces gives back the device memory that sw_sim and sw_sim_batch keep
    between calls; the calls after it allocate again and give the same results."""
    torch = pytest.importorskip("torch")
    probs = _instances()
    a = _lib.run_batch(probs)
    one = _lib.run(probs[0])
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    _lib.release_workspaces()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after > free_before
    _lib.release_workspaces()                  # nothing left to free: still fine
    b = _lib.run_batch(probs)
    again = _lib.run(probs[0])
    for k, (pr, x, y) in enumerate(zip(probs, a, b)):
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(x[key], y[key]), (k, key)
    for key in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(one[key], again[key]), key


@pytest.mark.gpu
def test_batch_of_many_instances_with_empty_ones():
    """Eighty instances (more than the batch reads back in pieces, some with no spins, first and
    last among them) of different sizes, FoV scales and sequences: the fused launches find every
    block's instance and every instance equals its own sw_sim run bit for bit."""
    mask, field = _phantom()
    xyz0 = _lib.initial_positions([FOV] * 3, 10, 400)
    rng = np.random.default_rng(17)
    gre = dict(TR_us=4050, TE_us=(2000, 4000), timestep_us=50)
    se = dict(TR_us=4050, TE_us=(4000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
              RF_us=(0, 2000), timestep_us=50, pXY=[[1, 0.3], [0.2, 1]])
    probs = []
    for i in range(80):
        n = 0 if i in (0, 33, 79) else int(rng.integers(1, 400))
        s32 = np.float32(0.5 + 0.02 * i)
        probs.append(Problem(mask, [float(s32 * np.float32(FOV))] * 3, field, n_spins=n, seed=10,
                             XYZ0=(xyz0[:n] * s32).astype(np.float32), **(gre if i % 2 else se)))
    batch = _lib.run_batch(probs, fill=np.nan)
    for k, (pr, b) in enumerate(zip(probs, batch)):
        if pr.params.n_spins == 0:
            continue
        one = _lib.run(pr, fill=np.nan)
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(b[key], one[key]), (k, key)


@pytest.mark.gpu
def test_batch_of_one_instance():
    """A batch of a single instance (one read-back piece) equals its sw_sim run."""
    pr = _instances()[0]
    b = _lib.run_batch([pr], fill=np.nan)[0]
    one = _lib.run(pr, fill=np.nan)
    for key in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(b[key], one[key]), key
