"""Walk tuning: Morton re-sort of the spins (sw_order.cu), walk block size, sw_autotune. The tuning
only changes which thread walks which spin, so every result must equal the id-order run bit for
bit, through every entry point that walks."""
import numpy as np
import pytest

from spinwalk_gb300 import _lib
from spinwalk_gb300.problem import Problem, cylinder_phantom
from tests.helpers import bits_equal, load_golden


@pytest.fixture
def tuning():
    """Restores the default tuning after the test (the setting is process-wide)."""
    yield _lib.set_tuning
    _lib.set_tuning(0, 256, 0, 0)


def test_tuning_roundtrip_and_validation(tuning):
    tuning(3, 128, 5, 2, 7, 300, 3)
    want = dict(resort_interval=3, walk_block=128, seed_chunks=5, round_streams=2,
                jump_min_kwords=7, ring_steps=300, walk_blocks_per_sm=3)
    assert _lib.get_tuning() == want
    for bad in (dict(resort_interval=1, walk_block=100), dict(resort_interval=1, walk_block=512),
                dict(resort_interval=1 << 21, walk_block=256), dict(seed_chunks=65),
                dict(round_streams=3), dict(ring_steps=31), dict(ring_steps=4097),
                dict(walk_blocks_per_sm=17)):
        with pytest.raises(_lib.SpinWalkError):
            _lib.set_tuning(**bad)
    assert _lib.get_tuning() == want


def _dense_problem(n_spins=20000, TE_us=(3000, 9000), **kw):
    """Many spins per voxel (20000 spins in 16^3 voxels): sorted warps share voxels."""
    mask, field = cylinder_phantom(16, 32e-6, 3e-6, 0.2, seed=4)
    return Problem(mask, [32e-6] * 3, field, n_spins=n_spins, seed=7, TR_us=12050, TE_us=TE_us,
                   timestep_us=20, pXY=[[1, 0.4], [0.3, 1]], **kw)


def _same(a, b, keys=("M1", "XYZ1", "T", "status")):
    for k in keys:
        assert bits_equal(a[k], b[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["permeable", "se_multi_te", "lost_spins", "pgse_gradients",
                                  "out_of_bounds_reflect", "trajectory"])
@pytest.mark.parametrize("interval,block", [(1, 256), (3, 128), (2, 64)])
def test_sim_results_independent_of_walk_order(tuning, case, interval, block):
    pr, _ = load_golden(case)
    want = _lib.run(pr, fill=np.nan)
    tuning(interval, block)
    got = _lib.run(pr, fill=np.nan)
    _same(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_dense_sim_all_precisions_independent_of_walk_order(tuning, precision):
    pr = _dense_problem()
    want = _lib.run(pr, precision=precision, fp64_shadow=True, fill=np.nan)
    tuning(1, 256)
    got = _lib.run(pr, precision=precision, fp64_shadow=True, fill=np.nan)
    _same(got, want, ("M1", "XYZ1", "T", "status", "M1_fp64"))
    assert got["timing"]["n_launches"] > want["timing"]["n_launches"]    # the sorts ran


@pytest.mark.gpu
def test_batch_and_engine_independent_of_walk_order(tuning):
    probs = [_dense_problem(n) for n in (20000, 5000, 777)]
    want = [_lib.run(p, fill=np.nan) for p in probs]
    tuning(1, 128)
    got = _lib.run_batch(probs, fill=np.nan)
    for g, w in zip(got, want):
        _same(g, w)


@pytest.mark.gpu
def test_signal_mode_independent_of_walk_order(tuning):
    pr = _dense_problem()
    sig0, cnt0, st0 = _lib.run_signal(pr)
    tuning(1, 256)
    sig1, cnt1, st1 = _lib.run_signal(pr)
    assert np.array_equal(cnt1, cnt0)
    assert np.array_equal(st1, st0)
    # double sums of the same float terms in another order
    np.testing.assert_allclose(sig1, sig0, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_autotune_measures_every_candidate_and_applies(tuning):
    pr = _dense_problem(n_spins=50000)
    want = _lib.run(pr, fill=np.nan)
    best, table = _lib.autotune(pr, apply=True)
    assert len(table) == 12
    assert {(e["resort_interval"], e["walk_block"], e["ring_steps"]) for e in table} == {
        (i, b, 256) for i in (0, 1, 2, 4, 8) for b in (128, 256)} | {(0, 256, 128), (0, 256, 512)}
    assert all(e["ms_per_round"] > 0 for e in table)
    fastest = min(table, key=lambda e: e["ms_per_round"])
    assert (best["resort_interval"], best["walk_block"]) == (fastest["resort_interval"],
                                                           fastest["walk_block"])
    assert best["ring_steps"] == fastest["ring_steps"]
    assert _lib.get_tuning() == best
    _same(_lib.run(pr, fill=np.nan), want)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["permeable", "se_multi_te", "lost_spins", "pgse_gradients",
                                  "trajectory", "three_substrates", "bssfp_phase_cycling"])
@pytest.mark.parametrize("ring_steps", [32, 100, 256, 4096])
def test_sim_results_independent_of_ring_steps(tuning, case, ring_steps):
    """Rounds of any length (the steps one refill of a spin's Gaussian ring lasts, an autotuner
    candidate) give the results of the default rounds, in both generator flavours."""
    pr, _ = load_golden(case)
    for flavour in (0, 0x100):
        want = _lib.run(pr, precision=flavour, fill=np.nan)
        tuning(0, 256, 0, 0, 0, ring_steps)
        got = _lib.run(pr, precision=flavour, fill=np.nan)
        tuning()
        _same(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("ring_steps", [32, 256, 1000])
def test_engine_entry_points_independent_of_ring_steps(tuning, ring_steps):
    """Engines take the ring length in force when they are created: sw_sim_spins and
    sw_sim_signal (through the one-call engine) and a serving engine give the results of
    sw_sim with the default rounds, bit for bit (the signal's sums up to their order)."""
    pr, _ = load_golden("permeable")
    want = _lib.run(pr, fill=np.nan)
    want_sig = _lib.run_signal(pr)
    n = pr.params.n_spins
    tuning(0, 256, 0, 0, 0, ring_steps)
    got = _lib.run_spins(pr, 0, n, fill=np.nan)
    _same(got, want)
    sig, cnt, status = _lib.run_signal(pr)
    assert np.array_equal(cnt, want_sig[1]) and np.array_equal(status, want_sig[2])
    # the sums are float atomics: their order, not their terms, may differ
    assert np.allclose(sig, want_sig[0], rtol=1e-12, atol=1e-12 * max(1, int(cnt.max())))
    eng = _lib.Engine(n_slots=2, slot_spins=max(1, n // 3))
    try:
        pid = eng.add_phantom(pr)
        _, out = eng.submit(pr, pid, fill=np.nan)
        assert all(rc == 0 for _, rc, _ in eng.run_all())
        _same(out, want)
    finally:
        eng.close()


@pytest.mark.gpu
def test_dense_ring_steps_with_halves_resort_and_shadow(tuning):
    pr = _dense_problem(n_spins=150000)
    want = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    tuning(2, 128, 3, 2, 0, 77)
    got = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    _same(got, want, ("M1", "XYZ1", "T", "status", "M1_fp64"))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["permeable", "se_multi_te", "lost_spins", "trajectory",
                                  "out_of_bounds_periodic", "three_substrates"])
@pytest.mark.parametrize("chunks", [1, 3, 8, 64])
def test_sim_results_independent_of_seed_chunks(tuning, case, chunks):
    """The seed/walk pipeline (spins seeded in chunks beside the walk of earlier chunks) gives
    the results of seeding everything first; more chunks than spins included."""
    pr, _ = load_golden(case)
    tuning(0, 256, 1)
    want = _lib.run(pr, fill=np.nan)
    tuning(0, 256, chunks)
    got = _lib.run(pr, fill=np.nan)
    _same(got, want)


@pytest.mark.gpu
def test_dense_pipeline_with_resort_and_fp64_shadow(tuning):
    pr = _dense_problem(n_spins=150000)
    tuning(0, 256, 1)
    want = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    tuning(2, 128, 7)
    got = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    _same(got, want, ("M1", "XYZ1", "T", "status", "M1_fp64"))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["permeable", "se_multi_te", "lost_spins", "trajectory",
                                  "bssfp_phase_cycling"])
@pytest.mark.parametrize("chunks", [1, 3])
def test_sim_results_independent_of_round_streams(tuning, case, chunks):
    """The rounds as two independent halves on two streams give the one-stream results."""
    pr, _ = load_golden(case)
    tuning(0, 256, 1, 1)
    want = _lib.run(pr, fill=np.nan)
    tuning(0, 256, chunks, 2)
    got = _lib.run(pr, fill=np.nan)
    _same(got, want)



@pytest.mark.gpu
@pytest.mark.parametrize("cap", [1, 2, 3])
def test_dense_walk_grid_cap(tuning, cap):
    """A capped walk grid (blocks striding over the spins) walks every spin as the full grid."""
    pr = _dense_problem(n_spins=150000)
    want = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    tuning(0, 256, 1, 2, 0, 0, cap)
    got = _lib.run(pr, precision=2, fp64_shadow=True, fill=np.nan)
    _same(got, want, ("M1", "XYZ1", "T", "status", "M1_fp64"))


@pytest.mark.gpu
def test_batch_persistent_walk_equals_default(tuning):
    """With a cap on the walk's blocks per SM, the fused batch walk runs as persistent blocks that
    stride over the instances' work blocks (here 4 x 47 work blocks on at most one block per SM);
    every instance equals the uncapped batch bit for bit."""
    probs = []
    for k, s in enumerate((1.0, 0.8, 1.25, 1.1)):
        pr = _dense_problem(n_spins=12000, TE_us=(3000, 9000), RF_FA=(90.0, 180.0),
                            RF_PH=(0.0, 90.0), RF_us=(0, 4500))
        s32 = np.float32(s)
        pr.params.fov[0] = pr.params.fov[1] = pr.params.fov[2] = float(s32 * np.float32(32e-6))
        pr.XYZ0 = (pr.XYZ0 * s32).astype(np.float32)
        probs.append(pr)
    want = _lib.run_batch(probs, fill=np.nan)
    tuning(walk_blocks_per_sm=1)
    got = _lib.run_batch(probs, fill=np.nan)
    for a, b in zip(want, got):
        _same(a, b)
