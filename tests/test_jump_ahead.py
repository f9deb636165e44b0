"""Jump-ahead seeding: the state of mt19937(seed + spin) after discard(seed + spin)
(src/sim/kernels.cu:82-88) computed through x^J mod phi instead of seed + spin generated words,
for large discard counts (sw_mtjump.h, k_seed_jump; by default from 1408 x 1024 words).

CPU: the host polynomials against libstdc++'s own discard, at the edges of a regeneration and
far out (a random 32-bit seed, the reference's SEED = 0 case). GPU: walks of high spin ids, of
large seeds and of ranges across the threshold, against the oracle (which discards word by
word), and through the serving engine with a distinct seed per request."""
import numpy as np
import pytest

from spinwalk_gb300 import _lib
from spinwalk_gb300.problem import Problem, cylinder_phantom
from tests import oracle_lib
from tests.helpers import bits_equal, m_close

JUMP_MIN_Z = 1408 * 1024
NEVER = 0xffffffff              # jump_min_kwords beyond any discard count: every spin discards


@pytest.fixture
def tuning():
    """Restores the default tuning after the test (the setting is process-wide)."""
    yield _lib.set_tuning
    _lib.set_tuning()


@pytest.mark.parametrize("z", [1, 623, 624, 625, 1247, 1248, 5000, JUMP_MIN_Z - 1, JUMP_MIN_Z,
                               JUMP_MIN_Z + 623, 7_000_001, 2 ** 27 + 5])
def test_host_jump_matches_discard(z):
    got, pos = _lib.debug_mt_jump(z)
    want, wpos = oracle_lib.mt_discard(z)
    assert pos == wpos
    assert np.array_equal(got, want)


def test_host_jump_matches_discard_for_a_random_32bit_seed():
    z = 3_000_000_017 + 41          # SEED = 0 draws a seed like this (simulation_parameters.cuh:233)
    got, pos = _lib.debug_mt_jump(z)
    want, wpos = oracle_lib.mt_discard(z)
    assert pos == wpos and np.array_equal(got, want)


def _problem(n_spins, seed, **kw):
    mask, field = cylinder_phantom(20, 40e-6, 4e-6, 0.15, seed=5)
    return Problem(mask, [40e-6] * 3, field, n_spins=n_spins, seed=seed, TR_us=6050,
                   TE_us=(3000, 6000), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0), RF_us=(0, 1500),
                   timestep_us=50, pXY=[[1, 0.3], [0.3, 1]], **kw)


def _check_rows(got, pr, lo, hi):
    want = oracle_lib.run(pr, spin_ids=np.arange(lo, hi, dtype=np.uint32))
    for k in ("XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k][lo:hi]), k
    ok, rel = m_close(got["M1"], want["M1"][lo:hi])
    assert ok, rel


@pytest.mark.gpu
@pytest.mark.parametrize("lo", [2_000_003, 5_500_000, 9_999_800])
def test_gpu_high_spin_ids_jump(lo):
    """Spin ids in [2e6, 1e7) with seed 10: every spin of the range jumps."""
    pr = _problem(10_000_000, 10)
    hi = lo + 160
    got = _lib.run_spins(pr, lo, hi)
    _check_rows(got, pr, lo, hi)


@pytest.mark.gpu
def test_gpu_range_across_the_jump_boundary():
    """Spins on both sides of the default threshold in one call: the lower ones discard, the
    upper ones jump, and both match."""
    seed = 10
    lo, hi = JUMP_MIN_Z - seed - 150, JUMP_MIN_Z - seed + 170
    pr = _problem(hi + 10, seed)
    got = _lib.run_spins(pr, lo, hi)
    _check_rows(got, pr, lo, hi)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 2])
def test_gpu_large_seed_whole_problem(precision):
    """A seed of 1.3e8 (all spins jump) through sw_sim, FP32 and Kahan."""
    pr = _problem(96, 2 ** 27 + 7)
    got = _lib.run(pr, precision=precision)
    want = oracle_lib.run(pr, precision=precision)
    for k in ("XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k]), k
    ok, rel = m_close(got["M1"], want["M1"])
    assert ok, rel


@pytest.mark.gpu
def test_gpu_engine_requests_with_distinct_seeds_equal_their_runs_alone():
    """Serving with a distinct seed per request (no request shares another's generator states):
    each result equals the request's own sw_sim run bit for bit, small seeds (discard) and
    large ones (jump) in the same mix."""
    seeds = [10, 77, 3_000_017, 2 ** 24 + 3, 12_345_678, 999]
    reqs = [_problem(n, s) for n, s in zip((300, 1200, 50, 100, 64, 2000), seeds)]
    alone = [_lib.run(pr) for pr in reqs]
    eng = _lib.Engine(n_slots=3, slot_spins=512)
    try:
        pid = eng.add_phantom(reqs[0])
        jobs = [eng.submit(pr, pid) for pr in reqs]
        done = eng.run_all()
        assert sorted(j for j, rc, _ in done) == sorted(j for j, _ in jobs)
        assert all(rc == 0 for _, rc, _ in done)
        for (jid, out), want in zip(jobs, alone):
            for k in ("M1", "XYZ1", "T", "status"):
                assert bits_equal(out[k], want[k]), (jid, k)
    finally:
        eng.close()
    # and the large-seed requests match the oracle
    for pr, out in zip(reqs, alone):
        if pr.params.seed > JUMP_MIN_Z:
            want = oracle_lib.run(pr)
            assert bits_equal(out["XYZ1"], want["XYZ1"])


@pytest.mark.gpu
@pytest.mark.parametrize("seed,n", [(10, 5000), (2 ** 31 + 5, 1500)])
def test_gpu_jump_equals_discard_on_every_spin(tuning, seed, n):
    """The same spins seeded by discard (threshold out of reach) and by jump-ahead (threshold
    1024 words: nearly every spin jumps) walk identically, bit for bit -- including a seed of
    2^31 + 5, where the discard regenerates over 2e9 words per spin."""
    pr = _problem(n, seed)
    tuning(jump_min_kwords=NEVER)
    want = _lib.run(pr, fill=np.nan)
    t_discard = want["timing"]["seed_ms"]
    tuning(jump_min_kwords=1)
    got = _lib.run(pr, fill=np.nan)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k]), k
    if seed > 2 ** 30:           # the whole point: far cheaper than the discard
        assert got["timing"]["seed_ms"] < 0.2 * t_discard


@pytest.mark.gpu
def test_gpu_engine_jump_equals_discard(tuning):
    """The serving engine's seeding takes the same path: a request with a large seed gives the
    same result with and without jump-ahead."""
    pr = _problem(3000, 5_000_003)
    outs = []
    for kw in (NEVER, 1):
        tuning(jump_min_kwords=kw)
        eng = _lib.Engine(n_slots=2, slot_spins=1024)
        try:
            pid = eng.add_phantom(pr)
            _, out = eng.submit(pr, pid)
            assert all(rc == 0 for _, rc, _ in eng.run_all())
            outs.append(out)
        finally:
            eng.close()
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(outs[0][k], outs[1][k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("offset,count", [(0, 1), (623, 1), (622, 3), (620, 9), (1, 624),
                                          (311, 625), (0, 1249)])
def test_gpu_jump_pairs_at_regeneration_edges(tuning, offset, count):
    """k_seed_jump seeds two spins that share R per thread block: R changes where
    (seed + spin) % 624 == 1, so a range splits into segments of 624 spins paired from their
    start. Ranges that begin or end at such an edge, single spins and odd segments (one spin
    computed alone) seed the same by jump-ahead as by discard, bit for bit."""
    seed = 5000
    base = (1 - seed) % 624 + 624 * 2           # (seed + base) % 624 == 1
    lo = base + offset
    hi = lo + count
    pr = _problem(hi + 5, seed)
    tuning(jump_min_kwords=NEVER)
    want = _lib.run_spins(pr, lo, hi)
    tuning(jump_min_kwords=1)
    got = _lib.run_spins(pr, lo, hi)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k]), k
