"""sw_engine: jobs cut into spin-range chunks on concurrent slots, phantoms resident, one seeding
per simulation seed. Every job must equal its own sw_sim run bit for bit."""
import ctypes as C

import numpy as np
import pytest

from spinwalk_gb300 import _lib, abi
from spinwalk_gb300.problem import Problem, cylinder_phantom, sphere_phantom
from tests.helpers import bits_equal

pytestmark = pytest.mark.gpu
FOV = 40e-6


def _jobs():
    mask, field = cylinder_phantom(24, FOV, 4e-6, 0.12, seed=5)
    mask2, field2 = sphere_phantom(20, 30e-6, 2e-6, 5e-6, 0.1, seed=6)
    gre = dict(TR_us=5050, TE_us=(2000, 5000), timestep_us=50)
    se = dict(TR_us=5050, TE_us=(5000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
              RF_us=(0, 2500), timestep_us=50, pXY=[[1, 0.3], [0.2, 1]])
    pgse = dict(se, gradient_us=(500, 1500, 3000, 4000),
                gradient_xyz=[[40, 0, 0], [0, 0, 0], [40, 0, 0], [0, 0, 0]])
    jobs = []
    for (m, f, fov), n, seed, kw, extra in (
            ((mask, field, FOV), 1000, 10, gre, {}),
            ((mask, field, FOV), 700, 10, se, {}),
            ((mask, field, 2 * FOV), 513, 10, se, {}),
            ((mask, field, FOV), 1000, 77, pgse, {}),
            ((mask, field, FOV), 300, 10, gre, dict(record_trajectory=True, n_dummy_scan=1)),
            ((mask2, field2, 30e-6), 900, 10, gre, dict(n_dummy_scan=2, linear_phase_cycling=7.5)),
            ((mask, field, FOV), 0, 10, gre, {})):
        jobs.append(Problem(m, [fov] * 3, f, n_spins=n, seed=seed, **kw, **extra))
    return jobs


@pytest.mark.parametrize("slots,slot_spins", [(3, 256), (1, 4096)])
def test_engine_jobs_equal_single_runs(slots, slot_spins):
    jobs = _jobs()
    eng = _lib.Engine(n_slots=slots, slot_spins=slot_spins)
    pids = {}
    outs = []
    for pr in jobs:
        key = (pr.mask.shape, float(pr.mask.sum()))
        if key not in pids:
            pids[key] = eng.add_phantom(pr)
        outs.append(eng.submit(pr, pids[key]))
    done = eng.run_all()
    assert sorted(j for j, rc, _ in done) == sorted(j for j, _ in outs)
    assert all(rc == 0 for _, rc, _ in done)
    for pr, (jid, o) in zip(jobs, outs):
        if pr.params.n_spins == 0:
            continue
        one = _lib.run(pr)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(o[k], one[k]), (jid, k)
    eng.close()


@pytest.mark.parametrize("prec", [abi.SW_PREC_FP64, abi.SW_PREC_KAHAN])
def test_engine_precision_modes(prec):
    pr = _jobs()[1]
    eng = _lib.Engine(n_slots=2, slot_spins=200)
    pid = eng.add_phantom(pr)
    _, o = eng.submit(pr, pid, precision=prec)
    eng.run_all()
    one = _lib.run(pr, precision=prec)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(o[k], one[k]), k
    eng.close()


def test_engine_rejects_bad_jobs():
    jobs = _jobs()
    eng = _lib.Engine(n_slots=1, slot_spins=128)
    pid = eng.add_phantom(jobs[0])
    with pytest.raises(_lib.SpinWalkError, match="unknown phantom"):
        eng.submit(jobs[0], pid + 5)
    with pytest.raises(_lib.SpinWalkError, match="phantom_size"):
        eng.submit(jobs[5], pid)
    bad = np.ascontiguousarray(jobs[0].mask.copy())
    bad[0, 0, 0] = 7                       # label >= n_substrate: refused at upload
    dims = (C.c_uint64 * 3)(*bad.shape)
    pid2 = C.c_int32()
    rc = _lib.lib().sw_engine_add_phantom(eng._h, bad.ctypes.data_as(C.c_void_p), None, dims, 2,
                                          C.byref(pid2))
    assert rc != 0 and b"substrate" in _lib.lib().sw_last_error()
    eng.close()


def test_engine_results_same_alone_and_in_a_mix_of_arrivals():
    """Continuous batching: jobs submitted while others run (polled in between) give the same
    results as each alone."""
    jobs = _jobs()[:6]
    alone = [_lib.run(pr) for pr in jobs]
    eng = _lib.Engine(n_slots=2, slot_spins=300)
    pids, outs = {}, []
    for i, pr in enumerate(jobs):
        key = (pr.mask.shape, float(pr.mask.sum()))
        if key not in pids:
            pids[key] = eng.add_phantom(pr)
        outs.append(eng.submit(pr, pids[key])[1])
        eng.poll(wait=1 if i % 2 else 0)          # let earlier jobs run before the next arrives
    eng.run_all()
    for k, (o, a) in enumerate(zip(outs, alone)):
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(o[key], a[key]), (k, key)
    eng.close()


def test_engine_evicts_idle_seed_caches_under_its_budget():
    """Requests with distinct seeds each need their own generator-state cache (2.5 KB per spin);
    under a small HBM budget the engine frees the caches no queued job uses, least recently used
    first, instead of refusing the next request. Every result still equals its run alone."""
    mask, field = cylinder_phantom(24, FOV, 4e-6, 0.12, seed=5)
    gre = dict(TR_us=3050, TE_us=(3000,), timestep_us=50)
    reqs = [Problem(mask, [FOV] * 3, field, n_spins=4000, seed=1000 + 17 * i, **gre)
            for i in range(6)]
    alone = [_lib.run(pr) for pr in reqs]
    probe = _lib.Engine(n_slots=2, slot_spins=2048)
    probe.add_phantom(reqs[0])
    base = probe.stats()["hbm_used"]            # slots and the resident phantom
    probe.close()
    cache = 4000 * (624 * 4 + 4)                 # one seed cache of 4000 spins
    eng = _lib.Engine(n_slots=2, slot_spins=2048, hbm_budget=base + int(2.5 * cache))
    try:
        pid = eng.add_phantom(reqs[0])
        for pr, want in zip(reqs, alone):
            _, out = eng.submit(pr, pid)
            assert all(rc == 0 for _, rc, _ in eng.run_all())
            for k in ("M1", "XYZ1", "T", "status"):
                assert bits_equal(out[k], want[k]), k
            st = eng.stats()
            assert st["hbm_used"] <= st["hbm_budget"] and st["seed_caches"] <= 2
        assert eng.stats()["seedings"] >= len(reqs)
    finally:
        eng.close()
