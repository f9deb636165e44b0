"""Parity at the benchmark workloads' full sizes (the workloads bench.py measures).

The oracle cannot walk a million spins in seconds, so at full size the CUDA path is checked in
two ways that do not depend on the size:

* a stratified sample of spin ids (evenly spread over the whole id range, so the largest
  discard(seed + spin) counts are included) is run by the oracle and compared with the same
  rows of the full GPU run: trajectories, echo substrates and status bit for bit, M1 within
  the FP32 bar (1e-5 of |M| + 1e-7), as in the small parity tests;
* properties of the whole run: |M| <= 1 for every spin (rotations keep the norm, relaxation
  towards (0, 0, 1) does not increase it); spin-range shards (sw_sim_spins) equal the rows of
  the full run bit for bit; the fused signal sums (sw_sim_signal) equal the per-tissue
  reduction of the full run's M1; the FP32 run's error against the FP64 shadow of the same
  walk is below 1e-5, and below 1e-6 with compensated (Kahan) phase sums on the spin echo
  workload (2001 time points), which leaves trajectories unchanged.

Workloads: gradient echo, 200^3 cylinders, 1e5 spins, 401 time points; spin echo, 500^3 spheres,
1e6 spins, 2001 time points, permeability 0.01; the 64-instance FoV sweep (32 radii x GRE/SE,
1e4-1e6 spins each) through sw_sim_batch; bSSFP on 300^3 cylinders with 2e5 spins and 210 TRs
of 200 time points, through sw_sim_tracks (a subset of the 640 phase-cycle x dummy-scan
instances); requests of the serving trace on its resident 100^3, 200^3 and 800^3 phantoms
through one engine (each the same alone and in the mix).
"""
import numpy as np
import pytest

import bench
from spinwalk_gb300 import _lib, abi
from tests import oracle_lib
from tests.helpers import bits_equal, m_close

pytestmark = pytest.mark.gpu

N_SAMPLE = 2048


def _sample_ids(n, k=N_SAMPLE):
    return bench.cpu_sample_ids(n, k)


def _oracle_rows(pr, ids):
    """Oracle outputs of the spins `ids` (their rows only)."""
    o = oracle_lib.run(pr, spin_ids=ids, fill=np.nan)
    return {k: o[k][ids] for k in ("M1", "XYZ1", "T", "status")}


def _check_rows(got, ref, ids, what):
    for k in ("XYZ1", "T", "status"):
        assert bits_equal(got[k][ids], ref[k]), f"{what}: {k} of the sampled spins differs"
    ok, rel = m_close(got["M1"][ids], ref["M1"])
    assert ok, f"{what}: M1 of the sampled spins differs from the oracle by {rel:.3e} of |M|"


def _norm_bound(m1, status):
    m = m1[status == abi.SW_SPIN_OK].astype(np.float64)
    return float(np.max(np.linalg.norm(m, axis=-1))) if m.size else 0.0


@pytest.fixture(scope="module", params=["gre", "se"])
def plain(request):
    pr, desc = bench.workload(request.param)
    out = _lib.run(pr, fill=np.nan)         # unreached echoes stay NaN
    return request.param, pr, out


def test_full_size_sample_equals_oracle(plain):
    name, pr, out = plain
    ids = _sample_ids(pr.params.n_spins)
    _check_rows(out, _oracle_rows(pr, ids), ids, name)


def test_full_size_properties(plain):
    name, pr, out = plain
    st = out["status"]
    assert np.all(np.isin(st, (abi.SW_SPIN_OK, abi.SW_SPIN_LOST, abi.SW_SPIN_OOB,
                               abi.SW_SPIN_START_OOB)))
    assert np.mean(st == abi.SW_SPIN_OK) > 0.99
    assert _norm_bound(out["M1"], st) <= 1.0 + 1e-6
    # the echo substrate is a mask label
    assert int(out["T"][st == abi.SW_SPIN_OK].max()) < pr.params.n_substrate


def test_full_size_shards_equal_rows(plain):
    name, pr, out = plain
    n = pr.params.n_spins
    for lo, hi in ((0, 4096), (n // 2 - 1000, n // 2 + 3000), (n - 5000, n)):
        s = _lib.run_spins(pr, lo, hi, fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(s[k], out[k][lo:hi]), f"{name}: shard [{lo}, {hi}) {k} differs"


def test_full_size_signal_equals_reduction(plain):
    name, pr, out = plain
    sig, cnt, st = _lib.run_signal(pr)
    assert bits_equal(st, out["status"])
    ns = pr.params.n_substrate
    for e in range(pr.n_te):                 # every echo a spin reached, by its substrate there
        m = out["M1"][:, e, :].astype(np.float64)
        reached = ~np.isnan(m[:, 0])
        t = out["T"][reached, e].astype(np.int64)
        ref = np.zeros((ns, 3))
        np.add.at(ref, t, m[reached])
        assert np.array_equal(cnt[e], np.bincount(t, minlength=ns).astype(np.uint64))
        # double sums of up to 1e6 floats in a different order
        assert np.allclose(sig[e], ref, rtol=1e-9, atol=1e-9 * max(1, len(t))), (name, e)


def test_full_size_error_against_fp64(plain):
    name, pr, out = plain
    sh = _lib.run(pr, fp64_shadow=True, fill=np.nan)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(sh[k], out[k]), f"{name}: the FP64 shadow changed the FP32 {k}"
    ok = out["status"] == abi.SW_SPIN_OK
    err32 = float(np.max(np.abs(out["M1"][ok].astype(np.float64) - sh["M1_fp64"][ok])))
    assert err32 <= 1e-5, f"{name}: FP32 error against FP64 {err32:.3e}"
    if name == "se":
        kh = _lib.run(pr, precision=abi.SW_PREC_KAHAN, fp64_shadow=True, fill=np.nan)
        assert bits_equal(kh["XYZ1"], out["XYZ1"]) and bits_equal(kh["T"], out["T"])
        errk = float(np.max(np.abs(kh["M1"][ok].astype(np.float64) - kh["M1_fp64"][ok])))
        assert errk <= 1e-6, f"Kahan error against FP64 {errk:.3e}"
        assert errk < err32


def test_full_size_fov_sweep_batch():
    """64 instances (32 FoV scales x GRE/SE, 1e4-1e6 spins each) in one sw_sim_batch call:
    sampled spins of every instance equal the oracle's run of that instance."""
    probs, desc = bench.c3_instances()
    outs = _lib.run_batch(probs, fill=np.nan)
    for i, (pr, o) in enumerate(zip(probs, outs)):
        ids = _sample_ids(pr.params.n_spins, 128)
        _check_rows(o, _oracle_rows(pr, ids), ids, f"instance {i}")
        assert _norm_bound(o["M1"], o["status"]) <= 1.0 + 1e-6


def test_full_size_bssfp_tracks():
    """bSSFP on the 300^3 phantom, 2e5 spins, 200 time points per TR: phase-cycling x
    DUMMY_SCAN instances on one walk; sampled spins of four instances equal the oracle run of
    that instance (42,000 time points each for DUMMY_SCAN 209)."""
    pr, desc = bench.workload("bssfp")
    tracks = [dict(linear_phase_cycling=5.625 * i, n_dummy_scan=d)
              for i in (0, 17, 40, 63) for d in (200, 209)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan)
    # one walk: instances with the same scan count end at the same positions and substrates
    for j, t in enumerate(tracks):
        first = next(i for i, u in enumerate(tracks) if u["n_dummy_scan"] == t["n_dummy_scan"])
        for k in ("XYZ1", "T", "status"):
            assert bits_equal(outs[j][k], outs[first][k]), (j, k)
    for j in (0, 3, 4, 7):
        t = tracks[j]
        pr.params.linear_phase_cycling = t["linear_phase_cycling"]
        pr.params.n_dummy_scan = t["n_dummy_scan"]
        ids = _sample_ids(pr.params.n_spins, 256)
        _check_rows(outs[j], _oracle_rows(pr, ids), ids, f"track {j}")
    for o in outs:
        assert _norm_bound(o["M1"], o["status"]) <= 1.0 + 1e-6


def test_full_size_serving_trace():
    """Requests of the serving trace (GRE / SE / PGSE along x, y, z on the resident 100^3,
    200^3 and 800^3 phantoms, 1e4-2e6 spins) submitted to one engine in arrival order while the
    earlier ones run, with the serving benchmark's slots (8 x 2^20 spins, so the larger jobs run
    in chunks): each result equals the request run alone bit for bit, and sampled spins equal
    the oracle."""
    reqs, phantoms, arrivals, kinds, desc = bench.serve_requests(40)
    picked = [pr for pr in reqs if pr.params.n_spins <= 2_000_000][:12]
    assert len({pr.mask.shape for pr in picked}) > 1
    eng = _lib.Engine(n_slots=8, slot_spins=1 << 20)
    pids, outs, done = {}, [], []
    for pr in picked:
        if pr.mask.shape not in pids:
            pids[pr.mask.shape] = eng.add_phantom(pr)
        outs.append(eng.submit(pr, pids[pr.mask.shape], fill=np.nan)[1])
        done += eng.poll(wait=0)
    done += eng.run_all()
    eng.close()
    assert len(done) == len(picked) and all(rc == 0 for _, rc, _ in done)
    for k, (pr, o) in enumerate(zip(picked, outs)):
        alone = _lib.run(pr, fill=np.nan)
        for key in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(o[key], alone[key]), f"request {k}: {key} differs in the mix"
        ids = _sample_ids(pr.params.n_spins, 64)
        _check_rows(alone, _oracle_rows(pr, ids), ids, f"request {k}")
