"""Randomised configurations for parity runs of the CUDA path against the oracle: sequences with
several RF pulses and echoes, dephasing and multi-axis gradient events, dummy scans with linear
and quadratic phase cycling, two or three substrates with permeabilities and zero
diffusivities, periodic or reflecting boundaries, recorded trajectories, the precision modes,
both generator flavours, bfloat16 field records and the walk tunings. Used by
tests/test_gpu_fuzz.py (a few seeded trials) and for longer campaigns (`python -m
tests.fuzz_configs N`)."""
import sys

import numpy as np

from spinwalk_gb300 import abi
from spinwalk_gb300.problem import Problem, cylinder_phantom


def bf16_round(a):
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def random_case(rng):
    """(Problem, precision flags, fp64 shadow, tuning tuple, whether to run through the batch
    path) for one random configuration."""
    n = int(rng.integers(8, 33))
    ns = int(rng.choice([2, 2, 3]))
    mask, field = cylinder_phantom(n, n * 1e-6, float(rng.uniform(1.5e-6, 5e-6)),
                                   float(rng.uniform(0.05, 0.25)), seed=int(rng.integers(1 << 30)))
    if ns == 3:
        mask = mask + (rng.random(mask.shape) < 0.1).astype(np.uint8) * (mask == 0) * 2
    dt = int(rng.choice([20, 25, 50]))
    n_tp = int(rng.integers(20, 200))
    TR = n_tp * dt + dt
    n_rf = int(rng.integers(1, 4))
    rf_us = [0] + sorted(int(x) * dt for x in rng.choice(np.arange(1, n_tp), n_rf - 1, replace=False))
    rf_fa = [float(rng.choice([30.0, 90.0, 180.0, float(rng.uniform(5, 175))])) for _ in range(n_rf)]
    rf_ph = [float(rng.choice([0.0, 90.0, 180.0, 270.0, float(rng.uniform(0, 360))]))
             for _ in range(n_rf)]
    n_te = int(rng.integers(0, 4))
    te = sorted(set(int(x) * dt for x in rng.integers(1, n_tp, n_te)))
    # discard(seed + spin) costs the oracle ~1 ns per word per spin: seeds below 1e5, or (one case
    # in ten) a seed up to 2^31 with at most 4 spins
    if rng.random() < 0.1:
        n_spins, seed = int(rng.integers(1, 5)), int(rng.integers(1, (1 << 31) - 8))
    else:
        n_spins, seed = int(rng.integers(1, 1500)), int(rng.integers(1, 100000))
    kw = dict(timestep_us=dt, TR_us=TR, TE_us=tuple(te), RF_FA=tuple(rf_fa), RF_PH=tuple(rf_ph),
              RF_us=tuple(rf_us), n_spins=n_spins, seed=seed, n_dummy_scan=int(rng.integers(0, 3)),
              linear_phase_cycling=float(rng.choice([0.0, float(rng.uniform(0, 360))])),
              quadratic_phase_cycling=float(rng.choice([0.0, float(rng.uniform(0, 30))])),
              cross_fov=bool(rng.integers(0, 2)), record_trajectory=bool(rng.random() < 0.15),
              diffusivity=tuple(float(rng.choice([0.0, 1e-9, 2e-9, float(rng.uniform(2e-10, 3e-9))]))
                                for _ in range(ns)),
              T1_ms=tuple(float(rng.choice([-1.0, float(rng.uniform(100, 3000))])) for _ in range(ns)),
              T2_ms=tuple(float(rng.uniform(10, 100)) for _ in range(ns)),
              pXY=rng.uniform(0, 1, (ns, ns)) * (rng.random((ns, ns)) < 0.8))
    if rng.random() < 0.4:                                   # dephasing events
        k = int(rng.integers(1, 4))
        kw["dephasing_us"] = tuple(sorted(int(x) * dt for x in rng.integers(0, n_tp, k)))
        kw["dephasing_deg"] = tuple(float(rng.uniform(-180, 180)) for _ in range(k))
    if rng.random() < 0.5:                                   # gradient events
        k = int(rng.integers(1, min(60, n_tp)))
        g_us = sorted(set(int(x) * dt for x in rng.integers(0, n_tp, k)))
        g = rng.uniform(-100, 100, (len(g_us), 3)).astype(np.float32)
        g *= (rng.random((len(g_us), 3)) < 0.6)              # some axes zero (single-axis lobes)
        kw["gradient_us"] = tuple(g_us)
        kw["gradient_xyz"] = g
    with_field = rng.random() < 0.85
    pr = Problem(mask, [n * 1e-6] * 3, field if with_field else None, **kw)
    prec = int(rng.choice([abi.SW_PREC_FP32, abi.SW_PREC_FP32, abi.SW_PREC_KAHAN, abi.SW_PREC_FP64]))
    if rng.random() < 0.25:
        prec |= abi.SW_RNG_MINSTD
    bf16 = with_field and rng.random() < 0.2
    if bf16:
        prec |= abi.SW_FIELD_BF16
    shadow = bool(rng.random() < 0.3)
    tuning = (int(rng.choice([0, 0, 1, 3])), int(rng.choice([64, 128, 256])),
              int(rng.choice([0, 1, 3])), int(rng.choice([0, 1, 2])))
    batch = bool(rng.random() < 0.2) and not kw["record_trajectory"]
    return pr, prec, shadow, tuning, batch, bf16


def check_case(pr, prec, shadow, tuning, batch, bf16):
    """Runs one case on the GPU and the oracle; returns None or a description of a mismatch."""
    import copy

    from spinwalk_gb300 import _lib
    from tests import oracle_lib
    from tests.helpers import bits_equal, m_close
    _lib.set_tuning(*tuning)
    try:
        if batch:
            g = _lib.run_batch([pr], precision=prec, fill=np.nan)[0]
        else:
            g = _lib.run(pr, precision=prec, fp64_shadow=shadow, fill=np.nan)
    finally:
        _lib.set_tuning(0, 256, 0, 0)
    q = pr
    if bf16:
        q = copy.copy(pr)
        q.field = bf16_round(pr.field)
    o = oracle_lib.run(q, precision=prec & ~abi.SW_FIELD_BF16, fp64_shadow=shadow and not batch,
                       fill=np.nan)
    for k in ("XYZ1", "T", "status"):
        if not bits_equal(g[k], o[k]):
            return f"{k} differs"
    ok, rel = m_close(g["M1"], o["M1"])
    if not ok:
        return f"M1 rel {rel:.3e}"
    if shadow and not batch:
        d = np.nanmax(np.abs(g["M1_fp64"] - o["M1_fp64"])) if g["M1_fp64"].size else 0.0
        if d > 1e-12:
            return f"M1_fp64 {d:.3e}"
    return None


def main(n_trials, seed=2024):
    rng = np.random.default_rng(seed)
    bad = 0
    for trial in range(n_trials):
        case = random_case(rng)
        err = check_case(*case)
        if err:
            bad += 1
            pr = case[0]
            print(f"trial {trial}: {err}; precision {case[1]:#x} shadow {case[2]} tuning "
                  f"{case[3]} batch {case[4]} n_spins {pr.params.n_spins}", flush=True)
    print(f"{n_trials} trials, {bad} mismatches", flush=True)
    return bad


if __name__ == "__main__":
    sys.exit(1 if main(int(sys.argv[1]) if len(sys.argv) > 1 else 100) else 0)
