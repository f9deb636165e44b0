"""sw_sim_tracks (one walk, many instances) against independent per-instance runs: each track's
outputs must equal sw_sim on that instance alone, bit for bit (same device arithmetic), and the
oracle within the magnetisation tolerance."""
import copy

import numpy as np
import pytest

from spinwalk_gb300 import _lib
from spinwalk_gb300.problem import Problem
from tests import oracle_lib
from tests.helpers import bits_equal, load_golden, m_close

pytestmark = pytest.mark.gpu


def _instance(pr, t):
    """The Problem the reference would run for track t."""
    q = copy.copy(pr)
    p = type(pr.params)()
    C = __import__("ctypes")
    C.memmove(C.byref(p), C.byref(pr.params), C.sizeof(p))
    p.n_dummy_scan = t["n_dummy_scan"]
    p.linear_phase_cycling = t.get("linear_phase_cycling", 0.0)
    p.quadratic_phase_cycling = t.get("quadratic_phase_cycling", 0.0)
    q.params = p
    return q


@pytest.mark.parametrize("case", ["bssfp_phase_cycling", "se_multi_te", "lost_spins", "pgse_gradients"])
def test_tracks_equal_independent_runs(case):
    pr, _ = load_golden(case)
    tracks = [dict(linear_phase_cycling=lpc, quadratic_phase_cycling=qpc, n_dummy_scan=nd)
              for lpc in (0.0, 45.0, 180.0) for qpc in (0.0, 7.5) for nd in (0, 2, 3)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan)
    for t, got in zip(tracks, outs):
        inst = _instance(pr, t)
        want = _lib.run(inst, fill=np.nan)
        assert bits_equal(got["M1"], want["M1"]), (case, t)
        assert bits_equal(got["T"], want["T"]), (case, t)
        assert bits_equal(got["XYZ1"], want["XYZ1"]), (case, t)
        assert np.array_equal(got["status"], want["status"]), (case, t)
    # one track against the oracle
    t = tracks[-1]
    o = oracle_lib.run(_instance(pr, t), fill=np.nan)
    ok, rel = m_close(outs[-1]["M1"], o["M1"])
    assert ok, rel
    assert bits_equal(outs[-1]["XYZ1"], o["XYZ1"])


def test_tracks_per_pulse_rf_variants():
    pr, _ = load_golden("se_multi_te")
    tracks = [dict(n_dummy_scan=1, RF_FA_deg=[90.0, fa], RF_PH_deg=[0.0, ph])
              for fa in (120.0, 180.0) for ph in (0.0, 90.0, 33.0)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan)
    for t, got in zip(tracks, outs):
        inst = _instance(pr, t)
        seq = dict(inst.seq.arrays)
        from spinwalk_gb300 import abi
        inst.seq = abi.Sequence(**{**seq, "RF_FA_deg": t["RF_FA_deg"], "RF_PH_deg": t["RF_PH_deg"]})
        want = _lib.run(inst, fill=np.nan)
        assert bits_equal(got["M1"], want["M1"]), t
        assert bits_equal(got["XYZ1"], want["XYZ1"]), t


def test_tracks_reject_duplicates():
    pr, _ = load_golden("gre")
    with pytest.raises(_lib.SpinWalkError):
        _lib.run_tracks(pr, [dict(n_dummy_scan=0), dict(n_dummy_scan=0)])


@pytest.mark.parametrize("case", ["bssfp_phase_cycling", "se_multi_te", "pgse_gradients",
                                  "ste_dephasing"])
@pytest.mark.parametrize("precision", ["kahan", "fp32_shadow", "fp64"])
def test_tracks_precision_modes_equal_independent_runs(case, precision):
    """Compensated phase sums, the FP64 shadow and FP64 output of the tracks path are those of
    sw_sim on each instance alone, bit for bit (the steady-state recurrence carried in double)."""
    from spinwalk_gb300 import abi
    prec = {"kahan": abi.SW_PREC_KAHAN, "fp32_shadow": abi.SW_PREC_FP32,
            "fp64": abi.SW_PREC_FP64}[precision]
    shadow = precision != "kahan"
    pr, _ = load_golden(case)
    tracks = [dict(linear_phase_cycling=lpc, n_dummy_scan=nd)
              for lpc in (0.0, 90.0, 200.0) for nd in (0, 3)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan, precision=prec, fp64=shadow)
    for t, got in zip(tracks, outs):
        want = _lib.run(_instance(pr, t), precision=prec, fp64_shadow=shadow, fill=np.nan)
        assert bits_equal(got["M1"], want["M1"]), (case, precision, t)
        assert bits_equal(got["T"], want["T"]), (case, precision, t)
        assert bits_equal(got["XYZ1"], want["XYZ1"]), (case, precision, t)
        if shadow:
            assert bits_equal(got["M1_fp64"], want["M1_fp64"]), (case, precision, t)


def test_tracks_shadow_leaves_fp32_results_unchanged():
    pr, _ = load_golden("bssfp_phase_cycling")
    tracks = [dict(linear_phase_cycling=lpc, n_dummy_scan=nd) for lpc in (0.0, 120.0) for nd in (1, 4)]
    plain = _lib.run_tracks(pr, tracks, fill=np.nan)
    shadowed = _lib.run_tracks(pr, tracks, fill=np.nan, fp64=True)
    for a, b in zip(plain, shadowed):
        assert bits_equal(a["M1"], b["M1"])
        assert bits_equal(a["XYZ1"], b["XYZ1"])
        # FP32 against its FP64 shadow: the stated per-spin error bound of the float path
        err = np.nanmax(np.abs(b["M1"].astype(np.float64) - b["M1_fp64"]))
        assert err < 1e-4, err


@pytest.mark.parametrize("flags", ["minstd", "bf16", "minstd_bf16_kahan"])
def test_tracks_generator_flavour_and_field_records(flags):
    """SW_RNG_MINSTD and SW_FIELD_BF16 in the tracks path equal sw_sim with the same flags on
    each instance, bit for bit."""
    from spinwalk_gb300 import abi
    prec = {"minstd": abi.SW_RNG_MINSTD, "bf16": abi.SW_FIELD_BF16,
            "minstd_bf16_kahan": abi.SW_RNG_MINSTD | abi.SW_FIELD_BF16 | abi.SW_PREC_KAHAN}[flags]
    pr, _ = load_golden("bssfp_phase_cycling")
    tracks = [dict(linear_phase_cycling=lpc, n_dummy_scan=nd) for lpc in (0.0, 150.0)
              for nd in (0, 2)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan, precision=prec)
    for t, got in zip(tracks, outs):
        want = _lib.run(_instance(pr, t), precision=prec, fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(got[k], want[k]), (flags, t, k)


def test_tracks_reject_unknown_flag_bits():
    pr, _ = load_golden("gre")
    with pytest.raises(_lib.SpinWalkError):
        _lib.run_tracks(pr, [dict(n_dummy_scan=0)], precision=0x400)


def _scaled(pr, t):
    """The instance the reference's gradient scale loop runs: the sequence's gradients times the
    scale, a float multiply (src/sim/monte_carlo.cu:287-290)."""
    from spinwalk_gb300 import abi
    inst = _instance(pr, t)
    if t.get("gradient_scale") is not None:
        sc = np.float32(t["gradient_scale"])
        seq = dict(inst.seq.arrays)
        for k in ("gradientX_mTm", "gradientY_mTm", "gradientZ_mTm"):
            seq[k] = (np.asarray(seq[k], np.float32) * sc).astype(np.float32)
        inst.seq = abi.Sequence(**seq)
    return inst


@pytest.mark.parametrize("scales", [(0.0, 0.5, 1.0, 2.0), (0.25,), (1.0, 3.0), (0.1, 0.2, 0.3, 0.4, 0.6, 0.7, 0.8)])
def test_tracks_gradient_scales_equal_independent_runs(scales):
    """Gradient-scale sweeps (the DWI b-value series) on one walk: each scale keeps its own phase
    sums and equals sw_sim with the scaled gradients, bit for bit."""
    pr, _ = load_golden("pgse_gradients")
    tracks = [dict(gradient_scale=s, n_dummy_scan=0) for s in scales]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan)
    for t, got in zip(tracks, outs):
        want = _lib.run(_scaled(pr, t), fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(got[k], want[k]), (t, k)


def test_tracks_gradient_scales_with_phase_cycling_and_dummy_scans():
    pr, _ = load_golden("pgse_gradients")
    tracks = [dict(gradient_scale=s, linear_phase_cycling=lpc, n_dummy_scan=nd)
              for s in (1.0, 3.0) for lpc in (0.0, 90.0) for nd in (0, 1)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan)
    for t, got in zip(tracks, outs):
        want = _lib.run(_scaled(pr, t), fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(got[k], want[k]), (t, k)


def test_tracks_gradient_scale_limits():
    from spinwalk_gb300 import abi
    pr, _ = load_golden("pgse_gradients")
    with pytest.raises(_lib.SpinWalkError):          # more than 8 distinct scales
        _lib.run_tracks(pr, [dict(gradient_scale=0.1 * i, n_dummy_scan=0) for i in range(9)])
    with pytest.raises(_lib.SpinWalkError):          # several scales: no FP64 arithmetic / shadow
        _lib.run_tracks(pr, [dict(gradient_scale=s, n_dummy_scan=0) for s in (1.0, 2.0)],
                        precision=abi.SW_PREC_FP64)
    with pytest.raises(_lib.SpinWalkError):
        _lib.run_tracks(pr, [dict(gradient_scale=s, n_dummy_scan=0) for s in (1.0, 2.0)], fp64=True)


@pytest.mark.parametrize("scales", [(0.0, 1.0), (0.5, 1.0, 1.5, 2.0, 2.5)])
def test_tracks_gradient_scales_kahan(scales):
    from spinwalk_gb300 import abi
    pr, _ = load_golden("pgse_gradients")
    tracks = [dict(gradient_scale=s, n_dummy_scan=nd) for s in scales for nd in (0, 1)]
    outs = _lib.run_tracks(pr, tracks, fill=np.nan, precision=abi.SW_PREC_KAHAN)
    for t, got in zip(tracks, outs):
        want = _lib.run(_scaled(pr, t), precision=abi.SW_PREC_KAHAN, fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(got[k], want[k]), (t, k)


def _large(case, n_spins=70000):
    """A golden case's phantom and sequence with n_spins >= 2^16: the tracks path then runs its
    rounds as two halves of the spins on two streams."""
    import json
    import os
    from spinwalk_gb300.problem import Problem
    from tests.helpers import GOLDEN_DIR
    z = np.load(os.path.join(GOLDEN_DIR, case + ".npz"))
    kw = json.loads(str(z["kwargs"]))
    kw = {k: (tuple(v) if isinstance(v, list) and k not in ("pXY", "gradient_xyz") else v)
          for k, v in kw.items()}
    kw["n_spins"] = n_spins
    field = z["field_T"] if z["field_T"].size else None
    return Problem(z["mask"], [float(z["fov"])] * 3, field, **kw)


@pytest.mark.parametrize("case,tracks,precision,fp64", [
    ("bssfp_phase_cycling", [dict(linear_phase_cycling=l, n_dummy_scan=d)
                             for l in (0.0, 120.0) for d in (0, 2)], 0, False),
    ("bssfp_phase_cycling", [dict(linear_phase_cycling=l, n_dummy_scan=1) for l in (0.0, 45.0)], 2, True),
    ("pgse_gradients", [dict(gradient_scale=s, n_dummy_scan=0) for s in (0.0, 0.5, 1.0, 2.0)], 0, False),
])
def test_tracks_two_halves_equal_independent_runs(case, tracks, precision, fp64):
    pr = _large(case)
    outs = _lib.run_tracks(pr, tracks, fill=np.nan, precision=precision, fp64=fp64)
    for t, got in zip(tracks, outs):
        want = _lib.run(_scaled(pr, t), precision=precision, fp64_shadow=fp64, fill=np.nan)
        for k in ("M1", "XYZ1", "T", "status") + (("M1_fp64",) if fp64 else ()):
            assert bits_equal(got[k], want[k]), (case, t, k)
