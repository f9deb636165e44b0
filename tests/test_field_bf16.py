"""SW_FIELD_BF16: phantoms packed as 4-byte voxel records with the field rounded to bfloat16.
Such a run must equal the float-record run on the field rounded to bfloat16 beforehand, bit for
bit (the rounding is the only change), and keep the trajectories of the unrounded run."""
import copy

import numpy as np
import pytest

from spinwalk_gb300 import _lib, abi
from tests.helpers import bits_equal, load_golden

BF16 = abi.SW_FIELD_BF16


def bf16_round(a):
    """float32 -> nearest bfloat16 (ties to even) -> float32, for finite values."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def test_bf16_round_reference_points():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, -0.0,
                  1.0 + 2 ** -8 + 2 ** -20, 3.0e-3], np.float32)
    got = bf16_round(x)
    assert got[0] == 1.0 and got[3] == -2.5 and got[4] == 0.0
    assert got[1] == 1.0                           # tie -> even (mantissa ...0)
    assert got[2] == np.float32(1.0 + 2 ** -6)     # tie -> even (rounds up)
    assert got[6] == np.float32(1.0 + 2 ** -7)     # above the tie
    assert np.signbit(got[5])
    assert abs(got[7] - x[7]) <= x[7] * 2 ** -8    # half an ulp of an 8-bit significand


def _rounded(pr):
    q = copy.copy(pr)
    q.field = bf16_round(pr.field)
    return q


FIELD_CASES = ["gre", "permeable", "se_multi_te", "three_substrates", "pgse_gradients",
               "trajectory", "lost_spins"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", FIELD_CASES)
@pytest.mark.parametrize("precision", [abi.SW_PREC_FP32, abi.SW_PREC_KAHAN, abi.SW_PREC_FP64])
def test_bf16_equals_float_run_on_rounded_field(case, precision):
    pr, _ = load_golden(case)
    assert pr.field is not None and np.any(pr.field != bf16_round(pr.field))
    got = _lib.run(pr, precision=precision | BF16, fill=np.nan)
    want = _lib.run(_rounded(pr), precision=precision, fill=np.nan)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k]), k
    plain = _lib.run(pr, precision=precision, fill=np.nan)
    for k in ("XYZ1", "T", "status"):              # the walk itself is unchanged
        assert bits_equal(got[k], plain[k]), k


@pytest.mark.gpu
def test_bf16_batch_spins_signal_paths():
    pr, _ = load_golden("se_multi_te")
    want = _lib.run(_rounded(pr), fill=np.nan)
    got = _lib.run_batch([pr], precision=BF16, fill=np.nan)[0]
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(got[k], want[k]), k
    n = pr.params.n_spins
    part = _lib.run_spins(pr, n // 3, n, precision=BF16, fill=np.nan)
    assert bits_equal(part["M1"], want["M1"][n // 3:])
    sig, cnt, st = _lib.run_signal(pr, precision=BF16)
    sig_w, cnt_w, st_w = _lib.run_signal(_rounded(pr))
    assert np.array_equal(cnt, cnt_w) and np.array_equal(st, st_w)
    np.testing.assert_allclose(sig, sig_w, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_bf16_engine_phantom():
    pr, _ = load_golden("permeable")
    want = _lib.run(_rounded(pr), fill=np.nan)
    eng = _lib.Engine(n_slots=2, slot_spins=1 << 12)
    pid = eng.add_phantom(pr, bf16=True)
    pid_f = eng.add_phantom(pr)
    outs = [eng.submit(pr, pid, fill=np.nan), eng.submit(pr, pid, precision=BF16, fill=np.nan)]
    with pytest.raises(_lib.SpinWalkError):
        eng.submit(pr, pid_f, precision=BF16)
    done = eng.run_all()
    assert sorted(j for j, rc, _ in done) == sorted(j for j, _ in outs)
    assert all(rc == 0 for _, rc, _ in done)
    for _, o in outs:
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(o[k], want[k]), k
    eng.close()
