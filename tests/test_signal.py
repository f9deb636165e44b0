"""Signal mode (sw_sim_signal / sw_engine_submit_signal): the reduction of M1 / T over spins
(sum of M per echo and substrate, and the count) fused into the walk. It must equal the
reduction of sw_sim's per-spin results: counts exactly, sums to 1e-12 (the order of the double
additions is not fixed)."""
import numpy as np
import pytest

from spinwalk_gb300 import _lib, abi
from tests.helpers import load_golden

pytestmark = pytest.mark.gpu
CASES = ["se_multi_te", "lost_spins", "three_substrates", "permeable", "bssfp_phase_cycling",
         "out_of_bounds_periodic", "gre_seed7_sph"]


def host_reduction(pr, precision=abi.SW_PREC_FP32):
    fp64 = precision == abi.SW_PREC_FP64       # the sums then add the double magnetisation
    full = _lib.run(pr, precision=precision, fp64_shadow=fp64, fill=np.nan)
    ns, nte = pr.params.n_substrate, pr.n_te
    sig = np.zeros((nte, ns, 3))
    cnt = np.zeros((nte, ns), np.uint64)
    for te in range(nte):
        m = (full["M1_fp64"] if fp64 else full["M1"])[:, te, :].astype(np.float64)
        ok = ~np.isnan(m[:, 0])
        t = full["T"][ok, te].astype(np.int64)
        np.add.at(sig[te], t, m[ok])
        np.add.at(cnt[te], t, 1)
    return sig, cnt, full["status"]


def check(sig, cnt, ref):
    rs, rc, _ = ref
    assert np.array_equal(cnt, rc)
    assert np.allclose(sig, rs, rtol=1e-12, atol=1e-12 * max(1, int(rc.max())))


@pytest.mark.parametrize("case", CASES)
def test_signal_equals_reduction_of_per_spin_results(case):
    pr, _ = load_golden(case)
    ref = host_reduction(pr)
    sig, cnt, status = _lib.run_signal(pr)
    check(sig, cnt, ref)
    assert np.array_equal(status, ref[2])


def test_signal_fp64_mode():
    pr, _ = load_golden("se_multi_te")
    check(*_lib.run_signal(pr, precision=abi.SW_PREC_FP64)[:2], host_reduction(pr, abi.SW_PREC_FP64))


def test_engine_signal_jobs_in_chunks():
    eng = _lib.Engine(n_slots=3, slot_spins=97)
    for case in ("lost_spins", "three_substrates"):
        pr, _ = load_golden(case)
        pid = eng.add_phantom(pr)
        _, o = eng.submit_signal(pr, pid)
        eng.run_all()
        check(o["signal"], o["count"], host_reduction(pr))
    eng.close()
