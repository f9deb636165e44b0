"""GPU parity: the sm_103a kernels against the reference's golden outputs and the oracle.

Bar: trajectories (XYZ1), substrates at the echoes (T) and per-spin status are bit-exact;
magnetisation within M_RTOL = 1e-5 of |M| (+1e-7 absolute) in the FP32 path.
"""
import copy

import numpy as np
import pytest

from spinwalk_gb300 import _lib, abi
from spinwalk_gb300.problem import Problem, cylinder_phantom
from tests import oracle_lib
from tests.helpers import GOLDEN_CASES, bits_equal, load_golden, m_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_matches_reference_golden(case):
    pr, ref = load_golden(case)
    out = _lib.run(pr, fill=np.nan)
    assert bits_equal(out["XYZ1"], ref["XYZ1"]), f"{case}: trajectories differ"
    assert bits_equal(out["T"], ref["T"]), f"{case}: substrates differ"
    ok, rel = m_close(out["M1"], ref["M1"])
    assert ok, f"{case}: M1 max relative error {rel:.3e}"
    st = oracle_lib.run(pr)["status"]
    assert np.array_equal(out["status"], st), f"{case}: status differs"


@pytest.mark.parametrize("case", ["gre", "se_multi_te", "bssfp_phase_cycling", "pgse_gradients",
                                  "permeable", "ste_dephasing"])
@pytest.mark.parametrize("prec", [abi.SW_PREC_FP64, abi.SW_PREC_KAHAN])
def test_gpu_precision_modes_match_oracle(case, prec):
    pr, _ = load_golden(case)
    g = _lib.run(pr, precision=prec, fp64_shadow=True)
    o = oracle_lib.run(pr, precision=prec, fp64_shadow=True)
    assert bits_equal(g["XYZ1"], o["XYZ1"]) and bits_equal(g["T"], o["T"])
    # the FP64 shadow differs from the oracle's only by libm-vs-CUDA double sin/cos/exp
    d = np.abs(g["M1_fp64"] - o["M1_fp64"])
    assert d.max() <= 1e-12, d.max()
    ok, rel = m_close(g["M1"], o["M1"])
    assert ok, rel


def test_gpu_fp64_shadow_reports_fp32_error():
    """The FP64 run of the same walk is what the FP32 error is stated against."""
    pr, _ = load_golden("se_multi_te")
    g = _lib.run(pr, fp64_shadow=True)
    err = np.abs(g["M1"] - g["M1_fp64"]).max()
    assert 0 < err < 1e-4


def test_gpu_random_configs_match_oracle():
    rng = np.random.default_rng(7)
    for trial in range(4):
        n = int(rng.integers(12, 40))
        mask, field = cylinder_phantom(n, n * 1e-6, float(rng.uniform(2e-6, 5e-6)), 0.12,
                                       seed=trial)
        kw = dict(n_spins=int(rng.integers(1, 700)), seed=int(rng.integers(1, 10 ** 6)),
                  TR_us=4050, TE_us=(1000, 2000, 4000), RF_FA=(90.0, 180.0),
                  RF_PH=(0.0, float(rng.choice([0.0, 90.0, 37.5]))), RF_us=(0, 1500),
                  pXY=rng.uniform(0, 1, (2, 2)), n_dummy_scan=int(rng.integers(0, 3)),
                  linear_phase_cycling=float(rng.uniform(0, 200)),
                  cross_fov=bool(rng.integers(0, 2)))
        pr = Problem(mask, [n * 1e-6] * 3, field, **kw)
        g = _lib.run(pr, fill=np.nan)
        o = oracle_lib.run(pr, fill=np.nan)
        assert bits_equal(g["XYZ1"], o["XYZ1"]), trial
        assert bits_equal(g["T"], o["T"]), trial
        assert np.array_equal(g["status"], o["status"]), trial
        ok, rel = m_close(g["M1"], o["M1"])
        assert ok, (trial, rel)


def test_gpu_large_seed_and_spin_ids():
    """Spin ids near 2^20 with a large seed: long discard() runs in the seeding kernel."""
    mask, field = cylinder_phantom(16, 16e-6, 3e-6, 0.1, seed=5)
    pr = Problem(mask, [16e-6] * 3, field, n_spins=1 << 20, seed=123456, TR_us=550,
                 TE_us=(500,))
    ids = np.array([0, 1, 623, 624, 625, 99999, (1 << 20) - 2, (1 << 20) - 1], np.uint32)
    g = _lib.run(pr)
    o = oracle_lib.run(pr, spin_ids=ids)
    for k in ("XYZ1", "T"):
        assert bits_equal(g[k][ids], o[k][ids]), k
    ok, rel = m_close(g["M1"][ids], o["M1"][ids])
    assert ok, rel


def test_gpu_phantom_beyond_2e31_voxels():
    """A 1300^3 phantom (2.197e9 voxels > 2^31, the reference's int64 voxel index): spins near
    the far corner, where the index exceeds 2^31, against the oracle. Mask only (a 17.6 GB packed
    phantom on the device)."""
    n = 1300
    mask = np.zeros((n, n, n), np.uint8)
    mask[n - 25:n - 10, n - 60:, :] = 1                  # a slab in the high-index corner
    fov = 1300e-6
    rng = np.random.default_rng(9)
    off = rng.uniform(0.005, 0.06, (512, 3))
    off[:, 0] = rng.uniform(0.004, 0.018, 512)         # x >= 1271: index > 2^31
    xyz0 = (fov * (1.0 - off)).astype(np.float32)
    pr = Problem(mask, [fov] * 3, None, n_spins=512, seed=77, TR_us=10050, TE_us=(5000, 10000),
                 diffusivity=(2e-9, 1e-9), T1_ms=(1500.0, 1200.0), T2_ms=(60.0, 30.0),
                 pXY=[[1.0, 0.2], [0.1, 1.0]], XYZ0=xyz0)
    idx = (xyz0.astype(np.float64) * (n / fov)).astype(np.int64)
    assert (idx[:, 0] * n * n + idx[:, 1] * n + idx[:, 2]).min() > 2 ** 31
    g = _lib.run(pr, fill=np.nan)
    o = oracle_lib.run(pr, fill=np.nan)
    for k in ("XYZ1", "T", "status"):
        assert bits_equal(g[k], o[k]), k
    assert (o["T"] == 1).any() and (o["T"] == 0).any()    # both substrates reached
    ok, rel = m_close(g["M1"], o["M1"])
    assert ok, rel


def test_gpu_deterministic_and_spin_independent():
    pr, _ = load_golden("permeable")
    a = _lib.run(pr)
    b = _lib.run(pr)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(a[k], b[k]), k
    # the first k spins of a run alone equal the same spins in the full run
    z = np.load(__import__("os").path.join(__import__("tests.helpers", fromlist=["x"]).GOLDEN_DIR,
                                           "permeable.npz"))
    kw = __import__("json").loads(str(z["kwargs"]))
    kw["n_spins"] = 40
    pr40 = Problem(z["mask"], [float(z["fov"])] * 3, z["field_T"], XYZ0=z["XYZ0"][:40],
                   **{k: (tuple(v) if isinstance(v, list) and k != "pXY" else v)
                      for k, v in kw.items()})
    c = _lib.run(pr40)
    for k in ("M1", "XYZ1", "T"):
        assert bits_equal(c[k], a[k][:40]), k


def test_gpu_logf_matches_host_libm_exhaustively():
    """Device logf == host libm logf on every float in [2^-48, 1] (the polar-method domain)."""
    torch = pytest.importorskip("torch")
    lo, hi = 0x27800000, 0x3F800000
    chunk = 1 << 26
    start = lo
    while start <= hi:
        stop = min(hi + 1, start + chunk)
        bits = np.arange(start, stop, dtype=np.uint32)
        x = bits.view(np.float32)
        want = oracle_lib.host_logf(x)
        dx = torch.from_numpy(x).cuda()
        dy = torch.empty_like(dx)
        _lib.debug_logf(dx.data_ptr(), dy.data_ptr(), x.size)
        torch.cuda.synchronize()
        got = dy.cpu().numpy()
        bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, f"{bad.size} mismatches, first x={x[bad[0]]!r}"
        start = stop


def test_gpu_device_api_matches_host_api():
    torch = pytest.importorskip("torch")
    pr, _ = load_golden("se_multi_te")
    h = _lib.run(pr)
    n, nte = pr.params.n_spins, pr.n_te
    dev = "cuda"
    d_field = torch.from_numpy(pr.field).to(dev)
    d_mask = torch.from_numpy(pr.mask).to(dev)
    d_M0 = torch.from_numpy(pr.M0).to(dev)
    d_XYZ0 = torch.from_numpy(pr.XYZ0).to(dev)
    d_M1 = torch.zeros((n, nte, 3), dtype=torch.float32, device=dev)
    d_XYZ1 = torch.zeros((n, pr.traj_len, 3), dtype=torch.float32, device=dev)
    d_T = torch.zeros((n, nte), dtype=torch.uint8, device=dev)
    d_st = torch.zeros(n, dtype=torch.int32, device=dev)
    _lib.run_device(pr, d_field.data_ptr(), d_mask.data_ptr(), d_M0.data_ptr(),
                    d_XYZ0.data_ptr(), d_M1.data_ptr(), d_XYZ1.data_ptr(), d_T.data_ptr(),
                    d_st.data_ptr())
    torch.cuda.synchronize()
    assert bits_equal(d_M1.cpu().numpy(), h["M1"])
    assert bits_equal(d_XYZ1.cpu().numpy(), h["XYZ1"])
    assert bits_equal(d_T.cpu().numpy(), h["T"])
    assert np.array_equal(d_st.cpu().numpy(), h["status"])


def test_gpu_device_call_waits_for_inputs_on_the_callers_stream():
    """sw_sim_device starts seeding at once, but its walk is ordered after the caller's stream:
    start positions, phantom and M0 that arrive late on that stream (after ~20 ms of other work
    there) are the ones the walk reads."""
    torch = pytest.importorskip("torch")
    pr, _ = load_golden("se_multi_te")
    h = _lib.run(pr)
    n, nte = pr.params.n_spins, pr.n_te
    dev = "cuda"
    src = {k: torch.from_numpy(getattr(pr, k)).to(dev) for k in ("field", "mask", "M0", "XYZ0")}
    dst = {k: torch.zeros_like(v) for k, v in src.items()}
    d_M1 = torch.zeros((n, nte, 3), dtype=torch.float32, device=dev)
    d_XYZ1 = torch.zeros((n, pr.traj_len, 3), dtype=torch.float32, device=dev)
    d_T = torch.zeros((n, nte), dtype=torch.uint8, device=dev)
    d_st = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        torch.cuda._sleep(40_000_000)                # the caller's stream is busy for a while
        for k in src:
            dst[k].copy_(src[k])                     # then produces the inputs
    _lib.run_device(pr, dst["field"].data_ptr(), dst["mask"].data_ptr(), dst["M0"].data_ptr(),
                    dst["XYZ0"].data_ptr(), d_M1.data_ptr(), d_XYZ1.data_ptr(), d_T.data_ptr(),
                    d_st.data_ptr(), stream=s.cuda_stream)
    torch.cuda.synchronize()
    assert bits_equal(d_XYZ1.cpu().numpy(), h["XYZ1"])
    assert bits_equal(d_M1.cpu().numpy(), h["M1"])
    assert bits_equal(d_T.cpu().numpy(), h["T"])
    assert np.array_equal(d_st.cpu().numpy(), h["status"])


def test_gpu_host_call_after_refused_mask_matches():
    """sw_sim launches its seeding before it copies the inputs in. A call refused afterwards (a
    mask label >= n_substrate, found by the pack) leaves the device usable, and later calls,
    of other sizes too (the device copies of the buffers are reused and grown), equal the ones
    made before it bit for bit."""
    pr, _ = load_golden("permeable")
    big, _ = load_golden("se_multi_te")
    a, a_big = _lib.run(pr), _lib.run(big)
    bad = copy.copy(pr)
    bad.mask = pr.mask.copy()
    bad.mask.flat[0] = 7
    with pytest.raises(_lib.SpinWalkError, match="substrate labels"):
        _lib.run(bad)
    b = _lib.run(pr)
    b_big = _lib.run(big)
    c = _lib.run(pr)
    for k in ("M1", "XYZ1", "T", "status"):
        assert bits_equal(a[k], b[k]), k
        assert bits_equal(a[k], c[k]), k
        assert bits_equal(a_big[k], b_big[k]), k


def test_gpu_rejects_bad_arguments():
    pr, _ = load_golden("gre")
    pr.params.matrix_length += 1
    with pytest.raises(_lib.SpinWalkError):
        _lib.run(pr)
    pr.params.matrix_length -= 1
    with pytest.raises(_lib.SpinWalkError):
        _lib.run(pr, precision=7)


def test_gpu_integer_double_add_matches_ieee():
    """Device dadd_int (the walk's position update) == IEEE double addition (numpy) on walk-like
    operands, cancellations, ties and random bit patterns."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    n = 1 << 22
    x = rng.random(n) * 5e-4
    g = (rng.random(n) - 0.5) * 8e-7
    ea = rng.integers(900, 1100, n, dtype=np.uint64)
    eb = ea + np.uint64(3) - rng.integers(0, 70, n, dtype=np.uint64)
    fr = np.uint64(0x800fffffffffffff)
    a = ((rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2)) & fr | (ea << np.uint64(52))).view(np.float64)
    b = ((rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + np.uint64(1)) & fr | (eb << np.uint64(52))).view(np.float64)
    tie = ((ea - np.uint64(53)) << np.uint64(52)).view(np.float64)
    rnd = rng.integers(0, 2**63, (2, n), dtype=np.uint64).view(np.float64)
    A = np.concatenate([x, g, -x, a, a, a, a, rnd[0]])
    B = np.concatenate([g, x, g, b, -a, -b, tie, rnd[1]])
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dY = torch.empty_like(dA)
    _lib.debug_dadd(dA.data_ptr(), dB.data_ptr(), dY.data_ptr(), A.size)
    torch.cuda.synchronize()
    got = dY.cpu().numpy()
    with np.errstate(all="ignore"):
        want = A + B
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{(~same).sum()} mismatches, first a={A[~same][0]!r} b={B[~same][0]!r}"


def test_gpu_integer_double_to_float_matches_ieee():
    """Device d2f_exact (the walk's gradient-phase conversion) == IEEE double -> float rounding to
    nearest even (numpy) on every exponent, ties, carries into the exponent, the float range's
    edges (overflow, subnormal results), zeros and non-finite values."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    n = 1 << 21
    e = rng.integers(0, 2047, n, dtype=np.uint64)
    frac = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    rnd = (sign | (e << np.uint64(52)) | frac).view(np.float64)
    near = (sign | (rng.integers(880, 1170, n, dtype=np.uint64) << np.uint64(52)) | frac)
    # ties (low 29 bits exactly half), just above / below, all-ones significands (carry)
    tie = (near & ~np.uint64(0x1fffffff)) | np.uint64(0x10000000)
    above, below = tie + np.uint64(1), tie - np.uint64(1)
    ones = near | np.uint64(0x000fffffffffffff)
    walk = (rng.standard_normal(n) * 1e3).astype(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38,
                        3.4028234663852886e38, 1.1754943508222875e-38, 1.1754942e-38, 1e-45,
                        7e-46, 1.4e-45, 5e-324, -5e-324], np.float64)
    X = np.concatenate([rnd, near.view(np.float64), tie.view(np.float64), above.view(np.float64),
                        below.view(np.float64), ones.view(np.float64), walk, special])
    dX = torch.from_numpy(X).cuda()
    dY = torch.empty(X.size, dtype=torch.float32, device="cuda")
    _lib.debug_d2f(dX.data_ptr(), dY.data_ptr(), X.size)
    torch.cuda.synchronize()
    got = dY.cpu().numpy()
    with np.errstate(all="ignore"):
        want = X.astype(np.float32)
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{(~same).sum()} mismatches, first x={X[~same][0]!r}"


def test_smoke_entry_point_passes():
    """The build's smoke check (one small GRE walk against the oracle) passes."""
    import __graft_entry__
    __graft_entry__.smoke()
