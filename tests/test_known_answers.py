"""Known answers, end to end through the simulation (oracle on the CPU, the CUDA path on the GPU):

* the rotation / relaxation conventions and the row-major index of the reference's unit tests
  (tests/test_kernel.cpp:17-89: xrot(90)(0,0,1) = (0,-1,0), yrot(90)(1,0,0) = (0,0,-1),
  zrot(90)(1,0,0) = (0,1,0), relax(e1,e2), sub2ind), each within 1e-5 as there;
* analytic answers from the physics: a GRE without diffusion in a uniform field, spin-echo
  refocusing of static fields, and the PGSE attenuation of free diffusion, which for the
  discrete Gaussian walk is exp(-var/2) with var the exact variance of the gradient phase.

Time-point semantics (src/sim/kernels.cu:107-232): at every time point tp = 0 .. n_tp-1 the spin
moves, then `phase += field`, then the events at tp; an echo at tp relaxes over
(tp - tp_last_event) * dt with the phase summed since the last RF / echo (tp + 1 additions for
the first event of a scan, since tp = 0 adds too)."""
import math

import numpy as np
import pytest

from spinwalk_gb300.problem import GAMMA, Problem
from tests import oracle_lib

FOV = 40e-6
N = 8


def _problem(n_spins=4, TE_us=(500,), TR_us=550, timestep_us=50, RF_FA=(90.0,), RF_PH=(0.0,),
             RF_us=(0,), D=0.0, T1=(-1.0,), T2=(-1.0,), field_deg=None, M0=None, mask=None,
             fov=FOV, XYZ0=None, **kw):
    mask = np.zeros((N, N, N), np.uint8) if mask is None else mask
    ns = int(mask.max()) + 1
    pr = Problem(mask, [fov] * 3, np.zeros(mask.shape, np.float32), timestep_us=timestep_us,
                 TR_us=TR_us, TE_us=TE_us, RF_FA=RF_FA, RF_PH=RF_PH, RF_us=RF_us,
                 diffusivity=(D,) * ns, T1_ms=T1 * ns if len(T1) == 1 else T1,
                 T2_ms=T2 * ns if len(T2) == 1 else T2, n_spins=n_spins, seed=11, XYZ0=XYZ0, **kw)
    if field_deg is not None:
        pr.field = np.ascontiguousarray(np.broadcast_to(np.asarray(field_deg, np.float32),
                                                        mask.shape))
    if M0 is not None:
        pr.M0 = np.ascontiguousarray(np.broadcast_to(np.asarray(M0, np.float32), (n_spins, 3)))
    return pr


def _impls():
    """(name, runner) pairs: the oracle always, the reference built from source where present,
    the CUDA path under the gpu marker."""
    out = [pytest.param(oracle_lib.run, id="oracle")]
    try:
        oracle_lib.ref()
        out.append(pytest.param(lambda pr, fill=np.nan: oracle_lib.run_ref(pr, fill=fill),
                                id="reference"))
    except Exception:
        pass

    def gpu(pr, fill=np.nan):
        from spinwalk_gb300 import _lib
        return _lib.run(pr, fill=fill)
    out.append(pytest.param(gpu, id="gpu", marks=pytest.mark.gpu))
    return out


IMPLS = _impls()


def _m(run, pr):
    return run(pr, fill=np.nan)["M1"].astype(np.float64)


@pytest.mark.parametrize("run", IMPLS)
def test_rf_x_rotation_convention(run):
    """RF phase 0 (xrot): (0,0,1) -> (0,-1,0)."""
    m = _m(run, _problem())
    np.testing.assert_allclose(m[:, 0], np.tile([0.0, -1.0, 0.0], (4, 1)), atol=1e-5)


@pytest.mark.parametrize("run", IMPLS)
def test_rf_y_rotation_convention(run):
    """RF phase 90 (yrot): (1,0,0) -> (0,0,-1)."""
    m = _m(run, _problem(RF_PH=(90.0,), M0=(1.0, 0.0, 0.0)))
    np.testing.assert_allclose(m[:, 0], np.tile([0.0, 0.0, -1.0], (4, 1)), atol=1e-5)


@pytest.mark.parametrize("run", IMPLS)
def test_phase_z_rotation_convention(run):
    """Accumulated phase of +90 deg (zrot): (1,0,0) -> (0,1,0). 11 additions reach the echo at
    tp 10."""
    m = _m(run, _problem(RF_FA=(0.0,), M0=(1.0, 0.0, 0.0), field_deg=90.0 / 11))
    np.testing.assert_allclose(m[:, 0], np.tile([0.0, 1.0, 0.0], (4, 1)), atol=1e-5)


@pytest.mark.parametrize("run", IMPLS)
def test_relaxation_convention(run):
    """relax(e1, e2): (mx e2, my e2, 1 + e1 (mz - 1)) over TE = 10 dt, e1 = 0.9, e2 = 0.8."""
    te_ms = 0.5
    T1, T2 = -te_ms / math.log(0.9), -te_ms / math.log(0.8)
    m0 = np.array([1.0, 0.5, -0.5])
    m = _m(run, _problem(RF_FA=(0.0,), M0=m0, T1=(T1,), T2=(T2,)))
    want = np.array([m0[0] * 0.8, m0[1] * 0.8, 1.0 + 0.9 * (m0[2] - 1.0)])
    np.testing.assert_allclose(m[:, 0], np.tile(want, (4, 1)), atol=1e-5)


@pytest.mark.parametrize("run", IMPLS)
def test_row_major_voxel_index(run):
    """sub2ind: voxel (x, y, z) of an Nx x Ny x Nz phantom is x Ny Nz + y Nz + z (z fastest),
    seen through the substrate recorded at the echo on a non-cubic phantom."""
    shape = (4, 5, 6)
    mask = np.zeros(shape, np.uint8)
    mask[1, 2, 3] = 1
    fov = (40e-6, 50e-6, 60e-6)
    centre = lambda v: [(v[i] + 0.5) * fov[i] / shape[i] for i in range(3)]   # noqa: E731
    xyz0 = np.array([centre((1, 2, 3)), centre((3, 2, 1)), centre((2, 1, 3)), centre((1, 3, 2))],
                    np.float32)
    pr = Problem(mask, fov, None, TR_us=550, TE_us=(500,), diffusivity=(0.0, 0.0),
                 T1_ms=(-1.0, -1.0), T2_ms=(-1.0, -1.0), n_spins=4, seed=3, XYZ0=xyz0)
    out = run(pr, fill=np.nan)
    assert out["T"][:, 0].tolist() == [1, 0, 0, 0]


@pytest.mark.parametrize("run", IMPLS)
def test_gre_without_diffusion_in_uniform_field(run):
    """D = 0, uniform field f per step, T2 decay: M(TE) = e^(-TE/T2) zrot(11 f)(0,-1,0) and
    Mz = 1 - e^(-TE/T1)."""
    f, T1, T2 = 7.3, 100.0, 20.0
    m = _m(run, _problem(field_deg=f, T1=(T1,), T2=(T2,)))
    acc = np.float32(0.0)                            # 11 float additions up to the echo
    for _ in range(11):
        acc = np.float32(acc + np.float32(f))
    ph = math.radians(float(acc))
    e2, e1 = math.exp(-0.5 / T2), math.exp(-0.5 / T1)
    want = np.array([math.sin(ph) * e2, -math.cos(ph) * e2, 1.0 - e1])
    np.testing.assert_allclose(m[:, 0], np.tile(want, (4, 1)), atol=1e-5)


@pytest.mark.parametrize("run", IMPLS)
def test_spin_echo_refocuses_static_fields(run):
    """D = 0, a different static field in every voxel: after 90 - TE/2 - 180(y) - TE/2 each spin
    keeps |Mxy| = e^(-TE/T2) and the phases realign to within one step's field (the echo adds
    the field of its own time point once more than the first half), while the same spins
    without the 180 (GRE) dephase."""
    rng = np.random.default_rng(4)
    field = rng.uniform(-0.4, 0.4, (N, N, N)).astype(np.float32)
    n, T2 = 512, 40.0
    kw = dict(n_spins=n, TR_us=20050, TE_us=(20000,), T1=(1000.0,), T2=(T2,), field_deg=field)
    se = _m(run, _problem(RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0), RF_us=(0, 10000), **kw))[:, 0]
    gre = _m(run, _problem(**kw))[:, 0]
    e2 = math.exp(-20.0 / T2)
    np.testing.assert_allclose(np.hypot(se[:, 0], se[:, 1]), e2, rtol=1e-5)
    s_se = abs(np.mean(se[:, 0] + 1j * se[:, 1])) / e2
    s_gre = abs(np.mean(gre[:, 0] + 1j * gre[:, 1])) / e2
    assert s_se > math.cos(math.radians(0.4)) - 1e-6, s_se
    assert s_gre < 0.6, s_gre


@pytest.mark.parametrize("run", IMPLS)
def test_pgse_attenuation_of_free_diffusion(run):
    """Free diffusion (no structure, no field), PGSE with two 5 ms lobes 10 ms apart around a
    180 at 10 ms, gradient along x. The phase is a linear combination of the Gaussian steps, so
    S/S0 = exp(-var/2) exactly, var = sigma^2 sum_i (sum_{k >= i} g_k)^2 with g_k the phase per
    metre of time point k (sign flipped before the refocusing pulse) and sigma the step
    deviation per axis; checked within the sampling error of 20000 spins."""
    dt, G, D = 50, 150.0, 2e-9                       # us, mT/m, m^2/s
    lobe1 = list(range(2000, 7000, dt))
    lobe2 = list(range(12000, 17000, dt))
    g_us = lobe1 + [7000] + lobe2 + [17000]
    gx = [G if t not in (7000, 17000) else 0.0 for t in g_us]
    grad = np.zeros((len(g_us), 3), np.float32)
    grad[:, 0] = gx
    n = 20000
    pr = _problem(n_spins=n, TR_us=20050, TE_us=(20000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 10000), D=D, T1=(-1.0,), T2=(-1.0,), fov=1e-3,
                  gradient_us=g_us, gradient_xyz=grad)
    m = _m(run, pr)[:, 0]
    ok = np.isfinite(m[:, 0])
    s = abs(np.mean(m[ok, 0] + 1j * m[ok, 1]))
    # phase (rad) per metre at each time point: G 1e-3 dt 1e-6 gamma, negated before the 180
    n_tp = 20050 // dt
    g = np.zeros(n_tp)
    for t_us, gv in zip(g_us, gx):
        k = t_us // dt
        g[k] = gv * 1e-3 * dt * 1e-6 * GAMMA * (-1.0 if k < 200 else 1.0)
    te = 400
    tail = np.cumsum(g[:te + 1][::-1])[::-1]         # sum_{k >= i, k <= TE} g_k
    sigma2 = (1e-3 * math.sqrt(2.0 * D * dt)) ** 2   # the step variance per axis (m^2)
    want = math.exp(-0.5 * sigma2 * float(np.sum(tail ** 2)))
    assert 0.2 < want < 0.8                          # a measurable attenuation
    assert abs(s - want) < 4.0 / math.sqrt(n), (s, want)


@pytest.mark.parametrize("run", IMPLS)
def test_pgse_b_sweep_recovers_the_diffusivity(run):
    """The DWI demo's check (demo/spinwalk_dwi.ipynb: simulated D = 1e-9 m^2/s, fitted 9.79e-10):
    a PGSE b-value sweep on free diffusion, log S linear in b with slope -D. b is the exact
    value of the discrete waveform (var = 2 b D for the Gaussian walk); the fit must recover D
    within 3 %."""
    dt, D, n = 50, 1e-9, 20000
    lobe1, lobe2 = list(range(2000, 7000, dt)), list(range(12000, 17000, dt))
    g_us = lobe1 + [7000] + lobe2 + [17000]
    n_tp, te = 20050 // dt, 400
    sigma2 = (1e-3 * math.sqrt(2.0 * D * dt)) ** 2
    bs, logs = [], []
    for G in (0.0, 60.0, 100.0, 140.0, 180.0):
        gx = [G if t not in (7000, 17000) else 0.0 for t in g_us]
        grad = np.zeros((len(g_us), 3), np.float32)
        grad[:, 0] = gx
        pr = _problem(n_spins=n, TR_us=20050, TE_us=(20000,), RF_FA=(90.0, 180.0),
                      RF_PH=(0.0, 90.0), RF_us=(0, 10000), D=D, fov=1e-3, gradient_us=g_us,
                      gradient_xyz=grad)
        m = _m(run, pr)[:, 0]
        logs.append(math.log(abs(np.mean(m[:, 0] + 1j * m[:, 1]))))
        g = np.zeros(n_tp)
        for t_us, gv in zip(g_us, gx):
            g[t_us // dt] = gv * 1e-3 * dt * 1e-6 * GAMMA * (-1.0 if t_us // dt < 200 else 1.0)
        tail = np.cumsum(g[:te + 1][::-1])[::-1]
        bs.append(sigma2 * float(np.sum(tail ** 2)) / (2.0 * D))   # s/m^2
    slope = np.polyfit(np.array(bs), np.array(logs), 1)[0]
    assert abs(-slope / D - 1.0) < 0.03, -slope
    # the discrete b agrees with Stejskal-Tanner, gamma^2 G^2 delta^2 (Delta - delta/3)
    b_st = (GAMMA * 0.18 * 5e-3) ** 2 * (10e-3 - 5e-3 / 3)
    assert abs(bs[-1] / b_st - 1.0) < 0.02, (bs[-1], b_st)        # ~483 s/mm^2
