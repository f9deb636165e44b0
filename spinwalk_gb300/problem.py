"""Problem set-up in the reference driver's terms.

``Problem`` holds one simulation exactly as ``sim::monte_carlo::run`` prepares it before calling
the per-spin kernel (src/sim/monte_carlo.cu:199-305): the parameter struct after
``config_reader::timing_scale`` (src/sim/config_reader.cpp:39-46) and ``parameters::prepare``
(src/sim/simulation_parameters.cuh:227-245), the fieldmap scaled from Tesla to degree per time step
(monte_carlo.cu:241-244), the initial positions of ``initialize_position`` (monte_carlo.cu:141-151)
and M0 = (0, 0, 1) (monte_carlo.cu:162-164).

Synthetic phantoms (seeded cylinders / spheres with analytic dipole fields, after
src/phantom/phantom_cylinder.cpp:183-275 and phantom_sphere.cpp:121-198) stand in for the
reference's HDF5 phantoms.
"""
import math

import numpy as np

from . import abi

GAMMA = 267515315.0          # rad/s/T, src/definitions.h:20
DEG2RAD = 0.0174532925199433  # simulation_parameters.cuh:24
RAD2DEG = 57.2957795130823    # simulation_parameters.cuh:25


def fieldmap_scale(B0, timestep_us):
    """float(B0 * dt * 1e-6 * GAMMA * RAD2DEG) with the reference's operand types
    (src/sim/monte_carlo.cu:241): B0 (float) * timestep (int32) is a float product."""
    f = np.float32(np.float32(B0) * np.float32(timestep_us))
    return np.float32(float(f) * 1e-6 * GAMMA * RAD2DEG)


def _libm():
    import ctypes
    import ctypes.util
    lib = ctypes.CDLL(ctypes.util.find_library("m"))
    lib.sinf.restype = ctypes.c_float
    lib.sinf.argtypes = [ctypes.c_float]
    lib.cosf.restype = ctypes.c_float
    lib.cosf.argtypes = [ctypes.c_float]
    return lib


_LIBM = None


def host_sincosf(x):
    """glibc sinf/cosf of a float (the reference calls them through libm)."""
    global _LIBM
    if _LIBM is None:
        _LIBM = _libm()
    xf = float(np.float32(x))
    return np.float32(_LIBM.sinf(xf)), np.float32(_LIBM.cosf(xf))


class Problem:
    """One scale of one phantom: everything sim::sim reads, as numpy arrays + ctypes structs."""

    def __init__(self, mask, fov, field_T=None, *, B0=9.4, timestep_us=50, TR_us=20050,
                 TE_us=(20000,), RF_FA=(90.0,), RF_PH=(0.0,), RF_us=(0,),
                 dephasing_deg=(), dephasing_us=(), gradient_xyz=None, gradient_us=(),
                 diffusivity=(1e-9, 1e-9), T1_ms=(2000.0, 2000.0), T2_ms=(40.0, 20.0),
                 pXY=None, n_spins=1000, seed=10, n_dummy_scan=0, linear_phase_cycling=0.0,
                 quadratic_phase_cycling=0.0, cross_fov=True, record_trajectory=False,
                 max_iterations=9999, XYZ0=None):
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        assert mask.ndim == 3
        self.mask = mask
        ns = len(diffusivity)
        if pXY is None:
            pXY = np.eye(ns, dtype=np.float32)
        pXY = np.asarray(pXY, dtype=np.float32).reshape(-1)
        assert pXY.size == ns * ns
        if int(mask.max()) + 1 > ns:                   # monte_carlo.cu:113-118
            raise ValueError("mask holds more substrates than the config defines")

        p = abi.SwParams()
        fov = [float(np.float32(f)) for f in fov]       # phantom fov is float in the h5 file
        for i in range(3):
            p.fov[i] = fov[i]
            p.phantom_size[i] = mask.shape[i]
        p.B0 = B0
        p.linear_phase_cycling = linear_phase_cycling
        p.quadratic_phase_cycling = quadratic_phase_cycling
        p.timestep_us = int(timestep_us)
        p.TR_us = int(TR_us)
        p.n_dummy_scan = int(n_dummy_scan)
        p.n_spins = int(n_spins)
        p.n_substrate = ns
        p.n_scales = 1
        p.matrix_length = mask.size
        p.enCrossFOV = 1 if cross_fov else 0
        p.enRecordTrajectory = 1 if record_trajectory else 0
        p.max_iterations = int(max_iterations)
        if seed == 0:                                   # simulation_parameters.cuh:233-234
            seed = int(np.random.SeedSequence().entropy % (1 << 32))
        p.seed = int(seed)

        # parameters::prepare (simulation_parameters.cuh:227-245)
        s, c = host_sincosf(RF_FA[0] * DEG2RAD)
        p.s, p.c = float(s), float(c)
        p.n_timepoints = int(TR_us) // int(timestep_us)
        diff = np.array([1e-3 * math.sqrt(2.0 * float(d) * timestep_us) for d in diffusivity],
                        dtype=np.float64)
        if p.n_dummy_scan < 0:
            p.n_dummy_scan = int(5.0 * float(np.float32(T1_ms[0])) /
                                 float(np.float32(TR_us * 1e-3)))

        # config_reader::timing_scale: microseconds -> time points by integer division
        def tp(v):
            return [int(x) // int(timestep_us) for x in v]

        if gradient_xyz is None:
            gradient_xyz = np.zeros((len(gradient_us), 3), dtype=np.float32)
        g = np.asarray(gradient_xyz, dtype=np.float32).reshape(-1, 3)
        self.seq = abi.Sequence(
            diffusivity=diff, T1_ms=T1_ms, T2_ms=T2_ms, pXY=pXY,
            RF_FA_deg=RF_FA, RF_PH_deg=RF_PH, RF_us=tp(RF_us), TE_us=tp(TE_us),
            dephasing_deg=dephasing_deg, dephasing_us=tp(dephasing_us),
            gradientX_mTm=g[:, 0], gradientY_mTm=g[:, 1], gradientZ_mTm=g[:, 2],
            gradient_us=tp(gradient_us))
        self.params = p

        if field_T is not None:
            fs = fieldmap_scale(B0, timestep_us)
            self.field = np.ascontiguousarray(np.asarray(field_T, np.float32) * fs,
                                              dtype=np.float32)
            p.fieldmap_exist = 1
        else:
            self.field = None
            p.fieldmap_exist = 0

        if XYZ0 is None:
            XYZ0 = initial_positions(fov, p.seed, n_spins)
        self.XYZ0 = np.ascontiguousarray(XYZ0, dtype=np.float32).reshape(n_spins, 3)
        self.M0 = np.zeros((n_spins, 3), np.float32)
        self.M0[:, 2] = 1.0

    @property
    def n_te(self):
        return int(self.seq.struct.n_TE)

    @property
    def traj_len(self):
        p = self.params
        return (p.n_dummy_scan + 1) * p.n_timepoints if p.enRecordTrajectory else 1

    def outputs(self, fill=0.0):
        n = self.params.n_spins
        M1 = np.full((n, self.n_te, 3), fill, np.float32)
        XYZ1 = np.full((n, self.traj_len, 3), fill, np.float32)
        T = np.zeros((n, self.n_te), np.uint8)
        status = np.full(n, -1, np.int32)
        return M1, XYZ1, T, status

    def spin_steps(self):
        p = self.params
        return p.n_spins * p.n_timepoints * (p.n_dummy_scan + 1)


def initial_positions(fov, seed, n_spins):
    """monte_carlo::initialize_position (src/sim/monte_carlo.cu:141-151), computed by the
    library's host code (same std::mt19937 + uniform_real_distribution<float>)."""
    from . import _lib
    return _lib.initial_positions(fov, seed, n_spins)


# ----------------------------------------------------------------------------------------------
# Synthetic phantoms (seeded numpy; small sizes for tests, the library generator for big ones)
# ----------------------------------------------------------------------------------------------
def cylinder_phantom(n, fov_m, radius_m, volume_fraction, seed, dchi=0.11e-6 * 0.4, Y=0.75,
                     random_orientation=True, B0_dir=(0.0, 0.0, 1.0)):
    """uint8 mask (1 inside infinite cylinders) + dipole field in T at B0 = 1 T.

    Field of one cylinder (phantom_cylinder.cpp:262-265): outside 2*pi*dchi*(1-Y)*(r^2/rho^2)*
    cos(2 phi)*sin^2(theta); inside 2*pi*dchi*(1-Y)*(cos^2(theta) - 1/3); superposed."""
    rng = np.random.default_rng(seed)
    v = fov_m / n
    ax = (np.arange(n) + 0.5) * v
    X, Yg, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    P = np.stack([X, Yg, Z], -1).reshape(-1, 3)
    mask = np.zeros(n ** 3, np.uint8)
    field = np.zeros(n ** 3, np.float64)
    b0 = np.asarray(B0_dir, float)
    b0 /= np.linalg.norm(b0)
    target = volume_fraction * fov_m ** 3
    vol = 0.0
    k = 2 * np.pi * dchi * (1 - Y)
    while vol < target:
        c = rng.uniform(0, fov_m, 3)
        if random_orientation:
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
        else:
            d = np.array([0.0, 0.0, 1.0])
        rel = P - c
        along = rel @ d
        perp = rel - along[:, None] * d
        rho2 = np.einsum("ij,ij->i", perp, perp)
        inside = rho2 <= radius_m ** 2
        mask[inside] = 1
        ct = float(np.dot(d, b0))
        st2 = 1 - ct * ct
        bp = b0 - ct * d
        nb = np.linalg.norm(bp)
        if nb > 1e-12:
            bp /= nb
            cphi = (perp @ bp) / np.sqrt(np.maximum(rho2, 1e-30))
        else:
            cphi = np.zeros_like(rho2)
        out = k * (radius_m ** 2 / np.maximum(rho2, 1e-30)) * (2 * cphi * cphi - 1) * st2
        field += np.where(inside, k * (ct * ct - 1.0 / 3.0), out)
        vol += np.pi * radius_m ** 2 * fov_m      # infinite cylinder, approx length = fov
    return mask.reshape(n, n, n), field.astype(np.float32).reshape(n, n, n)


def sphere_phantom(n, fov_m, rmin_m, rmax_m, volume_fraction, seed, dchi=0.11e-6 * 0.4,
                   Y=0.75, B0_dir=(0.0, 0.0, 1.0)):
    """uint8 mask + superposed sphere dipole field (phantom_sphere.cpp:185-187 form):
    outside 4*pi*(1-Y)*dchi*r^3/d^3*(cos^2(phi) - 1/3), 0 inside."""
    rng = np.random.default_rng(seed)
    v = fov_m / n
    ax = (np.arange(n) + 0.5) * v
    X, Yg, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    P = np.stack([X, Yg, Z], -1).reshape(-1, 3)
    mask = np.zeros(n ** 3, np.uint8)
    field = np.zeros(n ** 3, np.float64)
    b0 = np.asarray(B0_dir, float)
    b0 /= np.linalg.norm(b0)
    target = volume_fraction * fov_m ** 3
    vol = 0.0
    k = 4 * np.pi * (1 - Y) * dchi
    while vol < target:
        r = rng.uniform(rmin_m, rmax_m)
        c = rng.uniform(0, fov_m, 3)
        rel = P - c
        d2 = np.einsum("ij,ij->i", rel, rel)
        inside = d2 <= r * r
        mask[inside] = 1
        dp = rel @ b0
        c2 = dp * dp / np.maximum(d2, 1e-30)
        field += np.where(inside, 0.0, k * r ** 3 / np.maximum(d2, 1e-30) ** 1.5 * (c2 - 1 / 3))
        vol += 4 / 3 * np.pi * r ** 3
    return mask.reshape(n, n, n), field.astype(np.float32).reshape(n, n, n)
