"""ctypes binding of libspinwalk_gpu.so (the C ABI declared in include/spinwalk_gpu.h).

The library is loaded from this package directory only. There is no fallback: if the library
is missing, or no GPU is visible, every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspinwalk_gpu.so")
_lib = None


class SpinWalkError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SpinWalkError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'`")
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.sw_abi_version.restype = C.c_int
        L.sw_last_error.restype = C.c_char_p
        L.sw_device_count.argtypes = [P(C.c_int)]
        L.sw_device_info.argtypes = [C.c_int, C.c_char_p, C.c_uint64]
        L.sw_prepare_params.argtypes = [P(abi.SwParams), P(C.c_double), P(C.c_float),
                                        P(C.c_float)]
        L.sw_fieldmap_scale.restype = C.c_float
        L.sw_fieldmap_scale.argtypes = [C.c_float, C.c_int32]
        L.sw_initial_positions.argtypes = [P(C.c_float), C.c_uint64, C.c_uint32, P(C.c_float)]
        L.sw_logf_exception_count.argtypes = [P(C.c_uint64), P(C.c_uint64)]
        set_phantom_argtypes(L)
        sim_args = [P(abi.SwParams), P(abi.SwSequence), C.c_void_p, C.c_void_p, C.c_void_p,
                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                    C.c_void_p]
        L.sw_sim.argtypes = sim_args
        L.sw_sim_device.argtypes = sim_args + [C.c_void_p]
        L.sw_sim_device_noalloc.argtypes = sim_args[:10] + [C.c_void_p]
        L.sw_sim_tracks.argtypes = [P(abi.SwParams), P(abi.SwSequence), P(abi.SwTrack), C.c_uint32,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.sw_sim_batch.argtypes = [P(abi.SwInstance), C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]
        L.sw_engine_create.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_uint64, P(C.c_void_p)]
        L.sw_engine_destroy.argtypes = [C.c_void_p]
        L.sw_engine_add_phantom.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, P(C.c_uint64),
                                            C.c_uint32, P(C.c_int32)]
        L.sw_engine_get_stats.argtypes = [C.c_void_p, P(abi.SwEngineStats)]
        L.sw_engine_add_phantom_ex.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, P(C.c_uint64),
                                               C.c_uint32, C.c_int, P(C.c_int32)]
        L.sw_engine_submit.argtypes = [C.c_void_p, C.c_int32, P(abi.SwParams), P(abi.SwSequence),
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, P(C.c_int64)]
        L.sw_engine_poll.argtypes = [C.c_void_p, C.c_int, P(abi.SwJobResult), C.c_uint32,
                                     P(C.c_uint32)]
        L.sw_engine_pending.argtypes = [C.c_void_p, P(C.c_uint32)]
        L.sw_sim_spins.argtypes = [P(abi.SwParams), P(abi.SwSequence), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        for f in (L.sw_phantom_cylinder, L.sw_phantom_cylinder_device):
            f.argtypes = [C.c_float, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float,
                          C.c_float, C.c_int32, C.c_void_p, C.c_void_p, P(C.c_float)]
        for f in (L.sw_phantom_sphere, L.sw_phantom_sphere_device):
            f.argtypes = [C.c_float, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float,
                          C.c_int32, C.c_void_p, C.c_void_p, P(C.c_float)]
        L.sw_sim_signal.argtypes = [P(abi.SwParams), P(abi.SwSequence), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int]
        L.sw_engine_submit_signal.argtypes = [C.c_void_p, C.c_int32, P(abi.SwParams),
                                              P(abi.SwSequence), C.c_int, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, P(C.c_int64)]
        L.sw_config_dump.argtypes = [C.c_char_p, C.c_char_p]
        L.sw_run_config.argtypes = [C.c_char_p, C.c_int]
        L.sw_h5_write.argtypes = [C.c_char_p, C.c_int, P(C.c_char_p), P(C.c_int), P(C.c_int),
                                  P(C.c_uint64), P(C.c_void_p)]
        L.sw_h5_read.argtypes = [C.c_char_p, C.c_char_p, P(C.c_int), P(C.c_int), P(C.c_uint64),
                                 C.c_void_p, C.c_uint64]
        L.sw_sync.argtypes = [C.c_void_p]
        L.sw_last_timing.argtypes = [P(abi.SwTiming)]
        L.sw_set_tuning.argtypes = [P(abi.SwTuning)]
        L.sw_get_tuning.argtypes = [P(abi.SwTuning)]
        L.sw_autotune.argtypes = [P(abi.SwParams), P(abi.SwSequence), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_int, P(abi.SwTuning), P(abi.SwTuneEntry),
                                  C.c_uint32, P(C.c_uint32)]
        L.sw_debug_logf.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        L.sw_debug_ms_normal.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
        L.sw_debug_dadd.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        L.sw_debug_d2f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        L.sw_debug_mt_jump.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p]
        if L.sw_abi_version() != 1:
            raise SpinWalkError("libspinwalk_gpu ABI version mismatch")
        _lib = L
    return _lib


def check(rc):
    if rc != abi.SW_OK:
        raise SpinWalkError(f"spinwalk error {rc}: {lib().sw_last_error().decode()}")


def device_info(device=0):
    """(rc, text) of sw_device_info: CUDA versions, device count, the device's name, compute
    capability and memory (the reference CLI's -g/--gpu_info)."""
    buf = C.create_string_buffer(1024)
    rc = lib().sw_device_info(int(device), buf, len(buf))
    return rc, buf.value.decode()


def device_count():
    n = C.c_int(0)
    lib().sw_device_count(C.byref(n))
    return n.value


def fieldmap_scale(B0, timestep_us):
    return np.float32(lib().sw_fieldmap_scale(B0, timestep_us))


def initial_positions(fov, seed, n_spins):
    out = np.zeros((n_spins, 3), np.float32)
    f = (C.c_float * 3)(*[float(np.float32(x)) for x in fov])
    check(lib().sw_initial_positions(f, C.c_uint64(int(seed)), C.c_uint32(n_spins),
                                     out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def set_phantom_argtypes(L):
    """Argument types of sw_phantom_cylinders / sw_phantom_spheres on library handle L."""
    P = C.POINTER
    L.sw_phantom_cylinders.argtypes = [P(C.c_uint32), P(C.c_double), C.c_double, C.c_double,
                                       C.c_uint64, C.c_int, C.c_double, C.c_double,
                                       P(C.c_double), C.c_void_p, C.c_void_p]
    L.sw_phantom_spheres.argtypes = [P(C.c_uint32), P(C.c_double), C.c_double, C.c_double,
                                     C.c_double, C.c_uint64, C.c_double, C.c_double,
                                     P(C.c_double), C.c_double, C.c_void_p, C.c_void_p]


def _phantom_rc(rc, L, what):
    if rc == abi.SW_OK:
        return
    if L is None:
        check(rc)
    raise SpinWalkError(f"{what} failed with code {rc}")


def phantom_cylinders(n, fov_m, radius_m, volume_fraction, seed, random_orientation=True,
                      dchi=0.11e-6 * 0.4, Y=0.75, B0_dir=(0.0, 0.0, 1.0), L=None):
    """Seeded infinite cylinders: (mask uint8 [n,n,n], field float32 Tesla at 1 T). L: another
    library handle exporting sw_phantom_cylinders (default: this library)."""
    dims = (C.c_uint32 * 3)(n, n, n)
    fov = (C.c_double * 3)(fov_m, fov_m, fov_m)
    b0 = (C.c_double * 3)(*B0_dir)
    mask = np.empty((n, n, n), np.uint8)
    field = np.empty((n, n, n), np.float32)
    rc = (L or lib()).sw_phantom_cylinders(dims, fov, radius_m, volume_fraction, int(seed),
                                           1 if random_orientation else 0, dchi, Y, b0, _p(mask),
                                           _p(field))
    _phantom_rc(rc, L, "sw_phantom_cylinders")
    return mask, field


def phantom_spheres(n, fov_m, rmin_m, rmax_m, volume_fraction, seed, dchi=0.11e-6 * 0.4,
                    Y=0.75, B0_dir=(0.0, 0.0, 1.0), window=5.0, L=None):
    """Seeded spheres with superposed dipole fields: (mask uint8, field float32 Tesla at 1 T).
    L: another library handle exporting sw_phantom_spheres (default: this library)."""
    dims = (C.c_uint32 * 3)(n, n, n)
    fov = (C.c_double * 3)(fov_m, fov_m, fov_m)
    b0 = (C.c_double * 3)(*B0_dir)
    mask = np.empty((n, n, n), np.uint8)
    field = np.empty((n, n, n), np.float32)
    rc = (L or lib()).sw_phantom_spheres(dims, fov, rmin_m, rmax_m, volume_fraction, int(seed),
                                         dchi, Y, b0, window, _p(mask), _p(field))
    _phantom_rc(rc, L, "sw_phantom_spheres")
    return mask, field


def logf_exception_count():
    n, w = C.c_uint64(0), C.c_uint64(0)
    check(lib().sw_logf_exception_count(C.byref(n), C.byref(w)))
    return n.value, w.value


def config_dump(ini_path, out_path):
    """Parsed config as text (the reference's config_reader semantics); returns the rc."""
    return lib().sw_config_dump(str(ini_path).encode(), str(out_path).encode())


_H5_DTYPES = {0: np.uint8, 1: np.float32, 2: np.float64, 3: np.int8, 4: np.uint16, 5: np.int16,
              6: np.uint32, 7: np.int32, 8: np.uint64, 9: np.int64}
_H5_TYPES = {np.dtype(t): c for c, t in _H5_DTYPES.items()}


def h5_write(path, datasets):
    """Writes {name: numpy array (uint8/float32/float64)} as an HDF5 file (root datasets)."""
    items = [(k, np.ascontiguousarray(v)) for k, v in datasets.items()]
    n = len(items)
    names = (C.c_char_p * n)(*[k.encode() for k, _ in items])
    types = (C.c_int * n)(*[_H5_TYPES[v.dtype] for _, v in items])
    ranks = (C.c_int * n)(*[v.ndim for _, v in items])
    flat = [d for _, v in items for d in v.shape]
    dims = (C.c_uint64 * max(1, len(flat)))(*flat)
    data = (C.c_void_p * n)(*[v.ctypes.data for _, v in items])
    check(lib().sw_h5_write(str(path).encode(), n, names, types, ranks, dims, data))


def h5_read(path, name):
    t, r = C.c_int(0), C.c_int(0)
    dims = (C.c_uint64 * 8)()
    check(lib().sw_h5_read(str(path).encode(), name.encode(), C.byref(t), C.byref(r), dims, None, 0))
    out = np.empty([dims[i] for i in range(r.value)], _H5_DTYPES[t.value])
    check(lib().sw_h5_read(str(path).encode(), name.encode(), None, None, None,
                           out.ctypes.data_as(C.c_void_p), out.nbytes))
    return out


def run_config(ini_path, device=0):
    """sw_run_config: the whole `spinwalk sim -c ini` run (HDF5 in, HDF5 out)."""
    check(lib().sw_run_config(str(ini_path).encode(), int(device)))


def set_tuning(resort_interval=0, walk_block=256, seed_chunks=0, round_streams=0,
               jump_min_kwords=0, ring_steps=0, walk_blocks_per_sm=0):
    """sw_set_tuning: Morton re-sort interval (walk rounds, 0 = never), walk block size, seed
    chunks of the seed/walk pipeline (0 = auto), round halves (0 = auto), the discard count
    from which seeding jumps ahead (in 1024 words, 0 = default 1408) and the steps of one
    refill/walk round (0 = default 512) and a cap on the walk's blocks per SM (0 = none) for
    every later call of this process. Results do not depend on it."""
    t = abi.SwTuning(resort_interval=int(resort_interval), walk_block=int(walk_block),
                     seed_chunks=int(seed_chunks), round_streams=int(round_streams),
                     jump_min_kwords=int(jump_min_kwords), ring_steps=int(ring_steps),
                     walk_blocks_per_sm=int(walk_blocks_per_sm))
    check(lib().sw_set_tuning(C.byref(t)))


def _tuning_dict(t):
    return dict(resort_interval=t.resort_interval, walk_block=t.walk_block,
                seed_chunks=t.seed_chunks, round_streams=t.round_streams,
                jump_min_kwords=t.jump_min_kwords, ring_steps=t.ring_steps,
                walk_blocks_per_sm=t.walk_blocks_per_sm)


def get_tuning():
    t = abi.SwTuning()
    check(lib().sw_get_tuning(C.byref(t)))
    return _tuning_dict(t)


def autotune(problem, apply=False):
    """sw_autotune on `problem` (a problem.Problem): returns (best, table), best a dict as
    get_tuning(), table the measured candidates (resort_interval, walk_block, ms_per_round,
    sort_ms)."""
    best = abi.SwTuning()
    tab = (abi.SwTuneEntry * 32)()
    n = C.c_uint32(0)
    check(lib().sw_autotune(C.byref(problem.params), C.byref(problem.seq.struct),
                            _p(problem.field), _p(problem.mask), _p(problem.XYZ0), int(bool(apply)),
                            C.byref(best), tab, 32, C.byref(n)))
    table = [dict(resort_interval=e.resort_interval, walk_block=e.walk_block,
                  ms_per_round=e.ms_per_round, sort_ms=e.sort_ms, ring_steps=e.ring_steps)
             for e in tab[:n.value]]
    return _tuning_dict(best), table


def last_timing():
    t = abi.SwTiming()
    check(lib().sw_last_timing(C.byref(t)))
    return {k: getattr(t, k) for k, _ in abi.SwTiming._fields_}


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def run(problem, precision=abi.SW_PREC_FP32, fp64_shadow=False, fill=0.0):
    """sw_sim on host buffers: one scale of `problem` (a problem.Problem). Returns a dict with
    M1 [n, nTE, 3], XYZ1 [n, traj, 3], T [n, nTE], status [n] (+ M1_fp64, timing)."""
    M1, XYZ1, T, status = problem.outputs(fill)
    M1d = np.full(M1.shape, fill, np.float64) if fp64_shadow else None
    check(lib().sw_sim(C.byref(problem.params), C.byref(problem.seq.struct),
                       _p(problem.field), _p(problem.mask), _p(problem.M0), _p(problem.XYZ0),
                       _p(M1), _p(XYZ1), _p(T), _p(status), int(precision), _p(M1d)))
    out = dict(M1=M1, XYZ1=XYZ1, T=T, status=status, timing=last_timing())
    if M1d is not None:
        out["M1_fp64"] = M1d
    return out


def run_batch(problems, precision=abi.SW_PREC_FP32, fill=0.0, outs=None):
    """sw_sim_batch over problem.Problem instances that share the phantom and the seed (the
    phantom arrays of the first are used). Returns one output dict per instance, as run();
    `outs` (the dicts of an earlier call on the same problems) are written again in place."""
    if outs is None:
        outs = [dict(zip(("M1", "XYZ1", "T", "status"), pr.outputs(fill))) for pr in problems]
    arr = (abi.SwInstance * len(problems))()
    for a, pr, o in zip(arr, problems, outs):
        a.param = C.pointer(pr.params)
        a.seq = C.pointer(pr.seq.struct)
        a.M0, a.XYZ0 = _p(pr.M0), _p(pr.XYZ0)
        a.M1, a.XYZ1, a.T, a.status = _p(o["M1"]), _p(o["XYZ1"]), _p(o["T"]), _p(o["status"])
    pr0 = problems[0]
    check(lib().sw_sim_batch(arr, len(problems), _p(pr0.field), _p(pr0.mask), int(precision)))
    t = last_timing()
    for o in outs:
        o["timing"] = t
    return outs


def phantom_cylinder(fov_um, resolution, dchi=0.11e-6, Y=0.75, radius_um=8.0,
                     volume_fraction=4.0, orientation_deg=90.0, seed=10, field=True):
    """The reference's phantom::cylinder generated on the GPU: (mask u8, field f32 or None,
    actual volume fraction in percent), arrays of shape (res, res, res)."""
    n = int(resolution) ** 3
    mask = np.zeros(n, np.uint8)
    fld = np.zeros(n, np.float32) if field and Y >= 0 else None
    bvf = C.c_float()
    check(lib().sw_phantom_cylinder(fov_um, resolution, dchi, Y, radius_um, volume_fraction,
                                    orientation_deg, seed, _p(mask), _p(fld), C.byref(bvf)))
    shape = (resolution,) * 3
    return mask.reshape(shape), (fld.reshape(shape) if fld is not None else None), bvf.value


def phantom_sphere(fov_um, resolution, dchi=0.11e-6, Y=0.75, radius_um=8.0,
                   volume_fraction=4.0, seed=10, field=True):
    """The reference's phantom::sphere generated on the GPU (see phantom_cylinder)."""
    n = int(resolution) ** 3
    mask = np.zeros(n, np.uint8)
    fld = np.zeros(n, np.float32) if field and Y >= 0 else None
    bvf = C.c_float()
    check(lib().sw_phantom_sphere(fov_um, resolution, dchi, Y, radius_um, volume_fraction, seed,
                                  _p(mask), _p(fld), C.byref(bvf)))
    shape = (resolution,) * 3
    return mask.reshape(shape), (fld.reshape(shape) if fld is not None else None), bvf.value


def run_signal(problem, precision=abi.SW_PREC_FP32):
    """sw_sim_signal: (signal [nTE, n_substrate, 3] sums of M, count [nTE, n_substrate],
    status [n]) with the reduction fused into the walk (no per-spin M1 / T / XYZ1)."""
    ns, nte = problem.params.n_substrate, problem.n_te
    sig = np.zeros((nte, ns, 3), np.float64)
    cnt = np.zeros((nte, ns), np.uint64)
    status = np.full(problem.params.n_spins, -1, np.int32)
    check(lib().sw_sim_signal(C.byref(problem.params), C.byref(problem.seq.struct),
                              _p(problem.field), _p(problem.mask), _p(problem.M0),
                              _p(problem.XYZ0), _p(sig), _p(cnt), _p(status), int(precision)))
    return sig, cnt, status


def run_spins(problem, lo, hi, precision=abi.SW_PREC_FP32, fill=0.0):
    """sw_sim_spins: rows [lo, hi) of run(problem) (M1, XYZ1, T, status hold those rows only)."""
    M1, XYZ1, T, status = problem.outputs(fill)
    M1, XYZ1, T, status = (np.ascontiguousarray(a[lo:hi]) for a in (M1, XYZ1, T, status))
    M0 = np.ascontiguousarray(problem.M0[lo:hi])
    XYZ0 = np.ascontiguousarray(problem.XYZ0[lo:hi])
    check(lib().sw_sim_spins(C.byref(problem.params), C.byref(problem.seq.struct),
                             _p(problem.field), _p(problem.mask), _p(M0), _p(XYZ0), int(lo),
                             int(hi), _p(M1), _p(XYZ1), _p(T), _p(status), int(precision)))
    return dict(M1=M1, XYZ1=XYZ1, T=T, status=status)


class Engine:
    """sw_engine: resident phantoms, one seeding per simulation seed, jobs run in spin-range
    chunks on concurrent slots. Every job equals its own run() bit for bit."""

    def __init__(self, device=0, n_slots=4, slot_spins=1 << 20, hbm_budget=0):
        self._h = C.c_void_p()
        check(lib().sw_engine_create(int(device), int(n_slots), int(slot_spins),
                                     C.c_uint64(int(hbm_budget)), C.byref(self._h)))
        self._jobs = {}                 # job id -> (problem, outputs): keep buffers alive

    def add_phantom(self, problem, bf16=False):
        """Registers the phantom (mask, scaled field) of a problem.Problem; returns its id.
        bf16: 4-byte voxel records with the field rounded to bfloat16 (SW_FIELD_BF16)."""
        pid = C.c_int32()
        dims = (C.c_uint64 * 3)(*problem.mask.shape)
        check(lib().sw_engine_add_phantom_ex(self._h, _p(problem.mask), _p(problem.field), dims,
                                             int(problem.params.n_substrate),
                                             abi.SW_FIELD_BF16 if bf16 else 0, C.byref(pid)))
        return pid.value

    def submit(self, problem, phantom, precision=abi.SW_PREC_FP32, fill=0.0):
        o = dict(zip(("M1", "XYZ1", "T", "status"), problem.outputs(fill)))
        jid = C.c_int64()
        check(lib().sw_engine_submit(self._h, int(phantom), C.byref(problem.params),
                                     C.byref(problem.seq.struct), int(precision),
                                     _p(problem.M0), _p(problem.XYZ0), _p(o["M1"]),
                                     _p(o["XYZ1"]), _p(o["T"]), _p(o["status"]), C.byref(jid)))
        self._jobs[jid.value] = (problem, o)
        return jid.value, o

    def submit_signal(self, problem, phantom, precision=abi.SW_PREC_FP32):
        """Signal mode (see run_signal): returns (job id, dict(signal, count, status))."""
        ns, nte = problem.params.n_substrate, problem.n_te
        o = dict(signal=np.zeros((nte, ns, 3), np.float64), count=np.zeros((nte, ns), np.uint64),
                 status=np.full(problem.params.n_spins, -1, np.int32))
        jid = C.c_int64()
        check(lib().sw_engine_submit_signal(self._h, int(phantom), C.byref(problem.params),
                                            C.byref(problem.seq.struct), int(precision),
                                            _p(problem.M0), _p(problem.XYZ0), _p(o["signal"]),
                                            _p(o["count"]), _p(o["status"]), C.byref(jid)))
        self._jobs[jid.value] = (problem, o)
        return jid.value, o

    def poll(self, wait=0, max_done=256):
        """[(job id, rc, latency s)] of jobs finished since the last poll."""
        res = (abi.SwJobResult * max_done)()
        n = C.c_uint32()
        check(lib().sw_engine_poll(self._h, int(wait), res, max_done, C.byref(n)))
        out = [(r.job_id, r.rc, r.latency_s) for r in res[:n.value]]
        for jid, _, _ in out:
            self._jobs.pop(jid, None)
        return out

    def stats(self):
        """dict(launches, rounds, seedings) since the engine was created, and the HBM it holds
        (hbm_used of hbm_budget bytes, seed_caches held)."""
        s = abi.SwEngineStats()
        check(lib().sw_engine_get_stats(self._h, C.byref(s)))
        return dict(launches=s.launches, rounds=s.rounds, seedings=s.seedings,
                    hbm_used=s.hbm_used, hbm_budget=s.hbm_budget, seed_caches=s.seed_caches)

    def run_all(self):
        done = []
        while True:
            d = self.poll(wait=2)
            done += d
            n = C.c_uint32()
            check(lib().sw_engine_pending(self._h, C.byref(n)))
            if n.value == 0 and not d:
                return done

    def close(self):
        if self._h:
            lib().sw_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_device(problem, d_field, d_mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T, d_status=None,
               precision=abi.SW_PREC_FP32, d_M1d=None, stream=None):
    """sw_sim_device with raw device pointers (ints), e.g. torch tensors' data_ptr()."""
    check(lib().sw_sim_device(C.byref(problem.params), C.byref(problem.seq.struct),
                              d_field, d_mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T, d_status,
                              int(precision), d_M1d, stream))


def run_device_noalloc(problem, d_field, d_mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T,
                       d_status=None, stream=None):
    """sw_sim_device_noalloc: like run_device (FP32), with no device allocation by the library;
    its scratch is a fixed static device array (see include/spinwalk_gpu.h)."""
    check(lib().sw_sim_device_noalloc(C.byref(problem.params), C.byref(problem.seq.struct),
                                      d_field, d_mask, d_M0, d_XYZ0, d_M1, d_XYZ1, d_T,
                                      d_status, stream))


def run_tracks(problem, tracks, fill=0.0, precision=abi.SW_PREC_FP32, fp64=False):
    """sw_sim_tracks: many instances of `problem` sharing one walk. `tracks` is a list of dicts
    with keys linear_phase_cycling, quadratic_phase_cycling, n_dummy_scan and optionally
    RF_FA_deg / RF_PH_deg arrays and gradient_scale. Returns one output dict per track; with
    fp64=True each also holds "M1_fp64", the track's FP64 shadow."""
    n, nte = problem.params.n_spins, problem.n_te
    arr = (abi.SwTrack * len(tracks))()
    outs, keep = [], []
    for i, t in enumerate(tracks):
        o = dict(M1=np.full((n, nte, 3), fill, np.float32), XYZ1=np.full((n, 1, 3), fill, np.float32),
                 T=np.zeros((n, nte), np.uint8), status=np.full(n, -1, np.int32))
        outs.append(o)
        s = arr[i]
        s.linear_phase_cycling = t.get("linear_phase_cycling", 0.0)
        s.quadratic_phase_cycling = t.get("quadratic_phase_cycling", 0.0)
        s.n_dummy_scan = int(t.get("n_dummy_scan", 0))
        for key in ("RF_FA_deg", "RF_PH_deg"):
            if t.get(key) is not None:
                a = np.ascontiguousarray(t[key], np.float32)
                keep.append(a)
                setattr(s, key, abi.ptr(a, C.c_float))
            else:
                setattr(s, key, abi.ptr(None, C.c_float))
        s.M1 = abi.ptr(o["M1"], C.c_float)
        s.XYZ1 = abi.ptr(o["XYZ1"], C.c_float)
        s.T = abi.ptr(o["T"], C.c_uint8)
        s.status = abi.ptr(o["status"], C.c_int32)
        if t.get("gradient_scale") is not None:
            s.gradient_scale = float(t["gradient_scale"])
            s.options |= abi.SW_TRACK_GRADIENT_SCALE
        if fp64:
            o["M1_fp64"] = np.full((n, nte, 3), fill, np.float64)
            s.M1_fp64 = abi.ptr(o["M1_fp64"], C.c_double)
        else:
            s.M1_fp64 = abi.ptr(None, C.c_double)
    check(lib().sw_sim_tracks(C.byref(problem.params), C.byref(problem.seq.struct), arr,
                              len(tracks), _p(problem.field), _p(problem.mask), _p(problem.M0),
                              _p(problem.XYZ0), int(precision)))
    return outs


def debug_d2f(d_x, d_y, n, stream=None):
    check(lib().sw_debug_d2f(d_x, d_y, C.c_uint64(n), stream))


def release_workspaces():
    """sw_release_workspaces: frees the device memory the one-call entry points keep."""
    check(lib().sw_release_workspaces())


def debug_dadd(d_a, d_b, d_y, n, stream=None):
    check(lib().sw_debug_dadd(d_a, d_b, d_y, C.c_uint64(n), stream))


def debug_ms_normal(x_lo, n, d_y, stream=None):
    check(lib().sw_debug_ms_normal(int(x_lo), int(n), d_y, stream))


def debug_logf(d_x, d_y, n, stream=None):
    check(lib().sw_debug_logf(d_x, d_y, C.c_uint64(n), stream))


def debug_mt_jump(z):
    """sw_debug_mt_jump: (624-word buffer, position) of mt19937(z) after discard(z), computed on
    the host through the jump polynomial."""
    block = np.zeros(624, np.uint32)
    pos = np.zeros(1, np.uint32)
    check(lib().sw_debug_mt_jump(C.c_uint64(int(z)), _p(block), _p(pos)))
    return block, int(pos[0])
