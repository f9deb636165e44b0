"""ctypes mirror of include/spinwalk_gpu.h (struct layouts and constants).

The structs follow the reference's ``sim::parameters`` (src/sim/simulation_parameters.cuh:176-246)
and ``parameters_uvec`` (simulation_parameters.cuh:102-173) field for field, so a Python caller
fills them exactly as the reference's driver ``monte_carlo::run`` fills its own
(src/sim/monte_carlo.cu:199-336).
"""
import ctypes as C

import numpy as np

SW_OK = 0
SW_ERR_INVALID = -1
SW_ERR_CUDA = -2
SW_ERR_NOMEM = -3
SW_ERR_IO = -4
SW_ERR_CONFIG = -5
SW_ERR_TIMEOUT = -6

SW_SPIN_OK = 0
SW_SPIN_LOST = 1
SW_SPIN_OOB = 2
SW_SPIN_START_OOB = 3

SW_PREC_FP32 = 0
SW_PREC_FP64 = 1
SW_PREC_KAHAN = 2
SW_FIELD_BF16 = 0x200
SW_TRACK_GRADIENT_SCALE = 0x1
SW_RNG_MT19937 = 0x000
SW_RNG_MINSTD = 0x100


class SwParams(C.Structure):
    _fields_ = [
        ("fov", C.c_double * 3),
        ("B0", C.c_float),
        ("c", C.c_float),
        ("s", C.c_float),
        ("linear_phase_cycling", C.c_float),
        ("quadratic_phase_cycling", C.c_float),
        ("timestep_us", C.c_int32),
        ("TR_us", C.c_int32),
        ("n_dummy_scan", C.c_int32),
        ("n_spins", C.c_uint32),
        ("n_timepoints", C.c_uint32),
        ("n_substrate", C.c_uint32),
        ("n_scales", C.c_uint32),
        ("phantom_size", C.c_uint64 * 3),
        ("seed", C.c_uint64),
        ("max_iterations", C.c_uint64),
        ("matrix_length", C.c_int64),
        ("enCrossFOV", C.c_int32),
        ("enRecordTrajectory", C.c_int32),
        ("fieldmap_exist", C.c_int32),
        ("_pad", C.c_int32),
    ]


class SwSequence(C.Structure):
    _fields_ = [
        ("diffusivity", C.POINTER(C.c_double)),
        ("T1_ms", C.POINTER(C.c_float)),
        ("T2_ms", C.POINTER(C.c_float)),
        ("pXY", C.POINTER(C.c_float)),
        ("RF_FA_deg", C.POINTER(C.c_float)),
        ("RF_PH_deg", C.POINTER(C.c_float)),
        ("RF_us", C.POINTER(C.c_int32)),
        ("TE_us", C.POINTER(C.c_int32)),
        ("dephasing_deg", C.POINTER(C.c_float)),
        ("dephasing_us", C.POINTER(C.c_int32)),
        ("gradientX_mTm", C.POINTER(C.c_float)),
        ("gradientY_mTm", C.POINTER(C.c_float)),
        ("gradientZ_mTm", C.POINTER(C.c_float)),
        ("gradient_us", C.POINTER(C.c_int32)),
        ("n_RF", C.c_uint32),
        ("n_TE", C.c_uint32),
        ("n_dephasing", C.c_uint32),
        ("n_gradient", C.c_uint32),
    ]


class SwTrack(C.Structure):
    _fields_ = [
        ("linear_phase_cycling", C.c_float),
        ("quadratic_phase_cycling", C.c_float),
        ("n_dummy_scan", C.c_int32),
        ("_pad", C.c_int32),
        ("RF_FA_deg", C.POINTER(C.c_float)),
        ("RF_PH_deg", C.POINTER(C.c_float)),
        ("M1", C.POINTER(C.c_float)),
        ("XYZ1", C.POINTER(C.c_float)),
        ("T", C.POINTER(C.c_uint8)),
        ("status", C.POINTER(C.c_int32)),
        ("M1_fp64", C.POINTER(C.c_double)),
        ("gradient_scale", C.c_float),
        ("options", C.c_uint32),
    ]


class SwInstance(C.Structure):
    _fields_ = [
        ("param", C.POINTER(SwParams)),
        ("seq", C.POINTER(SwSequence)),
        ("M0", C.c_void_p),
        ("XYZ0", C.c_void_p),
        ("M1", C.c_void_p),
        ("XYZ1", C.c_void_p),
        ("T", C.c_void_p),
        ("status", C.c_void_p),
    ]


class SwJobResult(C.Structure):
    _fields_ = [("job_id", C.c_int64), ("rc", C.c_int32), ("_pad", C.c_int32),
                ("latency_s", C.c_double)]


class SwEngineStats(C.Structure):
    _fields_ = [
        ("launches", C.c_uint64),
        ("rounds", C.c_uint64),
        ("seedings", C.c_uint64),
        ("hbm_used", C.c_uint64),
        ("hbm_budget", C.c_uint64),
        ("seed_caches", C.c_uint64),
    ]


# sw_tuning.jump_min_kwords = 0 means this many 1024-word units (include/spinwalk_gpu.h)
JUMP_MIN_KWORDS_DEFAULT = 1408


class SwTuning(C.Structure):
    _fields_ = [
        ("resort_interval", C.c_uint32),
        ("walk_block", C.c_uint32),
        ("seed_chunks", C.c_uint32),
        ("round_streams", C.c_uint32),
        ("jump_min_kwords", C.c_uint32),
        ("ring_steps", C.c_uint32),
        ("walk_blocks_per_sm", C.c_uint32),
        ("reserved", C.c_uint32 * 1),
    ]


class SwTuneEntry(C.Structure):
    _fields_ = [
        ("resort_interval", C.c_uint32),
        ("walk_block", C.c_uint32),
        ("ms_per_round", C.c_float),
        ("sort_ms", C.c_float),
        ("ring_steps", C.c_uint32),
    ]


class SwTiming(C.Structure):
    _fields_ = [
        ("seed_ms", C.c_float),
        ("refill_ms", C.c_float),
        ("walk_ms", C.c_float),
        ("total_ms", C.c_float),
        ("n_chunks", C.c_uint32),
        ("n_launches", C.c_uint32),
    ]


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (or NULL for None)."""
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


_SEQ_ARRAYS = [
    ("diffusivity", np.float64, C.c_double),
    ("T1_ms", np.float32, C.c_float),
    ("T2_ms", np.float32, C.c_float),
    ("pXY", np.float32, C.c_float),
    ("RF_FA_deg", np.float32, C.c_float),
    ("RF_PH_deg", np.float32, C.c_float),
    ("RF_us", np.int32, C.c_int32),
    ("TE_us", np.int32, C.c_int32),
    ("dephasing_deg", np.float32, C.c_float),
    ("dephasing_us", np.int32, C.c_int32),
    ("gradientX_mTm", np.float32, C.c_float),
    ("gradientY_mTm", np.float32, C.c_float),
    ("gradientZ_mTm", np.float32, C.c_float),
    ("gradient_us", np.int32, C.c_int32),
]


class Sequence:
    """Owns the numpy arrays behind an SwSequence (keeps them alive while in use)."""

    def __init__(self, **arrays):
        self.arrays = {}
        for name, dt, _ in _SEQ_ARRAYS:
            a = arrays.get(name)
            a = np.ascontiguousarray(np.asarray([] if a is None else a, dtype=dt).ravel())
            self.arrays[name] = a
        self.struct = SwSequence()
        for name, _, ct in _SEQ_ARRAYS:
            a = self.arrays[name]
            setattr(self.struct, name, ptr(a, ct) if a.size else ptr(None, ct))
        self.struct.n_RF = self.arrays["RF_us"].size
        self.struct.n_TE = self.arrays["TE_us"].size
        self.struct.n_dephasing = self.arrays["dephasing_us"].size
        self.struct.n_gradient = self.arrays["gradient_us"].size

    def __getitem__(self, k):
        return self.arrays[k]
