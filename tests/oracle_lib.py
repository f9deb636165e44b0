"""ctypes access to the oracle (test infrastructure).

  oracle/liboracle.so        the project's CPU restatement of sim::sim (oracle/sim_oracle.cpp)
  oracle/_ref/libref_sim.so  the reference's own sim::sim compiled from its source tree (only
                             where that tree exists; see oracle/Makefile)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
import ctypes as C
import os

import numpy as np

from spinwalk_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_PATH = os.path.join(ROOT, "oracle", "liboracle.so")
SYNTH_PATH = os.path.join(ROOT, "oracle", "libsynth.so")
REF_PATH = os.path.join(ROOT, "oracle", "_ref", "libref_sim.so")
REF_NVCC_PATH = os.path.join(ROOT, "oracle", "_ref", "libref_sim_nvcc.so")

_ora = None
_synth = None
_ref = None
_ref_nvcc = None


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def oracle():
    global _ora
    if _ora is None:
        if not os.path.exists(ORACLE_PATH):
            from spinwalk_gb300 import _build
            _build.build_oracle()
        L = C.CDLL(ORACLE_PATH)
        L.oracle_sim.argtypes = [C.POINTER(abi.SwParams), C.POINTER(abi.SwSequence)] + \
            [C.c_void_p] * 8 + [C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_void_p]
        L.oracle_initial_positions.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p]
        L.oracle_logf.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
        L.oracle_logf.restype = None
        L.oracle_ms_normal.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p]
        L.oracle_ms_normal.restype = None
        L.oracle_mt_discard.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p]
        L.oracle_mt_discard.restype = None
        _ora = L
    return _ora


def synth():
    """oracle/libsynth.so: the synthetic phantom generator built alone (no CUDA library), so that
    the benchmark's CPU reference arm makes the same phantoms without loading the GPU library."""
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            from spinwalk_gb300 import _build
            _build.build_oracle()
        from spinwalk_gb300 import _lib
        L = C.CDLL(SYNTH_PATH)
        _lib.set_phantom_argtypes(L)
        _synth = L
    return _synth


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        L.ref_sim.argtypes = [C.POINTER(abi.SwParams), C.POINTER(abi.SwSequence)] + \
            [C.c_void_p] * 7 + [C.c_void_p, C.c_uint32, C.c_int]
        L.ref_config_dump.argtypes = [C.c_char_p, C.c_char_p]
        _ref = L
    return _ref


def _ids(spin_ids):
    if spin_ids is None:
        return None, 0
    ids = np.ascontiguousarray(spin_ids, dtype=np.uint32)
    return ids, ids.size


def run(problem, precision=abi.SW_PREC_FP32, fp64_shadow=False, spin_ids=None, n_threads=0,
        fill=0.0, outputs=None):
    """oracle_sim on `problem` (all spins, or only `spin_ids`, written at their own slots)."""
    M1, XYZ1, T, status = outputs if outputs is not None else problem.outputs(fill)
    M1d = np.full(M1.shape, fill, np.float64) if fp64_shadow else None
    ids, n_ids = _ids(spin_ids)
    oracle().oracle_sim(C.byref(problem.params), C.byref(problem.seq.struct), _p(problem.field),
                        _p(problem.mask), _p(problem.M0), _p(problem.XYZ0), _p(M1), _p(XYZ1),
                        _p(T), _p(status), _p(ids), n_ids, int(n_threads), int(precision),
                        _p(M1d))
    out = dict(M1=M1, XYZ1=XYZ1, T=T, status=status)
    if M1d is not None:
        out["M1_fp64"] = M1d
    return out


def ref_nvcc_available():
    return os.path.exists(REF_NVCC_PATH)


def run_ref_nvcc(problem, fill=0.0):
    """The reference's own sim::sim as its nvcc host (--use_cpu) path builds it: the generator
    flavour of its CUDA build (oracle/_ref/libref_sim_nvcc.so)."""
    global _ref_nvcc
    if _ref_nvcc is None:
        L = C.CDLL(REF_NVCC_PATH)
        L.ref_sim.argtypes = [C.POINTER(abi.SwParams), C.POINTER(abi.SwSequence)] + \
            [C.c_void_p] * 7 + [C.c_void_p, C.c_uint32, C.c_int]
        _ref_nvcc = L
    M1, XYZ1, T, _ = problem.outputs(fill)
    _ref_nvcc.ref_sim(C.byref(problem.params), C.byref(problem.seq.struct), _p(problem.field),
                      _p(problem.mask), _p(problem.M0), _p(problem.XYZ0), _p(M1), _p(XYZ1), _p(T),
                      None, 0, 0)
    return dict(M1=M1, XYZ1=XYZ1, T=T)


def run_ref(problem, spin_ids=None, n_threads=0, fill=0.0):
    """The reference's own sim::sim (oracle/_ref) on `problem`."""
    M1, XYZ1, T, _ = problem.outputs(fill)
    ids, n_ids = _ids(spin_ids)
    ref().ref_sim(C.byref(problem.params), C.byref(problem.seq.struct), _p(problem.field),
                  _p(problem.mask), _p(problem.M0), _p(problem.XYZ0), _p(M1), _p(XYZ1), _p(T),
                  _p(ids), n_ids, int(n_threads))
    return dict(M1=M1, XYZ1=XYZ1, T=T)


def initial_positions(fov, seed, n):
    out = np.zeros((n, 3), np.float32)
    f = np.asarray(fov, np.float32)
    oracle().oracle_initial_positions(_p(f), C.c_uint64(int(seed)), C.c_uint32(n), _p(out))
    return out


def host_ms_normal(x_lo, n):
    """The minstd flavour's deviates of engine outputs x_lo .. x_lo+n-1 (CUDA's host erfcinvf)."""
    y = np.empty(n, np.float32)
    oracle().oracle_ms_normal(int(x_lo), int(n), _p(y))
    return y


def host_logf(x):
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    oracle().oracle_logf(_p(x), _p(y), x.size)
    return y


def mt_discard(z):
    """(624-word buffer, position) of std::mt19937(z) after discard(z) (libstdc++)."""
    block = np.zeros(624, np.uint32)
    pos = np.zeros(1, np.uint32)
    oracle().oracle_mt_discard(C.c_uint64(int(z)), _p(block), _p(pos))
    return block, int(pos[0])
