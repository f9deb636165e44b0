"""Fixtures of the reference's CUDA-build generator flavour (thrust::minstd_rand +
thrust::normal_distribution, src/sim/kernels.cu:76-80) on the inputs of every tests/golden
case, computed by the reference's own sim::sim as its nvcc host (--use_cpu) path builds it
(oracle/_ref/libref_sim_nvcc.so, `make -C oracle ref`). Writes tests/golden/minstd_outputs.npz.

    python tests/golden/make_golden_minstd.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from tests import oracle_lib                                   # noqa: E402
from tests.helpers import GOLDEN_CASES, load_golden            # noqa: E402


def main():
    L = C.CDLL(os.path.join(HERE, "..", "..", "oracle", "_ref", "libref_sim_nvcc.so"))
    L.ref_sim.argtypes = oracle_lib.ref().ref_sim.argtypes
    p = lambda x: None if x is None else x.ctypes.data_as(C.c_void_p)        # noqa: E731
    out = {}
    for case in GOLDEN_CASES:
        pr, _ = load_golden(case)
        M1, XYZ1, T, _ = pr.outputs()
        L.ref_sim(C.byref(pr.params), C.byref(pr.seq.struct), p(pr.field), p(pr.mask), p(pr.M0),
                  p(pr.XYZ0), p(M1), p(XYZ1), p(T), None, 0, 0)
        out[case + "/M1"], out[case + "/XYZ1"], out[case + "/T"] = M1, XYZ1, T
    np.savez_compressed(os.path.join(HERE, "minstd_outputs.npz"), **out)


if __name__ == "__main__":
    main()
