"""spinwalk_gb300 -- SpinWalk's `sim` hot path (Monte-Carlo spin random walk over a voxel
phantom with the Bloch update) as hand-written CUDA kernels for GB300 (sm_103a), behind the C ABI
in include/spinwalk_gpu.h.

    from spinwalk_gb300 import Problem, run
    out = run(Problem(mask, fov, field_T, ...))     # bit-exact with the reference's CPU path

Python here is a thin binding for tests and benchmarks; the product is libspinwalk_gpu.so and the
`spinwalk` command-line host.
"""
from . import abi  # noqa: F401
from ._lib import SpinWalkError, device_count, run, run_device  # noqa: F401
from .problem import Problem, cylinder_phantom, sphere_phantom  # noqa: F401

__version__ = "0.1.0"
