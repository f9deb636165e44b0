"""sw_sim_device_noalloc: the entry point for callers that may not allocate device memory (a
process whose device memory is reserved up front by a pool or another framework, a real-time loop
that cannot take cudaMalloc's device-wide synchronisation, a host application that forbids
libraries from allocating). Its scratch is one fixed static device array.

Checked through the C ABI against the regular device entry point, sw_sim_device, on two calls in
a row (the second call finds the first call's leftovers in the shared array), and the library
must not allocate device memory during a call. This file is collected last so that a failing run
that stops at the first failure has already run every other test.
"""
import numpy as np
import pytest

from spinwalk_gb300 import _lib
from tests.helpers import bits_equal, load_golden

pytestmark = pytest.mark.gpu


def _device_buffers(torch, pr, fill):
    n, nte = pr.params.n_spins, pr.n_te
    dev = "cuda"
    return dict(
        field=torch.from_numpy(pr.field).to(dev), mask=torch.from_numpy(pr.mask).to(dev),
        M0=torch.from_numpy(pr.M0).to(dev), XYZ0=torch.from_numpy(pr.XYZ0).to(dev),
        M1=torch.full((n, nte, 3), fill, dtype=torch.float32, device=dev),
        XYZ1=torch.full((n, pr.traj_len, 3), fill, dtype=torch.float32, device=dev),
        T=torch.zeros((n, nte), dtype=torch.uint8, device=dev),
        status=torch.full((n,), -1, dtype=torch.int32, device=dev))


def _ptrs(d):
    return (d["field"].data_ptr(), d["mask"].data_ptr(), d["M0"].data_ptr(),
            d["XYZ0"].data_ptr(), d["M1"].data_ptr(), d["XYZ1"].data_ptr(), d["T"].data_ptr(),
            d["status"].data_ptr())


def _host(d):
    return {k: d[k].cpu().numpy() for k in ("M1", "XYZ1", "T", "status")}


@pytest.mark.parametrize("case", ["se_multi_te", "lost_spins"])
def test_noalloc_matches_device_entry_point_twice(case):
    torch = pytest.importorskip("torch")
    pr, _ = load_golden(case)
    ref_bufs = _device_buffers(torch, pr, float("nan"))
    _lib.run_device(pr, *_ptrs(ref_bufs))
    torch.cuda.synchronize()
    want = _host(ref_bufs)
    for call in range(2):
        bufs = _device_buffers(torch, pr, float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        _lib.run_device_noalloc(pr, *_ptrs(bufs))
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        got = _host(bufs)
        assert bits_equal(got["XYZ1"], want["XYZ1"]), (case, call)
        assert bits_equal(got["T"], want["T"]), (case, call)
        assert np.array_equal(got["status"], want["status"]), (case, call)
        # same kernels, same inputs: the magnetisation is bit-identical too
        assert bits_equal(got["M1"], want["M1"]), (case, call)
        if call == 1:     # after set-up, a call allocates no device memory at all
            assert free_after == free_before, (free_before, free_after)


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    pr, _ = load_golden("gre")
    p = pr.params
    n_big = 40_000                      # ~240 MiB of generator state: beyond the static array
    p.n_spins = n_big
    d = dict(field=torch.from_numpy(pr.field).cuda(), mask=torch.from_numpy(pr.mask).cuda(),
             M0=torch.zeros((n_big, 3), device="cuda"), XYZ0=torch.zeros((n_big, 3), device="cuda"),
             M1=torch.zeros((n_big, pr.n_te, 3), device="cuda"),
             XYZ1=torch.zeros((n_big, 1, 3), device="cuda"),
             T=torch.zeros((n_big, pr.n_te), dtype=torch.uint8, device="cuda"),
             status=torch.zeros(n_big, dtype=torch.int32, device="cuda"))
    with pytest.raises(_lib.SpinWalkError, match="static"):
        _lib.run_device_noalloc(pr, *_ptrs(d))
