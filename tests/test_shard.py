"""Sharding one job across ranks (spinwalk_gb300.shard): world-size-2 gloo ranks on the CPU,
each computing its spin range with the oracle; rank 0 reassembles the job, which must equal the
unsharded oracle run bit for bit. The GPU test checks sw_sim_spins rows against one sw_sim."""
import os
import socket

import numpy as np
import pytest

from spinwalk_gb300 import shard
from tests.helpers import bits_equal, load_golden


def test_balanced_ranges_cover_and_balance():
    for n, world, seed, steps in ((1000, 2, 10, 401), (10, 4, 0, 1), (3, 5, 7, 100),
                                  (1_000_000, 8, 10, 2001), (0, 3, 1, 1)):
        r = shard.balanced_ranges(n, world, seed, steps)
        assert len(r) == world and r[0][0] == 0 and r[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        assert all(lo <= hi for lo, hi in r)
        if n >= 1000:
            costs = [shard.spin_cost(np.arange(lo, hi), seed, steps).sum() for lo, hi in r]
            assert max(costs) / min(costs) < 1.01
    # seeding makes later spins costlier: the last range of a large job is the shortest
    r = shard.balanced_ranges(1_000_000, 4, 10, 100)
    assert r[-1][1] - r[-1][0] < r[0][1] - r[0][0]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case, q):
    import torch.distributed as dist
    from tests import oracle_lib
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pr, _ = load_golden(case)

    def compute(problem, lo, hi):
        ids = np.arange(lo, hi, dtype=np.uint32)
        full = oracle_lib.run(problem, spin_ids=ids, n_threads=1)
        return {k: np.ascontiguousarray(full[k][lo:hi]) for k in ("M1", "XYZ1", "T", "status")}

    out = shard.run_sharded(pr, compute)
    if rank == 0:
        ref = oracle_lib.run(pr, n_threads=1)
        q.put(all(bits_equal(out[k], ref[k]) for k in ("M1", "XYZ1", "T", "status")))
    dist.destroy_process_group()


@pytest.mark.parametrize("case", ["gre", "permeable", "lost_spins"])
def test_sharded_job_equals_one_run_gloo_world2(case):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, case, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True


@pytest.mark.gpu
def test_gpu_spin_ranges_equal_rows_of_one_run():
    from spinwalk_gb300 import _lib
    pr, _ = load_golden("permeable")
    full = _lib.run(pr)
    n = pr.params.n_spins
    for lo, hi in ((0, n), (0, 1), (n // 3, n // 3 + 7), (n - 5, n), *shard.balanced_ranges(n, 3, pr.params.seed, 100)):
        rows = _lib.run_spins(pr, lo, hi)
        for k in ("M1", "XYZ1", "T", "status"):
            assert bits_equal(rows[k], full[k][lo:hi]), (lo, hi, k)
