"""Sharding one `sim` job across processes / GPUs.

Spins are independent: a spin's generators are seeded from seed + spin id and its walk reads
only shared, read-only data (src/sim/kernels.cu:72-233). A job is therefore split into
contiguous spin ranges, one per rank; every rank computes its rows (sw_sim_spins on its GPU)
and rank 0 gathers them. There is no collective on the data path: the only exchange is the
final gather of the results, which live in host memory, over a gloo group.

The ranges balance the two per-spin costs of the GB300 path rather than the spin count: the
walk (proportional to the time points) and the seeding of spin s (seed + s generator words,
so later spins cost more).
"""
import numpy as np

# GB300 costs per spin-step of the walk + refill and per generator word of the seeding
# (SE workload: 86 ms per 2e9 spin-steps, 120 ms per 5e11 discarded words)
C_WALK_S = 4.3e-11
C_SEED_S = 2.4e-13


def spin_cost(spins, seed, steps_per_spin):
    """Modelled cost of each spin id in `spins`."""
    s = np.asarray(spins, dtype=np.float64)
    return steps_per_spin * C_WALK_S + (float(seed) + s) * C_SEED_S


def balanced_ranges(n_spins, world, seed=0, steps_per_spin=1):
    """Contiguous [lo, hi) per rank covering [0, n_spins), with equal modelled cost."""
    if world < 1:
        raise ValueError("world must be >= 1")
    if n_spins == 0:
        return [(0, 0)] * world
    a = steps_per_spin * C_WALK_S + float(seed) * C_SEED_S          # cost(s) = a + b s
    b = C_SEED_S

    def cum(x):                                                        # cost of spins [0, x)
        return a * x + b * x * (x - 1) / 2.0

    total = cum(n_spins)
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        # solve b/2 x^2 + (a - b/2) x - target = 0 for x
        qa, qb = b / 2.0, a - b / 2.0
        x = (-qb + np.sqrt(qb * qb + 4 * qa * target)) / (2 * qa) if qa > 0 else target / a
        bounds.append(int(min(max(round(x), bounds[-1]), n_spins)))
    bounds.append(n_spins)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def gather_rows(rows, lo, hi, n_spins, group=None):
    """Gathers every rank's rows (a dict of arrays whose first axis is its spins [lo, hi)) on
    rank 0; returns the full arrays there and None elsewhere."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    objs = [None] * world if rank == 0 else None
    dist.gather_object((lo, hi, rows), objs, dst=0, group=group)
    if rank != 0:
        return None
    out = {}
    for lo_r, hi_r, rows_r in objs:
        for k, v in rows_r.items():
            if k not in out:
                out[k] = np.zeros((n_spins,) + v.shape[1:], v.dtype)
            out[k][lo_r:hi_r] = v
    return out


def run_sharded(problem, compute=None, group=None):
    """One job over all ranks of `group` (torch.distributed, initialised by the caller).
    compute(problem, lo, hi) -> dict of row arrays; default: the GPU (sw_sim_spins)."""
    import torch.distributed as dist
    if compute is None:
        from . import _lib
        compute = _lib.run_spins
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    p = problem.params
    steps = p.n_timepoints * (p.n_dummy_scan + 1)
    lo, hi = balanced_ranges(p.n_spins, world, p.seed, steps)[rank]
    rows = compute(problem, lo, hi)
    return gather_rows(rows, lo, hi, p.n_spins, group)
