"""Benchmark of the SpinWalk `sim` hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W]
                    [--workload se|gre|c3|bssfp|serve|dwi|phantom|dense|small]
                    [--impl ours|reference] [--no-legs]

A "step" is one full pass of the hot path over one batch of synthetic input: per-spin generator
seeding (mt19937(seed+spin) + discard), the walk over all time points and the Bloch update for
every spin -- exactly the work of the reference's per-scale loop (src/sim/monte_carlo.cu:310-335).

The default run (`--workload se`) prints ONE line whose headline `value` is the plain kernel on
the spin-echo workload (500^3 spheres, 1e6 spins, 2001 time points), and whose `legs` hold the
other measurements of the metric, each with its own error against FP64:
  gre      plain gradient echo, 200^3 cylinders, 1e5 spins, 401 time points
  batched  64-instance FoV sweep (32 radii x GRE/SE, 1e4..1e6 spins each) in one sw_sim_batch
  tracks   bSSFP, 64 phase cycles x DUMMY_SCAN 200..209 on one walk (sw_sim_tracks)
  served   Poisson trace of 100 requests (GRE/SE/PGSE, 1e4..1e7 spins, three resident phantoms)
           through the serving engine: warm (generator states cached), cold (first pass,
           seeding inside the trace) and the service start-up
The batched and served rates are also given as ratios to the plain headline value.

Metric unit: spin-steps/s (spins x time points x scans per second; for batches, summed over the
instances). `value` is timed with CUDA events with every input already in HBM; `e2e` goes through
the public host-buffer entry point sw_sim (host->device copies of the inputs and device->host
copies of the results inside the timed region). Inputs (packed phantom, generator state) are
larger than L2, so no explicit flush is needed between steps.

--impl reference times the reference algorithm's CPU path (the oracle port of sim::sim, with
std::mt19937) on all host cores on a bounded, stratified sample of the same workload's spin ids.
It builds its inputs with oracle/libsynth.so (the synthetic phantom generator compiled alone)
and the oracle's initial positions, and never loads the CUDA library.
Multi-GPU: spins are independent, so each rank walks its own spin range (weak scaling, no
collective on the data path).
"""
import argparse
import copy
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spin-steps/s/GPU (batched+served vs plain) at ≤1e-5 err vs FP64; p50/p99 latency"
UNIT = "spin-steps/s"

GATHER_BYTES_PER_SPIN_STEP = 32   # one DRAM sector per random voxel lookup (mask + field record)
USEFUL_BYTES_PER_SPIN_STEP = 5    # 1 B mask + 4 B field at the visited voxel
SEED_BYTES_PER_SPIN = 2 * 624 * 4 + 6 * 4   # two mt19937 states + 6 ring/index words written
# DRAM traffic per unit from ncu on the small SE case (profiles/launches_small_se_300cubed_2e5spins.md),
# scaled to a full launch by the units it processes (both grow in proportion)
SEED_DRAM_BYTES_PER_SPIN = 4704.0
MT_BYTES_PER_SPIN_STEP = 3.82 * 8        # MT words drawn per step x (4 B read + 4 B write)
WALK_FP64_OPS_PER_SPIN_STEP = 6          # x, y, z step multiplies and position additions
FP64_PEAK_GFLOPS = 152 * 2 * 2070e6 / 1e9  # 2 FP64 lanes per clock per SM at 2070 MHz
WALK_DRAM_BYTES_PER_SPIN_STEP = 24.5
SEED_LANE_INST_PER_WORD = 7.7            # ncu, k_seed: lane instructions per regenerated MT word
# k_seed_jump: three correlations of 336 (padded) outputs over 32 x 15 groups of 21 steps, one
# ALU lane operation per output word per triple of steps on average (a three-input xor adds two
# windows), per spin
JUMP_XOR_LANE_OPS_PER_SPIN = 3 * 336 * 32 * 15 * 21 / 3
SEED_LIMITER = ("integer instruction issue (ncu: ALU pipe 83 %, issue 74 %, DRAM 2 %): "
                "7.7 lane instructions per MT word, not HBM")
JUMP_LIMITER = ("jump-ahead: integer ALU pipe (ncu: ALU 71 %, issue 59 %, DRAM 0.2 %) on the "
                "xor work of three 312-output correlations per spin, not HBM")
WALK_LIMITER = ("FP64 pipe (ncu: 64 %, 3 position additions + 3 step multiplies per step at 2 "
                "lanes/clock/SM) and the latency of the voxel gather (issue 38 %, long-scoreboard "
                "stalls, DRAM 10 %)")


# ------------------------------------------------------------------------------------------
# Inputs
# ------------------------------------------------------------------------------------------
class Inputs:
    """Where the synthetic inputs come from. The GPU arm uses the library (sw_phantom_*,
    sw_initial_positions); the CPU reference arm the same generator source built alone
    (oracle/libsynth.so) and the oracle's restatement of the reference driver's initial
    positions, so that it never loads the CUDA library. Both give identical arrays."""

    def __init__(self, oracle_side=False):
        self.oracle_side = oracle_side

    def _L(self):
        if not self.oracle_side:
            return None
        from tests import oracle_lib
        return oracle_lib.synth()

    def spheres(self, n, fov, rmin, rmax, vf, seed):
        from spinwalk_gb300 import _lib
        return _lib.phantom_spheres(n, fov, rmin, rmax, vf, seed=seed, L=self._L())

    def cylinders(self, n, fov, r, vf, seed):
        from spinwalk_gb300 import _lib
        return _lib.phantom_cylinders(n, fov, r, vf, seed=seed, L=self._L())

    def positions(self, fov, seed, n):
        if self.oracle_side:
            from tests import oracle_lib
            return oracle_lib.initial_positions(fov, seed, n)
        from spinwalk_gb300 import _lib
        return _lib.initial_positions(fov, seed, n)


def workload(name, rank=0, inputs=None, seed=None):
    from spinwalk_gb300.problem import Problem
    inputs = inputs or Inputs()
    if name == "se":
        n, fov = 500, 500e-6
        mask, field = inputs.spheres(n, fov, 2e-6, 8e-6, 0.05, seed=2)
        n_spins = 1_000_000
        kw = dict(TR_us=40020, TE_us=(40000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 20000), timestep_us=20, pXY=[[1.0, 0.01], [0.01, 1.0]],
                  T2_ms=(40.0, 20.0), T1_ms=(2000.0, 2000.0))
        desc = dict(workload="se_spheres_500cubed_1e6spins_2001tp", phantom="500^3 spheres r2-8um 5%",
                    n_spins=n_spins, time_points=2001, sequence="SE 90/180, TE 40 ms, dt 20 us",
                    permeability=0.01)
    elif name == "gre":
        n, fov = 200, 200e-6
        mask, field = inputs.cylinders(n, fov, 5e-6, 0.03, seed=1)
        n_spins = 100_000
        kw = dict(TR_us=20050, TE_us=(20000,), timestep_us=50)
        desc = dict(workload="gre_cylinders_200cubed_1e5spins_401tp",
                    phantom="200^3 cylinders r5um 3% random orientation", n_spins=n_spins,
                    time_points=401, sequence="GRE 90, TE 20 ms, dt 50 us", permeability=0.0)
    elif name == "bssfp":      # config 4 phantom/sequence; batched by leg_tracks()
        n, fov = 300, 300e-6
        mask, field = inputs.cylinders(n, fov, 5e-6, 0.03, seed=4)
        n_spins = 200_000
        kw = dict(TR_us=5000, TE_us=(2500,), RF_FA=(30.0,), timestep_us=25, n_dummy_scan=209)
        desc = dict(workload="bssfp_cylinders_300cubed_2e5spins_64pc_x_10tr",
                    phantom="300^3 cylinders r5um 3%", n_spins=n_spins, time_points=200,
                    sequence="bSSFP FA 30, TR 5 ms, TE 2.5 ms, dt 25 us, 64 phase cycles "
                             "(5.625 deg steps) x DUMMY_SCAN 200..209")
    elif name in ("dense", "dense_small"):   # many spins per voxel: the Morton re-sort's case
        n, fov = 100, 100e-6
        mask, field = inputs.cylinders(n, fov, 5e-6, 0.03, seed=1)
        n_spins = 2_000_000 if name == "dense" else 500_000
        kw = dict(TR_us=40050, TE_us=(40000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 20000), timestep_us=50)
        desc = dict(workload=f"{name}_se_cylinders_100cubed_{n_spins:.0e}spins_801tp".replace("+0", ""),
                    phantom="100^3 cylinders r5um 3% (the serving trace's smallest phantom)",
                    n_spins=n_spins, spins_per_voxel=n_spins / n ** 3, time_points=801,
                    sequence="SE 90/180, TE 40 ms, dt 50 us", permeability=0.0)
    elif name == "small":      # profiling case: > L2 phantom, few GB on the device
        n, fov = 300, 300e-6
        mask, field = inputs.spheres(n, fov, 2e-6, 8e-6, 0.05, seed=2)
        n_spins = 200_000
        kw = dict(TR_us=4020, TE_us=(4000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 2000), timestep_us=20, pXY=[[1.0, 0.01], [0.01, 1.0]])
        desc = dict(workload="small_se_300cubed_2e5spins_201tp", n_spins=n_spins, time_points=201)
    else:
        raise SystemExit(f"unknown workload {name}")
    if seed is None:
        seed = 10 + 1_000_003 * rank      # each rank: its own disjoint spin population
    xyz0 = inputs.positions([fov] * 3, seed, n_spins)
    pr = Problem(mask, [fov] * 3, field, n_spins=n_spins, seed=seed, XYZ0=xyz0, **kw)
    return pr, desc


def bench_config(args, desc):
    """The `config` object of both arms' lines: the workload and nothing that differs between
    them (how the GPU arm shards is in its own `parallelism` key)."""
    return dict(desc, l2="inputs larger than L2 (packed phantom + generator state)",
                field_records="bfloat16, 4 B per voxel" if args.field_bf16
                else "float32 fieldmap",
                generators="thrust minstd_rand + erfcinv normal (the reference's CUDA build)"
                if args.rng == "minstd" else
                "std::mt19937 + polar normal (the reference's CPU build)")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.dev = device_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx = float(c[2])
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# Error against FP64
# ------------------------------------------------------------------------------------------
def _signal(m, ok):
    """|mean over spins of Mx + iMy| per echo."""
    return np.abs(m[ok, :, 0].mean(0) + 1j * m[ok, :, 1].mean(0))


def fp64_error(pr, prec, rng=0):
    """Error of one run in precision `prec` against the FP64 shadow of the same walk (computed by
    the library alongside): the largest per-spin |M - M_fp64| (|M| <= 1) and the largest
    relative error of the echo signal |mean Mxy| over all echoes."""
    from spinwalk_gb300 import _lib
    r = _lib.run(pr, precision=prec | rng, fp64_shadow=True)
    m, d = r["M1"].astype(np.float64), r["M1_fp64"]
    ok = r["status"] == 0
    if not ok.any():
        return {"max_abs_per_spin": 0.0, "signal_rel": 0.0}
    s32, s64 = _signal(m, ok), _signal(d, ok)
    return {"max_abs_per_spin": float(np.abs(m[ok] - d[ok]).max()),
            "signal_rel": float((np.abs(s32 - s64) / np.maximum(s64, 1e-30)).max())}


def precision_errors(pr, rng=0):
    """fp32 and compensated-FP32 (Kahan) phase sums against FP64, on one problem."""
    from spinwalk_gb300 import abi
    return {name: fp64_error(pr, prec, rng)
            for name, prec in (("fp32", abi.SW_PREC_FP32), ("kahan", abi.SW_PREC_KAHAN))}


def max_errors(problems, rng=0):
    """FP32 and compensated-FP32 (Kahan) errors against FP64 over several problems (the worst of
    each figure)."""
    from spinwalk_gb300 import abi
    out = {}
    for name, prec in (("fp32", abi.SW_PREC_FP32), ("kahan", abi.SW_PREC_KAHAN)):
        errs = [fp64_error(p, prec, rng) for p in problems]
        out[name] = {"max_abs_per_spin": max(e["max_abs_per_spin"] for e in errs),
                     "signal_rel": max(e["signal_rel"] for e in errs)}
    return out


def bf16_field_errors(pr):
    """Error of the bfloat16 fieldmap records (SW_FIELD_BF16) on this workload: M of the FP32
    run with bf16 records against the FP32 run with float records (same walk, same arithmetic)
    and against the FP64 shadow of the float-record run; largest per-spin |dM| and largest
    relative error of the echo signal |mean Mxy|."""
    from spinwalk_gb300 import _lib, abi
    ref = _lib.run(pr, precision=abi.SW_PREC_FP32, fp64_shadow=True)
    got = _lib.run(pr, precision=abi.SW_PREC_FP32 | abi.SW_FIELD_BF16)
    ok = (ref["status"] == 0) & (got["status"] == 0)
    m = got["M1"].astype(np.float64)[ok]

    def sig(a):
        return np.abs(a[:, :, 0].mean(0) + 1j * a[:, :, 1].mean(0))
    out = {}
    for name, r in (("vs_float_field", ref["M1"].astype(np.float64)[ok]),
                    ("vs_fp64", ref["M1_fp64"][ok])):
        out[name] = {"max_abs_per_spin": float(np.abs(m - r).max()),
                     "signal_rel": float((np.abs(sig(m) - sig(r)) / np.maximum(sig(r), 1e-30)).max())}
    out["trajectories_equal"] = bool(np.array_equal(got["XYZ1"], ref["XYZ1"]))
    return out


# ------------------------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference's CPU path)
# ------------------------------------------------------------------------------------------
def cpu_sample_ids(n_spins, n_sample):
    """Stratified sample: evenly spaced spin ids over the whole range (the per-spin discard()
    cost grows with the spin id, so a prefix would under-count it)."""
    return np.unique(np.linspace(0, n_spins - 1, n_sample).round().astype(np.uint32))


def time_cpu(pr, n_sample, threads=0, lowest=False, rng=0):
    """The oracle port on `threads` host threads over n_sample spin ids: stratified over the
    whole range (end to end, the per-spin discard included), or the lowest ids (lowest=True:
    discard(seed + spin) of a few thousand words, i.e. the walk-only rate)."""
    from tests import oracle_lib
    ids = (np.arange(min(n_sample, pr.params.n_spins), dtype=np.uint32) if lowest
           else cpu_sample_ids(pr.params.n_spins, n_sample))
    outs = pr.outputs()
    t = time.perf_counter()
    oracle_lib.run(pr, precision=rng, spin_ids=ids, n_threads=threads, outputs=outs)
    dt = time.perf_counter() - t
    steps = len(ids) * pr.params.n_timepoints * (pr.params.n_dummy_scan + 1)
    return steps / dt, len(ids), dt


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rng_flag(args):
    from spinwalk_gb300 import abi
    return abi.SW_RNG_MINSTD if args.rng == "minstd" else abi.SW_RNG_MT19937


def run_reference(args, world, rank):
    """CPU reference arm: the oracle port on all host cores, rank 0 only. Its inputs come from
    oracle/libsynth.so and the oracle (the CUDA library is never loaded)."""
    if rank != 0:
        return
    pr, desc = workload(args.workload, inputs=Inputs(oracle_side=True), seed=args.seed)
    rng = rng_flag(args)
    cores = os.cpu_count()
    n_sample = args.ref_sample
    for _ in range(args.warmup):
        time_cpu(pr, max(16, n_sample // 8), cores, rng=rng)
    rates, secs = [], []
    for _ in range(args.steps):
        r, n, dt = time_cpu(pr, n_sample, cores, rng=rng)
        rates.append(r)
        secs.append(dt)
    v = float(np.mean(rates))
    sample = (f"{n} stratified spin ids of {pr.params.n_spins} per step, "
              f"{pr.params.n_timepoints} time points each, extrapolated as spin-steps/s")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(secs)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, desc),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def apply_tuning(args, pr=None):
    """Walk tuning for the run: --autotune measures every candidate on `pr` (sw_autotune) and
    installs the fastest; --resort-interval / --walk-block set it directly. Returns what was
    applied (and the measured table)."""
    from spinwalk_gb300 import _lib
    info = {}
    if args.autotune and pr is not None:
        t0 = time.perf_counter()
        best, table = _lib.autotune(pr, apply=True)
        info = {"autotuned": True, "probe_s": time.perf_counter() - t0, "table": table}
    if args.resort_interval is not None or args.walk_block is not None or \
            args.seed_chunks is not None or args.round_streams is not None or \
            args.jump_min_kwords is not None or args.ring_steps is not None or \
            args.walk_blocks_per_sm is not None:
        cur = _lib.get_tuning()
        _lib.set_tuning(cur["resort_interval"] if args.resort_interval is None else args.resort_interval,
                        cur["walk_block"] if args.walk_block is None else args.walk_block,
                        cur["seed_chunks"] if args.seed_chunks is None else args.seed_chunks,
                        cur["round_streams"] if args.round_streams is None else args.round_streams,
                        cur["jump_min_kwords"] if args.jump_min_kwords is None else args.jump_min_kwords,
                        cur["ring_steps"] if args.ring_steps is None else args.ring_steps,
                        cur["walk_blocks_per_sm"] if args.walk_blocks_per_sm is None
                        else args.walk_blocks_per_sm)
    info["applied"] = _lib.get_tuning()
    return info


# ------------------------------------------------------------------------------------------
# Plain kernel (the headline) and the plain GRE leg
# ------------------------------------------------------------------------------------------
def device_buffers(pr, dev):
    import torch
    p = pr.params
    n, nte = p.n_spins, pr.n_te
    return dict(field=torch.from_numpy(pr.field).to(dev), mask=torch.from_numpy(pr.mask).to(dev),
                M0=torch.from_numpy(pr.M0).to(dev), XYZ0=torch.from_numpy(pr.XYZ0).to(dev),
                M1=torch.zeros((n, nte, 3), dtype=torch.float32, device=dev),
                XYZ1=torch.zeros((n, pr.traj_len, 3), dtype=torch.float32, device=dev),
                T=torch.zeros((n, nte), dtype=torch.uint8, device=dev),
                status=torch.zeros(n, dtype=torch.int32, device=dev))


def time_plain(pr, prec, steps, warmup, world, local, clocks=True):
    """The plain kernel on device buffers: `steps` passes timed with CUDA events on the
    launching stream (barrier + synchronize on both sides), then the same pass end to end
    through sw_sim with host buffers. Returns a dict of the figures."""
    import torch
    from spinwalk_gb300 import _lib
    dev = torch.device("cuda", local)
    d = device_buffers(pr, dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        _lib.run_device(pr, d["field"].data_ptr(), d["mask"].data_ptr(), d["M0"].data_ptr(),
                        d["XYZ0"].data_ptr(), d["M1"].data_ptr(), d["XYZ1"].data_ptr(),
                        d["T"].data_ptr(), d["status"].data_ptr(), precision=prec,
                        stream=stream.cuda_stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    timings = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local) if clocks else None
    if sampler:
        sampler.__enter__()
    barrier(world)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        step()
        timings.append(_lib.last_timing())
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    if sampler:
        sampler.__exit__()
    ms = max_over_ranks(world, ev0.elapsed_time(ev1))
    st = d["status"].cpu().numpy()
    del d

    # end to end through the host-buffer entry point, inputs in pinned host memory
    n, nte = pr.params.n_spins, pr.n_te
    h2d = pr.mask.nbytes + (pr.field.nbytes if pr.field is not None else 0) + pr.M0.nbytes + pr.XYZ0.nbytes
    d2h = n * nte * 12 + n * nte + n * pr.traj_len * 12 + n * 4
    pinned = []

    def pin(a):
        if a is None:
            return None
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        pinned.append(t)
        return t.numpy()

    hp = copy.copy(pr)
    hp.mask, hp.field, hp.M0, hp.XYZ0 = pin(pr.mask), pin(pr.field), pin(pr.M0), pin(pr.XYZ0)
    _lib.run(hp, precision=prec)                     # warm (host staging)
    e2e_times = []
    for _ in range(max(1, steps)):
        barrier(world)
        t = time.perf_counter()
        out = _lib.run(hp, precision=prec)
        e2e_times.append(time.perf_counter() - t)
    e2e_s = max_over_ranks(world, float(np.mean(e2e_times)))
    assert np.array_equal(out["status"], st)
    return dict(ms=ms, timings=timings, status=st, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                clocks=sampler.summary() if sampler else None)


def leg_gre(args, local=0):
    """Config 1, plain: GRE on 200^3 cylinders, 1e5 spins, 401 time points."""
    from spinwalk_gb300 import abi
    pr, desc = workload("gre")
    steps = max(3, min(args.steps, 10))
    r = time_plain(pr, abi.SW_PREC_FP32 | rng_flag(args), steps, max(3, args.warmup), 1, local,
                   clocks=False)
    ss = pr.spin_steps()
    return {"workload": desc["workload"], "value": ss * steps / (r["ms"] * 1e-3), "unit": UNIT,
            "ms_per_step": r["ms"] / steps, "steps": steps,
            "e2e": {"value": ss / r["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                    "d2h_bytes_per_step": int(r["d2h"])},
            "gpu_launches": int(sum(t["n_launches"] for t in r["timings"])),
            "error_vs_fp64": precision_errors(pr, rng_flag(args))}


# ------------------------------------------------------------------------------------------
# Batched: the config-3 FoV sweep in one sw_sim_batch
# ------------------------------------------------------------------------------------------
def c3_instances(rank=0, max_spins=None):
    """Config 3: the config-1 phantom (200^3 random-orientation cylinders, r 5 um, 3 %), 32 FoV
    scales giving vessel radii 1-100 um (log-spaced; scale = r / 5 um, WHAT_TO_SCALE = 0) x
    {GRE, SE}; spins per instance log-uniform in [1e4, 1e6] (seed 3); TE = 5, 10, ..., 40 ms,
    dt 50 us, SE refocusing at 20 ms. One simulation seed for all (as one config's scales)."""
    from spinwalk_gb300 import _lib
    from spinwalk_gb300.problem import Problem
    n, fov = 200, 200e-6
    mask, field = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=1)
    rng = np.random.default_rng(3)
    radii = np.logspace(0, 2, 32)
    spins = np.round(10 ** rng.uniform(4, 6, 64)).astype(int)
    if max_spins:                      # a smaller case of the same sweep (profiling)
        spins = np.minimum(spins, max_spins)
    te = tuple(range(5000, 40001, 5000))
    seqs = {"gre": dict(TR_us=40050, TE_us=te, timestep_us=50),
            "se": dict(TR_us=40050, TE_us=te, RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                       RF_us=(0, 20000), timestep_us=50)}
    seed = 10 + 1_000_003 * rank
    xyz0 = _lib.initial_positions([fov] * 3, seed, int(spins.max()))
    probs = []
    for i, r in enumerate(radii):
        s32 = np.float32(r / 5.0)
        f = float(s32 * np.float32(fov))
        for j, name in enumerate(("gre", "se")):
            ns = int(spins[2 * i + j])
            probs.append(Problem(mask, [f] * 3, field, n_spins=ns, seed=seed,
                                 XYZ0=(xyz0[:ns] * s32).astype(np.float32), **seqs[name]))
    desc = dict(workload="c3_fov_sweep_32radii_x_gre_se_200cubed",
                phantom="200^3 cylinders r5um 3% random orientation",
                instances=len(probs), spins_per_instance="log-uniform [1e4, 1e6], seed 3",
                sequence="GRE / SE (refocus 20 ms), TE 5..40 ms, dt 50 us, 801 time points",
                radii_um="1..100 log-spaced (FoV scale r / 5 um)")
    return probs, desc


def leg_batched(args, rank=0, world=1):
    """Config 3 batched (sw_sim_batch: phantom packed once, pooled generator streams seeded once
    for all 64 instances, every round one refill of the streams and one fused uniform-refill and
    walk launch over all instances, replayed as a CUDA graph) against the same instances run one
    sw_sim each. `value` is the whole call as the library times it (from its entry to its
    return: phantom upload, seeding, rounds and the copies to and from the host staging);
    `e2e` the host time around it from Python (output arrays allocated once, outside)."""
    from spinwalk_gb300 import _lib
    probs, desc = c3_instances(rank, args.max_spins)
    tuning = apply_tuning(args, max(probs, key=lambda q: q.params.n_spins))
    steps = sum(p.spin_steps() for p in probs)
    reps = max(3, min(args.steps, 5))
    for _ in range(max(3, min(args.warmup, 3))):
        outs = _lib.run_batch(probs)
    dev_ms, wall, launches, seed_ms, round_ms = [], [], [], [], []
    for _ in range(reps):
        t = time.perf_counter()
        _lib.run_batch(probs, outs=outs)          # the caller's output arrays, reused
        wall.append(time.perf_counter() - t)
        lt = _lib.last_timing()
        dev_ms.append(lt["total_ms"])
        launches.append(lt["n_launches"])
        seed_ms.append(lt["seed_ms"])
        round_ms.append(lt["walk_ms"])
    plain_ms, plain_wall = 0.0, 0.0
    for p in probs:
        t = time.perf_counter()
        _lib.run(p)
        plain_wall += time.perf_counter() - t
        plain_ms += _lib.last_timing()["total_ms"]
    value = world * steps / (np.mean(dev_ms) * 1e-3)
    plain = steps / (plain_ms * 1e-3)
    # error against FP64 on the smallest, a middle and the largest radius, GRE and SE, and the
    # largest instance (a batch instance is bit-identical to its own sw_sim run)
    err_idx = sorted({0, 1, 30, 31, 62, 63} | {int(np.argmax([p.params.n_spins for p in probs]))})
    return {"workload": desc["workload"], "value": value, "unit": UNIT,
            "ms_per_step": float(np.mean(dev_ms)), "steps": reps,
            "stage_ms": {"seeding": float(np.mean(seed_ms)),
                         "rounds": float(np.mean(round_ms)),
                         "rest": float(np.mean(dev_ms) - np.mean(seed_ms) - np.mean(round_ms)),
                         "note": "CUDA events on the batch's main stream; rest = the call's "
                                 "wall time minus both (the phantom upload and the input "
                                 "staging overlap the seeding; then the output copies to the "
                                 "caller's buffers)"},
            "rounds_instance_spin_steps_per_s": steps / (np.mean(round_ms) * 1e-3),
            "config": dict(desc, instance_spin_steps=int(steps)),
            "plain_one_call_per_instance": {"value": plain, "ms": plain_ms,
                                            "e2e_value": steps / plain_wall},
            "batched_over_one_call_per_instance": value / plain,
            "e2e": {"value": world * steps / float(np.mean(wall)), "unit": UNIT,
                    "note": "sw_sim_batch with host buffers (the caller's arrays, allocated once)"},
            "gpu_launches": int(sum(launches)),
            "error_vs_fp64": dict(max_errors([probs[i] for i in err_idx], rng_flag(args)),
                                  instances=err_idx, timed_precision="fp32"),
            "tuning": tuning}


# ------------------------------------------------------------------------------------------
# Tracks: config 4 (bSSFP phase cycles x dummy scans on one walk)
# ------------------------------------------------------------------------------------------
def bssfp_cycle_errors(pr, tracks):
    """Error of the float steady-state recurrence against its FP64 shadow, per phase cycle: the
    given tracks (one per cycle) run once with plain float and once with compensated (Kahan)
    phase sums, each beside the FP64 shadow of the same walk (sw_sim_tracks M1_fp64). Per cycle:
    the relative error of the signal (complex mean of Mx + iMy over spins, first echo) and the
    largest per-spin |M - M_fp64|."""
    from spinwalk_gb300 import _lib, abi
    res = {"cycles": len(tracks), "n_dummy_scan": tracks[0]["n_dummy_scan"],
           "definition": "signal: |S - S64| / |S64|, S = mean over spins of Mx + iMy at the "
                         "first echo; spin: max over spins of max |M - M64| (M0 = 1)"}
    for name, prec in (("fp32", abi.SW_PREC_FP32), ("kahan", abi.SW_PREC_KAHAN)):
        outs = _lib.run_tracks(pr, tracks, precision=prec, fp64=True)
        sig, spin = [], []
        for o in outs:
            ok = o["status"] == 0
            m, md = o["M1"][ok, 0].astype(np.float64), o["M1_fp64"][ok, 0]
            s32 = np.mean(m[:, 0] + 1j * m[:, 1])
            s64 = np.mean(md[:, 0] + 1j * md[:, 1])
            sig.append(abs(s32 - s64) / max(abs(s64), 1e-300))
            spin.append(float(np.max(np.abs(m - md))) if ok.any() else 0.0)
        res[name] = {"signal_rel_max": float(max(sig)), "signal_rel_median": float(np.median(sig)),
                     "spin_abs_max": float(max(spin)),
                     "signal_rel_per_cycle": [float(f"{v:.3g}") for v in sig]}
    return res


def leg_tracks(args, rank=0, world=1):
    """Config 4 batched: 64 phase-cycling scales x 10 sampled TRs (DUMMY_SCAN 200..209) = 640
    reference instances on ONE walk (sw_sim_tracks). Work is counted per instance, as the
    reference executes it: sum over instances of spins x time points x (DUMMY_SCAN + 1)."""
    from spinwalk_gb300 import _lib
    pr, desc = workload("bssfp", rank)
    p = pr.params
    tracks = [dict(linear_phase_cycling=5.625 * i, n_dummy_scan=d)
              for i in range(64) for d in range(200, 210)]
    inst_steps = sum(p.n_spins * p.n_timepoints * (t["n_dummy_scan"] + 1) for t in tracks)
    walk_steps = p.n_spins * p.n_timepoints * 210
    reps = max(2, min(args.steps, 3))
    for _ in range(max(3, min(args.warmup, 3))):
        _lib.run_tracks(pr, tracks)
    times, dev_ms, launches = [], [], []
    for _ in range(reps):
        t = time.perf_counter()
        _lib.run_tracks(pr, tracks)
        times.append(time.perf_counter() - t)
        dev_ms.append(_lib.last_timing()["total_ms"])
        launches.append(_lib.last_timing()["n_launches"])
    # the plain kernel on one instance of the same config, for the batched/plain ratio
    one = dict(tracks[-1])
    pr.params.linear_phase_cycling = one["linear_phase_cycling"]
    pr.params.n_dummy_scan = one["n_dummy_scan"]
    _lib.run(pr)
    t = time.perf_counter()
    _lib.run(pr)
    plain_s = time.perf_counter() - t
    plain_dev = _lib.last_timing()["total_ms"] * 1e-3
    plain_rate = p.n_spins * p.n_timepoints * (one["n_dummy_scan"] + 1) / plain_dev
    value = world * inst_steps / (np.mean(dev_ms) * 1e-3)
    pr.params.linear_phase_cycling = 0.0
    pr.params.n_dummy_scan = 0
    rec_err = bssfp_cycle_errors(pr, [t for t in tracks if t["n_dummy_scan"] == 209])
    return {"workload": desc["workload"], "value": value, "unit": UNIT,
            "ms_per_step": float(np.mean(dev_ms)), "steps": reps,
            "config": dict(desc, instances=len(tracks), instance_spin_steps=int(inst_steps),
                           distinct_walk_spin_steps=int(walk_steps)),
            "distinct_walk_steps_per_s": walk_steps / (np.mean(dev_ms) * 1e-3),
            "plain_kernel_one_instance": {"value": plain_rate, "e2e_s": plain_s},
            "tracks_over_one_instance": value / plain_rate,
            "e2e": {"value": inst_steps / float(np.mean(times)), "unit": UNIT,
                    "note": "includes the per-track host output copies"},
            "gpu_launches": int(sum(launches)),
            "error_vs_fp64": {"recurrence": rec_err}}


# ------------------------------------------------------------------------------------------
# Served: the config-5 trace through the serving engine
# ------------------------------------------------------------------------------------------
def serve_requests(n_req, rng_seed=5, rank=0):
    """Config 5 trace: Poisson arrivals (mean 20 / s), requests on resident phantoms, spins
    log-uniform in [1e4, 1e7], a mix of GRE, SE and PGSE (b = 1000 s/mm^2, delta 10 ms, Delta
    20 ms, lobes from 2 ms, G = 91.6 mT/m along x, y or z; TE 34 ms; dt 50 us). One simulation
    seed for the service."""
    from spinwalk_gb300 import _lib
    from spinwalk_gb300.problem import Problem
    rng = np.random.default_rng(rng_seed)
    phantoms = []
    for n, kind, s in ((100, "cyl", 1), (200, "sph", 2), (800, "ref_cyl", 3)):
        fov = n * 1e-6
        if kind == "cyl":
            m, f = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=s)
        elif kind == "sph":
            m, f = _lib.phantom_spheres(n, fov, 2e-6, 8e-6, 0.05, seed=s)
        else:      # the reference's cylinder phantom, generated on the GPU
            m, f, _ = _lib.phantom_cylinder(float(n), n, 0.11e-6 * 0.4, 0.75, 5.0, 3.0, 90.0, s)
        phantoms.append((m, f, fov))
    seed = 10 + 1_000_003 * rank
    gre = dict(TR_us=20050, TE_us=(20000,), timestep_us=50)
    se = dict(TR_us=40050, TE_us=(40000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
              RF_us=(0, 20000), timestep_us=50)
    lobe = lambda t0: list(range(t0, t0 + 10000, 50))                       # noqa: E731
    g_t = lobe(2000) + [12000] + lobe(22000) + [32000]
    pgse = {}
    for d, axis in enumerate("xyz"):
        g = np.zeros((len(g_t), 3), np.float32)
        for i, t in enumerate(g_t):
            if t not in (12000, 32000):
                g[i, d] = 91.6
        pgse[axis] = dict(TR_us=34050, TE_us=(34000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                          RF_us=(0, 17000), timestep_us=50, gradient_us=tuple(g_t),
                          gradient_xyz=g)
    spins = np.round(10 ** rng.uniform(4, 7, n_req)).astype(int)
    which = rng.integers(0, len(phantoms), n_req)
    kinds = rng.integers(0, 5, n_req)
    arrivals = np.cumsum(rng.exponential(1 / 20.0, n_req))
    xyz0 = {}
    reqs = []
    for i in range(n_req):
        m, f, fov = phantoms[which[i]]
        if fov not in xyz0:
            xyz0[fov] = _lib.initial_positions([fov] * 3, seed, int(spins.max()))
        kw = [gre, se, pgse["x"], pgse["y"], pgse["z"]][kinds[i]]
        reqs.append(Problem(m, [fov] * 3, f, n_spins=int(spins[i]), seed=seed,
                            XYZ0=xyz0[fov][:spins[i]], **kw))
    desc = dict(workload="c5_serving_poisson20_%dreq" % n_req,
                phantoms="100^3 cylinders, 200^3 spheres, 800^3 reference cylinders (resident)",
                spins_per_request="log-uniform [1e4, 1e7], seed 5",
                sequences="GRE 20 ms / SE 40 ms / PGSE b=1000 x,y,z", arrivals="Poisson, 20 / s")
    return reqs, phantoms, arrivals, kinds, desc


def distinct_seed_requests(reqs, rng_seed=6):
    """Copies of `reqs` with a random 32-bit seed each (seeded draw) and the start positions the
    reference driver derives from that seed (monte_carlo.cu:141-151)."""
    import copy

    from spinwalk_gb300 import _lib, abi
    rng = np.random.default_rng(rng_seed)
    out = []
    for pr in reqs:
        q = copy.copy(pr)
        q.params = abi.SwParams.from_buffer_copy(pr.params)
        q.params.seed = int(rng.integers(1, 2 ** 32))
        q.XYZ0 = _lib.initial_positions([q.params.fov[i] for i in range(3)], q.params.seed,
                                        q.params.n_spins)
        out.append(q)
    return out


def play_trace(eng, reqs, arrivals, submit):
    """Submits the requests at their arrival times (real time) and polls until every result is
    in the caller's buffers. Returns (makespan s, latencies s, engine stats delta)."""
    n_req = len(reqs)
    st0 = eng.stats()
    lat = []
    t_start = time.perf_counter()
    i = 0
    while i < n_req or len(lat) < n_req:
        now = time.perf_counter() - t_start
        while i < n_req and arrivals[i] <= now:
            submit(reqs[i])
            i += 1
        for jid, rc, lt in eng.poll(wait=0):
            assert rc == 0
            lat.append(lt)
        time.sleep(0.0005)
    makespan = time.perf_counter() - t_start
    st1 = eng.stats()
    return makespan, np.array(lat), {k: int(st1[k] - st0[k]) for k in st1}


def _lat(lat):
    return {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
            "max": float(lat.max())}


def leg_served(args, rank=0, world=1):
    """Config 5: the requests are submitted to one engine at their arrival times; latency =
    submit -> results in the caller's buffers (queueing included). Two passes of the same trace
    on one engine: `cold` is the first (generator states computed as requests need them, inside
    the trace), `value` the second (warm: every request's states come from the cache)."""
    from spinwalk_gb300 import _lib
    n_req = args.requests
    reqs, phantoms, arrivals, kinds, desc = serve_requests(n_req, rank=rank)
    tuning = apply_tuning(args, max(reqs, key=lambda q: q.params.n_spins))
    eng = _lib.Engine(n_slots=8, slot_spins=1 << 20)
    pids = {}
    t0 = time.perf_counter()
    for pr in reqs:
        key = pr.mask.shape
        if key not in pids:
            pids[key] = eng.add_phantom(pr, bf16=args.field_bf16)
    phantom_s = time.perf_counter() - t0

    def submit(pr):
        if args.signal:
            return eng.submit_signal(pr, pids[pr.mask.shape])
        return eng.submit(pr, pids[pr.mask.shape])
    steps = sum(p.spin_steps() for p in reqs)
    cold_s, cold_lat, cold_st = play_trace(eng, reqs, arrivals, submit)
    with ClockSampler(0) as clk:
        warm_s, warm_lat, warm_st = play_trace(eng, reqs, arrivals, submit)
    clocks = clk.summary()
    # capacity: the same requests all submitted at once (the 20 / s trace offers less work per
    # second than the engine can do, so its rate is bounded by the arrivals)
    sat_s, sat_lat, sat_st = play_trace(eng, reqs, np.zeros(n_req), submit)
    # distinct seeds: the first requests of the trace, each with its own random 32-bit seed (what
    # SEED = 0 draws, simulation_parameters.cuh:233-234) and its own start positions, so no
    # request can use another's generator states
    dreqs = distinct_seed_requests(reqs[:args.distinct_requests])
    dsteps = sum(p.spin_steps() for p in dreqs)
    dist_s, dist_lat, dist_st = play_trace(eng, dreqs, arrivals[:len(dreqs)], submit)
    eng.close()
    # error against FP64 on the smallest request of each kind (a served request is
    # bit-identical to its own sw_sim run)
    sample = []
    for k in range(5):
        idx = [i for i in range(n_req) if kinds[i] == k]
        if idx:
            sample.append(min(idx, key=lambda i: reqs[i].params.n_spins))
    value = world * steps / warm_s
    return {"workload": desc["workload"], "value": value, "unit": UNIT,
            "ms_per_step": warm_s * 1e3, "steps": 1,
            "config": dict(desc, requests=n_req, spin_steps=int(steps),
                           outputs="per-(echo, substrate) signal sums (signal mode)" if args.signal
                           else "per-spin M1, T, XYZ1, status",
                           field_records="bfloat16, 4 B per voxel" if args.field_bf16
                           else "float32, 8 B per voxel"),
            "latency_s": _lat(warm_lat),
            "cold": {"value": world * steps / cold_s, "makespan_s": cold_s,
                     "latency_s": _lat(cold_lat), "seedings": cold_st["seedings"],
                     "note": "first pass of the trace on a new engine: every generator state "
                             "is computed inside the trace, when a request first needs it"},
            "saturated": {"value": world * steps / sat_s, "makespan_s": sat_s,
                          "latency_s": _lat(sat_lat),
                          "note": "the same %d requests submitted at once: the engine's "
                                  "capacity on this mix (latency is queueing)" % n_req},
            "distinct_seeds": {"value": world * dsteps / dist_s, "makespan_s": dist_s,
                               "requests": len(dreqs), "spin_steps": int(dsteps),
                               "spins": int(sum(p.params.n_spins for p in dreqs)),
                               "latency_s": _lat(dist_lat), "seedings": dist_st["seedings"],
                               "note": "the first requests of the trace at their arrival times, "
                                       "each with its own random 32-bit seed and start "
                                       "positions: every spin is seeded inside the trace (by "
                                       "jump-ahead, the discard counts being ~1e9)"},
            "startup": {"phantom_upload_s": phantom_s,
                        "note": "phantoms packed and made resident before the first request"},
            "offered_spin_steps_per_s": steps / float(arrivals[-1]),
            "e2e": {"value": value, "unit": UNIT,
                    "note": "host buffers in and out through the engine, arrivals in real time"},
            "gpu_launches": int(warm_st["launches"]), "walk_rounds": int(warm_st["rounds"]),
            "seedings_warm": int(warm_st["seedings"]),
            "error_vs_fp64": dict(max_errors([reqs[i] for i in sample], rng_flag(args)),
                                  requests=sample, timed_precision="fp32"),
            "tuning": tuning, "clocks": clocks}


# ------------------------------------------------------------------------------------------
# The default line
# ------------------------------------------------------------------------------------------
def run_ours(args, world, rank, local):
    import torch
    from spinwalk_gb300 import _lib, abi

    torch.cuda.set_device(local)
    pr, desc = workload(args.workload, rank, seed=args.seed)
    tuning = apply_tuning(args, pr)
    p = pr.params
    n = p.n_spins
    rng = rng_flag(args)
    prec = abi.SW_PREC_FP32 | (abi.SW_FIELD_BF16 if args.field_bf16 else 0) | rng
    spin_steps = pr.spin_steps()
    r = time_plain(pr, prec, args.steps, args.warmup, world, local)
    ms, timings, st, clocks = r["ms"], r["timings"], r["status"], r["clocks"]
    value = world * spin_steps * args.steps / (ms * 1e-3)
    e2e = world * spin_steps / r["e2e_s"]

    if rank != 0:
        return
    walk_ms = sum(t["walk_ms"] for t in timings)
    refill_ms = sum(t["refill_ms"] for t in timings)
    seed_ms = sum(t["seed_ms"] for t in timings)
    n_walk = sum(t["n_chunks"] for t in timings)
    launches = sum(t["n_launches"] for t in timings)
    parts = {"walk": walk_ms, "refill": refill_ms, "seed+init+pack": seed_ms}
    dominant = max(parts, key=parts.get)
    peak, peak_kind = measured_peaks()
    n_chunks = n_walk / args.steps
    # k_seed (seed+init+pack stage): algorithmic bytes = the generator state it must write
    seed_launch_s = seed_ms / args.steps * 1e-3
    seed_roof = {"bound": "hbm", "kernel": "k_seed", "unit_of_work": "spin",
                 "algorithmic_bytes_per_unit": SEED_BYTES_PER_SPIN,
                 "achieved": n * SEED_BYTES_PER_SPIN / seed_launch_s / 1e9, "peak": peak,
                 "unit": "GB/s", "traffic": SEED_DRAM_BYTES_PER_SPIN * n,
                 "peak_source": peak_kind, "limiter": SEED_LIMITER}
    # k_walk: one 32 B DRAM sector per spin-step (random voxel gather)
    walk_launch_s = walk_ms / n_walk * 1e-3
    walk_units = spin_steps / n_chunks
    walk_roof = {"bound": "hbm", "kernel": "k_walk", "unit_of_work": "spin-step",
                 "algorithmic_bytes_per_unit": GATHER_BYTES_PER_SPIN_STEP,
                 "achieved": walk_units * GATHER_BYTES_PER_SPIN_STEP / walk_launch_s / 1e9,
                 "peak": peak, "unit": "GB/s",
                 "traffic": WALK_DRAM_BYTES_PER_SPIN_STEP * walk_units,
                 "peak_source": peak_kind, "limiter": WALK_LIMITER}
    for rf in (seed_roof, walk_roof):
        rf["frac"] = rf["achieved"] / peak
    # the seeding's own ceiling is instruction issue: the words the discards regenerate (624 per
    # regeneration, mt_discard_twists), at the measured instructions per word, against 4 warp
    # instructions per SM clock; spins at or above the jump threshold are seeded by k_seed_jump
    # instead, whose ceiling is the integer ALU pipe (16 lanes per clock per SM quarter) on its
    # xor work. frac = the time both ideals would take / the stage's time.
    from spinwalk_gb300 import abi
    kw = tuning["applied"]["jump_min_kwords"] or abi.JUMP_MIN_KWORDS_DEFAULT
    z = int(p.seed) + np.arange(n, dtype=np.int64)
    jumped = z >= kw * 1024
    zd = z[~jumped]
    regen_words = float(624 * np.where(zd > 0, 1 + (zd - 1) // 624, 0).sum())
    n_jump = int(jumped.sum())
    sm_hz = (clocks.get("sm_mhz") or 2070.0) * 1e6 if clocks else 2070e6
    issue_peak = 152 * 4 * sm_hz
    alu_peak = 152 * 64 * sm_hz
    t_ideal = (regen_words * SEED_LANE_INST_PER_WORD / 32 / issue_peak +
               n_jump * JUMP_XOR_LANE_OPS_PER_SPIN / alu_peak)
    seed_roof["issue_roofline"] = {
        "achieved_warp_inst_per_s": regen_words * SEED_LANE_INST_PER_WORD / 32 / seed_launch_s,
        "peak": issue_peak, "frac": t_ideal / seed_launch_s, "regenerated_words": regen_words,
        "jump_spins": n_jump, "jump_xor_lane_ops_per_spin": JUMP_XOR_LANE_OPS_PER_SPIN,
        "alu_peak_lane_ops_per_s": alu_peak,
        "note": "discarded words x 7.7 lane instructions (ncu) / 32 per warp instruction against "
                "4 warp instructions per SM clock, plus jumped spins' xor lane operations against "
                "64 ALU lanes per SM clock, at the sampled SM clock; frac = ideal time / stage time"}
    if n_jump:
        seed_roof["kernel"] = "k_seed + k_seed_jump" if regen_words else "k_seed_jump"
        seed_roof["limiter"] = (("discards: " + SEED_LIMITER + "; ") if regen_words else "") + \
            JUMP_LIMITER
    if rng != abi.SW_RNG_MT19937:          # minstd: O(log) seeding per spin, no such ceiling
        seed_roof.pop("issue_roofline")
        seed_roof["kernel"] = "k_seed_minstd"
    roof = {"seed+init+pack": seed_roof, "walk": walk_roof}.get(dominant, walk_roof)
    # walk-only rate: the call's wall time minus its seeding stage (the kernel times of the two
    # halves of the rounds overlap, so their sum would overstate it)
    walk_refill_s = ms / args.steps * 1e-3 - seed_ms / args.steps * 1e-3
    overlapped = tuning["applied"]["seed_chunks"] > 1     # the seeding runs beside the walk
    secondary = {
        "walk_only_spin_steps_per_s": None if overlapped else spin_steps / walk_refill_s,
        "refill_mt_state_gbs": spin_steps * MT_BYTES_PER_SPIN_STEP / (refill_ms / args.steps * 1e-3) / 1e9,
        "walk_fp64_gflops": spin_steps * WALK_FP64_OPS_PER_SPIN_STEP / (walk_ms / args.steps * 1e-3) / 1e9,
        "fp64_peak_gflops": FP64_PEAK_GFLOPS,
        "useful_gather_gbs": spin_steps * USEFUL_BYTES_PER_SPIN_STEP / (walk_ms / args.steps * 1e-3) / 1e9,
        "note": "walk-only = call time minus the seeding stage; the refill and walk kernel times "
                "of the two halves of the rounds overlap; ncu: k_walk L2 hit rate and FP64 pipe "
                "in profiles/",
    }
    errors = precision_errors(pr, rng) if args.workload in ("se", "small") else None
    bf16_err = bf16_field_errors(pr) if args.field_bf16 else None
    cpu = None
    if args.cpu_sample > 0:
        rate, ns, dt = time_cpu(pr, args.cpu_sample, os.cpu_count(), rng=rng)
        wrate, wns, wdt = time_cpu(pr, max(1, args.cpu_sample // 16), os.cpu_count(),
                                   lowest=True, rng=rng)
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{ns} stratified spin ids of {n} ({pr.params.n_timepoints} time "
                         f"points each, {dt:.1f} s wall on {os.cpu_count()} threads)",
               "walk_only": {"value": wrate, "unit": UNIT,
                             "sample": f"spin ids 0..{wns - 1} (discard of at most "
                                       f"{int(pr.params.seed) + wns} words), {wdt:.1f} s wall"}}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded phantom generator, reference-driver initial positions)",
        "config": bench_config(args, desc),
        "value_is": "the plain kernel (one sw_sim_device pass: seeding, walk and Bloch update of "
                    "every spin) on the spin-echo workload; legs.batched and legs.served are "
                    "the batched and served rates",
        "parallelism": f"spin-range shards x{world}",
        "kernel_ms_per_step": {k: v / args.steps for k, v in parts.items()},
        "kernel_ms_note": "sums of launch durations; the refill/walk rounds run as two halves on "
                          "two streams whose kernels overlap, so walk + refill exceed their wall "
                          "time",
        "roofline": dict(roof, dominant_stage=dominant),
        "roofline_walk": walk_roof,
        "secondary_ceilings": secondary,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                "d2h_bytes_per_step": int(r["d2h"])},
        "gpu_launches": int(launches),
        "tuning": tuning,
        "error_vs_fp64": errors,
        "field_bf16": bf16_err,
        "clocks": clocks,
        "status_counts": {str(k): int(v) for k, v in zip(*np.unique(st, return_counts=True))},
    }
    if args.workload == "se" and not args.no_legs and world == 1:
        legs = {}
        for name, fn in (("gre", leg_gre), ("batched", leg_batched), ("tracks", leg_tracks),
                         ("served", leg_served)):
            t = time.perf_counter()
            legs[name] = fn(args) if name != "gre" else fn(args, local)
            legs[name]["leg_wall_s"] = time.perf_counter() - t
        line["legs"] = legs
        line["batched_over_plain"] = legs["batched"]["value"] / value
        line["served_over_plain"] = legs["served"]["value"] / value
        line["served_cold_over_plain"] = legs["served"]["cold"]["value"] / value
        line["served_capacity_over_plain"] = legs["served"]["saturated"]["value"] / value
        line["tracks_over_plain"] = legs["tracks"]["value"] / value
        line["ratios_note"] = ("leg value / headline value (plain kernel on the spin-echo "
                               "workload); each leg also carries its ratio to the plain kernel "
                               "on its own instances")
    print(json.dumps(line), flush=True)


def print_leg(args, world, rank, leg):
    """One line for a leg run on its own (--workload c3 / bssfp / serve)."""
    if rank != 0:
        return
    line = {"metric": METRIC, "value": leg["value"], "unit": UNIT, "n_gpus": world,
            "steps": leg.get("steps", args.steps), "warmup": args.warmup,
            "ms_per_step": leg.get("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic"}
    line.update({k: v for k, v in leg.items() if k not in line})
    print(json.dumps(line), flush=True)


def run_dwi(args, world, rank):
    """DWI b-value sweep (the reference's gradient scale loop, WHAT_TO_SCALE = 1): PGSE along x
    (b = 1000 s/mm^2 at scale 1, delta 10 ms, Delta 20 ms) on the 200^3 cylinder phantom of
    config 1, 1e6 spins, 8 gradient scales 0 .. 1.4 (b 0 .. 1960 s/mm^2). One walk with a phase
    per scale (sw_sim_tracks) against one walk per scale with one seeding (sw_sim_batch); the
    work is counted per instance."""
    import torch  # noqa: F401
    from spinwalk_gb300 import _lib
    from spinwalk_gb300.problem import Problem
    n, fov = 200, 200e-6
    mask, field = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=1)
    lobe = lambda t0: list(range(t0, t0 + 10000, 50))                       # noqa: E731
    g_t = lobe(2000) + [12000] + lobe(22000) + [32000]
    g = np.zeros((len(g_t), 3), np.float32)
    for i, t in enumerate(g_t):
        if t not in (12000, 32000):
            g[i, 0] = 91.6
    kw = dict(TR_us=34050, TE_us=(34000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
              RF_us=(0, 17000), timestep_us=50, gradient_us=tuple(g_t), gradient_xyz=g)
    n_spins = 1_000_000
    pr = Problem(mask, [fov] * 3, field, n_spins=n_spins, seed=10 + 1_000_003 * rank, **kw)
    scales = [0.2 * i for i in range(8)]
    tracks = [dict(gradient_scale=sc, n_dummy_scan=0) for sc in scales]

    def scaled(sc):
        return Problem(mask, [fov] * 3, field, n_spins=n_spins, seed=10 + 1_000_003 * rank,
                       **dict(kw, gradient_xyz=g * np.float32(sc)))
    insts = [scaled(sc) for sc in scales]
    steps = len(scales) * pr.spin_steps()
    for _ in range(args.warmup):
        _lib.run_tracks(pr, tracks)
    t_ms, b_ms = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            _lib.run_tracks(pr, tracks)
            t_ms.append(_lib.last_timing()["total_ms"])
    clocks = clk.summary()
    _lib.run_batch(insts)
    for _ in range(max(1, args.steps // 2)):
        _lib.run_batch(insts)
        b_ms.append(_lib.last_timing()["total_ms"])
    value = world * steps / (np.mean(t_ms) * 1e-3)
    batch = steps / (np.mean(b_ms) * 1e-3)
    leg = {"value": value, "ms_per_step": float(np.mean(t_ms)), "steps": args.steps,
           "config": {"workload": "dwi_pgse_8_gradient_scales_200cubed_1e6spins",
                      "phantom": "200^3 cylinders r5um 3% (config 1)", "n_spins": n_spins,
                      "sequence": "PGSE x, delta 10 ms, Delta 20 ms, TE 34 ms, dt 50 us",
                      "gradient_scales": scales},
           "one_walk_per_scale": {"value": batch, "ms": float(np.mean(b_ms))},
           "shared_over_separate": value / batch,
           "error_vs_fp64": dict(max_errors([insts[0], insts[-1]], rng_flag(args)),
                                 scales=[scales[0], scales[-1]], timed_precision="fp32"),
           "clocks": clocks}
    print_leg(args, world, rank, leg)


def run_phantom(args, world, rank):
    """The reference's cylinder phantom (phantom::cylinder: 800 um FoV, 800^3 voxels, r 5 um,
    3 %, B0 perpendicular, with the dipole field) generated on the GPU; voxels per second."""
    from spinwalk_gb300 import _lib
    res = 800
    for _ in range(args.warmup):
        _lib.phantom_cylinder(float(res), res, 0.11e-6 * 0.4, 0.75, 5.0, 3.0, 90.0, 1)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        m, f, bvf = _lib.phantom_cylinder(float(res), res, 0.11e-6 * 0.4, 0.75, 5.0, 3.0, 90.0, 1)
        times.append(time.perf_counter() - t)
    s = float(np.mean(times))
    line = {"metric": "phantom voxels/s", "value": res ** 3 / s, "unit": "voxels/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "reference_cylinder_phantom_800cubed",
                       "generator": "phantom::cylinder (fov 800 um, r 5 um, 3 %, 90 deg, seed 1)",
                       "actual_volume_fraction": bvf},
            "e2e": {"value": res ** 3 / s, "unit": "voxels/s",
                    "note": "host placement + GPU mask/field + copy of 2.5 GB to the host"}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="se")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-legs", action="store_true",
                    help="se workload: skip the GRE / batched / tracks / served legs")
    ap.add_argument("--cpu-sample", type=int, default=262144,
                    help="spin ids of the GPU arm's CPU baseline (stratified over the range)")
    ap.add_argument("--ref-sample", type=int, default=32768,
                    help="spin ids per step of the CPU reference arm (stratified)")
    ap.add_argument("--seed", type=int, default=None,
                    help="plain workloads: simulation seed (default 10; a large one makes the "
                         "seeding jump ahead)")
    ap.add_argument("--max-spins", type=int, default=None,
                    help="c3 workload: cap on the spins of every instance (a smaller case)")
    ap.add_argument("--requests", type=int, default=100, help="served leg: trace length")
    ap.add_argument("--distinct-requests", type=int, default=20,
                    help="served leg: requests of the distinct-seed pass")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the walk tuning by sw_autotune on the workload before timing")
    ap.add_argument("--resort-interval", type=int, default=None,
                    help="walk rounds between Morton re-sorts of the spins (0 = never)")
    ap.add_argument("--walk-block", type=int, default=None, help="walk kernel block size")
    ap.add_argument("--signal", action="store_true",
                    help="served leg: requests in signal mode (no per-spin outputs)")
    ap.add_argument("--field-bf16", action="store_true",
                    help="bfloat16 fieldmap records (SW_FIELD_BF16); reports their error")
    ap.add_argument("--rng", default="mt19937", choices=["mt19937", "minstd"],
                    help="generator flavour: the reference's CPU build (default) or CUDA build")
    ap.add_argument("--round-streams", type=int, default=None,
                    help="refill/walk rounds as this many independent halves on own streams (1, 2)")
    ap.add_argument("--seed-chunks", type=int, default=None,
                    help="seed/walk pipeline chunks (1 = seed all first, 0 = auto)")
    ap.add_argument("--walk-blocks-per-sm", type=int, default=None,
                    help="cap on the walk kernel's blocks per SM (0 = none)")
    ap.add_argument("--ring-steps", type=int, default=None,
                    help="walk steps per refill/walk round (0 = default 512)")
    ap.add_argument("--jump-min-kwords", type=int, default=None,
                    help="seeding jumps ahead from this discard count (x 1024 words; 0 = default)")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload in ("bssfp", "c3", "serve"):
        import torch
        torch.cuda.set_device(local)
        fn = {"bssfp": leg_tracks, "c3": leg_batched, "serve": leg_served}[args.workload]
        print_leg(args, world, rank, fn(args, rank, world))
    elif args.workload == "dwi":
        run_dwi(args, world, rank)
    elif args.workload == "phantom":
        run_phantom(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
