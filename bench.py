"""Benchmark of the SpinWalk `sim` hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W]
                    [--workload se|gre|bssfp|c3|serve|phantom]
                    [--impl ours|reference]

A "step" is one full pass of the hot path over one batch of synthetic input: per-spin generator
seeding (mt19937(seed+spin) + discard), the walk over all time points and the Bloch update for
every spin -- exactly the work of the reference's per-scale loop (src/sim/monte_carlo.cu:310-335).

Workloads (synthetic, seeded; the reference publishes no dataset):
  se  (default) spin echo, 500^3 phantom of random spheres (r 2-8 um, 5 %), 1e6 spins, 2001 time
      points (TE 40 ms, dt 20 us, TR = TE + dt), permeability 0.01 both ways.
  gre gradient echo, 200^3 phantom of random-orientation cylinders (r 5 um, 3 %), 1e5 spins,
      401 time points (TE 20 ms, dt 50 us).

Metric: spin-steps/s (spins x time points x scans per second of the whole pass). `value` is
timed with CUDA events with every input already in HBM; `e2e` goes through the public host-buffer
entry point sw_sim (host->device copies of the inputs and device->host copies of the results
inside the timed region). Inputs (packed phantom, generator state) are larger than L2, so no
explicit flush is needed between steps.

--impl reference times the reference algorithm's CPU path (the oracle port of sim::sim, with
std::mt19937) on all host cores on a bounded, stratified sample of the same workload's spin ids.
Multi-GPU: spins are independent, so each rank walks its own spin range (weak scaling, no
collective on the data path).
"""
import argparse
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

GATHER_BYTES_PER_SPIN_STEP = 32   # one DRAM sector per random voxel lookup (mask + field record)
USEFUL_BYTES_PER_SPIN_STEP = 5    # 1 B mask + 4 B field
SEED_BYTES_PER_SPIN = 2 * 624 * 4 + 6 * 4   # two mt19937 states + 6 ring/index words written
# DRAM traffic per unit from ncu on the small SE case (profiles/kernels_small_se_300cubed_2e5spins.md),
# scaled to a full launch by the units it processes (both grow in proportion)
SEED_DRAM_BYTES_PER_SPIN = 4713.0
MT_BYTES_PER_SPIN_STEP = 3.82 * 8        # MT words drawn per step x (4 B read + 4 B write)
WALK_FP64_OPS_PER_SPIN_STEP = 6          # x, y, z step multiplies and position additions
FP64_PEAK_GFLOPS = 152 * 2 * 2070e6 / 1e9  # 2 FP64 lanes per clock per SM at 2070 MHz
USEFUL_BYTES_PER_SPIN_STEP = 5           # 1 B mask + 4 B field at the visited voxel
WALK_DRAM_BYTES_PER_SPIN_STEP = 26.0
SEED_LIMITER = ("integer instruction issue (ncu: ALU pipe 83 %, issue 74 %, DRAM 2 %): "
                "7.7 lane instructions per MT word, not HBM")
WALK_LIMITER = ("FP64 pipe (ncu: 64 %, 3 position additions + 3 step multiplies per step at 2 "
                "lanes/clock/SM) and the latency of the voxel gather (issue 38 %, long-scoreboard "
                "stalls, DRAM 10 %)")


def workload(name, rank=0):
    from spinwalk_gb300 import _lib
    from spinwalk_gb300.problem import Problem
    if name == "se":
        n, fov = 500, 500e-6
        mask, field = _lib.phantom_spheres(n, fov, 2e-6, 8e-6, 0.05, seed=2)
        n_spins = 1_000_000
        kw = dict(TR_us=40020, TE_us=(40000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 20000), timestep_us=20, pXY=[[1.0, 0.01], [0.01, 1.0]],
                  T2_ms=(40.0, 20.0), T1_ms=(2000.0, 2000.0))
        desc = dict(workload="se_spheres_500cubed_1e6spins_2001tp", phantom="500^3 spheres r2-8um 5%",
                    n_spins=n_spins, time_points=2001, sequence="SE 90/180, TE 40 ms, dt 20 us",
                    permeability=0.01)
    elif name == "gre":
        n, fov = 200, 200e-6
        mask, field = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=1)
        n_spins = 100_000
        kw = dict(TR_us=20050, TE_us=(20000,), timestep_us=50)
        desc = dict(workload="gre_cylinders_200cubed_1e5spins_401tp",
                    phantom="200^3 cylinders r5um 3% random orientation", n_spins=n_spins,
                    time_points=401, sequence="GRE 90, TE 20 ms, dt 50 us", permeability=0.0)
    elif name == "bssfp":      # config 4 phantom/sequence; batched by run_tracks()
        n, fov = 300, 300e-6
        mask, field = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=4)
        n_spins = 200_000
        kw = dict(TR_us=5000, TE_us=(2500,), RF_FA=(30.0,), timestep_us=25, n_dummy_scan=209)
        desc = dict(workload="bssfp_cylinders_300cubed_2e5spins_64pc_x_10tr",
                    phantom="300^3 cylinders r5um 3%", n_spins=n_spins, time_points=200,
                    sequence="bSSFP FA 30, TR 5 ms, TE 2.5 ms, dt 25 us, 64 phase cycles "
                             "(5.625 deg steps) x DUMMY_SCAN 200..209")
    elif name in ("dense", "dense_small"):   # many spins per voxel: the Morton re-sort's case
        n, fov = 100, 100e-6
        mask, field = _lib.phantom_cylinders(n, fov, 5e-6, 0.03, seed=1)
        n_spins = 2_000_000 if name == "dense" else 500_000
        kw = dict(TR_us=40050, TE_us=(40000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 20000), timestep_us=50)
        desc = dict(workload=f"{name}_se_cylinders_100cubed_{n_spins:.0e}spins_801tp".replace("+0", ""),
                    phantom="100^3 cylinders r5um 3% (the serving trace's smallest phantom)",
                    n_spins=n_spins, spins_per_voxel=n_spins / n ** 3, time_points=801,
                    sequence="SE 90/180, TE 40 ms, dt 50 us", permeability=0.0)
    elif name == "small":      # profiling case: > L2 phantom, few GB on the device
        n, fov = 300, 300e-6
        mask, field = _lib.phantom_spheres(n, fov, 2e-6, 8e-6, 0.05, seed=2)
        n_spins = 200_000
        kw = dict(TR_us=4020, TE_us=(4000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 2000), timestep_us=20, pXY=[[1.0, 0.01], [0.01, 1.0]])
        desc = dict(workload="small_se_300cubed_2e5spins_201tp", n_spins=n_spins, time_points=201)
    else:
        raise SystemExit(f"unknown workload {name}")
    seed = 10 + 1_000_003 * rank          # each rank: its own disjoint spin population
    pr = Problem(mask, [fov] * 3, field, n_spins=n_spins, seed=seed, **kw)
    return pr, desc


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


def precision_errors(pr, rng=0):
    """Error of the FP32 and compensated-FP32 (Kahan) phase sums against an FP64 run of the same
    walk (the FP64 shadow the library computes alongside): the largest per-spin |M - M_fp64|
    (|M| <= 1) and the largest relative error of the echo signal |mean Mxy| over all echoes."""
    from spinwalk_gb300 import _lib, abi
    out = {}
    for name, prec in (("fp32", abi.SW_PREC_FP32), ("kahan", abi.SW_PREC_KAHAN)):
        r = _lib.run(pr, precision=prec | rng, fp64_shadow=True)
        m, d = r["M1"].astype(np.float64), r["M1_fp64"]
        ok = r["status"] == 0
        sig = np.abs(m[ok, :, 0].mean(0) + 1j * m[ok, :, 1].mean(0))
        sig64 = np.abs(d[ok, :, 0].mean(0) + 1j * d[ok, :, 1].mean(0))
        out[name] = {"max_abs_per_spin": float(np.abs(m[ok] - d[ok]).max()),
                     "signal_rel": float((np.abs(sig - sig64) / np.maximum(sig64, 1e-30)).max())}
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


def run_reference(args, world, rank):
    """CPU reference arm: the oracle port on all host cores, rank 0 only."""
    if rank != 0:
        return
    pr, desc = workload(args.workload)
    cores = os.cpu_count()
    n_sample = args.cpu_sample
    for _ in range(args.warmup):
        time_cpu(pr, max(16, n_sample // 8), cores)
    rates, secs = [], []
    for _ in range(args.steps):
        r, n, dt = time_cpu(pr, n_sample, cores)
        rates.append(r)
        secs.append(dt)
    v = float(np.mean(rates))
    sample = (f"{n} stratified spin ids of {pr.params.n_spins} per step, "
              f"{pr.params.n_timepoints} time points each, extrapolated as spin-steps/s")
    line = {"impl": "reference", "metric": "spin-steps/s", "value": v, "unit": "spin-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(secs)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(desc, l2="inputs larger than L2"),
            "cpu_baseline": {"value": v, "unit": "spin-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "spin-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
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
            args.seed_chunks is not None or args.round_streams is not None:
        cur = _lib.get_tuning()
        _lib.set_tuning(cur["resort_interval"] if args.resort_interval is None else args.resort_interval,
                        cur["walk_block"] if args.walk_block is None else args.walk_block,
                        cur["seed_chunks"] if args.seed_chunks is None else args.seed_chunks,
                        cur["round_streams"] if args.round_streams is None else args.round_streams)
    info["applied"] = _lib.get_tuning()
    return info


def run_ours(args, world, rank, local):
    import torch
    from spinwalk_gb300 import _lib

    torch.cuda.set_device(local)
    pr, desc = workload(args.workload, rank)
    tuning = apply_tuning(args, pr)
    p = pr.params
    n, nte = p.n_spins, pr.n_te
    dev = torch.device("cuda", local)
    d = dict(field=torch.from_numpy(pr.field).to(dev), mask=torch.from_numpy(pr.mask).to(dev),
             M0=torch.from_numpy(pr.M0).to(dev), XYZ0=torch.from_numpy(pr.XYZ0).to(dev),
             M1=torch.zeros((n, nte, 3), dtype=torch.float32, device=dev),
             XYZ1=torch.zeros((n, pr.traj_len, 3), dtype=torch.float32, device=dev),
             T=torch.zeros((n, nte), dtype=torch.uint8, device=dev),
             status=torch.zeros(n, dtype=torch.int32, device=dev))
    stream = torch.cuda.current_stream(dev)

    from spinwalk_gb300 import abi
    rng = abi.SW_RNG_MINSTD if args.rng == "minstd" else abi.SW_RNG_MT19937
    prec = abi.SW_PREC_FP32 | (abi.SW_FIELD_BF16 if args.field_bf16 else 0) | rng

    def step():
        _lib.run_device(pr, d["field"].data_ptr(), d["mask"].data_ptr(), d["M0"].data_ptr(),
                        d["XYZ0"].data_ptr(), d["M1"].data_ptr(), d["XYZ1"].data_ptr(),
                        d["T"].data_ptr(), d["status"].data_ptr(), precision=prec,
                        stream=stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    spin_steps = pr.spin_steps()
    timings = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
            timings.append(_lib.last_timing())
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    clocks = clk.summary()
    ms = ev0.elapsed_time(ev1)
    ms = max_over_ranks(world, ms)
    value = world * spin_steps * args.steps / (ms * 1e-3)
    st = d["status"].cpu().numpy()

    # ---- end to end through the host-buffer entry point ----
    e2e_times = []
    h2d = pr.mask.nbytes + pr.field.nbytes + pr.M0.nbytes + pr.XYZ0.nbytes + \
        n * nte * 12 + n * nte + n * pr.traj_len * 12
    d2h = n * nte * 12 + n * nte + n * pr.traj_len * 12 + n * 4
    _lib.run(pr, precision=prec)                     # warm (host staging)
    for _ in range(max(1, args.steps)):
        barrier(world)
        t = time.perf_counter()
        out = _lib.run(pr, precision=prec)
        e2e_times.append(time.perf_counter() - t)
    e2e_s = max_over_ranks(world, float(np.mean(e2e_times)))
    e2e = world * spin_steps / e2e_s
    assert np.array_equal(out["status"], st)

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
    for r in (seed_roof, walk_roof):
        r["frac"] = r["achieved"] / peak
    roof = {"seed+init+pack": seed_roof, "walk": walk_roof}.get(dominant, walk_roof)
    # walk-only rate (refill + walk kernels, generator seeding excluded) and the secondary
    # ceilings: MT-state traffic of the refill (3.82 words of 8 B read+write per step) and the
    # FP64 work of the walk (3 position additions per step, 2 FP64 lanes per clock per SM)
    # wall time of the rounds: the call minus its seeding stage (the kernel times of the two
    # halves of the rounds overlap, so their sum would overstate it)
    walk_refill_s = ms / args.steps * 1e-3 - seed_ms / args.steps * 1e-3
    secondary = {
        "walk_only_spin_steps_per_s": spin_steps / walk_refill_s,
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
    if world == 1 or rank == 0:
        if args.cpu_sample > 0:
            rate, ns, dt = time_cpu(pr, args.cpu_sample, os.cpu_count(), rng=rng)
            wrate, wns, wdt = time_cpu(pr, max(1, args.cpu_sample // 4), os.cpu_count(),
                                       lowest=True, rng=rng)
            cpu = {"value": rate, "unit": "spin-steps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{ns} stratified spin ids of {n} ({pr.params.n_timepoints} time "
                             f"points each, {dt:.1f} s wall on {os.cpu_count()} threads)",
                   "walk_only": {"value": wrate, "unit": "spin-steps/s",
                                 "sample": f"spin ids 0..{wns - 1} (discard of at most "
                                           f"{int(pr.params.seed) + wns} words), {wdt:.1f} s wall"}}
    line = {
        "metric": "spin-steps/s", "value": value, "unit": "spin-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded phantom generator, reference-driver initial positions)",
        "config": dict(desc, parallelism=f"spin-range shards x{world}",
                       l2="inputs larger than L2 (packed phantom + generator state)",
                       field_records="bfloat16, 4 B per voxel" if args.field_bf16
                       else "float32, 8 B per voxel",
                       generators="thrust minstd_rand + erfcinv normal (the reference's CUDA "
                                  "build)" if args.rng == "minstd" else
                                  "std::mt19937 + polar normal (the reference's CPU build)"),
        "kernel_ms_per_step": {k: v / args.steps for k, v in parts.items()},
        "kernel_ms_note": "sums of launch durations; the refill/walk rounds run as two halves on "
                          "two streams whose kernels overlap, so walk + refill exceed their wall "
                          "time",
        "roofline": dict(roof, dominant_stage=dominant),
        "roofline_walk": walk_roof,
        "secondary_ceilings": secondary,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "spin-steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "tuning": tuning,
        "error_vs_fp64": errors,
        "field_bf16": bf16_err,
        "clocks": clocks,
        "status_counts": {str(k): int(v) for k, v in zip(*np.unique(st, return_counts=True))},
    }
    print(json.dumps(line), flush=True)


def run_batched(args, world, rank):
    """Config 4 batched: 64 phase-cycling scales x 10 sampled TRs (DUMMY_SCAN 200..209) = 640
    reference instances on ONE walk (sw_sim_tracks). Work is counted per instance, as the
    reference executes it: sum over instances of spins x time points x (DUMMY_SCAN + 1)."""
    import torch  # noqa: F401  (device selection only)
    from spinwalk_gb300 import _lib
    pr, desc = workload("bssfp", rank)
    p = pr.params
    tracks = [dict(linear_phase_cycling=5.625 * i, n_dummy_scan=d)
              for i in range(64) for d in range(200, 210)]
    inst_steps = sum(p.n_spins * p.n_timepoints * (t["n_dummy_scan"] + 1) for t in tracks)
    walk_steps = p.n_spins * p.n_timepoints * 210
    for _ in range(args.warmup):
        _lib.run_tracks(pr, tracks)
    times, dev_ms, launches = [], [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t = time.perf_counter()
            _lib.run_tracks(pr, tracks)
            times.append(time.perf_counter() - t)
            dev_ms.append(_lib.last_timing()["total_ms"])
            launches.append(_lib.last_timing()["n_launches"])
    clocks = clk.summary()
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
    value = inst_steps / (np.mean(dev_ms) * 1e-3)
    pr.params.linear_phase_cycling = 0.0
    pr.params.n_dummy_scan = 0
    rec_err = bssfp_cycle_errors(pr, [t for t in tracks if t["n_dummy_scan"] == 209])
    line = {"metric": "spin-steps/s (batched instances)", "value": value, "unit": "spin-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(dev_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(desc, instances=len(tracks), instance_spin_steps=int(inst_steps),
                           distinct_walk_spin_steps=int(walk_steps)),
            "distinct_walk_steps_per_s": walk_steps / (np.mean(dev_ms) * 1e-3),
            "plain_kernel_one_instance": {"value": plain_rate, "e2e_s": plain_s},
            "batched_over_plain": value / plain_rate,
            "e2e": {"value": inst_steps / float(np.mean(times)), "unit": "spin-steps/s",
                    "note": "includes the per-track host output copies"},
            "recurrence_error_vs_fp64": rec_err,
            "gpu_launches": int(sum(launches)),
            "clocks": clocks}
    print(json.dumps(line), flush=True)


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
        q = Problem(mask, [fov] * 3, field, n_spins=n_spins, seed=10 + 1_000_003 * rank,
                    **dict(kw, gradient_xyz=g * np.float32(sc)))
        return q
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
    line = {"metric": "spin-steps/s (gradient-scale sweep, per instance)", "value": value,
            "unit": "spin-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(t_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "dwi_pgse_8_gradient_scales_200cubed_1e6spins",
                       "phantom": "200^3 cylinders r5um 3% (config 1)", "n_spins": n_spins,
                       "sequence": "PGSE x, delta 10 ms, Delta 20 ms, TE 34 ms, dt 50 us",
                       "gradient_scales": scales},
            "one_walk_per_scale": {"value": batch, "ms": float(np.mean(b_ms))},
            "shared_over_separate": value / batch, "clocks": clocks}
    if rank == 0:
        print(json.dumps(line), flush=True)


def c3_instances(rank=0):
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


def run_batch_scales(args, world, rank):
    """Config 3 batched (sw_sim_batch: phantom packed once, generators seeded once for all 64
    instances, instances in spin-range chunks on concurrent slots) against the same instances
    run one sw_sim each. `value` is timed on the host around the whole call (staging copies
    included; every call uploads the phantom and seeds again)."""
    import torch  # noqa: F401
    from spinwalk_gb300 import _lib
    probs, desc = c3_instances(rank)
    tuning = apply_tuning(args, max(probs, key=lambda q: q.params.n_spins))
    steps = sum(p.spin_steps() for p in probs)
    for _ in range(args.warmup):
        _lib.run_batch(probs)
    dev_ms, wall, launches = [], [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t = time.perf_counter()
            _lib.run_batch(probs)
            wall.append(time.perf_counter() - t)
            dev_ms.append(_lib.last_timing()["total_ms"])
            launches.append(_lib.last_timing()["n_launches"])
    clocks = clk.summary()
    plain_ms, plain_wall = 0.0, 0.0
    for p in probs:
        t = time.perf_counter()
        _lib.run(p)
        plain_wall += time.perf_counter() - t
        plain_ms += _lib.last_timing()["total_ms"]
    value = world * steps / (np.mean(dev_ms) * 1e-3)
    plain = steps / (plain_ms * 1e-3)
    line = {"metric": "spin-steps/s (batched instances)", "value": value, "unit": "spin-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(dev_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(desc, instance_spin_steps=int(steps)),
            "plain_one_call_per_instance": {"value": plain, "ms": plain_ms,
                                            "e2e_value": steps / plain_wall},
            "batched_over_plain": value / plain,
            "batched_over_plain_e2e": float(np.mean(wall)) and (steps / float(np.mean(wall))) / (steps / plain_wall),
            "e2e": {"value": world * steps / float(np.mean(wall)), "unit": "spin-steps/s",
                    "note": "sw_sim_batch with host buffers"},
            "gpu_launches": int(sum(launches)),
            "tuning": tuning, "clocks": clocks}
    if rank == 0:
        print(json.dumps(line), flush=True)


def serve_requests(n_req, rng_seed=5, rank=0):
    """Config 5 trace: Poisson arrivals (mean 20 / s), requests on resident phantoms, spins
    log-uniform in [1e4, 1e7], a mix of GRE, SE and PGSE (b = 1000 s/mm^2, delta 10 ms, Delta
    20 ms, lobes from 2 ms, G = 91.6 mT/m along x, y or z; TE 34 ms; dt 50 us). One simulation
    seed for the service (its generator states are computed once, at start-up)."""
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
    return reqs, phantoms, arrivals, desc


def run_serve(args, world, rank):
    """Config 5: the requests are submitted to one engine at their arrival times; latency =
    submit -> results in the caller's buffers (queueing included)."""
    import torch  # noqa: F401
    from spinwalk_gb300 import _lib
    n_req = args.requests
    reqs, phantoms, arrivals, desc = serve_requests(n_req, rank=rank)
    tuning = apply_tuning(args, max(reqs, key=lambda q: q.params.n_spins))
    eng = _lib.Engine(n_slots=8, slot_spins=1 << 20)
    pids = {}
    t0 = time.perf_counter()
    for pr in reqs:
        key = pr.mask.shape
        if key not in pids:
            pids[key] = eng.add_phantom(pr, bf16=args.field_bf16)

    def submit(pr):
        if args.signal:
            return eng.submit_signal(pr, pids[pr.mask.shape])
        return eng.submit(pr, pids[pr.mask.shape])
    # service start-up: generator states of the largest request, computed once
    big = max(reqs, key=lambda p: p.params.n_spins)
    submit(big)
    eng.run_all()
    startup_s = time.perf_counter() - t0
    st0 = eng.stats()
    steps = sum(p.spin_steps() for p in reqs)
    lat = []
    with ClockSampler(0) as clk:
        t_start = time.perf_counter()
        i = 0
        while i < n_req or len(lat) < n_req:
            now = time.perf_counter() - t_start
            while i < n_req and arrivals[i] <= now:
                submit(reqs[i])
                i += 1
            for jid, rc, l in eng.poll(wait=0):
                assert rc == 0
                lat.append(l)
            time.sleep(0.0005)
        makespan = time.perf_counter() - t_start
    clocks = clk.summary()
    st1 = eng.stats()
    lat = np.array(lat)
    value = world * steps / makespan
    line = {"metric": "spin-steps/s (served)", "value": value, "unit": "spin-steps/s",
            "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": makespan * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": dict(desc, requests=n_req, spin_steps=int(steps),
                           outputs="per-(echo, substrate) signal sums (signal mode)" if args.signal
                           else "per-spin M1, T, XYZ1, status",
                           field_records="bfloat16, 4 B per voxel" if args.field_bf16
                           else "float32, 8 B per voxel"),
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "offered_spin_steps_per_s": steps / float(arrivals[-1]),
            "startup_s": startup_s,
            "e2e": {"value": value, "unit": "spin-steps/s",
                    "note": "host buffers in and out through the engine, arrivals in real time"},
            "gpu_launches": int(st1["launches"] - st0["launches"]),
            "walk_rounds": int(st1["rounds"] - st0["rounds"]),
            "tuning": tuning, "clocks": clocks}
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


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
    ap.add_argument("--cpu-sample", type=int, default=32768)
    ap.add_argument("--requests", type=int, default=100, help="serve workload: trace length")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the walk tuning by sw_autotune on the workload before timing")
    ap.add_argument("--resort-interval", type=int, default=None,
                    help="walk rounds between Morton re-sorts of the spins (0 = never)")
    ap.add_argument("--walk-block", type=int, default=None, help="walk kernel block size")
    ap.add_argument("--signal", action="store_true",
                    help="serve workload: requests in signal mode (no per-spin outputs)")
    ap.add_argument("--field-bf16", action="store_true",
                    help="bfloat16 fieldmap records (SW_FIELD_BF16); reports their error")
    ap.add_argument("--rng", default="mt19937", choices=["mt19937", "minstd"],
                    help="generator flavour: the reference's CPU build (default) or CUDA build")
    ap.add_argument("--round-streams", type=int, default=None,
                    help="refill/walk rounds as this many independent halves on own streams (1, 2)")
    ap.add_argument("--seed-chunks", type=int, default=None,
                    help="seed/walk pipeline chunks (1 = seed all first, 0 = auto)")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "bssfp":
        run_batched(args, world, rank)
    elif args.workload == "dwi":
        run_dwi(args, world, rank)
    elif args.workload == "c3":
        run_batch_scales(args, world, rank)
    elif args.workload == "serve":
        run_serve(args, world, rank)
    elif args.workload == "phantom":
        run_phantom(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
