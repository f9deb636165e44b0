"""Generates the golden fixtures in tests/golden/*.npz by running the REFERENCE's own per-spin
function sim::sim (SpinWalk 1.21.0 src/sim/kernels.cu:72-233, CPU-only build with std::mt19937),
compiled from the read-only source tree into oracle/_ref/libref_sim.so by oracle/Makefile.

    python tests/golden/make_golden.py        (needs the reference tree; run from the repo root)

Each fixture stores the inputs of one case (phantom, field in Tesla, initial positions, Problem
keyword arguments) and the reference outputs M1, XYZ1, T. The cases exercise every branch of the
hot path: GRE / SE / stimulated echo, dummy scans with linear + quadratic phase cycling,
permeable interfaces, reflecting and periodic boundaries, gradients and ideal dephasing,
trajectory recording, no fieldmap, a zero-diffusivity substrate, disabled relaxation, lost spins
(max_iterations exceeded) and out-of-bounds spins (steps larger than the field of view).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from spinwalk_gb300.problem import Problem, cylinder_phantom, sphere_phantom  # noqa: E402
from tests import oracle_lib  # noqa: E402


def cases():
    cyl_m, cyl_f = cylinder_phantom(32, 32e-6, 4e-6, 0.10, seed=1)
    sph_m, sph_f = sphere_phantom(24, 24e-6, 1.5e-6, 3e-6, 0.08, seed=2)
    tiny_m = np.zeros((4, 4, 4), np.uint8)
    tiny_m[1:3, 1:3, 1:3] = 1
    tiny_f = np.linspace(-1e-7, 1e-7, 64, dtype=np.float32).reshape(4, 4, 4)
    three_m = (np.arange(20 ** 3).reshape(20, 20, 20) % 3).astype(np.uint8)
    three_f = np.cos(np.arange(20 ** 3, dtype=np.float32)).reshape(20, 20, 20) * 2e-7
    cyl = dict(mask=cyl_m, field=cyl_f, fov=32e-6)
    sph = dict(mask=sph_m, field=sph_f, fov=24e-6)
    gre = dict(TR_us=10050, TE_us=(10000,))
    yield "gre", cyl, dict(gre, n_spins=256, seed=10)
    yield "gre_seed7_sph", sph, dict(gre, n_spins=200, seed=7)
    yield "se_multi_te", cyl, dict(TR_us=20050, TE_us=(5000, 10000, 15000, 20000),
                                   RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0), RF_us=(0, 10000),
                                   n_spins=256, seed=10)
    yield "ste_dephasing", sph, dict(TR_us=12000, TE_us=(4000, 8000), RF_FA=(90.0, 90.0, 90.0),
                                     RF_PH=(0.0, 90.0, 90.0), RF_us=(0, 2000, 6000),
                                     dephasing_deg=(360.0, 360.0, 720.0, 360.0),
                                     dephasing_us=(1000, 3000, 5000, 7000), n_spins=200, seed=10)
    yield "bssfp_phase_cycling", cyl, dict(TR_us=2500, TE_us=(1250,), RF_FA=(30.0,),
                                           timestep_us=25, n_dummy_scan=12,
                                           linear_phase_cycling=33.75,
                                           quadratic_phase_cycling=7.5, n_spins=128, seed=3)
    yield "bssfp_180_cycling", cyl, dict(TR_us=2500, TE_us=(1250,), RF_FA=(16.0,),
                                         timestep_us=25, n_dummy_scan=6,
                                         linear_phase_cycling=180.0, n_spins=128, seed=4)
    yield "permeable", cyl, dict(gre, pXY=[[1.0, 0.3], [0.2, 1.0]], n_spins=256, seed=11)
    yield "reflect", cyl, dict(gre, cross_fov=False, n_spins=256, seed=12)
    yield "trajectory", sph, dict(TR_us=2050, TE_us=(1000, 2000), record_trajectory=True,
                                  n_dummy_scan=1, n_spins=96, seed=13)
    yield "pgse_gradients", cyl, dict(
        TR_us=12050, TE_us=(12000,), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0), RF_us=(0, 6000),
        gradient_xyz=[[0, 0, 0]] + [[91.6, 0, 0]] * 40 + [[0, 0, 0], [0, 0, 0]] +
        [[91.6, 0, 0]] * 40 + [[0, 0, 0]],
        gradient_us=[950] + [1000 + 50 * i for i in range(40)] + [3000, 6950] +
        [7000 + 50 * i for i in range(40)] + [9000], n_spins=200, seed=14)
    yield "no_fieldmap", dict(cyl, field=None), dict(gre, n_spins=128, seed=15)
    yield "zero_diffusivity_norelax", cyl, dict(gre, diffusivity=(1e-9, 0.0),
                                                T1_ms=(-1.0, 2000.0), T2_ms=(-1.0, 30.0),
                                                n_spins=256, seed=16)
    yield "three_substrates", dict(mask=three_m, field=three_f, fov=20e-6), dict(
        gre, diffusivity=(1e-9, 2e-9, 0.5e-9), T1_ms=(1000.0, 1500.0, 2000.0),
        T2_ms=(40.0, 30.0, 20.0), pXY=[[1, .5, .1], [.4, 1, .2], [.3, .6, 1]],
        n_spins=256, seed=17)
    yield "lost_spins", cyl, dict(gre, max_iterations=1, n_spins=256, seed=18)
    yield "out_of_bounds_periodic", dict(mask=tiny_m, field=tiny_f, fov=0.4e-6), dict(
        TR_us=2050, TE_us=(1000, 2000), diffusivity=(3e-9, 3e-9), n_spins=64, seed=19,
        pXY=[[1, 1], [1, 1]])
    yield "out_of_bounds_reflect", dict(mask=tiny_m, field=tiny_f, fov=0.4e-6), dict(
        TR_us=2050, TE_us=(1000, 2000), diffusivity=(3e-9, 3e-9), n_spins=64, seed=20,
        cross_fov=False, pXY=[[1, 1], [1, 1]])


def make(name, ph, kw):
    fov = ph["fov"]
    n = kw["n_spins"]
    XYZ0 = oracle_lib.initial_positions([fov] * 3, kw.get("seed", 10), n)
    pr = Problem(ph["mask"], [fov] * 3, ph["field"], XYZ0=XYZ0, **kw)
    out = oracle_lib.run_ref(pr, fill=np.nan)
    kw_json = json.dumps({k: (np.asarray(v).tolist() if isinstance(v, (tuple, list, np.ndarray))
                              else v) for k, v in kw.items()})
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), mask=ph["mask"],
        field_T=(ph["field"] if ph["field"] is not None else np.zeros(0, np.float32)),
        fov=np.float64(fov), XYZ0=XYZ0, kwargs=np.array(kw_json), M1=out["M1"],
        XYZ1=out["XYZ1"], T=out["T"])
    return pr, out


def main():
    if not oracle_lib.ref_available():
        raise SystemExit("oracle/_ref/libref_sim.so missing: run `make -C oracle ref` first")
    for name, ph, kw in cases():
        pr, out = make(name, ph, kw)
        unreached = int(np.isnan(out["M1"]).any(axis=(1, 2)).sum())
        print(f"{name:28s} spins={pr.params.n_spins:4d} steps={pr.spin_steps():8d} "
              f"spins_with_unreached_echoes={unreached}")


if __name__ == "__main__":
    main()
