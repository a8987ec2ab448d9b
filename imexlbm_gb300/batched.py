"""Batched workload: many independent periodic Taylor-Green lattices of
uneven sizes advanced together, against the plain float64 path.

Default workload (seeded, numpy PCG64 seed 20261203): 64 cubic lattices,
edges uniform over {32, 48, 64, 96, 128}, Re uniform in [100, 3200] cast to
int as the deck does, u0 uniform in [0.02, 0.08], a phase offset uniform in
[0, 2 pi)^3 added to x, y, z of the Taylor-Green field, 500 steps each,
float32 storage, one persistent launch per step (captured in CUDA graphs,
launch shape from the autotuner).

Reported: the batch's aggregate MLUPS (sum of cells x steps / wall time of
the batched steps, after one warm-up step that includes the autotuner), the
plain float64 path's aggregate MLUPS on the same lattices (one lattice per
launch, one after the other), their ratio, and per lattice the kinetic-
energy error against its float64 run, mass drift and momentum.

Usage: python -m imexlbm_gb300.batched [--lattices 64] [--steps 500]
         [--precision f32|f16dev|mixed] [--seed 20261203] [--json out.json]
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

from . import _lib
from .lbm import LBM, Batch, System

EDGES = (32, 48, 64, 96, 128)


def workload(n=64, seed=20261203, precision="f32"):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        edge = int(rng.choice(EDGES))
        re = int(rng.uniform(100, 3200))
        u0 = float(rng.uniform(0.02, 0.08))
        phase = tuple(float(x) for x in rng.uniform(0.0, 2 * math.pi, 3))
        p = precision if precision != "mixed" else ("f32" if rng.uniform() < 0.5 else "f16dev")
        out.append({"edge": edge, "Re": re, "u0": u0, "phase": phase, "precision": p})
    return out


def tau_of(edge, re, u0):
    return System(text=f"1.0 0.1 {re}\n{u0} 1 1\n{edge} {edge} {edge}\n").tau


def run(n=64, steps=500, precision="f32", seed=20261203, log=print, check_fp64=True, row_launch=None, launch=None):
    import torch

    work = workload(n, seed, precision)
    pid = {"f32": _lib.IMEX_F32, "f16dev": _lib.IMEX_F16DEV}
    lats = []
    for w in work:
        lat = LBM(w["edge"], w["edge"], w["edge"], tau_of(w["edge"], w["Re"], w["u0"]), 1.0, w["u0"],
                  precision=pid[w["precision"]])
        lat.initialize_phase(*w["phase"])
        lats.append(lat)
    cells = sum(w["edge"] ** 3 for w in work)
    batch = Batch(max(2, n))
    if row_launch is not None:
        batch.set_row_launch(*row_launch)
    if launch is not None:
        batch.set_launch(*launch)
    for lat in lats:
        batch.add(lat)
    m0 = [lat.Conserved()[0] for lat in lats]
    launches0 = batch.kernel_launches()
    t0 = time.perf_counter()
    batch.step(1)          # autotuner + first (in-place) collision of every member
    batch.synchronize()
    t_warm = time.perf_counter() - t0
    launches1 = batch.kernel_launches()
    t0 = time.perf_counter()
    batch.step(steps - 1)
    batch.synchronize()
    t_batch = time.perf_counter() - t0
    launches = batch.kernel_launches() - launches1
    mlups = cells * (steps - 1) / t_batch / 1e6
    result = {"lattices": n, "steps": steps, "precision": precision, "seed": seed, "cells": cells,
              "batch_mlups": mlups, "batch_seconds": t_batch, "warmup_seconds": t_warm,
              "batch_launches_timed": launches, "launch_shape": batch.get_launch(),
              "row_launch": batch.get_row_launch()}
    cons = [lat.Conserved() for lat in lats]
    if check_fp64:
        ke_err, drift, mom = [], [], []
        t64 = 0.0
        for w, c, mm in zip(work, cons, m0):
            with LBM(w["edge"], w["edge"], w["edge"], tau_of(w["edge"], w["Re"], w["u0"]), 1.0, w["u0"]) as ref:
                ref.initialize_phase(*w["phase"])
                ref.get_launch()  # the launch-shape autotuner, outside the timed steps
                ref.step(1)
                ref.fence()
                t0 = time.perf_counter()
                ref.step(steps - 1)
                ref.fence()
                t64 += time.perf_counter() - t0
                r = ref.Conserved()
            ke_err.append(abs(c[4] - r[4]) / r[4])
            drift.append(abs(c[0] - mm) / mm)
            mom.append(max(abs(x) for x in c[1:4]))
        fp64_mlups = cells * (steps - 1) / t64 / 1e6
        result.update({"fp64_plain_mlups": fp64_mlups, "speedup_vs_fp64_plain": mlups / fp64_mlups,
                       "ke_rel_err_max": max(ke_err), "ke_rel_err_median": float(np.median(ke_err)),
                       "mass_drift_max": max(drift), "momentum_abs_max": max(mom)})
    log(json.dumps(result))
    batch.close()
    for lat in lats:
        lat.close()
    return result


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--lattices", type=int, default=64)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--precision", choices=["f32", "f16dev", "mixed"], default="f32")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--row-launch", default=None, metavar="STAGES,KB,CTAS",
                    help="pin the row kernel's shape (-1,0,0: off) instead of autotuning it")
    ap.add_argument("--launch", default=None, metavar="THREADS,CPT,CTAS",
                    help="pin the one-thread-per-cell kernel's shape instead of autotuning it")
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    rl = tuple(int(v) for v in a.row_launch.split(",")) if a.row_launch else None
    cl = tuple(int(v) for v in a.launch.split(",")) if a.launch else None
    r = run(a.lattices, a.steps, a.precision, a.seed, check_fp64=not a.no_fp64, row_launch=rl, launch=cl)
    if a.json:
        with open(a.json, "w") as fp:
            json.dump(r, fp, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
