"""Precision sweep: float64 vs float32 vs float16-deviation storage on one
periodic Taylor-Green lattice, all resident on the GPU at once.

Default workload: 512^3, Re = 1600, u0 = 0.05, 2000 steps, reporting every
100 - three runs side by side:
  (a) float64 storage (the reference's precision; fixed-point engine),
  (b) float32 storage, float32 collision,
  (c) float16 storage of 2^12 (f - w), float32 collision, rounded to nearest,
  (d) the same with stochastic rounding.
Every report step prints, for (b) and (c) against (a): the relative
kinetic-energy error, the largest velocity difference over all cells (in
units of u0) and the relative mass drift of each run; at the end, each
run's MLUPS (CUDA events around its own steps, each lattice's launch shape
tuned before the first) and the worst errors.
Mass, momentum and ke are float64 reductions in every run.

Usage: python -m imexlbm_gb300.sweep [--size 512] [--steps 2000] [--report 100]
                                     [--re 1600] [--u0 0.05] [--json out.json]
Needs about 27 x 18 bytes per cell of device memory (130 GB at 512^3).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

from . import _lib
from .lbm import LBM, System


def run(size=512, steps=2000, report=100, re=1600, u0=0.05, out=None, log=print):
    import torch

    deck = System(text=f"1.0 0.1 {re}\n{u0} {steps} {report}\n{size} {size} {size}\n")
    names = [("f64", _lib.IMEX_F64), ("f32", _lib.IMEX_F32), ("f16dev", _lib.IMEX_F16DEV),
             ("f16dev_sr", _lib.IMEX_F16DEV)]
    lats, streams = {}, {}
    for name, prec in names:
        streams[name] = torch.cuda.Stream()
        lat = LBM(size, size, size, deck.tau, deck.rho0, deck.u0, precision=prec)
        lat.set_stream(streams[name].cuda_stream)
        lat.set_rounding(_lib.IMEX_ROUND_STOCHASTIC if name.endswith("_sr") else _lib.IMEX_ROUND_NEAREST)
        lat.Initialize()
        lat.get_launch()  # the launch-shape autotuner, outside the timed steps (it leaves the state as it is)
        lats[name] = lat
    m0 = {k: v.Conserved()[0] for k, v in lats.items()}
    ms = {k: 0.0 for k in lats}
    rows = []
    low = [n for n, _ in names if n != "f64"]
    worst = {k: {"ke_rel": 0.0, "u_max_over_u0": 0.0, "mass_drift_rel": 0.0} for k in low}
    done = 0
    while done < steps:
        k = min(report, steps - done)
        for name, lat in lats.items():
            s = streams[name]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            lat.step(k)
            e1.record(s)
            e1.synchronize()
            ms[name] += e0.elapsed_time(e1)
        done += k
        cons = {name: lat.Conserved() for name, lat in lats.items()}
        row = {"step": done, "ke_f64": cons["f64"][4]}
        for name in low:
            ke_rel = abs(cons[name][4] - cons["f64"][4]) / cons["f64"][4]
            du, _ = lats[name].velocity_max_diff(lats["f64"])
            drift = abs(cons[name][0] - m0[name]) / m0[name]
            row[name] = {"ke_rel": ke_rel, "u_max_over_u0": du / u0, "mass_drift_rel": drift,
                         "momentum_abs": max(abs(x) for x in cons[name][1:4])}
            for key, val in (("ke_rel", ke_rel), ("u_max_over_u0", du / u0), ("mass_drift_rel", drift)):
                worst[name][key] = max(worst[name][key], val)
        row["f64_mass_drift_rel"] = abs(cons["f64"][0] - m0["f64"]) / m0["f64"]
        rows.append(row)
        log(json.dumps(row))
    cells = size ** 3
    summary = {"size": size, "steps": steps, "report_every": report, "Re": re, "u0": u0, "tau": deck.tau,
               "mlups": {k: cells * steps / (v * 1e-3) / 1e6 for k, v in ms.items()},
               "worst": worst,
               "f64_fallback_cells": lats["f64"].fallback_cells()}
    log(json.dumps({"summary": summary}))
    for lat in lats.values():
        lat.close()
    if out:
        with open(out, "w") as fp:
            json.dump({"rows": rows, "summary": summary}, fp, indent=1)
    return summary


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--report", type=int, default=100)
    ap.add_argument("--re", type=int, default=1600)
    ap.add_argument("--u0", type=float, default=0.05)
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    run(a.size, a.steps, a.report, a.re, a.u0, a.json)
    return 0


if __name__ == "__main__":
    sys.exit(main())
