"""Served workload: Poisson arrivals of Taylor-Green solves into the
continuous-batching server, with time-to-result percentiles.

Default trace (seeded, numpy PCG64 seed 20261203): arrivals at 50 requests/s
for 60 s; each request a periodic Taylor-Green solve with cubic edge from
{32, 64, 96, 128, 192, 256} (weights 0.3, 0.25, 0.2, 0.12, 0.08, 0.05), Re
log-uniform in [100, 5000] (cast to int as the deck does), u0 uniform in
[0.02, 0.08], steps uniform in [200, 5000], storage float32 or float16
deviations (50/50; float16 with stochastic rounding).  Admission against a
120 GB device-memory budget.

Reported: p50 / p99 / max time-to-result (submission to result, queueing
included), the aggregate MLUPS over the run, the batch's own MLUPS while
busy, the peak number of requests in flight, and checks on sampled
requests - the kinetic-energy error of the served result against the same
solve in float64 alone (whose steps, timed after its launch shape is tuned,
also give the plain float64 path's MLUPS on the sample), and that the served result
equals the same request run alone in its own precision, bit for bit.

The offered load (about 1.9 M cells x 2600 steps per request, 50 per
second) is several times what one GPU can serve, so the queue grows for the
whole minute; the percentiles say so.

Usage: python -m imexlbm_gb300.serve [--rate 50] [--duration 60]
          [--budget-gb 120] [--max-active 256] [--steps-per-tick 25]
          [--spot 16] [--policy arrival|least-work] [--json out.json]
       small trace: --edges 16,24,32 --steps-min 20 --steps-max 80
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

from . import _lib
from .lbm import LBM, Server, System

EDGES = (32, 64, 96, 128, 192, 256)
WEIGHTS = (0.3, 0.25, 0.2, 0.12, 0.08, 0.05)


def trace(rate=50.0, duration=60.0, seed=20261203, edges=EDGES, weights=WEIGHTS, re_range=(100, 5000),
          u0_range=(0.02, 0.08), steps_range=(200, 5000)):
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    w = np.asarray(weights, float)
    w = w / w.sum()
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        edge = int(rng.choice(edges, p=w))
        re = int(math.exp(rng.uniform(math.log(re_range[0]), math.log(re_range[1]))))
        u0 = float(rng.uniform(*u0_range))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        prec = "f32" if rng.uniform() < 0.5 else "f16dev"
        out.append({"t": t, "edge": edge, "Re": re, "u0": u0, "steps": steps, "precision": prec})
    return out


def tau_of(edge, re, u0):
    return System(text=f"1.0 0.1 {re}\n{u0} 1 1\n{edge} {edge} {edge}\n").tau


PREC = {"f32": _lib.IMEX_F32, "f16dev": _lib.IMEX_F16DEV}


def run_alone(req, precision, timed=False):
    """One request on its own lattice: its diagnostics, and with timed the
    seconds of its steps alone (the launch shape tuned before them, creation,
    initialisation and the diagnostics outside)."""
    with LBM(req["edge"], req["edge"], req["edge"], tau_of(req["edge"], req["Re"], req["u0"]), 1.0, req["u0"],
             precision=precision) as lat:
        lat.Initialize()
        lat.get_launch()
        lat.fence()
        t0 = time.perf_counter()
        lat.step(req["steps"])
        lat.fence()
        seconds = time.perf_counter() - t0
        cons = lat.Conserved(allow_nonfinite=True)
    return (cons, seconds) if timed else cons


def run(rate=50.0, duration=60.0, budget_gb=120.0, max_active=256, steps_per_tick=25, spot=16, seed=20261203,
        edges=EDGES, steps_range=(200, 5000), drain_timeout=3600.0, log=print, policy="arrival"):
    reqs = trace(rate, duration, seed, edges=edges, weights=WEIGHTS[:len(edges)] if len(edges) <= len(WEIGHTS)
                 else [1.0] * len(edges), steps_range=steps_range)
    results = {}
    peak_active = 0
    with Server(budget_gb * 1e9, max_active, steps_per_tick) as srv:
        srv.set_policy({"arrival": _lib.IMEX_POLICY_ARRIVAL, "least-work": _lib.IMEX_POLICY_LEAST_WORK}[policy])
        t0 = time.perf_counter()
        ids = {}
        for i, r in enumerate(reqs):
            while True:
                lag = r["t"] - (time.perf_counter() - t0)
                if lag <= 0:
                    break
                time.sleep(min(lag, 0.005))
            rid = srv.submit(r["edge"], r["edge"], r["edge"], tau_of(r["edge"], r["Re"], r["u0"]), r["u0"],
                             r["steps"], PREC[r["precision"]], tag=i)
            ids[rid] = i
            if i % 16 == 0:
                for res in srv.poll():
                    results[res["tag"]] = res
                peak_active = max(peak_active, srv.stats()["active"])
        t_submitted = time.perf_counter() - t0
        while len(results) < len(reqs) and time.perf_counter() - t0 < drain_timeout:
            for res in srv.poll():
                results[res["tag"]] = res
            st = srv.stats()
            peak_active = max(peak_active, st["active"])
            if st["failed"]:
                break
            time.sleep(0.02)
        st = srv.stats()
    done = [results[i] for i in sorted(results)]
    ok = [r for r in done if r["status"] == 0]
    # A solve whose diagnostics are NaN / Inf diverged (BGK at tau near 0 on
    # a coarse grid: high Re, small edge); it ran all its steps and gets its
    # result with status IMEX_ERR_NONFINITE.
    ran = [r for r in done if r["status"] in (0, _lib.IMEX_ERR_NONFINITE)]
    statuses = {}
    for r in done:
        statuses[str(r["status"])] = statuses.get(str(r["status"]), 0) + 1
    ttr = np.array([r["t_done"] - r["t_submit"] for r in ran]) if ran else np.array([float("nan")])
    span = max(r["t_done"] for r in ran) - min(r["t_submit"] for r in ran) if ran else float("nan")
    updates = sum(r["cells"] * r["steps"] for r in ran)
    out = {"requests": len(reqs), "completed": len(ok), "diverged": sum(r["status"] == _lib.IMEX_ERR_NONFINITE for r in done),
           "failed": len(done) - len(ran), "statuses": statuses, "unfinished": len(reqs) - len(done),
           "rate_per_s": rate, "duration_s": duration, "budget_gb": budget_gb, "max_active": max_active,
           "steps_per_tick": steps_per_tick, "policy": policy, "seed": seed, "submit_seconds": t_submitted,
           "ttr_p50_s": float(np.percentile(ttr, 50)), "ttr_p99_s": float(np.percentile(ttr, 99)),
           "ttr_max_s": float(ttr.max()), "aggregate_mlups": updates / span / 1e6 if ran else None,
           "busy_mlups": st["cell_updates"] / st["busy_seconds"] / 1e6 if st["busy_seconds"] else None,
           "peak_active": peak_active, "offered_lups": sum(r["edge"] ** 3 * r["steps"] for r in reqs) / duration}
    # sampled checks
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    sample = sorted(rng.choice(len(ok), size=min(spot, len(ok)), replace=False).tolist()) if ok else []
    ke_err, same, spots = [], [], []
    f64_updates, f64_seconds = 0, 0.0
    for k in sample:
        r = ok[k]
        req = reqs[r["tag"]]
        ref64, sec = run_alone(req, _lib.IMEX_F64, timed=True)  # the plain float64 path, one request at a time
        f64_seconds += sec
        f64_updates += r["cells"] * r["steps"]
        err = abs(r["conserved"][4] - ref64[4]) / ref64[4]
        ke_err.append(err)
        spots.append({"edge": req["edge"], "Re": req["Re"], "u0": round(req["u0"], 5), "steps": req["steps"],
                      "precision": req["precision"], "tau": tau_of(req["edge"], req["Re"], req["u0"]),
                      "ke_rel_err": err})
        if len(same) < max(4, spot // 4):
            same.append(tuple(r["conserved"]) == tuple(run_alone(req, PREC[req["precision"]])))
    # diverged solves: does the same solve diverge in float64 too?
    div = [r for r in done if r["status"] == _lib.IMEX_ERR_NONFINITE]
    div_sample = sorted(rng.choice(len(div), size=min(max(2, spot // 4), len(div)), replace=False).tolist()) if div else []
    div_f64 = [not np.all(np.isfinite(run_alone(reqs[div[k]["tag"]], _lib.IMEX_F64))) for k in div_sample]
    out["diverged_checked"] = len(div_f64)
    out["diverged_also_in_f64"] = sum(div_f64)
    out["diverged_tau_max"] = max((tau_of(reqs[r["tag"]]["edge"], reqs[r["tag"]]["Re"], reqs[r["tag"]]["u0"]) for r in div),
                                  default=None)
    if f64_seconds > 0:
        out["fp64_plain_mlups_on_sample"] = f64_updates / f64_seconds / 1e6
        if out.get("aggregate_mlups"):
            out["aggregate_vs_fp64_plain"] = out["aggregate_mlups"] / out["fp64_plain_mlups_on_sample"]
    out.update({"spot_checks": len(ke_err), "ke_rel_err_vs_f64_max": max(ke_err) if ke_err else None,
                "ke_rel_err_vs_f64_median": float(np.median(ke_err)) if ke_err else None,
                "alone_equals_mix": all(same) if same else None, "alone_checks": len(same), "spots": spots})
    log(json.dumps(out))
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--max-active", type=int, default=256)
    ap.add_argument("--steps-per-tick", type=int, default=25)
    ap.add_argument("--spot", type=int, default=16)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--edges", default=",".join(map(str, EDGES)))
    ap.add_argument("--steps-min", type=int, default=200)
    ap.add_argument("--steps-max", type=int, default=5000)
    ap.add_argument("--drain-timeout", type=float, default=3600.0)
    ap.add_argument("--policy", choices=["arrival", "least-work"], default="arrival",
                    help="admission order: first come first served, or least work (cells x steps) first")
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    r = run(a.rate, a.duration, a.budget_gb, a.max_active, a.steps_per_tick, a.spot, a.seed,
            edges=tuple(int(x) for x in a.edges.split(",")), steps_range=(a.steps_min, a.steps_max),
            drain_timeout=a.drain_timeout, policy=a.policy)
    if a.json:
        with open(a.json, "w") as fp:
            json.dump(r, fp, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
