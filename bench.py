"""Benchmark of the IMEXLBM time step on GB300.

Workload: the shipped deck size - 256^3 fully periodic Taylor-Green vortex,
rho0 = 1, Re = 1600, u0 = 0.05, float64 distributions (two arrays of
27 x 256^3 doubles, 3.62 GB each), reporting every 100 steps.  One "step" is
one reference time step (collision + pull streaming) of the whole lattice.

  value  MLUPS of K device-resident steps, CUDA events on the lattice's
         stream (the reference's MLUPS, src/main.cpp:71-80, also excludes
         the diagnostics); the arrays are larger than L2, so no flush.
  e2e    the same metric through the public C ABI with host buffers: upload
         f0 from pinned host memory, K steps with the Conserved diagnostics
         read back every 100 steps, download f at the end - all timed.
  roofline  the fused step kernel: algorithmic 432 B/cell (27 float64 read
         + 27 written) x cells / average launch time, against the measured
         HBM copy bandwidth.
  cpu_baseline  the reference's own code - its unmodified src/*.cpp built
         against single-process Kokkos / MPI stand-ins (oracle/_ref), OpenMP
         on all host cores - on a bounded slab of the workload; the CPU
         oracle (a C restatement) where the reference's sources are absent.

--impl reference times that build of the reference on the full 256^3
lattice (its own MLUPS line of a bounded report interval).

Multi-GPU: the path does not shard on one GPU; under torchrun each
rank advances its own independent lattice (replicas, weak scaling) and
value = all ranks' cell updates / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes per cell update: 27 values read + 27 written
BYTES_PER_CELL = {"f64": 432, "f32": 216, "f16dev": 108}
FLOP_PER_CELL = 594       # the reference's own count (src/profile.cpp:38)
DECK = "1.0 0.1 1600\n0.05 1000 100\n256 256 256\n"
FALLBACK_HBM_GBS = 6800.0


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--engine", choices=["auto", "native", "fixed"], default="auto")
    ap.add_argument("--precision", choices=["f64", "f32", "f16dev"], default="f64",
                    help="storage precision (f64: the reference's; f32 / f16dev: the reduced-precision variants)")
    ap.add_argument("--rounding", choices=["nearest", "stochastic"], default="nearest",
                    help="float16-deviation storage rounding")
    ap.add_argument("--size", type=int, default=256, help="cubic lattice edge (default: the shipped deck's 256)")
    ap.add_argument("--report-every", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--launch", default=None, metavar="STAGES,ROWS,CTAS",
                    help="pin the fused step's launch shape instead of autotuning it (stages 0: one thread per cell)")
    ap.add_argument("--blocks", type=int, default=0,
                    help="time the lattice decomposed into this many blocks (imex_domain_*) instead")
    ap.add_argument("--quick", action="store_true",
                    help="skip the precision sweep, batched and served workloads (added to the line by default)")
    return ap.parse_args(argv)


# ----------------------------------------------------------------- helpers --
def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fp:
            d = json.load(fp)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def load_traffic(kernel: str):
    """Per-cell DRAM bytes of `kernel` from the committed ncu summary and the
    lattice size it was captured at, if any."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(p) as fp:
            d = json.load(fp)
        return d[kernel], d.get("captured_at", {}).get(kernel, "?")
    except Exception:
        return None, None


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for ln in out.splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) == 8:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        # median under load: samples at or above half the max clock
        top = max(sm) if sm else 0.0
        load = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks (the job's time is its slowest rank's);
    x itself on one rank.  Works on any process-group backend."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mlups(cells: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job throughput: every rank advances its own `cells` lattice
    `steps` steps (replicas), in the slowest rank's `seconds`."""
    return cells * steps * world / seconds / 1e6


# -------------------------------------------------------------- CPU timing --
def time_cpu_oracle(n: int, tau: float, steps: int, warmup: int, budget_s: float):
    """Time the oracle on an n x n x nz slab with nz chosen so that
    steps + warmup slab steps fit in about budget_s seconds."""
    import numpy as np

    from oracle import oracle as o
    o.build()
    threads = o.max_threads()
    o.set_threads(threads)
    # calibrate on a thin slab
    nz_cal = max(1, min(n, 8))
    f = o.init(n, n, nz_cal, 1.0, 0.05)
    ft = np.empty_like(f)
    o.step_pingpong(f, ft, tau)
    t = time.perf_counter()
    o.step_pingpong(ft, f, tau)
    per_cell = (time.perf_counter() - t) / (n * n * nz_cal)
    total = max(1, steps + warmup)
    nz = int(max(1, min(n, budget_s / total / max(per_cell * n * n, 1e-12))))
    f = o.init(n, n, nz, 1.0, 0.05)
    ft = np.empty_like(f)
    for _ in range(warmup):
        o.step_pingpong(f, ft, tau)
        f, ft = ft, f
    t = time.perf_counter()
    for _ in range(steps):
        o.step_pingpong(f, ft, tau)
        f, ft = ft, f
    dt = time.perf_counter() - t
    cells = n * n * nz
    return {"value": cells * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{n}x{n}x{nz} slab (of {n}^3), {steps} steps after {warmup} warm-up, "
                      f"float64 collide+stream, OpenMP {threads} threads",
            "seconds": dt}


def time_reference_build(n: int, nz: int, interval: int):
    """Time the reference's own code (oracle/_ref: its unmodified src/*.cpp
    with the single-process Kokkos / MPI stand-ins) on one rank with every
    host core: the deck's n x n x nz lattice for two report intervals of
    `interval` steps; its own MLUPS line of the second interval is the
    figure (the first absorbs start-up, as tools/parse_scaling.sh:60 of the
    reference discards it).  None when the reference's sources are absent."""
    import tempfile

    from oracle import oracle as o
    exe = o.build_ref()
    if not exe:
        return None
    cores = os.cpu_count() or 1
    deck = f"1.0 0.1 1600\n0.05 {2 * interval} {interval}\n{n} {n} {nz}\n"
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        text = o.run_ref(deck, d, ranks=1, threads=cores, mode="main", timeout=1200, bind=True)
        wall = time.perf_counter() - t0
    mlups = o.parse_mlups(text)
    if len(mlups) < 2:
        raise RuntimeError("the reference's run printed no second interval:\n" + text[-1000:])
    return {"value": mlups[1], "unit": "MLUPS", "cores": cores, "kind": "reference",
            "sample": f"the reference's src/*.cpp (unmodified, single-process Kokkos/MPI stand-ins, OpenMP "
                      f"{cores} threads bound as its job scripts bind them, 1 rank) on a {n}x{n}x{nz} lattice: "
                      f"its own MLUPS over the second {interval}-step report interval of {2 * interval} steps",
            "seconds": interval * n * n * nz / (mlups[1] * 1e6), "wall_s": wall}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    steps = max(1, a.steps)
    interval = min(steps, 10)   # a bounded sample: two report intervals of at most 10 steps
    cb = time_reference_build(a.size, a.size, interval)
    note = ("the reference's own src/*.cpp built unmodified against single-process Kokkos / MPI stand-ins "
            "(oracle/refshim); genuine Kokkos and MPI are not installed")
    if cb is None:
        d = parse_deck_text(a.size)
        cb = time_cpu_oracle(a.size, d["tau"], steps, max(0, a.warmup), budget_s=120.0)
        note = "the reference's sources are absent on this machine: the CPU oracle (a C restatement of " \
               "src/lbm.cpp:78-207) with OpenMP on all host cores"
    line = {"impl": "reference", "metric": "MLUPS", "value": round(cb["value"], 3), "unit": "MLUPS",
            "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
            "ms_per_step": round(a.size ** 3 / (cb["value"] * 1e6) * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic: Taylor-Green initial field",
            "config": workload_config(a, "reference" if cb["kind"] == "reference" else "oracle"),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": round(cb["value"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": note}
    print(json.dumps(line), flush=True)
    return 0


def parse_deck_text(n):
    from oracle import oracle as o
    o.build()
    d = o.parse_deck(f"1.0 0.1 1600\n0.05 1000 100\n{n} {n} {n}\n")
    return {"tau": d.tau, "rho0": d.rho0, "u0": d.u0}


def workload_config(a, engine):
    prec = getattr(a, "precision", "f64")
    desc = {"f64": "float64 distributions", "f32": "float32 distributions",
            "f16dev": "float16 deviations 2^12 (f - w)"}[prec]
    esize = {"f64": 8, "f32": 4, "f16dev": 2}[prec]
    if prec == "f16dev":
        desc += ", %s rounding" % getattr(a, "rounding", "nearest")
    return {"workload": f"taylor-green {a.size}^3 periodic D3Q27, Re=1600, u0=0.05, {desc}",
            "grid": [a.size] * 3, "precision": prec, "engine": engine, "report_every": a.report_every,
            "l2": "inputs larger than L2 (2 arrays x %.2f GB), no flush" % (27 * a.size ** 3 * esize / 1e9),
            "parallelism": "replicas (one independent lattice per GPU)"}


# ------------------------------------------------- the other configurations --
def extended_precision(hbm: float):
    """Precision sweep: 512^3 Taylor-Green, Re 1600, u0 0.05, 2000 steps,
    float64 against float32 and float16 deviations (nearest and stochastic
    rounding), all resident at once; errors against the float64 run at every
    500 steps."""
    from imexlbm_gb300 import sweep
    r = sweep.run(size=512, steps=2000, report=500, log=lambda _: None)
    bpc = {"f64": 432, "f32": 216, "f16dev": 108, "f16dev_sr": 108}
    out = {"workload": "taylor-green 512^3, Re=1600, u0=0.05, 2000 steps, errors vs the float64 run every 500 steps",
           "runs": {}}
    for name, mlups in r["mlups"].items():
        achieved = mlups * 1e6 * bpc[name] / 1e9
        run = {"glups": round(mlups / 1e3, 3), "bytes_per_cell": bpc[name], "roofline_frac": round(achieved / hbm, 4)}
        if name in r["worst"]:
            w = r["worst"][name]
            run.update({"ke_rel_err_max": w["ke_rel"], "u_max_err_over_u0": w["u_max_over_u0"],
                        "mass_drift_rel_max": w["mass_drift_rel"]})
        out["runs"][name] = run
    out["f64_fallback_cells"] = r["f64_fallback_cells"]
    return out


def extended_batched():
    """64 uneven float32 lattices (edges 32-128, seeded), 500 steps in the
    batch kernels against the plain float64 path on the same lattices."""
    from imexlbm_gb300 import batched
    r = batched.run(n=64, steps=500, precision="f32", log=lambda _: None)
    return {"workload": "64 taylor-green lattices, edges {32,48,64,96,128}, Re U[100,3200], u0 U[0.02,0.08], "
                        "random phases, seed 20261203, 500 steps, float32 storage",
            "glups": round(r["batch_mlups"] / 1e3, 3), "fp64_plain_glups": round(r["fp64_plain_mlups"] / 1e3, 3),
            "multiple_of_fp64_plain": round(r["speedup_vs_fp64_plain"], 3), "ke_rel_err_max": r["ke_rel_err_max"],
            "mass_drift_max": r["mass_drift_max"], "cells": r["cells"], "row_launch": list(r["row_launch"]),
            "cell_launch": list(r["launch_shape"])}


def extended_served():
    """The served trace: Poisson arrivals at 50 requests/s for 60 s into the
    continuous-batching server (120 GB budget), float32 / float16-deviation
    solves, 16 float64 spot checks."""
    from imexlbm_gb300 import serve
    r = serve.run(rate=50.0, duration=60.0, budget_gb=120.0, spot=16, log=lambda _: None)
    keys = ("requests", "completed", "diverged", "failed", "unfinished", "ttr_p50_s", "ttr_p99_s", "ttr_max_s",
            "aggregate_mlups", "busy_mlups", "fp64_plain_mlups_on_sample", "aggregate_vs_fp64_plain",
            "ke_rel_err_vs_f64_max", "ke_rel_err_vs_f64_median", "spot_checks", "alone_equals_mix",
            "diverged_checked", "diverged_also_in_f64", "peak_active", "offered_lups")
    out = {"workload": "poisson 50 req/s for 60 s, edges {32..256} weighted, Re log-U[100,5000], u0 U[0.02,0.08], "
                       "steps U[200,5000], f32/f16dev 50/50, 120 GB budget, seed 20261203"}
    out.update({k: r.get(k) for k in keys})
    return out


def run_extended(hbm: float):
    out = {}
    for key, fn in (("precision", lambda: extended_precision(hbm)), ("batched", extended_batched),
                    ("served", extended_served)):
        t0 = time.perf_counter()
        try:
            out[key] = fn()
        except Exception as e:  # keep the main measurement; say what failed
            out[key] = {"error": f"{type(e).__name__}: {e}"}
        out[key]["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def pinned_copy_gbs(nbytes: int, stream):
    """One plain pinned-host <-> device copy of nbytes each way (torch's
    copy_ is a cudaMemcpyAsync), best of three: the link the e2e copies use."""
    import torch
    host = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    dev = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
    best = {"h2d": 0.0, "d2h": 0.0}
    with torch.cuda.stream(stream):
        for _ in range(3):
            for key, (dst, src) in (("h2d", (dev, host)), ("d2h", (host, dev))):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                dst.copy_(src, non_blocking=True)
                e1.record(stream)
                e1.synchronize()
                best[key] = max(best[key], nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    del host, dev
    return {"pinned_h2d_gbs": round(best["h2d"], 1), "pinned_d2h_gbs": round(best["d2h"], 1)}


# ------------------------------------------------------------------ GPU arm --
def run_ours(a):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import imexlbm_gb300 as m
    m.load()
    d = parse_deck_text(a.size)
    n = a.size
    cells = n ** 3
    engine = {"auto": m.IMEX_ENGINE_AUTO, "native": m.IMEX_ENGINE_NATIVE, "fixed": m.IMEX_ENGINE_FIXED}[a.engine]
    prec = {"f64": m.IMEX_F64, "f32": m.IMEX_F32, "f16dev": m.IMEX_F16DEV}[a.precision]
    if prec != m.IMEX_F64:
        engine = m.IMEX_ENGINE_AUTO
    stream = torch.cuda.Stream()
    lat = m.LBM(n, n, n, d["tau"], d["rho0"], d["u0"], precision=prec, engine=engine)
    lat.set_stream(stream.cuda_stream)
    if a.precision == "f16dev":
        lat.set_rounding(m.IMEX_ROUND_STOCHASTIC if a.rounding == "stochastic" else m.IMEX_ROUND_NEAREST)
    if a.launch:
        lat.set_launch(*(int(v) for v in a.launch.split(",")))
    lat.Initialize()
    eng_name = "fixed" if (engine == m.IMEX_ENGINE_FIXED) else "native" if engine == m.IMEX_ENGINE_NATIVE else "auto"
    if prec != m.IMEX_F64:
        eng_name = "float32"
    elif engine == m.IMEX_ENGINE_AUTO:
        eng_name = "fixed" if d["rho0"] >= 0.75 and d["rho0"] <= 1.25 else "native"

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up (includes the first-step collide-only kernel and the launch-shape
    # autotuner, which times each candidate on this lattice)
    lat.step(max(3, a.warmup))
    launch_shape = lat.get_launch()
    lat.fence()
    torch.cuda.synchronize()
    barrier()
    lat.fallback_cells(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = lat.kernel_launches()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier()
        ev0.record(stream)
        lat.step(a.steps)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    gpu_launches = lat.kernel_launches() - launches0
    ms = ev0.elapsed_time(ev1)
    fallback = lat.fallback_cells(reset=True)
    t_max = max_over_ranks(ms, world)
    value = job_mlups(cells, a.steps, world, t_max * 1e-3)
    cons = lat.Conserved()

    # roofline of the fused step kernel: every timed launch is that kernel (the
    # fixed-point engine's run of steps: k_step_fxs, whose first and last
    # launches read / write float64)
    hbm, peak_kind = load_peaks()
    bpc = BYTES_PER_CELL[a.precision]
    # algorithmic bytes per step over the time per step (a launch is one step,
    # or two for the pinned two-steps-per-launch shape)
    achieved = bpc * cells * a.steps / (ms * 1e-3) / 1e9
    kname = {"fixed": "step_fxs", "native": "step_f64", "float32": "step_lowp_" + a.precision}[eng_name]
    if eng_name == "fixed" and launch_shape[0] == 1:
        kname = "two_fxs"
    tr, tr_size = load_traffic(kname)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "peak_kind": peak_kind,
            "traffic": round(tr * cells, 0) if tr is not None else None,
            "traffic_from": (f"ncu dram bytes per cell of a {tr_size} capture ({tr} B), times this launch's "
                             f"{cells} cells (profiles/dram_traffic.json)") if tr is not None else None,
            "kernel": kname, "algorithmic_bytes_per_launch": bpc * cells * (2 if kname == "two_fxs" else 1)}

    # end-to-end through the public API with host buffers
    e2e = None
    if not a.no_e2e:
        nval = 27 * cells
        host = torch.empty(nval, dtype=torch.float64, pin_memory=True)
        lat2 = m.LBM(n, n, n, d["tau"], d["rho0"], d["u0"], precision=prec, engine=engine)
        lat2.set_stream(stream.cuda_stream)
        if a.precision == "f16dev":
            lat2.set_rounding(m.IMEX_ROUND_STOCHASTIC if a.rounding == "stochastic" else m.IMEX_ROUND_NEAREST)
        lat2.Initialize()
        import ctypes
        L = m.load()
        dp = ctypes.cast(host.data_ptr(), ctypes.POINTER(ctypes.c_double))
        L.imex_get_f(lat2.handle, dp, nval)     # f0 into pinned host memory (untimed)
        lat2.step(3)                             # warm the path
        lat2.fence()
        barrier()
        t0 = time.perf_counter()
        m._lib.check(L.imex_set_f(lat2.handle, dp, nval), lat2.handle)
        reports = 0
        done = 0
        while done < a.steps:
            k = min(a.report_every, a.steps - done)
            lat2.step(k)
            done += k
            if done % a.report_every == 0:
                lat2.Conserved()
                reports += 1
        m._lib.check(L.imex_get_f(lat2.handle, dp, nval), lat2.handle)
        dt = max_over_ranks(time.perf_counter() - t0, world)
        lat2.close()
        e2e = {"value": round(job_mlups(cells, a.steps, world, dt), 2), "unit": "MLUPS",
               "h2d_bytes_per_step": round(nval * 8 / a.steps, 1),
               "d2h_bytes_per_step": round((nval * 8 + 40 * reports) / a.steps, 1),
               "what": f"imex_set_f from pinned host, {a.steps} steps with imex_conserved every "
                       f"{a.report_every}, imex_get_f to pinned host (a pending streaming is applied by the "
                       f"kernel that writes the pinned buffer)"}
        del host
        e2e.update(pinned_copy_gbs(nval * 8, stream))

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        # the reference's own code on a 256 x 256 x 32 slab of the lattice
        # (about 10 s), else the oracle port on a bounded slab
        cb = time_reference_build(n, max(1, min(n, 32)), 2)
        if cb is None:
            cb = time_cpu_oracle(n, d["tau"], steps=2, warmup=1, budget_s=20.0)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    lat.close()
    extended = run_extended(hbm) if (rank == 0 and world == 1 and not a.quick and a.size == 256
                                     and a.precision == "f64") else None
    if rank == 0:
        line = {"metric": "MLUPS", "value": round(value, 2), "unit": "MLUPS", "n_gpus": world, "steps": a.steps,
                "warmup": max(3, a.warmup), "ms_per_step": round(t_max / a.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": {"fixed": "s64 fixed-point arithmetic, f64 storage", "native": "f64",
                          "float32": "f32 arithmetic, %s storage" % a.precision}[eng_name],
                "data": "synthetic: Taylor-Green initial field (deterministic, no seed)",
                "config": dict(workload_config(a, eng_name),
                               launch={"stages": launch_shape[0], "rows_per_stage": launch_shape[1],
                                       "ctas_per_sm": launch_shape[2], "threads": launch_shape[3]}),
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": gpu_launches, "clocks": clk.summary(),
                "fallback_cells": fallback, "mass": cons[0], "ke": cons[4],
                "roofline_glups_at_peak": round(hbm / bpc, 3)}
        if extended:
            line.update(extended)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_blocks(a):
    """The lattice decomposed into a.blocks blocks on this GPU (the
    reference's rank layout, imex_domain_*): MLUPS of a.steps steps, wall
    clock around the steps and a final synchronisation."""
    import imexlbm_gb300 as m
    m.load()
    d = parse_deck_text(a.size)
    n = a.size
    with m.Domain(n, n, n, a.blocks, d["tau"], d["rho0"], d["u0"]) as dom:
        dom.Initialize()
        dom.step(max(3, a.warmup))
        dom.fence()
        info0 = dom.info()
        t0 = time.perf_counter()
        dom.step(a.steps)
        dom.fence()
        dt = time.perf_counter() - t0
        info = dom.info()
        cons = dom.Conserved()
    hbm, peak_kind = load_peaks()
    halo = info["halo_values_per_step"]
    line = {"metric": "MLUPS", "value": round(n ** 3 * a.steps / dt / 1e6, 2), "unit": "MLUPS", "n_gpus": 1,
            "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": round(dt / a.steps * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "s64 fixed-point arithmetic, f64 storage", "data": "synthetic: Taylor-Green initial field",
            "config": {"workload": f"taylor-green {n}^3 periodic D3Q27, Re=1600, u0=0.05, float64, decomposed into "
                                   f"{a.blocks} blocks (rank grid {info['grid']})", "blocks": a.blocks,
                       "grid": list(info["grid"]), "halo_values_per_step": halo,
                       "timing": "wall clock around the steps and a synchronisation"},
            "roofline": {"bound": "hbm", "unit": "GB/s", "peak": hbm, "peak_kind": peak_kind,
                         "achieved": round((432 * n ** 3 + 16 * halo) * a.steps / dt / 1e9, 1),
                         "note": "432 B per cell update plus 16 B (read + write) per halo value"},
            "gpu_launches": info["launches"] - info0["launches"], "mass": cons[0], "ke": cons[4]}
    line["roofline"]["frac"] = round(line["roofline"]["achieved"] / hbm, 4)
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    a = parse_args(argv)
    if a.impl == "reference":
        return run_reference(a)
    if a.blocks > 0:
        return run_blocks(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
