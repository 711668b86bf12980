#!/usr/bin/env python
"""Benchmark of the GB300 LES time step (grid-point-steps per second).

Workload: the 128^3 half-channel case (Lx=2pi, Ly=pi, Lz=1; Lagrangian
scale-dependent SGS updated every 5 steps, equilibrium wall model z0=1e-4,
dt=2e-4, seeded log-law IC).  The timed region is the steady state of a run
(jt >= dyn_init), so one step in five carries the dynamic SGS update; the
number of timed steps is rounded up to a multiple of 5.

Our arm (default) times, on the GPU:
  * value       -- the plain FP64 drop-in, fused step with CUDA-graph replay,
                   fields resident in HBM (CUDA events on the library's stream);
  * e2e         -- the same through the C ABI with the prognostic state
                   (u, v, w) copied from pinned host memory before each step
                   and back after it;
  * forms       -- the same measurement for the mixed form (FP32 bulk, FP64
                   pressure solve), and its ratio to the FP64 plain form;
  * roofline    -- the dominant kernel's algorithmic bytes / duration, timed
                   with CUDA events on the launching stream in a profiled pass;
  * cpu_baseline-- the FP64 oracle port (numpy/scipy, threaded FFTs) timed on
                   the host cores on a bounded sample (rank 0, N=1 only).
`--impl reference` times the oracle port alone (the reference itself, Fortran
+ MPI + FFTW, cannot be built here).  Under torchrun each rank runs an
independent replica (the path does not shard; no collective on the data path).
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

METRIC = "grid-pt-steps/s on 1 GB300: FP32 batched vs FP64 plain at <=1% profile error"
UNIT = "grid-pt-steps/s"
WORKLOAD = dict(nx=128, ny=128, Nz=128, dyn_init=5, cs_count=5)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--forms", default="fp64,mixed,batched")
    ap.add_argument("--serve", action="store_true", help="run the served request stream instead")
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--validate", choices=["B", "C"], help="long-run statistics of the mixed form vs FP64: "
                    "B = 128^3 half channel, C = 256x256x192 wind farm with 12 actuator disks")
    ap.add_argument("--val-steps", type=int, default=None)
    ap.add_argument("--val-window", type=int, default=2000)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, idx: int):
        self.idx = idx
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{idx}.csv") if os.path.isdir(
            os.path.join(ROOT, "gpurun_out")) else f"/tmp/lesgo_clocks_{os.getpid()}.csv"

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def time_form(precision, args, torch, world):
    """Device-resident throughput of the fused step (CUDA events on the
    library's stream), plus a profiled pass for the per-kernel roofline."""
    from lesgo_gb300.solver import LesgoGPU
    n = args.grid
    cfg = dict(WORKLOAD, nx=n, ny=n, Nz=n, precision=precision)
    g = LesgoGPU(**cfg)
    g.init_ic(1)
    steps = max(5, (args.steps + 4) // 5 * 5)
    warm = max(args.warmup, cfg["dyn_init"] + 1)
    warm = (warm + 4) // 5 * 5   # timed region starts at a multiple of 5 (phase of the SGS update)
    g.step(warm)
    g.sync()
    stream = torch.cuda.ExternalStream(g.stream_ptr())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    g.step(steps)
    e1.record(stream)
    g.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = (4 * g.launches_per_step(False) + g.launches_per_step(True)) * steps // 5
    # profiled pass (eager, event pair per kernel) for the roofline
    g.profile(True)
    g.step(5)
    rep = g.profile_report()
    g.profile(False)
    diag = g.diag()
    g.close()
    return dict(ms=ms, steps=steps, pts=n * n * n, launches=launches, profile=rep, diag=diag, cfg=cfg)


BATCH_GRIDS = [(48, 48, 48), (64, 64, 64), (96, 96, 64), (128, 64, 64)]


def batch_instances(n=48, seed=2024):
    """The 48-instance ensemble: grid drawn from BATCH_GRIDS, z0 log-uniform
    in [1e-5, 1e-3], own IC seed."""
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        g = BATCH_GRIDS[int(rng.integers(len(BATCH_GRIDS)))]
        zo = math.exp(rng.uniform(math.log(1e-5), math.log(1e-3)))
        out.append((g, zo, 5000 + i))
    return out


def time_batched(args, torch):
    """All 48 instances in the mixed form: one batch handle per grid size
    (every kernel advances the whole class in one launch), classes on their
    own streams and overlapping; against the same instances run one at a
    time in the plain FP64 form."""
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    inst = batch_instances()
    by_grid = {}
    for g, zo, seed in inst:
        by_grid.setdefault(g, []).append((zo, seed))
    batches = []
    for g, lst in by_grid.items():
        b = LesgoBatch(len(lst), nx=g[0], ny=g[1], Nz=g[2], precision="mixed", dyn_init=5, cs_count=5)
        for zo, seed in lst:
            b.add(zo, seed)
        batches.append((g, len(lst), b))
    for _, _, b in batches:
        b.step(10)
    for _, _, b in batches:
        b.sync()
    steps = max(5, (args.steps + 4) // 5 * 5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for _, _, b in batches:
            b.step(1)
    for _, _, b in batches:
        b.sync()
    dt = time.perf_counter() - t0
    pts = sum(g[0] * g[1] * g[2] * n for g, n, _ in batches)
    launches = sum((4 * b.launches_per_step(False) + b.launches_per_step(True)) for _, _, b in batches) * steps // 5
    for _, _, b in batches:
        b.close()
    # plain FP64, one instance at a time: steady-state step time per grid
    t64 = {}
    for g in by_grid:
        s = LesgoGPU(nx=g[0], ny=g[1], Nz=g[2], precision="fp64", dyn_init=5, cs_count=5)
        s.init_ic(1)
        s.step(10)
        s.sync()
        t1 = time.perf_counter()
        s.step(10)
        s.sync()
        t64[g] = (time.perf_counter() - t1) / 10
        s.close()
    seq_time = sum(t64[g] for g, _, _ in inst)
    fp64_one_at_a_time = sum(g[0] * g[1] * g[2] for g, _, _ in inst) / seq_time
    return dict(value=pts * steps / dt, ms_per_step=dt * 1e3 / steps, instances=len(inst),
                grids={f"{g[0]}x{g[1]}x{g[2]}": n for g, n, _ in batches}, launches=launches,
                fp64_one_at_a_time=fp64_one_at_a_time, ratio_vs_fp64_one_at_a_time=pts * steps / dt / fp64_one_at_a_time)


def time_e2e(args, torch):
    """Through the C ABI with host buffers: per step, u, v, w go host->device
    from pinned memory, one fused step runs, and u, v, w come back."""
    from lesgo_gb300.solver import LesgoGPU
    n = args.grid
    g = LesgoGPU(**dict(WORKLOAD, nx=n, ny=n, Nz=n, precision="fp64"))
    g.init_ic(1)
    g.step(10)
    g.sync()
    shape = (g.nz + 1, g.ny, g.ld)
    host = {k: torch.empty(shape, dtype=torch.float64, pin_memory=True) for k in ("u", "v", "w")}
    for k, t in host.items():
        g.get_ptr(k, t.data_ptr(), 0, g.nz)
    steps = max(5, (args.steps + 4) // 5 * 5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for k, t in host.items():
            g.set_ptr(k, t.data_ptr(), 0, g.nz)
        g.step(1)
        for k, t in host.items():
            g.get_ptr(k, t.data_ptr(), 0, g.nz)
    g.sync()
    dt = time.perf_counter() - t0
    nbytes = 3 * shape[0] * shape[1] * shape[2] * 8
    g.close()
    return dict(value=n * n * n * steps / dt, h2d=nbytes, d2h=nbytes)


def cpu_baseline(args, steps=2):
    from oracle.lesgo_oracle import Oracle, Params
    n = args.grid
    cores = os.cpu_count() or 1
    o = Oracle(Params(nx=n, ny=n, Nz=n, dyn_init=1, cs_count=2))
    o.workers = cores
    o.set_ic(1)
    o.step()          # first step (Euler, Cs init)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()      # one of the two carries the dynamic SGS update (cs_count=2)
    dt = time.perf_counter() - t0
    return dict(value=n * n * n * steps / dt, unit=UNIT, cores=cores, kind="port",
                sample=f"{steps} steps of the {n}^3 FP64 oracle (numpy + scipy.fft with {cores} workers), "
                       "one with the dynamic SGS update")


def dominant(rep, hbm):
    name, (cnt, tot_ms, tot_b) = max(rep.items(), key=lambda kv: kv[1][1])
    per_ms = tot_ms / cnt
    per_b = tot_b / cnt
    achieved = per_b / (per_ms * 1e-3) / 1e9
    total_ms = sum(v[1] for v in rep.values())
    return name, dict(bound="hbm", achieved=achieved, peak=hbm, unit="GB/s", frac=achieved / hbm,
                      traffic=None, kernel=name, share=tot_ms / total_ms, bytes_per_launch=per_b,
                      ms_per_launch=per_ms)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from lesgo_gb300 import _lib
    _lib.load()
    hbm, peak_kind = peaks()
    forms = [f for f in args.forms.split(",") if f]
    with Clocks(local) as clk:
        res = {f: time_form(f, args, torch, world) for f in forms if f in ("fp64", "mixed")}
    clocks = clk.summary()
    head = res.get("fp64") or next(iter(res.values()))
    ms = head["ms"]
    if world > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = head["pts"] * head["steps"] * world / (ms * 1e-3)
    batched = time_batched(args, torch) if "batched" in forms else None
    e2e = time_e2e(args, torch) if rank == 0 else None
    cpu = cpu_baseline(args) if (rank == 0 and world == 1 and not args.no_cpu) else None
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    kname, roof = dominant(head["profile"], hbm)
    roof["peak_kind"] = peak_kind
    traffic = load_traffic(kname, args.grid, "fp64")
    roof["traffic"] = traffic
    out_forms = {}
    for f, r in res.items():
        v = r["pts"] * r["steps"] * world / (r["ms"] * 1e-3)
        kn, rf = dominant(r["profile"], hbm)
        out_forms[f] = dict(value=v, ms_per_step=r["ms"] / r["steps"], dominant_kernel=kn,
                            dominant_frac=rf["frac"], dominant_share=rf["share"], diag=r["diag"],
                            kernels=r["profile"])
    if "fp64" in out_forms and "mixed" in out_forms:
        out_forms["mixed_vs_fp64"] = out_forms["mixed"]["value"] / out_forms["fp64"]["value"]
    if batched:
        out_forms["mixed_batched"] = batched
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": head["steps"],
        "warmup": args.warmup, "ms_per_step": ms / head["steps"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded log-law + noise IC)",
        "config": {"workload": f"half-channel LES {args.grid}^3, plain FP64 drop-in (fused, graph-replayed)",
                   "grid": [args.grid, args.grid, args.grid], "dt": 2e-4, "sgs": "Lagrangian scale-dependent, every 5 steps",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": "working set > L2 (about 0.9 GB of fields)"},
        "e2e": {"value": e2e["value"], "unit": UNIT, "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"]},
        "gpu_launches": head["launches"],
        "roofline": roof,
        "forms": out_forms,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "kernels": head["profile"],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def load_traffic(kernel, grid, form):
    """dram bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(f"{form}:{grid}:{kernel}")
    except Exception:
        return None


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.lesgo_oracle import Oracle, Params
    n = args.grid
    cores = os.cpu_count() or 1
    o = Oracle(Params(nx=n, ny=n, Nz=n, dyn_init=1, cs_count=5))
    o.workers = cores
    o.set_ic(1)
    for _ in range(max(1, args.warmup // 5)):
        o.step()
    steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    value = n * n * n * steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded log-law + noise IC)",
        "config": {"workload": f"half-channel LES {n}^3, plain FP64 drop-in (fused, graph-replayed)",
                   "grid": [n, n, n]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{steps} full {n}^3 steps of the FP64 oracle port (numpy + scipy.fft, "
                                   f"{cores} workers); the Fortran reference needs gfortran + MPI + FFTW, absent"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Served stream: Poisson arrivals; grid from {64^3, 128x128x96,
    192x192x128}; z0 log-uniform in [1e-5, 1e-3]; 0-16 actuator disks;
    200-2000 steps; 150 GB admission budget; mixed form.  Reports p50/p99
    completion latency and aggregate grid-point-steps/s next to the plain FP64
    form run one request at a time (from measured steady-state step times)."""
    import torch
    torch.cuda.set_device(0)
    from lesgo_gb300.serve import GpuBackend, Server, poisson_requests
    from lesgo_gb300.solver import LesgoGPU
    grids = [(64, 64, 64), (128, 128, 96), (192, 192, 128)]
    base = dict(dyn_init=100, cs_count=5)
    # arrival rate sized to keep the GPU busy: mean work / mean service time
    reqs = poisson_requests(args.requests, rate=4.0, grids=grids, steps_range=(200, 2000), seed=7, turbines_max=16)
    srv = Server(GpuBackend("mixed", **base), budget_bytes=150e9, chunk_slots=8, cs_count=5)
    rep = srv.run(reqs)
    t64 = {}
    for g in grids:
        s = LesgoGPU(nx=g[0], ny=g[1], Nz=g[2], precision="fp64", **base)
        s.init_ic(1)
        s.step(5)
        s.sync()
        t1 = time.perf_counter()
        s.step(10)
        s.sync()
        t64[g] = (time.perf_counter() - t1) / 10
        s.close()
    seq = sum(r.steps * t64[r.grid] for r in reqs)
    one_at_a_time = sum(r.points * r.steps for r in reqs) / seq
    line = {"metric": "served LES requests: aggregate grid-pt-steps/s and completion latency", "unit": UNIT,
            "value": rep["throughput"], "p50_s": rep["p50_s"], "p99_s": rep["p99_s"], "requests": rep["requests"],
            "wall_s": rep["wall_s"], "busy_frac": rep["busy_frac"], "fp64_one_at_a_time": one_at_a_time,
            "ratio_vs_fp64_one_at_a_time": rep["throughput"] / one_at_a_time, "budget_gb": 150,
            "config": {"grids": [list(g) for g in grids], "steps": [200, 2000], "turbines": [0, 16],
                       "arrival_rate_per_s": 4.0, "form": "mixed (FP32 bulk, FP64 pressure solve)"}}
    print(json.dumps(line), flush=True)


def run_validate(args):
    """Mean profile <u>(z), resolved <u'w'>(z) and (C) per-turbine power of
    the mixed form against the plain FP64 form over a long run, sampled every
    10 steps over the last `--val-window` steps."""
    import torch
    torch.cuda.set_device(0)
    from lesgo_gb300.validate import compare, long_run, wind_farm_4x3
    if args.validate == "B":
        kw = dict(nx=128, ny=128, Nz=128)
        turbines = None
        steps = args.val_steps or 4000
    else:
        # the time step the reference's own configuration uses: use_cfl_dt
        # with cfl = 0.0625.  A fixed dt = 2e-4 is unstable at this
        # resolution (NaN near step 110), and dt = 1e-4 with the 12 disks
        # near step 1900, in both forms
        kw = dict(nx=256, ny=256, Nz=192, use_cfl_dt=True, cfl=0.0625)
        turbines = wind_farm_4x3()
        steps = args.val_steps or 3000
    window = min(args.val_window, steps)
    runs = {prec: long_run(prec, steps, window, 10, 1, turbines, **kw) for prec in ("fp64", "mixed")}
    nz = kw["Nz"] + 1
    r = compare(runs["mixed"], runs["fp64"], nz)
    line = {"validate": args.validate, "grid": [kw["nx"], kw["ny"], kw["Nz"]], "steps": steps, "window": window,
            "nskip": 10, "samples": runs["fp64"]["samples"], "turbines": len(turbines or []),
            "bar": "u_linf <= 0.01 and uw_linf <= 0.01", "pass": r["u_linf"] <= 0.01 and r["uw_linf"] <= 0.01,
            **r,
            "rmsdiv": {k: v["diag"]["rmsdiv"] for k, v in runs.items()},
            "wall_s": {k: v["wall_s"] for k, v in runs.items()},
            "profile_u_fp64": runs["fp64"]["u"].tolist(), "profile_u_mixed": runs["mixed"]["u"].tolist(),
            "profile_upwp_fp64": runs["fp64"]["upwp"].tolist(),
            "profile_upwp_mixed": runs["mixed"]["upwp"].tolist()}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.validate:
        run_validate(args)
    elif args.serve:
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
