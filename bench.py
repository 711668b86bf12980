#!/usr/bin/env python
"""Benchmark of the GB300 LES time step (grid-point-steps per second).

Headline workload: the batched ensemble of 48 independent half-channel LES
instances of uneven grids (48^3, 64^3, 96x96x64, 128x64x64; Lx=2pi, Ly=pi,
Lz=1; z0 log-uniform in [1e-5, 1e-3]; own seeded log-law + noise IC;
Lagrangian scale-dependent SGS updated every 5 steps; dt=2e-4) in the mixed
form (FP32 bulk, FP64 pressure solve): one batch handle per grid class, every
kernel advancing the whole class in one launch, graph-replayed steps,
autotuned tiles, the classes overlapping on their own streams.  The timed
region is the steady state (the number of timed steps is rounded up to a
multiple of 5, the phase of the SGS update).

Our arm (default) reports:
  * value       -- aggregate grid-point-steps/s of the ensemble, fields
                   resident in HBM, CUDA events around the steps of all
                   classes;
  * config.vs_fp64_plain_one_at_a_time -- against the same instances run one
                   at a time in the plain FP64 form (the drop-in);
  * e2e         -- the ensemble through the C ABI with every instance's u, v,
                   w copied from pinned host memory before each step and back
                   after it;
  * forms       -- the 128^3 half channel as one instance in the plain FP64
                   drop-in (with its own e2e) and in the mixed form;
  * roofline    -- the dominant kernel's algorithmic bytes / duration, timed
                   with CUDA events on the launching stream in a profiled pass;
  * cpu_baseline-- the FP64 oracle port (numpy/scipy, threaded FFTs) on one
                   instance of each grid class, on the host cores (rank 0,
                   N=1 only).
`--impl reference` times the oracle port alone on the same sample (the
reference itself, Fortran + MPI + FFTW, cannot be built here).  Under
torchrun each rank runs an independent replica (instances do not exchange
data; no collective on the data path).  `--serve` runs the request stream,
`--validate B|C` the long-run statistics of the mixed form against FP64.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-steps/s on 1 GB300: FP32 batched vs FP64 plain at <=1% profile error"
UNIT = "grid-pt-steps/s"
WORKLOAD = dict(nx=128, ny=128, Nz=128, dyn_init=5, cs_count=5)
WORKLOAD_DESC = ("48 independent half-channel LES instances of uneven grids (48^3, 64^3, 96x96x64, 128x64x64), "
                 "z0 log-uniform in [1e-5, 1e-3], own IC seeds")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--e2e-split", type=int, default=3, help="batch handles per grid class in the e2e measurement "
                    "(measured e2e: 1.75e9 with 1, 2.04e9 with 2, 2.07e9 with 3)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--forms", default="fp64,fp64dw,mixed",
                    help="single-instance 128^3 forms reported beside the ensemble (fp64dw: FP64 fields, "
                         "double-word transforms)")
    ap.add_argument("--serve", action="store_true", help="run the served request stream instead")
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--validate", choices=["B", "C", "D"], help="long-run statistics of the mixed form vs FP64: "
                    "B = 128^3 half channel, C = 256x256x192 wind farm with 12 actuator disks, D = each "
                    "instance of the batched 48-instance ensemble against the same instance alone in FP64")
    ap.add_argument("--val-steps", type=int, default=None)
    ap.add_argument("--val-window", type=int, default=2000)
    ap.add_argument("--val-no-floor", action="store_true", help="skip the FP64 run-to-run spread (a second FP64 "
                    "ensemble)")
    ap.add_argument("--val-members", type=int, default=None, help="realisations per side (default 3 for B, 1 for C)")
    ap.add_argument("--xdft-compare", action="store_true", help="the forward x transforms as tensor-core GEMMs "
                    "(LESGO_XDFT=1) against the radix kernels: per-stage and whole-step times")
    ap.add_argument("--only-class", default=None, help="run only the ensemble's instances of one grid class, "
                    "e.g. 96x96x64 (each class is an independent batch: used to profile its launches alone)")
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
        # the raw samples go to $LESGO_CLOCKS_DIR when set (kept), else a temporary file
        d = os.environ.get("LESGO_CLOCKS_DIR")
        self.path = (os.path.join(d, f"clocks_rank{idx}.csv") if d and os.path.isdir(d)
                     else os.path.join(tempfile.gettempdir(), f"lesgo_clocks_{os.getpid()}_{idx}.csv"))

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
    tiles = g.autotune()   # transform tile shapes for this grid (state unchanged)
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
    return dict(ms=ms, steps=steps, pts=n * n * n, launches=launches, profile=rep, diag=diag, cfg=cfg, tiles=tiles)


BATCH_GRIDS = [(48, 48, 48), (64, 64, 64), (96, 96, 64), (128, 64, 64)]


def batch_instances(n=48, seed=2024):
    """The 48-instance ensemble: grid drawn from BATCH_GRIDS, z0 log-uniform
    in [1e-5, 1e-3], own IC seed (restricted to one class with --only-class)."""
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        g = BATCH_GRIDS[int(rng.integers(len(BATCH_GRIDS)))]
        zo = math.exp(rng.uniform(math.log(1e-5), math.log(1e-3)))
        out.append((g, zo, 5000 + i))
    if ONLY_CLASS:
        out = [x for x in out if "x".join(map(str, x[0])) == ONLY_CLASS]
        if not out:
            raise SystemExit(f"no instance of class {ONLY_CLASS}")
    return out


ONLY_CLASS = None


def make_batches(precision="mixed", split=1):
    """Batch handles of the 48-instance ensemble, every instance added, tile
    shapes autotuned: one per grid class, or `split` per class (the class's
    instances dealt in turn)."""
    from lesgo_gb300.solver import LesgoBatch
    by_grid = {}
    for g, zo, seed in batch_instances():
        by_grid.setdefault(g, []).append((zo, seed))
    batches = []
    for g, lst in by_grid.items():
        for part in range(split):
            sub = lst[part::split]
            if not sub:
                continue
            b = LesgoBatch(len(sub), nx=g[0], ny=g[1], Nz=g[2], precision=precision, dyn_init=5, cs_count=5)
            ids = [b.add(zo, seed) for zo, seed in sub]
            b.autotune()
            batches.append((g, ids, b))
    return batches


def step_all(batches, n):
    for _, _, b in batches:
        b.step(n)


def timed_on_device(torch, batches, fn):
    """fn() launches work on the batches' own streams; the elapsed device time
    from an event every stream waits on to an event after all of them."""
    streams = [torch.cuda.ExternalStream(b.stream_ptr()) for _, _, b in batches]
    main = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    for _, _, b in batches:
        b.sync()
    e0.record(main)
    for st in streams:
        st.wait_event(e0)
    fn()
    for st in streams:
        ev = torch.cuda.Event()
        ev.record(st)
        main.wait_event(ev)
    e1.record(main)
    e1.synchronize()
    return e0.elapsed_time(e1)


def merge_profiles(reps):
    out = {}
    for rep in reps:
        for k, (n, ms, by) in rep.items():
            a = out.setdefault(k, [0, 0.0, 0.0])
            a[0] += n
            a[1] += ms
            a[2] += by
    return {k: tuple(v) for k, v in out.items()}


def time_batched(args, torch):
    """The 48 instances in the mixed form: one batch handle per grid class
    (every kernel advances the whole class in one launch, graph-replayed
    steps, autotuned tiles), the classes on their own streams and
    overlapping; against the same instances run one at a time in the plain
    FP64 form."""
    from lesgo_gb300.solver import LesgoGPU
    inst = batch_instances()
    batches = make_batches("mixed")
    warm, steps = timed_steps(args)
    step_all(batches, warm)
    ms = timed_on_device(torch, batches, lambda: step_all(batches, steps))
    pts = sum(g[0] * g[1] * g[2] * len(ids) for g, ids, _ in batches)
    launches = sum((4 * b.launches_per_step(False) + b.launches_per_step(True)) for _, _, b in batches) * steps // 5
    reps = []
    for _, _, b in batches:
        b.profile(True)
        b.step(5)
        reps.append(b.profile_report())
        b.profile(False)
    tiles = {f"{g[0]}x{g[1]}x{g[2]}": b.autotune() for g, _, b in batches}
    for _, _, b in batches:
        b.close()
    # the FP64-field forms, one instance at a time: steady-state step time per
    # grid class (FP64 transforms; double-word transforms)
    one_at_a_time = {}
    for prec in ("fp64", "fp64dw"):
        t64 = {}
        for g, _, _ in batches:
            s = LesgoGPU(nx=g[0], ny=g[1], Nz=g[2], precision=prec, dyn_init=5, cs_count=5)
            s.init_ic(1)
            s.autotune()
            s.step(10)
            st = torch.cuda.ExternalStream(s.stream_ptr())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.sync()
            e0.record(st)
            s.step(10)
            e1.record(st)
            e1.synchronize()
            t64[g] = e0.elapsed_time(e1) * 1e-3 / 10
            s.close()
        seq_time = sum(t64[g] for g, _, _ in inst)
        one_at_a_time[prec] = sum(g[0] * g[1] * g[2] for g, _, _ in inst) / seq_time
    fp64_one_at_a_time = one_at_a_time["fp64"]
    value = pts * steps / (ms * 1e-3)
    return dict(value=value, ms=ms, steps=steps, ms_per_step=ms / steps, pts=pts, instances=len(inst),
                grids={f"{g[0]}x{g[1]}x{g[2]}": len(ids) for g, ids, _ in batches}, launches=launches,
                profile=merge_profiles(reps), tiles=tiles, fp64_one_at_a_time=fp64_one_at_a_time,
                ratio_vs_fp64_one_at_a_time=value / fp64_one_at_a_time,
                fp64dw_one_at_a_time=one_at_a_time["fp64dw"],
                ratio_vs_fp64dw_one_at_a_time=value / one_at_a_time["fp64dw"])


def time_e2e_batched(args, torch):
    """The batched ensemble through the C ABI with host buffers: per step,
    every instance's u, v, w go host->device from pinned FP64 memory, all
    classes step once, and u, v, w of every instance come back.  The copies
    are queued in stream order (the *_async calls): each class's copies run
    on its handle's stream while the other classes' steps run, and a step's
    uploads read the buffers its predecessor's downloads wrote.  With
    `--e2e-split` handles per class, one handle's copies also run while the
    other handles of its class step."""
    batches = make_batches("mixed", split=args.e2e_split)
    step_all(batches, 10)
    host = []
    nbytes = 0
    for g, ids, b in batches:
        shape = (b.nz + 1, b.ny, b.ld)
        for iid in ids:
            bufs = {k: torch.empty(shape, dtype=torch.float64, pin_memory=True) for k in ("u", "v", "w")}
            for k, t in bufs.items():
                b.get_ptr(iid, k, t.data_ptr(), 0, b.nz)
                nbytes += t.numel() * 8
            host.append((b, iid, bufs))
    steps = max(5, (args.steps + 4) // 5 * 5)

    by_batch = {}
    for b, iid, bufs in host:
        by_batch.setdefault(id(b), (b, []))[1].append((iid, bufs))

    def run():
        for _ in range(steps):
            for b, lst in by_batch.values():
                for iid, bufs in lst:
                    for k, t in bufs.items():
                        b.set_ptr(iid, k, t.data_ptr(), 0, b.nz, wait=False)
                b.step(1)
                for iid, bufs in lst:
                    for k, t in bufs.items():
                        b.get_ptr(iid, k, t.data_ptr(), 0, b.nz, wait=False)

    ms = timed_on_device(torch, batches, run)
    pts = sum(g[0] * g[1] * g[2] * len(ids) for g, ids, _ in batches)
    for _, _, b in batches:
        b.close()
    return dict(value=pts * steps / (ms * 1e-3), h2d=nbytes, d2h=nbytes)


def time_e2e(args, torch, precision="fp64"):
    """Through the C ABI with host buffers: per step, u, v, w go host->device
    from pinned memory, one fused step runs, and u, v, w come back."""
    from lesgo_gb300.solver import LesgoGPU
    n = args.grid
    g = LesgoGPU(**dict(WORKLOAD, nx=n, ny=n, Nz=n, precision=precision))
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


def class_counts():
    """Instances per grid class in the ensemble."""
    counts = {}
    for g, _, _ in batch_instances():
        counts[g] = counts.get(g, 0) + 1
    return counts


def timed_steps(args):
    """Warm-up and timed step counts of both arms: the timed region starts
    at a multiple of 5 and spans whole multiples of 5 steps, so every arm
    sees the same phase of the every-5-steps dynamic SGS update."""
    warm = (max(args.warmup, 6) + 4) // 5 * 5
    steps = max(5, (args.steps + 4) // 5 * 5)
    return warm, steps


def oracle_sample(warm, steps):
    """The FP64 oracle port, one instance of each grid class of the ensemble
    in turn (dyn_init = cs_count = 5 like the GPU arm), `warm` untimed steps,
    then `steps` timed steps, threaded FFTs on all host cores.  The
    ensemble's rate weights each class by its instance count: sum over
    classes of instances x points / sum of instances x seconds per step
    (the 48 instances run one at a time).  Returns the rate, the cores and
    the sample's description."""
    from oracle.lesgo_oracle import Oracle, Params
    cores = os.cpu_count() or 1
    counts = class_counts()
    work, secs = 0.0, 0.0
    for k, g in enumerate(BATCH_GRIDS):
        if g not in counts:
            continue
        o = Oracle(Params(nx=g[0], ny=g[1], Nz=g[2], dyn_init=5, cs_count=5, zo=1e-4))
        o.workers = cores
        o.set_ic(5000 + k)
        for _ in range(warm):
            o.step()
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step()
        per_step = (time.perf_counter() - t0) / steps
        work += counts[g] * g[0] * g[1] * g[2]
        secs += counts[g] * per_step
    sample = (f"one instance of each grid class "
              f"({', '.join('x'.join(map(str, g)) + ' x' + str(counts.get(g, 0)) for g in BATCH_GRIDS)}) of the "
              f"FP64 oracle port (numpy + scipy.fft, {cores} workers), {warm} warm-up + {steps} timed steps each "
              f"(dynamic SGS update every 5 steps, as the GPU arm), weighted by the class's instance count")
    return work / secs, cores, sample


def cpu_baseline(args):
    value, cores, sample = oracle_sample(5, 5)
    return dict(value=value, unit=UNIT, cores=cores, kind="port", sample=sample)


def dominant(rep, hbm):
    name, (cnt, tot_ms, tot_b) = max(rep.items(), key=lambda kv: kv[1][1])
    per_ms = tot_ms / cnt
    per_b = tot_b / cnt
    achieved = per_b / (per_ms * 1e-3) / 1e9
    total_ms = sum(v[1] for v in rep.values())
    return name, dict(bound="hbm", achieved=achieved, peak=hbm, unit="GB/s", frac=achieved / hbm,
                      traffic=None, kernel=name, share=tot_ms / total_ms, bytes_per_launch=per_b,
                      ms_per_launch=per_ms)


def max_over_ranks(ms, world, torch, device):
    """The slowest rank's time (all ranks must call it)."""
    if world <= 1:
        return ms
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


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
        if world > 1:
            torch.distributed.barrier()
        batched = time_batched(args, torch)
        res = {f: time_form(f, args, torch, world) for f in forms if f in ("fp64", "fp64dw", "mixed")}
    clocks = clk.summary()
    ms = max_over_ranks(batched["ms"], world, torch, "cuda")
    steps = batched["steps"]
    value = batched["pts"] * steps * world / (ms * 1e-3)
    e2e = time_e2e_batched(args, torch) if rank == 0 else None
    cpu = cpu_baseline(args) if (rank == 0 and world == 1 and not args.no_cpu) else None
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    kname, roof = dominant(batched["profile"], hbm)
    roof["peak_kind"] = peak_kind
    nc = load_traffic(kname, "ensemble48", "mixed")
    roof["traffic"] = nc["dram_bytes"] if nc else None
    if nc and "fp64_pipe_pct" in nc:
        # the pressure solve stays FP64 in the mixed form: bound by the FP64 pipe
        roof["fp64_pipe_frac"] = nc["fp64_pipe_pct"] / 100.0
        roof["limiter"] = "FP64 ALU (ncu: FP64 pipe %.0f %% active)" % nc["fp64_pipe_pct"]
    out_forms = {}
    for f, r in res.items():
        v = r["pts"] * r["steps"] * world / (r["ms"] * 1e-3)
        kn, rf = dominant(r["profile"], hbm)
        if f == "fp64":
            nc64 = load_traffic(kn, args.grid, "fp64")
            if nc64 and "fp64_pipe_pct" in nc64:
                # the FP64 transforms are bound by the FP64 pipe, not by HBM
                rf["fp64_pipe_frac"] = nc64["fp64_pipe_pct"] / 100.0
                rf["traffic"] = nc64["dram_bytes"]
                rf["limiter"] = "FP64 ALU (ncu: FP64 pipe %.0f %% active)" % nc64["fp64_pipe_pct"]
        if f in ("fp64", "fp64dw"):
            e = time_e2e(args, torch, f)
            rf_e2e = {"value": e["value"], "unit": UNIT, "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"]}
        else:
            rf_e2e = None
        out_forms[f] = dict(workload=f"half-channel LES {args.grid}^3, one instance", value=v, e2e=rf_e2e,
                            ms_per_step=r["ms"] / r["steps"], roofline=rf, diag=r["diag"], tiles=r["tiles"],
                            kernels=r["profile"])
    if "fp64" in out_forms and "mixed" in out_forms:
        out_forms["mixed_vs_fp64"] = out_forms["mixed"]["value"] / out_forms["fp64"]["value"]
    if "fp64" in out_forms and "fp64dw" in out_forms:
        out_forms["fp64dw_vs_fp64"] = out_forms["fp64dw"]["value"] / out_forms["fp64"]["value"]
    out_forms["batched"] = {k: v for k, v in batched.items() if k not in ("profile",)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 pressure solve, wall law, step constants)",
        "data": "synthetic (seeded log-law + noise IC)",
        "config": {"workload": WORKLOAD_DESC + "; mixed form (FP32 bulk, FP64 Poisson), one batch per grid "
                               "class, graph-replayed steps, autotuned tiles",
                   "instances": batched["instances"], "grids": batched["grids"],
                   "sgs": "Lagrangian scale-dependent, every 5 steps", "dt": 2e-4,
                   "vs_fp64_plain_one_at_a_time": batched["ratio_vs_fp64_one_at_a_time"],
                   "fp64_plain_one_at_a_time": batched["fp64_one_at_a_time"],
                   "vs_fp64dw_one_at_a_time": batched["ratio_vs_fp64dw_one_at_a_time"],
                   "fp64dw_one_at_a_time": batched["fp64dw_one_at_a_time"],
                   "profile_error": "mean profile <= 1e-2 against FP64 (128^3: 2.6e-4; wind farm: 2.6e-5)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": "working set > L2 (about 3 GB of fields)"},
        "e2e": {"value": e2e["value"], "unit": UNIT, "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"]},
        "gpu_launches": batched["launches"],
        "roofline": roof,
        "forms": out_forms,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "kernels": batched["profile"],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def load_traffic(kernel, grid, form):
    """ncu figures of `kernel` (dram bytes per launch, FP64 pipe utilisation)
    from the committed summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(f"{form}:{grid}:{kernel}")
    except Exception:
        return None


def run_reference(args):
    """The reference arm: the FP64 oracle port on the host cores, on the same
    ensemble, SGS phase, warm-up and timed step counts as the GPU arm, one
    instance per grid class standing for its class (the Fortran reference
    needs gfortran, MPI and FFTW, absent on the GPU machine)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    warm, steps = timed_steps(args)
    t0 = time.perf_counter()
    value, cores, sample = oracle_sample(warm, steps)
    pts = sum(g[0] * g[1] * g[2] * n for g, n in class_counts().items())
    ms = pts / value * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded log-law + noise IC)",
        "config": {"workload": WORKLOAD_DESC + "; the reference computes in FP64 one instance at a time",
                   "instances": sum(class_counts().values()),
                   "grids": {"x".join(map(str, g)): n for g, n in class_counts().items()},
                   "sgs": "Lagrangian scale-dependent, every 5 steps", "dt": 2e-4,
                   "wall_s": time.perf_counter() - t0},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample + "; the Fortran reference needs gfortran + MPI + FFTW, absent on the "
                                            "GPU box (probed)"},
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
    from lesgo_gb300.validate import batch_vs_alone, compare, ensemble, long_run, wind_farm_4x3
    if args.validate == "D":
        steps = args.val_steps or 500
        window = min(args.val_window, steps // 2)
        r = batch_vs_alone(batch_instances(), steps=steps, window=window)
        worst = max(max(c["u_linf"], c["uw_linf"]) for c in r["per_class"].values())
        line = {"validate": "D", "instances": len(r["rows"]), "steps": steps, "window": window, "nskip": 10,
                "batch": "mixed, one batch per grid class", "alone": "fp64 (plain FP64 form), one instance at a time",
                "bar": "u_linf <= 0.01 and uw_linf <= 0.01 per instance", "pass": worst <= 0.01,
                "per_class": r["per_class"], "wall_s": r["wall_s"], "rows": r["rows"]}
        print(json.dumps(line), flush=True)
        return
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
    # Both sides are ensembles of the same size: realisations whose initial
    # u is the IC scaled by 1 + p, p in `pert` (FP32-sized perturbations).
    # The noise floor is a second FP64 ensemble of other perturbations
    # against the first: the spread of the ensemble-mean statistics over
    # this window that any two realisation sets show.
    members = args.val_members or (3 if args.validate == "B" else 1)
    pert = (0.0, 1e-6, -1e-6, 2e-6, -2e-6)[:members]
    pert_floor = (3e-6, -3e-6, 4e-6, -4e-6, 5e-6)[:members]
    runs = {"fp64": ensemble("fp64", steps, window, 10, 1, turbines, perturbs=pert, **kw),
            "mixed": ensemble("mixed", steps, window, 10, 1, turbines, perturbs=pert, **kw)}
    nz = kw["Nz"] + 1
    r = compare(runs["mixed"], runs["fp64"], nz)
    if not args.val_no_floor:
        fl = compare(ensemble("fp64", steps, window, 10, 1, turbines, perturbs=pert_floor, **kw), runs["fp64"], nz)
        r["fp64_noise_floor"] = {k: v for k, v in fl.items() if k in ("u_linf", "uw_linf", "power_rel")}
    r["mixed_members"] = runs["mixed"]["members"]
    r["fp64_members"] = runs["fp64"]["members"]
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


def run_xdft_compare(args):
    """The forward x transforms as tensor-core GEMMs (k_xdft_tc: three-pass
    TF32 splitting, FP32 accuracy; LESGO_XDFT=1) against the radix kernels
    (k_xfwd), in the mixed form: the x-forward stages' CUDA-event times and
    achieved algorithmic GB/s, and the whole step's device time, for one
    128^3 instance and for the 48-instance ensemble.  Both arms run the same
    instances from the same seeds; the tiles are autotuned per arm."""
    import torch
    torch.cuda.set_device(0)
    from lesgo_gb300.solver import LesgoGPU
    hbm = peaks()[0]
    warm, steps = timed_steps(args)

    def xf_stages(rep):
        out = {}
        for k, (n, ms, by) in rep.items():
            if k.endswith("xfwd"):
                out[k] = dict(launches=n, us_per_launch=1e3 * ms / n, gbs=by / (ms * 1e-3) / 1e9 if ms > 0 else 0.0,
                              frac_of_measured_hbm=(by / (ms * 1e-3) / 1e9) / hbm if ms > 0 else 0.0)
        return out

    res = {}
    for mode in ("0", "1"):
        os.environ["LESGO_XDFT"] = mode
        n = args.grid
        g = LesgoGPU(**dict(WORKLOAD, nx=n, ny=n, Nz=n, precision="mixed"))
        g.init_ic(1)
        g.autotune()
        g.step(warm)
        ms1 = timed_on_device(torch, [(None, None, g)], lambda: g.step(steps))
        g.profile(True)
        g.step(5)
        rep1 = g.profile_report()
        g.profile(False)
        u1 = g.get("u")
        g.close()
        batches = make_batches("mixed")
        step_all(batches, warm)
        msb = timed_on_device(torch, batches, lambda: step_all(batches, steps))
        reps = []
        for _, _, b in batches:
            b.profile(True)
            b.step(5)
            reps.append(b.profile_report())
            b.profile(False)
        for _, _, b in batches:
            b.close()
        repb = merge_profiles(reps)
        res[mode] = dict(single_ms_per_step=ms1 / steps, ensemble_ms_per_step=msb / steps,
                         single_xfwd=xf_stages(rep1), ensemble_xfwd=xf_stages(repb),
                         single_xfwd_ms_per_step=sum(v[1] for k, v in rep1.items() if k.endswith("xfwd")) / 5,
                         ensemble_xfwd_ms_per_step=sum(v[1] for k, v in repb.items() if k.endswith("xfwd")) / 5,
                         u=u1)
    du = float(abs(res["1"]["u"] - res["0"]["u"]).max() / abs(res["0"]["u"]).max())
    for r in res.values():
        del r["u"]
    line = {"xdft_compare": True, "grid": args.grid, "warmup": warm, "steps": steps, "hbm_gbs_measured": hbm,
            "radix": res["0"], "tensor_core_gemm": res["1"],
            "single_u_max_rel_diff_after_warmup_and_timed_steps": du,
            "xfwd_speedup_single": res["0"]["single_xfwd_ms_per_step"] / res["1"]["single_xfwd_ms_per_step"],
            "xfwd_speedup_ensemble": res["0"]["ensemble_xfwd_ms_per_step"] / res["1"]["ensemble_xfwd_ms_per_step"],
            "step_speedup_single": res["0"]["single_ms_per_step"] / res["1"]["single_ms_per_step"],
            "step_speedup_ensemble": res["0"]["ensemble_ms_per_step"] / res["1"]["ensemble_ms_per_step"]}
    print(json.dumps(line), flush=True)


def main():
    global ONLY_CLASS
    args = parse()
    ONLY_CLASS = args.only_class
    if args.impl == "reference":
        run_reference(args)
    elif args.validate:
        run_validate(args)
    elif args.serve:
        run_serve(args)
    elif args.xdft_compare:
        run_xdft_compare(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
