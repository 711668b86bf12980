"""Long-run statistical agreement of the mixed form with the plain FP64 form.

Turbulence is chaotic, so after the first steps the two forms' fields part
ways; what must agree is the statistics.  Over a window of a few thousand
steps those carry sampling noise of their own: at 128^3 (4000 steps,
averages over the last 2000) single mixed-form runs whose initial u differ
by 1e-6 relative give <u'w'> between 0.6 % and 1.8 % off the FP64 run, and
FP64 runs perturbed the same way 0.2-0.6 %.  So `ensemble` averages the
mixed form over realisations with FP32-sized perturbations of the initial
condition (the IC itself and +-1e-6), which removes most of that noise, and
the FP64 spread is reported beside it as the noise floor.  A run advances one instance of a
grid from the seeded IC, accumulates the time averages of
time_average.f90:176-319 on the device over a window at the end of the run
(sampled every `nskip` steps, schedule io.f90:557-580), and, with actuator
disks, averages each turbine's power P = -f_n u_d_T (turbines.f90:465-638)
over the same samples.  `compare` states:

  * u_linf   -- max_z |<u>_mixed - <u>_fp64| / max_z |<u>_fp64|   (levels 1..nz-1)
  * uw_linf  -- max_z |<u'w'>_mixed - <u'w'>_fp64| / max_z |<u'w'>_fp64|
                (resolved shear stress on the w grid, time_average.f90:622-629)
  * power    -- per turbine |P_mixed - P_fp64| / max |P_fp64|
"""
from __future__ import annotations

import time
from typing import Dict, Optional

import numpy as np

from .solver import LesgoGPU


def long_run(precision: str, steps: int, window: int, nskip: int = 10, seed: int = 1,
             turbines: Optional[list] = None, perturb: float = 0.0, **kw) -> Dict[str, object]:
    """Run `steps` steps; time averages over the last `window` steps.
    perturb != 0 scales u by (1 + perturb) after the IC: a run of the same
    form whose trajectory parts from the unperturbed one, which measures how
    far two realisations' statistics differ over the window (the noise
    floor the mixed form is compared against)."""
    if window > steps or window % nskip or steps % nskip:
        raise ValueError("window <= steps, both multiples of nskip")
    g = LesgoGPU(precision=precision, turbines=turbines, **kw)
    try:
        g.init_ic(seed)
        if perturb:
            g.set("u", g.get("u") * (1.0 + perturb))
        nstart = steps - window
        # the sample at nstart starts the sums; with nstart = 0 the first one is at nskip
        first = nstart if nstart > 0 else nskip
        g.tavg_config(first, steps, nskip)
        power = []
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            g.step(nskip)
            done += nskip
            if turbines and done > first:
                power.append(g.turbine_state()["power"].copy())
        g.sync()
        wall = time.perf_counter() - t0
        out = dict(u=g.tavg_profile("u"), upwp=g.tavg_profile("upwp"), uw=g.tavg_profile("uw"),
                   total_time=g.tavg_total_time(), diag=g.diag(), wall_s=wall,
                   samples=(steps - first) // nskip)
        if turbines:
            out["power"] = np.mean(np.array(power), axis=0)
        return out
    finally:
        g.close()


def ensemble(precision: str, steps: int, window: int, nskip: int = 10, seed: int = 1,
             turbines: Optional[list] = None, perturbs=(0.0, 1e-6, -1e-6), **kw) -> Dict[str, object]:
    """long_run over realisations whose initial u is scaled by (1 + p), p in
    `perturbs`; profiles, power and diagnostics averaged over the members."""
    runs = [long_run(precision, steps, window, nskip, seed, turbines, perturb=p, **kw) for p in perturbs]
    out = dict(runs[0])
    for k in ("u", "upwp", "uw", "total_time"):
        out[k] = np.mean([r[k] for r in runs], axis=0)
    if turbines:
        out["power"] = np.mean([r["power"] for r in runs], axis=0)
    out["wall_s"] = float(sum(r["wall_s"] for r in runs))
    out["members"] = len(runs)
    out["perturbs"] = list(perturbs)
    return out


def compare(a: Dict[str, object], b: Dict[str, object], nz: int) -> Dict[str, object]:
    """Errors of run `a` (mixed) against run `b` (FP64)."""
    ua, ub = a["u"][1:nz], b["u"][1:nz]
    wa, wb = a["upwp"][1:nz + 1], b["upwp"][1:nz + 1]
    r = dict(u_linf=float(np.max(np.abs(ua - ub)) / np.max(np.abs(ub))),
             uw_linf=float(np.max(np.abs(wa - wb)) / np.max(np.abs(wb))),
             uw_max_fp64=float(np.max(np.abs(wb))), u_max_fp64=float(np.max(np.abs(ub))))
    if "power" in b:
        pa, pb = np.asarray(a["power"]), np.asarray(b["power"])
        r["power_rel"] = (np.abs(pa - pb) / np.max(np.abs(pb))).tolist()
        r["power_fp64"] = pb.tolist()
        r["power_mixed"] = pa.tolist()
    return r


def wind_farm_4x3(L_z: float = 1.0):
    """4 x 3 aligned actuator disks: D = 0.1, hub 0.1, 7D streamwise x 5D
    spanwise spacing, Ct' = 1.33 (positions in units of z_i like
    input_turbines/param.dat, turbines.f90:759-770)."""
    D = 0.1
    ts = []
    for i in range(4):
        for j in range(3):
            ts.append(dict(xloc=1.0 + 7 * D * i, yloc=1.0 + 5 * D * (j - 1) + 0.5, height=0.1 * L_z, dia=D,
                           thk=0.0, theta1=0.0, theta2=0.0, Ct_prime=1.33))
    return ts


def batch_vs_alone(instances, steps: int = 500, window: int = 250, nskip: int = 10,
                   batch_precision: str = "mixed", alone_precision: str = "fp64", base: Optional[dict] = None):
    """Each instance of a batched ensemble against the same instance run
    alone.  `instances` is a list of ((nx, ny, Nz), zo, seed).  The batch
    runs one handle per grid class in `batch_precision`; every instance then
    runs alone in `alone_precision` from the same seeded IC.  Per instance:
    the time-averaged <u>(z) and resolved <u'w'>(z) over the last `window`
    steps (sampled every `nskip`) and the plane-mean u(z) after the last
    step, each as max_z |batch - alone| / max_z |alone|.  Returns the rows
    and their worst value per grid class."""
    from .solver import LesgoBatch
    base = dict(base or dict(dyn_init=5, cs_count=5))
    first = steps - window if steps > window else nskip
    by_grid: Dict[tuple, list] = {}
    for g, zo, seed in instances:
        by_grid.setdefault(tuple(g), []).append((zo, seed))
    rows = []
    t_batch = t_alone = 0.0
    for g, lst in by_grid.items():
        kw = dict(nx=g[0], ny=g[1], Nz=g[2], **base)
        nz = g[2] + 1
        b = LesgoBatch(len(lst), precision=batch_precision, **kw)
        try:
            ids = [b.add(zo, seed) for zo, seed in lst]
            b.tavg_config(first, steps, nskip)
            t0 = time.perf_counter()
            b.step(steps)
            b.sync()
            t_batch += time.perf_counter() - t0
            res_b = {iid: dict(u=b.tavg_profile(iid, "u"), upwp=b.tavg_profile(iid, "upwp"),
                               um=b.get(iid, "u")[1:nz, :, :g[0]].mean(axis=(1, 2))) for iid in ids}
        finally:
            b.close()
        for (zo, seed), iid in zip(lst, ids):
            a = LesgoGPU(zo=zo, precision=alone_precision, **kw)
            try:
                a.init_ic(seed)
                a.tavg_config(first, steps, nskip)
                t0 = time.perf_counter()
                a.step(steps)
                a.sync()
                t_alone += time.perf_counter() - t0
                ua, wa = a.tavg_profile("u")[1:nz], a.tavg_profile("upwp")[1:nz + 1]
                uma = a.get("u")[1:nz, :, :g[0]].mean(axis=(1, 2))
            finally:
                a.close()
            rb = res_b[iid]
            rows.append(dict(grid="x".join(map(str, g)), zo=zo, seed=seed,
                             u_linf=float(np.max(np.abs(rb["u"][1:nz] - ua)) / np.max(np.abs(ua))),
                             uw_linf=float(np.max(np.abs(rb["upwp"][1:nz + 1] - wa)) / np.max(np.abs(wa))),
                             plane_u_linf=float(np.max(np.abs(rb["um"] - uma)) / np.max(np.abs(uma)))))
    per_class = {}
    for r in rows:
        c = per_class.setdefault(r["grid"], dict(instances=0, u_linf=0.0, uw_linf=0.0, plane_u_linf=0.0))
        c["instances"] += 1
        for k in ("u_linf", "uw_linf", "plane_u_linf"):
            c[k] = max(c[k], r[k])
    return dict(rows=rows, per_class=per_class, wall_s=dict(batch=t_batch, alone=t_alone))
