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
