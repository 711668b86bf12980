"""Shared helpers for the GPU parity tests: matched oracle/GPU instances and
valid-entry comparisons (the reference's valid levels; pad columns and
BOGUS levels excluded)."""
from __future__ import annotations

import numpy as np

from oracle.lesgo_oracle import Oracle, Params

# valid levels per field after the stage that writes it
VALID = {
    "u": (1, -1), "v": (1, -1), "w": (1, 0),
    "dudx": (1, 0), "dudy": (1, 0), "dvdx": (1, 0), "dvdy": (1, 0), "dwdx": (1, 0), "dwdy": (1, 0),
    "dudz": (1, 0), "dvdz": (1, 0), "dwdz": (1, -1),
    "txx": (1, -1), "txy": (1, -1), "tyy": (1, -1), "tzz": (1, -1), "txz": (1, 0), "tyz": (1, 0),
    "S11": (1, 0), "S12": (1, 0), "S13": (1, 0), "S22": (1, 0), "S23": (1, 0), "S33": (1, 0),
    "Cs_opt2": (1, 0), "F_LM": (1, 0), "F_MM": (1, 0), "F_QN": (1, 0), "F_NN": (1, 0),
    "divtx": (1, -1), "divty": (1, -1), "divtz": (1, 0),
    "RHSx": (1, -1), "RHSy": (1, -1), "RHSz": (1, 0),
    "RHSx_f": (1, -1), "RHSy_f": (1, -1), "RHSz_f": (1, 0),
    "p": (0, 0), "dpdx": (1, -1), "dpdy": (1, -1), "dpdz": (1, 0),
    "fxa": (1, -1), "fya": (1, -1), "fza": (2, -1),
}
# stage-specific overrides: ddz_uv alone leaves levels 1 and nz to the wall model
STAGE_VALID = {"ddz_uv:u": {"dudz": (2, -1)}, "ddz_uv:v": {"dvdz": (2, -1)}}


def oracle_field(o: Oracle, name: str) -> np.ndarray:
    return o.pres if name == "p" else getattr(o, name)


def rel_err(p: Params, name: str, gpu: np.ndarray, ref: np.ndarray, lev=None) -> float:
    lo, hi = lev if lev is not None else VALID[name]
    hi = p.nz + hi
    a = gpu[lo:hi + 1, :, :p.nx]
    b = ref[lo:hi + 1, :, :p.nx]
    den = np.max(np.abs(b))
    if den == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)


def make_pair(precision: str = "fp64", seed: int = 1, **kw):
    from lesgo_gb300.solver import LesgoGPU
    turbines = kw.pop("turbines", None)
    p = Params(**kw)
    o = Oracle(p)
    o.set_ic(seed)
    gkw = dict(nx=p.nx, ny=p.ny, Nz=p.Nz, L_x=p.L_x, L_y=p.L_y, L_z=p.L_z, z_i=p.z_i, u_star=p.u_star,
               vonk=p.vonk, zo=p.zo, dt=p.dt, cs_count=p.cs_count, dyn_init=p.dyn_init, lbc_mom=p.lbc_mom,
               ubc_mom=p.ubc_mom, molec=p.molec, nu_molec=p.nu_molec, ubot=p.ubot, utop=p.utop,
               use_mean_p_force=p.use_mean_p_force, eval_mean_p_force=p.eval_mean_p_force,
               mean_p_force_x=p.mean_p_force_x_in, mean_p_force_y=p.mean_p_force_y_in,
               use_cfl_dt=p.use_cfl_dt, cfl=p.cfl, precision=precision)
    g = LesgoGPU(turbines=turbines, **gkw)
    g.init_ic(seed)
    return p, o, g
