"""Host-side mirror of LESGO's time-step subroutines over the C ABI.

``LesgoGPU`` exposes one method per reference subroutine on the hot path
(``filt_da``, ``ddx``, ``ddz_uv``, ``wallstress``, ``sgs_stag``,
``divstress_uv``, ``convec``, ``press_stag_array``, ``project`` ...) with
the same argument meaning, plus the fused ``step``.  Fields are addressed by
the reference's names (sim_param.f90 / sgs_param.f90).  Host arrays use the
shape ``(levels, ny, ld)`` in C order, which is byte-identical to the
reference's Fortran ``(ld, ny, lbz:nzhi)`` arrays.

Failures raise ``LesgoError`` carrying the library's status code, where the
reference would print and ``stop`` (messages.f90:228-239).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Iterable, Optional

import numpy as np

from . import _lib as L


# Time-averaged quantities in the order the library numbers them
# (time_average.f90:176-319), then the Reynolds stresses (:616-629).
TAVG_QUANTITIES = ["u", "v", "w", "u_w", "v_w", "w_uv", "u2", "v2", "w2", "uv", "uw", "vw",
                   "txx", "tyy", "tzz", "txy", "txz", "tyz", "p", "fx", "fy", "fz", "cs_opt2",
                   "vortx", "vorty", "vortz", "up2", "vp2", "wp2", "upvp", "upwp", "vpwp"]


class LesgoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lesgo_gpu error {code}: {msg}")
        self.code = code


# precision forms: FP64 throughout; FP32 bulk with the FP64 pressure solve;
# FP64 fields with double-word (FP32 pair) x-y transforms
PRECISIONS = {"fp64": L.LESGO_FP64, "mixed": L.LESGO_MIXED, "fp64dw": L.LESGO_FP64_DW}

PARAM_DEFAULTS = dict(
    nx=64, ny=64, Nz=64, L_x=2.0 * 3.1415926535897932384626433, L_y=3.1415926535897932384626433, L_z=1.0,
    z_i=1000.0, u_star=0.45, vonk=0.4, zo=1.0e-4, dt=2.0e-4, sgs_model=5, cs_count=5, dyn_init=100,
    ifilter=1, lbc_mom=2, ubc_mom=0, molec=False, nu_molec=1.14e-5, ubot=0.0, utop=0.0,
    use_mean_p_force=True, eval_mean_p_force=True, mean_p_force_x=1.0, mean_p_force_y=0.0,
    initu=False, precision="fp64", alpha1=1.5, alpha2=1.5, filter_cutoff=1e-2, T_avg_dim=-1.0,
    adm_correction=True, use_cfl_dt=False, cfl=0.05,
)


def make_params(**kw) -> L.Params:
    """lesgo_params_t from lesgo.conf-style keywords (defaults: PARAM_DEFAULTS)."""
    unknown = set(kw) - set(PARAM_DEFAULTS)
    if unknown:
        raise TypeError(f"unknown parameters: {sorted(unknown)}")
    cfg = dict(PARAM_DEFAULTS, **kw)
    p = L.Params()
    p.nx, p.ny, p.nz_tot = cfg["nx"], cfg["ny"], cfg["Nz"]
    for name in ("L_x", "L_y", "L_z", "z_i", "u_star", "vonk", "zo", "dt", "nu_molec", "ubot", "utop",
                 "mean_p_force_x", "mean_p_force_y", "alpha1", "alpha2", "filter_cutoff", "T_avg_dim", "cfl"):
        setattr(p, name, float(cfg[name]))
    for name in ("sgs_model", "cs_count", "dyn_init", "ifilter", "lbc_mom", "ubc_mom"):
        setattr(p, name, int(cfg[name]))
    for name in ("molec", "use_mean_p_force", "eval_mean_p_force", "initu", "adm_correction", "use_cfl_dt"):
        setattr(p, name, 1 if cfg[name] else 0)
    prec = cfg["precision"]
    p.precision = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
    return p, cfg


def make_turbines(turbines):
    tl = list(turbines or [])
    arr = (L.Turbine * max(1, len(tl)))()
    for i, t in enumerate(tl):
        for k in ("xloc", "yloc", "height", "dia", "thk", "theta1", "theta2", "Ct_prime"):
            setattr(arr[i], k, float(t.get(k, 1.33 if k == "Ct_prime" else 0.0)))
    return arr, len(tl)


def read_conf(path: str, with_turbines: bool = True, max_turbines: int = 4096):
    """<path>lesgo.conf -> (parameter keywords for LesgoGPU / make_params, run
    control dict, notes on unused blocks and keys).  `path` is a prefix like
    the reference's `path` ("" or a directory with its trailing '/')."""
    lib = L.load()
    p, run = L.Params(), L.Run()
    tb = (L.Turbine * max(1, max_turbines))()
    log = C.create_string_buffer(1 << 14)
    rc = lib.lesgo_gpu_read_conf(os.fsencode(path), 1 if with_turbines else 0, C.byref(p), C.byref(run),
                                 C.cast(tb, C.POINTER(L.Turbine)), max_turbines, log, len(log))
    if rc != L.LESGO_OK:
        raise LesgoError(rc, lib.lesgo_gpu_last_error(None).decode())
    kw = dict(nx=p.nx, ny=p.ny, Nz=p.nz_tot)
    for name in ("L_x", "L_y", "L_z", "z_i", "u_star", "vonk", "zo", "dt", "nu_molec", "ubot", "utop",
                 "mean_p_force_x", "mean_p_force_y", "alpha1", "alpha2", "filter_cutoff", "T_avg_dim"):
        kw[name] = getattr(p, name)
    for name in ("sgs_model", "cs_count", "dyn_init", "ifilter", "lbc_mom", "ubc_mom"):
        kw[name] = getattr(p, name)
    for name in ("molec", "use_mean_p_force", "eval_mean_p_force", "initu", "adm_correction", "use_cfl_dt"):
        kw[name] = bool(getattr(p, name))
    kw["cfl"] = p.cfl
    kw["turbines"] = [{k: getattr(tb[i], k) for k, _ in L.Turbine._fields_} for i in range(p.n_turbines)]
    rd = {k: getattr(run, k) for k, _ in L.Run._fields_}
    return kw, rd, log.value.decode()


SCHEDULES = {"theta1": 0, "theta2": 1, "Ct_prime": 2}


def _which(which) -> int:
    return SCHEDULES[which] if isinstance(which, str) else int(which)


def _set_schedule(check, fn, head, which, rows, nturb):
    a = np.ascontiguousarray(np.zeros((0, 1 + nturb)) if rows is None else rows, dtype=np.float64)
    if a.size and (a.ndim != 2 or a.shape[1] != 1 + nturb):
        raise ValueError("schedule rows need the time and %d values" % nturb)
    nt = a.shape[0] if a.size else 0
    check(fn(*head, _which(which), nt, a.ctypes.data_as(C.POINTER(C.c_double))))


def _get_controls(lib, check, h, iid, n):
    t1, t2, c = (np.zeros(max(n, 1)) for _ in range(3))
    dp = C.POINTER(C.c_double)
    check(lib.lesgo_gpu_turbine_controls(h, iid, t1.ctypes.data_as(dp), t2.ctypes.data_as(dp),
                                         c.ctypes.data_as(dp), n))
    return dict(theta1=t1[:n], theta2=t2[:n], Ct_prime=c[:n])


def read_turbine_schedule(path: str, which, n_turbines: int, max_rows: int = 1 << 16) -> np.ndarray:
    """<path>input_turbines/theta1.dat | theta2.dat | Ct_prime.dat ->
    rows of (time, one value per turbine) (read_control_files,
    turbines.f90:872-931)."""
    lib = L.load()
    buf = np.zeros((max_rows, 1 + n_turbines))
    nt = C.c_int()
    rc = lib.lesgo_gpu_read_turbine_schedule(os.fsencode(path), _which(which), n_turbines,
                                             buf.ctypes.data_as(C.POINTER(C.c_double)), max_rows, C.byref(nt))
    if rc != L.LESGO_OK:
        raise LesgoError(rc, lib.lesgo_gpu_last_error(None).decode())
    return buf[:nt.value].copy()


def conf_turbine_schedules(path: str, run: dict, n_turbines: int) -> dict:
    """The control schedules a lesgo.conf asks for (run["dyn_theta1"] etc.
    from read_conf), read from <path>input_turbines/: {which: rows}.  Pass
    each to turbine_schedule(which, rows)."""
    out = {}
    for which, flag in (("theta1", "dyn_theta1"), ("theta2", "dyn_theta2"), ("Ct_prime", "dyn_ct_prime")):
        if run.get(flag):
            out[which] = read_turbine_schedule(path, which, n_turbines)
    return out


def footprint_bytes(capacity: int = 1, **kw) -> int:
    """Device bytes a handle of this grid and capacity allocates."""
    lib = L.load()
    p, _ = make_params(**kw)
    b = C.c_longlong()
    rc = lib.lesgo_gpu_footprint(C.byref(p), capacity, C.byref(b))
    if rc != L.LESGO_OK:
        raise LesgoError(rc, lib.lesgo_gpu_last_error(None).decode())
    return b.value


class LesgoGPU:
    """One LES instance resident on the current CUDA device."""

    def __init__(self, turbines: Optional[Iterable[dict]] = None, **kw):
        p, cfg = make_params(**kw)
        self.cfg = cfg
        self._lib = L.load()
        self._turb, nt = make_turbines(turbines)
        p.n_turbines = nt
        p.turbines = C.cast(self._turb, C.POINTER(L.Turbine)) if nt else None
        self.n_turbines = nt
        h = C.c_void_p()
        rc = self._lib.lesgo_gpu_create(C.byref(p), C.byref(h))
        if rc != L.LESGO_OK:
            raise LesgoError(rc, self._lib.lesgo_gpu_last_error(None).decode())
        self._h = h
        nz, ld, lh, nx2, ny2 = (C.c_int() for _ in range(5))
        self._lib.lesgo_gpu_dims(h, C.byref(nz), C.byref(ld), C.byref(lh), C.byref(nx2), C.byref(ny2))
        self.nx, self.ny = cfg["nx"], cfg["ny"]
        self.nz, self.ld, self.lh, self.nx2, self.ny2 = nz.value, ld.value, lh.value, nx2.value, ny2.value

    # ---------------- lifetime -------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.lesgo_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != L.LESGO_OK:
            raise LesgoError(rc, self._lib.lesgo_gpu_last_error(self._h).decode())

    @staticmethod
    def _fid(name) -> int:
        return name if isinstance(name, int) else L.FIELD[name]

    # ---------------- field access ----------------------------------------------
    def get(self, name, lbz: int = 0, nzhi: Optional[int] = None) -> np.ndarray:
        nzhi = self.nz if nzhi is None else nzhi
        out = np.empty((nzhi - lbz + 1, self.ny, self.ld), dtype=np.float64)
        self._check(self._lib.lesgo_gpu_get_field(self._h, self._fid(name), out.ctypes.data, lbz, nzhi))
        return out

    def set(self, name, arr: np.ndarray, lbz: int = 0):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.ndim != 3 or a.shape[1:] != (self.ny, self.ld):
            raise ValueError(f"expected (levels, {self.ny}, {self.ld}), got {a.shape}")
        self._check(self._lib.lesgo_gpu_set_field(self._h, self._fid(name), a.ctypes.data, lbz, lbz + a.shape[0] - 1))

    def set_ptr(self, name, ptr: int, lbz: int, nzhi: int, wait: bool = True):
        """Copy levels lbz..nzhi from a host FP64 buffer at address ``ptr``.
        wait=False queues the copy in stream order (the buffer must stay
        unchanged until sync())."""
        fn = self._lib.lesgo_gpu_set_field if wait else self._lib.lesgo_gpu_set_field_async
        self._check(fn(self._h, self._fid(name), C.c_void_p(ptr), lbz, nzhi))

    def get_ptr(self, name, ptr: int, lbz: int, nzhi: int, wait: bool = True):
        """wait=False queues the copy; the buffer holds the data after sync()."""
        fn = self._lib.lesgo_gpu_get_field if wait else self._lib.lesgo_gpu_get_field_async
        self._check(fn(self._h, self._fid(name), C.c_void_p(ptr), lbz, nzhi))

    def init_ic(self, seed: int):
        self._check(self._lib.lesgo_gpu_init_ic(self._h, C.c_uint64(seed)))

    # ---------------- reference subroutines ---------------------------------------
    def filt_da(self, f, dfdx, dfdy):
        self._check(self._lib.lesgo_gpu_filt_da(self._h, self._fid(f), self._fid(dfdx), self._fid(dfdy)))

    def ddx(self, f, dfdx):
        self._check(self._lib.lesgo_gpu_ddx(self._h, self._fid(f), self._fid(dfdx)))

    def ddy(self, f, dfdy):
        self._check(self._lib.lesgo_gpu_ddy(self._h, self._fid(f), self._fid(dfdy)))

    def ddxy(self, f, dfdx, dfdy):
        self._check(self._lib.lesgo_gpu_ddxy(self._h, self._fid(f), self._fid(dfdx), self._fid(dfdy)))

    def ddz_uv(self, f, dfdz):
        self._check(self._lib.lesgo_gpu_ddz_uv(self._h, self._fid(f), self._fid(dfdz)))

    def ddz_w(self, f, dfdz):
        self._check(self._lib.lesgo_gpu_ddz_w(self._h, self._fid(f), self._fid(dfdz)))

    def test_filter(self, f, level: int):
        self._check(self._lib.lesgo_gpu_test_filter(self._h, self._fid(f), level))

    def wallstress(self):
        self._check(self._lib.lesgo_gpu_wallstress(self._h))

    def sgs_stag(self):
        self._check(self._lib.lesgo_gpu_sgs_stag(self._h))

    def divstress_uv(self):
        self._check(self._lib.lesgo_gpu_divstress_uv(self._h))

    def divstress_w(self):
        self._check(self._lib.lesgo_gpu_divstress_w(self._h))

    def convec(self):
        self._check(self._lib.lesgo_gpu_convec(self._h))

    def turbines_forcing(self):
        self._check(self._lib.lesgo_gpu_turbines_forcing(self._h))

    def begin_step(self):
        self._check(self._lib.lesgo_gpu_begin_step(self._h))

    def rhs_assemble(self):
        self._check(self._lib.lesgo_gpu_rhs_assemble(self._h))

    def ab2(self):
        self._check(self._lib.lesgo_gpu_ab2(self._h))

    def press_stag_array(self):
        self._check(self._lib.lesgo_gpu_press_stag_array(self._h))

    def rhs_sub_dp(self):
        self._check(self._lib.lesgo_gpu_rhs_sub_dp(self._h))

    def project(self):
        self._check(self._lib.lesgo_gpu_project(self._h))

    def tridag_array(self, a_ptr: int, b_ptr: int, c_ptr: int, r_ptr: int, u_ptr: int, lh: int, ny: int, n: int):
        """tridag_array.f90:166-246 on device arrays (addresses of FP64
        buffers in the reference layout)."""
        self._check(self._lib.lesgo_gpu_tridag_array(self._h, C.c_void_p(a_ptr), C.c_void_p(b_ptr), C.c_void_p(c_ptr),
                                                     C.c_void_p(r_ptr), C.c_void_p(u_ptr), lh, ny, n))

    def step_reference_order(self):
        """One time step through the stand-alone entry points in the order
        of main.f90:130-344 (the drop-in call sequence)."""
        self.begin_step()
        self.filt_da("u", "dudx", "dudy")
        self.filt_da("v", "dvdx", "dvdy")
        self.filt_da("w", "dwdx", "dwdy")
        self.ddz_uv("u", "dudz")
        self.ddz_uv("v", "dvdz")
        self.ddz_w("w", "dwdz")
        self.wallstress()
        self.sgs_stag()
        self.divstress_uv()
        self.divstress_w()
        self.convec()
        if self.n_turbines:
            self.turbines_forcing()
        self.rhs_assemble()
        self.ab2()
        self.press_stag_array()
        self.rhs_sub_dp()
        self.project()

    # ---------------- fused loop, diagnostics ----------------------------------------
    def step(self, nsteps: int = 1):
        self._check(self._lib.lesgo_gpu_step(self._h, nsteps))

    def sync(self):
        self._check(self._lib.lesgo_gpu_sync(self._h))

    def diag(self) -> Dict[str, float]:
        r, k, c, t = (C.c_double() for _ in range(4))
        self._check(self._lib.lesgo_gpu_diag(self._h, C.byref(r), C.byref(k), C.byref(c), C.byref(t)))
        return dict(rmsdiv=r.value, ke=k.value, cfl=c.value, tau_bot=t.value)

    def counters(self):
        a, b = C.c_int(), C.c_int()
        self._check(self._lib.lesgo_gpu_counters(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def turbine_state(self):
        n = self.n_turbines
        a, b, c = (np.zeros(max(n, 1)) for _ in range(3))
        dp = C.POINTER(C.c_double)
        self._check(self._lib.lesgo_gpu_turbine_state(self._h, a.ctypes.data_as(dp), b.ctypes.data_as(dp),
                                                      c.ctypes.data_as(dp), n))
        return dict(u_d_T=a[:n], f_n=b[:n], power=c[:n])

    def turbine_schedule(self, which, rows):
        """Time-varying yaw (which 0 or "theta1"), tilt (1, "theta2") or Ct'
        (2, "Ct_prime"): rows of (dimensional time, one value per turbine),
        as the lines of input_turbines/theta1.dat; None or [] removes it."""
        _set_schedule(self._check, self._lib.lesgo_gpu_turbine_schedule, (self._h,), which, rows, self.n_turbines)

    def turbine_controls(self):
        """Current yaw, tilt (degrees) and Ct' of each turbine."""
        return _get_controls(self._lib, self._check, self._h, -1, self.n_turbines)

    def profile(self, enable: bool = True):
        self._check(self._lib.lesgo_gpu_profile(self._h, 1 if enable else 0))

    def profile_report(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 16)
        self._check(self._lib.lesgo_gpu_profile_report(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.lesgo_gpu_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def launches_per_step(self, with_sgs_update: bool = False) -> int:
        return self._lib.lesgo_gpu_launches_per_step(self._h, 1 if with_sgs_update else 0)

    def autotune(self) -> Dict[str, int]:
        """Pick the transform tile shapes for this grid by timing them."""
        xt, yb = C.c_int(), C.c_int()
        self._check(self._lib.lesgo_gpu_autotune(self._h, C.byref(xt), C.byref(yb)))
        return dict(xtarget=xt.value, ybudget=yb.value)

    # ---------------- diagnostics log ---------------------------------------------------
    def diag_log_config(self, every: int, capacity: int = 1024):
        """Rows of (jt_total, total_time, rmsdiv, ke, cfl, tau_bot) every `every` steps."""
        self._check(self._lib.lesgo_gpu_diag_log_config(self._h, every, capacity))

    def diag_log_sample(self):
        self._check(self._lib.lesgo_gpu_diag_log_sample(self._h))

    def diag_log(self, maxrows: int = 65536) -> np.ndarray:
        out = np.zeros((maxrows, 6))
        n = C.c_int()
        self._check(self._lib.lesgo_gpu_diag_log_read(self._h, -1, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                      maxrows, C.byref(n)))
        return out[:n.value].copy()

    # ---------------- time averaging ---------------------------------------------------
    def tavg_config(self, nstart: int, nend: int, nskip: int):
        """tavg_nstart / tavg_nend / tavg_nskip of the reference's input."""
        self._check(self._lib.lesgo_gpu_tavg_config(self._h, nstart, nend, nskip))

    def tavg_sample(self):
        self._check(self._lib.lesgo_gpu_tavg_sample(self._h))

    def tavg_get(self, name: str, lbz: int = 1) -> np.ndarray:
        out = np.zeros((self.nz + 1 - lbz, self.ny, self.ld))
        self._check(self._lib.lesgo_gpu_tavg_get(self._h, TAVG_QUANTITIES.index(name),
                                                 out.ctypes.data_as(C.POINTER(C.c_double)), lbz, self.nz))
        return out

    def tavg_profile(self, name: str) -> np.ndarray:
        out = np.zeros(self.nz + 1)
        self._check(self._lib.lesgo_gpu_tavg_profile(self._h, TAVG_QUANTITIES.index(name),
                                                     out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    # ---------------- checkpoint / restart ---------------------------------------------
    def checkpoint_write(self, path: str, mpi_names: bool = False):
        """vel.out, grid.out, total_time.dat (and tavg.out) under the prefix `path`."""
        self._check(self._lib.lesgo_gpu_checkpoint_write(self._h, os.fsencode(path), 1 if mpi_names else 0))

    def checkpoint_read(self, path: str) -> bool:
        """Restart from the files under `path`; True when they were of this grid."""
        same = C.c_int()
        self._check(self._lib.lesgo_gpu_checkpoint_read(self._h, os.fsencode(path), C.byref(same)))
        return bool(same.value)

    def time_step(self) -> float:
        """dt of the last step (chosen on the device with use_cfl_dt)."""
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_time_step(self._h, -1, C.byref(t)))
        return t.value

    def sim_time(self) -> float:
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_sim_time(self._h, -1, C.byref(t)))
        return t.value

    def tavg_total_time(self) -> float:
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_tavg_total_time(self._h, -1, C.byref(t)))
        return t.value


class LesgoBatch:
    """A batch of independent LES instances of one grid size on the current
    device.  All active instances advance together; each has its own
    roughness length, IC seed, actuator disks and step counters."""

    def __init__(self, capacity: int, **kw):
        p, cfg = make_params(**kw)
        self.cfg = cfg
        self._lib = L.load()
        h = C.c_void_p()
        rc = self._lib.lesgo_gpu_batch_create(C.byref(p), capacity, C.byref(h))
        if rc != L.LESGO_OK:
            raise LesgoError(rc, self._lib.lesgo_gpu_last_error(None).decode())
        self._h = h
        nz, ld, lh, nx2, ny2 = (C.c_int() for _ in range(5))
        self._lib.lesgo_gpu_dims(h, C.byref(nz), C.byref(ld), C.byref(lh), C.byref(nx2), C.byref(ny2))
        self.nx, self.ny = cfg["nx"], cfg["ny"]
        self.nz, self.ld = nz.value, ld.value
        self.capacity = capacity
        self._nturb = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lesgo_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != L.LESGO_OK:
            raise LesgoError(rc, self._lib.lesgo_gpu_last_error(self._h).decode())

    def add(self, zo: float, seed: int, turbines: Optional[Iterable[dict]] = None) -> int:
        arr, nt = make_turbines(turbines)
        i = C.c_int()
        self._check(self._lib.lesgo_gpu_batch_add(self._h, float(zo), C.c_uint64(seed), nt,
                                                  C.cast(arr, C.POINTER(L.Turbine)) if nt else None, C.byref(i)))
        self._nturb[i.value] = nt
        return i.value

    def remove(self, iid: int):
        self._check(self._lib.lesgo_gpu_batch_remove(self._h, iid))
        self._nturb.pop(iid, None)

    def size(self):
        a, c = C.c_int(), C.c_int()
        self._check(self._lib.lesgo_gpu_batch_size(self._h, C.byref(a), C.byref(c)))
        return a.value, c.value

    def get(self, iid: int, name, lbz: int = 0, nzhi: Optional[int] = None) -> np.ndarray:
        nzhi = self.nz if nzhi is None else nzhi
        out = np.empty((nzhi - lbz + 1, self.ny, self.ld), dtype=np.float64)
        self._check(self._lib.lesgo_gpu_get_field_inst(self._h, iid, LesgoGPU._fid(name), out.ctypes.data, lbz, nzhi))
        return out

    def set_ptr(self, iid: int, name, ptr: int, lbz: int, nzhi: int, wait: bool = True):
        """Copy levels lbz..nzhi of instance iid from a host FP64 buffer at
        ``ptr``; wait=False queues it in stream order (see LesgoGPU.set_ptr)."""
        fn = self._lib.lesgo_gpu_set_field_inst if wait else self._lib.lesgo_gpu_set_field_inst_async
        self._check(fn(self._h, iid, LesgoGPU._fid(name), C.c_void_p(ptr), lbz, nzhi))

    def get_ptr(self, iid: int, name, ptr: int, lbz: int, nzhi: int, wait: bool = True):
        fn = self._lib.lesgo_gpu_get_field_inst if wait else self._lib.lesgo_gpu_get_field_inst_async
        self._check(fn(self._h, iid, LesgoGPU._fid(name), C.c_void_p(ptr), lbz, nzhi))

    def set(self, iid: int, name, arr: np.ndarray, lbz: int = 0):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(self._lib.lesgo_gpu_set_field_inst(self._h, iid, LesgoGPU._fid(name), a.ctypes.data, lbz,
                                                       lbz + a.shape[0] - 1))

    def step(self, nsteps: int = 1):
        self._check(self._lib.lesgo_gpu_step(self._h, nsteps))

    def sync(self):
        self._check(self._lib.lesgo_gpu_sync(self._h))

    def diag(self, iid: int) -> Dict[str, float]:
        r, k, c, t = (C.c_double() for _ in range(4))
        self._check(self._lib.lesgo_gpu_diag_inst(self._h, iid, C.byref(r), C.byref(k), C.byref(c), C.byref(t)))
        return dict(rmsdiv=r.value, ke=k.value, cfl=c.value, tau_bot=t.value)

    def counters(self, iid: int):
        a, b = C.c_int(), C.c_int()
        self._check(self._lib.lesgo_gpu_counters_inst(self._h, iid, C.byref(a), C.byref(b)))
        return a.value, b.value

    def turbine_state(self, iid: int):
        n = self._nturb.get(iid, 0)
        a, b, c = (np.zeros(max(n, 1)) for _ in range(3))
        dp = C.POINTER(C.c_double)
        self._check(self._lib.lesgo_gpu_turbine_state_inst(self._h, iid, a.ctypes.data_as(dp), b.ctypes.data_as(dp),
                                                           c.ctypes.data_as(dp), n))
        return dict(u_d_T=a[:n], f_n=b[:n], power=c[:n])

    def turbine_schedule(self, iid: int, which, rows):
        _set_schedule(self._check, self._lib.lesgo_gpu_turbine_schedule_inst, (self._h, iid), which, rows,
                      self._nturb.get(iid, 0))

    def turbine_controls(self, iid: int):
        return _get_controls(self._lib, self._check, self._h, iid, self._nturb.get(iid, 0))

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.lesgo_gpu_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def profile(self, enable: bool = True):
        self._check(self._lib.lesgo_gpu_profile(self._h, 1 if enable else 0))

    def profile_report(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 16)
        self._check(self._lib.lesgo_gpu_profile_report(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def launches_per_step(self, with_sgs_update: bool = False) -> int:
        return self._lib.lesgo_gpu_launches_per_step(self._h, 1 if with_sgs_update else 0)

    def autotune(self) -> Dict[str, int]:
        """Pick the transform tile shapes for this grid by timing them."""
        xt, yb = C.c_int(), C.c_int()
        self._check(self._lib.lesgo_gpu_autotune(self._h, C.byref(xt), C.byref(yb)))
        return dict(xtarget=xt.value, ybudget=yb.value)

    # ---------------- diagnostics log ---------------------------------------------------
    def diag_log_config(self, every: int, capacity: int = 1024):
        """Rows of (jt_total, total_time, rmsdiv, ke, cfl, tau_bot) every `every` steps."""
        self._check(self._lib.lesgo_gpu_diag_log_config(self._h, every, capacity))

    def diag_log_sample(self):
        self._check(self._lib.lesgo_gpu_diag_log_sample(self._h))

    def diag_log(self, iid: int, maxrows: int = 65536) -> np.ndarray:
        out = np.zeros((maxrows, 6))
        n = C.c_int()
        self._check(self._lib.lesgo_gpu_diag_log_read(self._h, iid, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                      maxrows, C.byref(n)))
        return out[:n.value].copy()

    # ---------------- time averaging ---------------------------------------------------
    def tavg_config(self, nstart: int, nend: int, nskip: int):
        """tavg_nstart / tavg_nend / tavg_nskip of the reference's input."""
        self._check(self._lib.lesgo_gpu_tavg_config(self._h, nstart, nend, nskip))

    def tavg_sample(self):
        self._check(self._lib.lesgo_gpu_tavg_sample(self._h))

    def tavg_get(self, iid: int, name: str, lbz: int = 1) -> np.ndarray:
        out = np.zeros((self.nz + 1 - lbz, self.ny, self.ld))
        self._check(self._lib.lesgo_gpu_tavg_get_inst(self._h, iid, TAVG_QUANTITIES.index(name),
                                                 out.ctypes.data_as(C.POINTER(C.c_double)), lbz, self.nz))
        return out

    def tavg_profile(self, iid: int, name: str) -> np.ndarray:
        out = np.zeros(self.nz + 1)
        self._check(self._lib.lesgo_gpu_tavg_profile_inst(self._h, iid, TAVG_QUANTITIES.index(name),
                                                     out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    # ---------------- checkpoint / restart ---------------------------------------------
    def checkpoint_write(self, iid: int, path: str, mpi_names: bool = False):
        """vel.out, grid.out, total_time.dat (and tavg.out) under the prefix `path`."""
        self._check(self._lib.lesgo_gpu_checkpoint_write_inst(self._h, iid, os.fsencode(path), 1 if mpi_names else 0))

    def checkpoint_read(self, iid: int, path: str) -> bool:
        """Restart from the files under `path`; True when they were of this grid."""
        same = C.c_int()
        self._check(self._lib.lesgo_gpu_checkpoint_read_inst(self._h, iid, os.fsencode(path), C.byref(same)))
        return bool(same.value)

    def time_step(self, iid: int) -> float:
        """dt of the last step (chosen on the device with use_cfl_dt)."""
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_time_step(self._h, iid, C.byref(t)))
        return t.value

    def sim_time(self, iid: int) -> float:
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_sim_time(self._h, iid, C.byref(t)))
        return t.value

    def tavg_total_time(self, iid: int) -> float:
        t = C.c_double()
        self._check(self._lib.lesgo_gpu_tavg_total_time(self._h, iid, C.byref(t)))
        return t.value
