"""ctypes binding of the C ABI in include/lesgo_gpu.h.

The library is the product: nothing here computes the step on the host.  If
``liblesgo_gpu.so`` is missing the import fails loudly (build it with
``python -m lesgo_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

# status codes and enums (include/lesgo_gpu.h)
LESGO_OK, LESGO_ERR_ARG, LESGO_ERR_CUDA, LESGO_ERR_UNSUPPORTED, LESGO_ERR_NOMEM, LESGO_ERR_NUMERIC = range(6)
LESGO_FP64, LESGO_MIXED, LESGO_FP64_DW = 0, 1, 2

FIELD_NAMES = [
    "u", "v", "w", "dudx", "dudy", "dudz", "dvdx", "dvdy", "dvdz", "dwdx", "dwdy", "dwdz",
    "RHSx", "RHSy", "RHSz", "RHSx_f", "RHSy_f", "RHSz_f",
    "txx", "txy", "txz", "tyy", "tyz", "tzz", "divtx", "divty", "divtz",
    "p", "dpdx", "dpdy", "dpdz", "fxa", "fya", "fza",
    "S11", "S12", "S13", "S22", "S23", "S33", "Nu_t", "Cs_opt2",
    "F_LM", "F_MM", "F_QN", "F_NN", "Beta", "Tn_all", "ee_now",
]
FIELD = {n: i for i, n in enumerate(FIELD_NAMES)}
NFIELDS = len(FIELD_NAMES)


class Turbine(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("xloc", "yloc", "height", "dia", "thk", "theta1", "theta2", "Ct_prime")]


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz_tot", C.c_int),
        ("L_x", C.c_double), ("L_y", C.c_double), ("L_z", C.c_double), ("z_i", C.c_double),
        ("u_star", C.c_double), ("vonk", C.c_double), ("zo", C.c_double), ("dt", C.c_double),
        ("sgs_model", C.c_int), ("cs_count", C.c_int), ("dyn_init", C.c_int), ("ifilter", C.c_int),
        ("lbc_mom", C.c_int), ("ubc_mom", C.c_int),
        ("molec", C.c_int),
        ("nu_molec", C.c_double), ("ubot", C.c_double), ("utop", C.c_double),
        ("use_mean_p_force", C.c_int), ("eval_mean_p_force", C.c_int),
        ("mean_p_force_x", C.c_double), ("mean_p_force_y", C.c_double),
        ("initu", C.c_int),
        ("precision", C.c_int),
        ("n_turbines", C.c_int),
        ("turbines", C.POINTER(Turbine)),
        ("alpha1", C.c_double), ("alpha2", C.c_double), ("filter_cutoff", C.c_double), ("T_avg_dim", C.c_double),
        ("adm_correction", C.c_int),
        ("use_cfl_dt", C.c_int), ("cfl", C.c_double),
    ]


class Run(C.Structure):
    """lesgo_run_t: run control read from lesgo.conf."""
    _fields_ = [(n, C.c_int) for n in ("nproc", "uniform_spacing", "wall_damp_exp", "sgs")] + [
        ("Co", C.c_double)] + [(n, C.c_int) for n in ("nsteps", "runtime", "use_cfl_dt")] + [
        ("cfl", C.c_double)] + [(n, C.c_int) for n in (
            "cumulative_time", "inilag", "wbase", "nenergy", "lag_cfl_count", "checkpoint_data", "checkpoint_nskip",
            "tavg_calc", "tavg_nstart", "tavg_nend", "tavg_nskip", "dyn_theta1", "dyn_theta2", "dyn_ct_prime")]


# exported symbol -> (restype, argtypes); every function include/lesgo_gpu.h declares
_H = C.c_void_p
_I = C.c_int
_D = C.POINTER(C.c_double)
SIGNATURES = {
    "lesgo_gpu_params_default": (_I, [C.POINTER(Params)]),
    "lesgo_gpu_create": (_I, [C.POINTER(Params), C.POINTER(_H)]),
    "lesgo_gpu_destroy": (_I, [_H]),
    "lesgo_gpu_last_error": (C.c_char_p, [_H]),
    "lesgo_gpu_dims": (_I, [_H, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "lesgo_gpu_set_field": (_I, [_H, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_get_field": (_I, [_H, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_set_field_async": (_I, [_H, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_get_field_async": (_I, [_H, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_bind_field": (_I, [_H, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_upload": (_I, [_H, _I]),
    "lesgo_gpu_download": (_I, [_H, _I]),
    "lesgo_gpu_init_ic": (_I, [_H, C.c_uint64]),
    "lesgo_gpu_filt_da": (_I, [_H, _I, _I, _I]),
    "lesgo_gpu_ddx": (_I, [_H, _I, _I]),
    "lesgo_gpu_ddy": (_I, [_H, _I, _I]),
    "lesgo_gpu_ddxy": (_I, [_H, _I, _I, _I]),
    "lesgo_gpu_ddz_uv": (_I, [_H, _I, _I]),
    "lesgo_gpu_ddz_w": (_I, [_H, _I, _I]),
    "lesgo_gpu_test_filter": (_I, [_H, _I, _I]),
    "lesgo_gpu_wallstress": (_I, [_H]),
    "lesgo_gpu_sgs_stag": (_I, [_H]),
    "lesgo_gpu_divstress_uv": (_I, [_H]),
    "lesgo_gpu_divstress_w": (_I, [_H]),
    "lesgo_gpu_convec": (_I, [_H]),
    "lesgo_gpu_turbines_forcing": (_I, [_H]),
    "lesgo_gpu_begin_step": (_I, [_H]),
    "lesgo_gpu_rhs_assemble": (_I, [_H]),
    "lesgo_gpu_ab2": (_I, [_H]),
    "lesgo_gpu_press_stag_array": (_I, [_H]),
    "lesgo_gpu_rhs_sub_dp": (_I, [_H]),
    "lesgo_gpu_project": (_I, [_H]),
    "lesgo_gpu_tridag_array": (_I, [_H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _I, _I, _I]),
    "lesgo_gpu_tridag_array_noalloc": (_I, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _I, _I, _I,
                                            C.c_void_p]),
    "lesgo_gpu_step": (_I, [_H, _I]),
    "lesgo_gpu_sync": (_I, [_H]),
    "lesgo_gpu_diag": (_I, [_H, _D, _D, _D, _D]),
    "lesgo_gpu_counters": (_I, [_H, C.POINTER(_I), C.POINTER(_I)]),
    "lesgo_gpu_turbine_state": (_I, [_H, _D, _D, _D, _I]),
    "lesgo_gpu_launches_per_step": (_I, [_H, _I]),
    "lesgo_gpu_batch_create": (_I, [C.POINTER(Params), _I, C.POINTER(_H)]),
    "lesgo_gpu_batch_add": (_I, [_H, C.c_double, C.c_uint64, _I, C.POINTER(Turbine), C.POINTER(_I)]),
    "lesgo_gpu_batch_remove": (_I, [_H, _I]),
    "lesgo_gpu_batch_size": (_I, [_H, C.POINTER(_I), C.POINTER(_I)]),
    "lesgo_gpu_set_field_inst": (_I, [_H, _I, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_get_field_inst": (_I, [_H, _I, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_set_field_inst_async": (_I, [_H, _I, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_get_field_inst_async": (_I, [_H, _I, _I, C.c_void_p, _I, _I]),
    "lesgo_gpu_diag_inst": (_I, [_H, _I, _D, _D, _D, _D]),
    "lesgo_gpu_counters_inst": (_I, [_H, _I, C.POINTER(_I), C.POINTER(_I)]),
    "lesgo_gpu_turbine_state_inst": (_I, [_H, _I, _D, _D, _D, _I]),
    "lesgo_gpu_turbine_schedule": (_I, [_H, _I, _I, _D]),
    "lesgo_gpu_turbine_schedule_inst": (_I, [_H, _I, _I, _I, _D]),
    "lesgo_gpu_turbine_controls": (_I, [_H, _I, _D, _D, _D, _I]),
    "lesgo_gpu_read_turbine_schedule": (_I, [C.c_char_p, _I, _I, _D, _I, C.POINTER(_I)]),
    "lesgo_gpu_footprint": (_I, [C.POINTER(Params), _I, C.POINTER(C.c_longlong)]),
    "lesgo_gpu_autotune": (_I, [_H, C.POINTER(_I), C.POINTER(_I)]),
    "lesgo_gpu_diag_log_config": (_I, [_H, _I, _I]),
    "lesgo_gpu_diag_log_sample": (_I, [_H]),
    "lesgo_gpu_diag_log_read": (_I, [_H, _I, _D, _I, C.POINTER(_I)]),
    "lesgo_gpu_tavg_config": (_I, [_H, _I, _I, _I]),
    "lesgo_gpu_tavg_sample": (_I, [_H]),
    "lesgo_gpu_tavg_get": (_I, [_H, _I, _D, _I, _I]),
    "lesgo_gpu_tavg_get_inst": (_I, [_H, _I, _I, _D, _I, _I]),
    "lesgo_gpu_tavg_profile": (_I, [_H, _I, _D, _I]),
    "lesgo_gpu_tavg_profile_inst": (_I, [_H, _I, _I, _D, _I]),
    "lesgo_gpu_tavg_total_time": (_I, [_H, _I, _D]),
    "lesgo_gpu_checkpoint_write": (_I, [_H, C.c_char_p, _I]),
    "lesgo_gpu_checkpoint_write_inst": (_I, [_H, _I, C.c_char_p, _I]),
    "lesgo_gpu_checkpoint_read": (_I, [_H, C.c_char_p, C.POINTER(_I)]),
    "lesgo_gpu_checkpoint_read_inst": (_I, [_H, _I, C.c_char_p, C.POINTER(_I)]),
    "lesgo_gpu_sim_time": (_I, [_H, _I, _D]),
    "lesgo_gpu_time_step": (_I, [_H, _I, _D]),
    "lesgo_gpu_read_conf": (_I, [C.c_char_p, _I, C.POINTER(Params), C.POINTER(Run), C.POINTER(Turbine), _I,
                                 C.c_char_p, _I]),
    "lesgo_gpu_profile": (_I, [_H, _I]),
    "lesgo_gpu_profile_report": (_I, [_H, C.c_char_p, _I]),
    "lesgo_gpu_get_stream": (_I, [_H, C.POINTER(C.c_void_p)]),
}

_lib = None


def load(path: str = LIB) -> C.CDLL:
    """Load the library (once) and attach the prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: the CUDA library must be built (python -m lesgo_gb300.build)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
