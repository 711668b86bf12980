"""The C-ABI library: it builds, loads, exports every symbol the header
declares, its struct layout matches the ctypes mirror, and without a GPU it
fails loudly with a status code (no CPU fallback).  CPU only."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "lesgo_gpu.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(lesgo_gpu_\w+)\s*\(", txt, re.M)))


def test_header_declares_the_stage_entry_points():
    fns = header_functions()
    for name in ("filt_da", "ddx", "ddy", "ddxy", "ddz_uv", "ddz_w", "convec", "press_stag_array", "sgs_stag",
                 "divstress_uv", "divstress_w", "wallstress", "turbines_forcing", "project", "step", "diag"):
        assert "lesgo_gpu_" + name in fns


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    for name in header_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lesgo_gpu_\w+)", out))
    assert set(header_functions()) <= exported


def test_ctypes_signatures_cover_header():
    from lesgo_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(header_functions())


def test_params_layout_matches_c(tmp_path):
    from lesgo_gb300 import _lib
    src = tmp_path / "lay.c"
    fields = [f[0] for f in _lib.Params._fields_]
    body = "\n".join(f'printf("%zu\\n", offsetof(lesgo_params_t, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "lesgo_gpu.h"\n'
                   f'int main(void){{printf("%zu\\n", sizeof(lesgo_params_t)); printf("%zu\\n", sizeof(lesgo_turbine_t));\n{body}\nreturn 0;}}\n')
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(_lib.Params)
    assert vals[1] == C.sizeof(_lib.Turbine)
    for f, off in zip(fields, vals[2:]):
        assert getattr(_lib.Params, f).offset == off, f


def test_run_layout_matches_c(tmp_path):
    from lesgo_gb300 import _lib
    src = tmp_path / "run.c"
    fields = [f[0] for f in _lib.Run._fields_]
    body = "\n".join(f'printf("%zu\\n", offsetof(lesgo_run_t, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "lesgo_gpu.h"\n'
                   f'int main(void){{printf("%zu\\n", sizeof(lesgo_run_t));\n{body}\nreturn 0;}}\n')
    exe = tmp_path / "run"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(_lib.Run)
    for f, off in zip(fields, vals[1:]):
        assert getattr(_lib.Run, f).offset == off, f


def test_params_default_on_host(built_lib):
    from lesgo_gb300 import _lib
    lib = _lib.load()
    p = _lib.Params()
    assert lib.lesgo_gpu_params_default(C.byref(p)) == 0
    assert (p.lbc_mom, p.ubc_mom, p.sgs_model, p.cs_count, p.dyn_init) == (2, 0, 5, 5, 100)
    assert abs(p.dt - 2e-4) < 1e-18 and abs(p.zo - 1e-4) < 1e-18
    assert lib.lesgo_gpu_params_default(None) == _lib.LESGO_ERR_ARG


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_no_gpu_fails_loudly(built_lib):
    from lesgo_gb300.solver import LesgoError, LesgoGPU
    with pytest.raises(LesgoError) as ei:
        LesgoGPU(nx=32, ny=32, Nz=16)
    assert ei.value.code in (2, 4)


def test_null_handle_is_rejected(built_lib):
    from lesgo_gb300 import _lib
    lib = _lib.load()
    assert lib.lesgo_gpu_step(None, 1) == _lib.LESGO_ERR_ARG
    assert lib.lesgo_gpu_destroy(None) == _lib.LESGO_ERR_ARG
    assert lib.lesgo_gpu_filt_da(None, 0, 3, 4) == _lib.LESGO_ERR_ARG
