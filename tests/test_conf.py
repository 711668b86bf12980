"""lesgo.conf reader (input_util.f90:54-1023) and turbine placement
(turbines.f90:740-866), host only: no GPU needed.

Configurations are written by the tests in the reference's syntax: blocks
`NAME { ... }`, `key = value` lines, `!` comment lines, blanks and tabs
anywhere, case-insensitive keys, Fortran list-directed values (`.true.`,
`T`, `1.0d-4`).  Expected values are written out by hand; the placements of
every orientation are checked against a restatement in the test.
"""
import math
import os

import pytest

from lesgo_gb300 import _lib as L
from lesgo_gb300.solver import LesgoError, read_conf

FULL = """! channel with a wind farm
DOMAIN {
  nproc = 4
  Nx = 48
  Ny = 32
  Nz = 24\t
  z_i = 500.0
  Lx = 6.283185307
  Ly = 3.14159
  Lz = 1.0
  uniform_spacing = .false.
}
MODEL {
  SGS_MODEL = 5
  wall_damp_exp = 2
  cs_count = 3
  dyn_init = 50
  Co = 0.2
  ifilter = 1
  u_star = 0.5
  vonk = 0.41
  sgs = T
  molec = .false.
  nu_molec = 1.5d-5
}
CORIOLIS {
  coriolis_forcing = 0
  fc = 0.0001
}
TIME {
  nsteps = 1234
  runtime = -1
  use_cfl_dt = .true.
  cfl = 0.0625
  dt = 1.0d-4
  cumulative_time = .false.
}
FLOW_COND {
  initu = .false.
  inilag = .true.
  lbc_mom = 2
  ubc_mom = 0
  zo = 2e-4
  inflow_type = 0
  use_mean_p_force = .true.
  eval_mean_p_force = .true.
  mean_p_force_x = 1.0
  mean_p_force_y = 0.5
  u_file = './somewhere'
}
OUTPUT {
  wbase = 10
  nenergy = 20
  lag_cfl_count = 30
  checkpoint_data = .true.
  checkpoint_nskip = 500
  tavg_calc = .true.
  tavg_nstart = 100
  tavg_nend = 900
  tavg_nskip = 10
  point_loc = 0.1, 0.1, 0.1 // 0.5, 0.5, 0.5
  xplane_calc = .false.
  mystery_key = 3
}
LEVEL_SET {
  global_CA_calc = .true.
}
TURBINES {
  num_x = 4
  num_y = 3
  dia_all = 50
  height_all = 50
  thk_all = 5
  orientation = 1
  stag_perc = 50
  theta1_all = 10
  theta2_all = 0
  Ct_prime = 1.2
  read_param = .false.
  T_avg_dim = 100
  alpha1 = 1.2
  alpha2 = 1.3
  filter_cutoff = 1e-3
  adm_correction = .false.
}
"""


def write(tmp_path, text, name="lesgo.conf"):
    (tmp_path / name).write_text(text)
    return str(tmp_path) + os.sep


def test_full_configuration(built_lib, tmp_path):
    kw, run, log = read_conf(write(tmp_path, FULL))
    assert (kw["nx"], kw["ny"], kw["Nz"]) == (48, 32, 24)
    assert (kw["L_x"], kw["L_y"], kw["L_z"], kw["z_i"]) == (6.283185307, 3.14159, 1.0, 500.0)
    assert (kw["sgs_model"], kw["cs_count"], kw["dyn_init"], kw["ifilter"]) == (5, 3, 50, 1)
    assert (kw["u_star"], kw["vonk"], kw["nu_molec"], kw["molec"]) == (0.5, 0.41, 1.5e-5, False)
    assert (kw["dt"], kw["zo"], kw["lbc_mom"], kw["ubc_mom"], kw["initu"]) == (1e-4, 2e-4, 2, 0, False)
    assert (kw["use_mean_p_force"], kw["eval_mean_p_force"], kw["mean_p_force_y"]) == (True, True, 0.5)
    assert (kw["alpha1"], kw["alpha2"], kw["filter_cutoff"], kw["T_avg_dim"], kw["adm_correction"]) == \
        (1.2, 1.3, 1e-3, 100.0, False)
    assert (run["nproc"], run["wall_damp_exp"], run["Co"], run["sgs"]) == (4, 2, 0.2, 1)
    assert (run["nsteps"], run["runtime"], run["use_cfl_dt"], run["cfl"], run["cumulative_time"]) == \
        (1234, -1, 1, 0.0625, 0)
    assert (run["wbase"], run["nenergy"], run["lag_cfl_count"]) == (10, 20, 30)
    assert (run["checkpoint_data"], run["checkpoint_nskip"]) == (1, 500)
    assert (run["tavg_calc"], run["tavg_nstart"], run["tavg_nend"], run["tavg_nskip"]) == (1, 100, 900, 10)
    assert "Found unused input block: LEVEL_SET" in log
    assert "OUTPUT block: MYSTERY_KEY" in log
    ts = kw["turbines"]
    assert len(ts) == 12
    # orientation 1: a num_x x num_y grid, cells L/num centred, sizes / z_i
    assert ts[0]["xloc"] == pytest.approx(6.283185307 / 4 * 0.5, rel=1e-15)
    assert ts[4]["yloc"] == pytest.approx(3.14159 / 3 * 1.5, rel=1e-15)
    assert (ts[5]["dia"], ts[5]["height"], ts[5]["thk"], ts[5]["theta1"], ts[5]["Ct_prime"]) == \
        (0.1, 0.1, 0.01, 10.0, 1.2)


def test_defaults_are_the_references(built_lib, tmp_path):
    """An empty file: param.f90's defaults (lbc_mom = 1, eval_mean_p_force
    false, cfl a default-real 0.05, L_y = 2 pi, ...)."""
    kw, run, _ = read_conf(write(tmp_path, "! nothing\n"), with_turbines=False)
    assert (kw["nx"], kw["ny"], kw["Nz"], kw["lbc_mom"], kw["eval_mean_p_force"]) == (64, 64, 64, 1, False)
    assert kw["L_y"] == pytest.approx(2 * math.pi, rel=1e-16)
    assert run["cfl"] == float.fromhex("0x1.99999a0000000p-5")
    assert (run["tavg_nstart"], run["tavg_nend"], run["tavg_nskip"], run["nsteps"]) == (1, 50000, 100, 50000)
    assert kw["turbines"] == []


def test_uniform_spacing(built_lib, tmp_path):
    kw, _, _ = read_conf(write(tmp_path, "DOMAIN {\nNx=32\nNy=16\nNz=8\nLx=2.0\nuniform_spacing=.true.\n}\n"))
    assert kw["L_y"] == 16 * (2.0 / 32) and kw["L_z"] == 8 * (2.0 / 32)


def test_turbines_block_skipped_without_turbines(built_lib, tmp_path):
    kw, _, log = read_conf(write(tmp_path, FULL), with_turbines=False)
    assert kw["turbines"] == [] and "Found unused input block: TURBINES" in log


@pytest.mark.parametrize("text,code,msg", [
    ("Nx = 32\n", L.LESGO_ERR_ARG, "block entry not found"),
    ("DOMAIN {\nNx 32\n}\n", L.LESGO_ERR_ARG, "Bad read in block at line"),
    ("DOMAIN {\nNx =\n}\n", L.LESGO_ERR_ARG, "nothing after equals sign"),
    ("DOMAIN {\nNx = 32}\n", L.LESGO_ERR_ARG, "not formatted correctly"),
    ("DOMAIN {\nNx = 3x2\n}\n", L.LESGO_ERR_ARG, "not an integer"),
    ("DOMAIN {\nNx = 32\n", L.LESGO_ERR_ARG, "Bad read in block"),
    ("CORIOLIS {\ncoriolis_forcing = 1\n}\n", L.LESGO_ERR_UNSUPPORTED, "coriolis_forcing"),
    ("FLOW_COND {\nuse_sponge = .true.\n}\n", L.LESGO_ERR_UNSUPPORTED, "use_sponge"),
    ("MODEL {\nsgs = .false.\n}\n", L.LESGO_ERR_UNSUPPORTED, "sgs"),
    ("TURBINES {\nnum_x = 1\nnum_y = 1\nuse_rotation = T\n}\n", L.LESGO_ERR_UNSUPPORTED, "use_rotation"),
])
def test_errors(built_lib, tmp_path, text, code, msg):
    with pytest.raises(LesgoError) as ei:
        read_conf(write(tmp_path, text))
    assert ei.value.code == code and msg in str(ei.value)


def test_missing_file(built_lib, tmp_path):
    with pytest.raises(LesgoError) as ei:
        read_conf(str(tmp_path) + os.sep)
    assert ei.value.code == L.LESGO_ERR_ARG and "does not exist" in str(ei.value)


def place(num_x, num_y, orientation, stag, Lx, Ly, dia, height):
    """turbines.f90:790-866 restated (units of z_i already applied)."""
    sxx, syy = Lx / num_x, Ly / num_y
    xs, ys, hs = [], [], []
    for i in range(1, num_x + 1):
        for j in range(1, num_y + 1):
            xs.append(sxx * (2 * i - 1) / 2)
            ys.append(syy * (2 * j - 1) / 2)
            hs.append(height)
    if orientation == 2:
        for i in range(2, num_x + 1):
            for k in range(num_y * (i - 1), num_y * i):
                ys[k] = math.fmod(ys[k] + (i - 1) * syy * stag / 100.0, Ly)
    elif orientation == 3:
        for i in range(1, num_x + 1):
            for k in range(num_y * (i - 1), num_y * i):
                hs[k] = height * (1.0 + stag / 100.0) if i % 2 == 0 else height * (1.0 - stag / 100.0)
    elif orientation == 4:
        k = 0
        for i in range(1, num_x + 1):
            for j in range(1, num_y + 1):
                c = 2.0 * ((i + j) % 2) - 1.0
                hs[k] = height * (1.0 + c * stag / 100.0)
                k += 1
    elif orientation == 5:
        d = stag * (ys[1] - ys[0])
        k = 0
        for i in range(1, num_x + 1):
            for j in range(1, num_y + 1):
                ys[k] = math.fmod(ys[k] + d * (i - 1), Ly)
                k += 1
    return xs, ys, hs


@pytest.mark.parametrize("orientation", [1, 2, 3, 4, 5])
def test_turbine_orientations(built_lib, tmp_path, orientation):
    stag = 0.3 if orientation == 5 else 40.0
    text = ("DOMAIN {\nLx = 6.0\nLy = 3.0\nz_i = 1000\n}\nTURBINES {\nnum_x = 3\nnum_y = 4\ndia_all = 100\n"
            f"height_all = 80\nthk_all = 10\norientation = {orientation}\nstag_perc = {stag}\n}}\n")
    kw, _, _ = read_conf(write(tmp_path, text))
    xs, ys, hs = place(3, 4, orientation, stag, 6.0, 3.0, 0.1, 0.08)
    got = kw["turbines"]
    assert [t["xloc"] for t in got] == pytest.approx(xs, rel=1e-15)
    assert [t["yloc"] for t in got] == pytest.approx(ys, rel=1e-15)
    assert [t["height"] for t in got] == pytest.approx(hs, rel=1e-15)


def test_turbines_from_param_dat(built_lib, tmp_path):
    (tmp_path / "input_turbines").mkdir()
    (tmp_path / "input_turbines" / "param.dat").write_text(
        "1000.0, 500.0, 100.0, 100.0, 10.0, 5.0, 0.0, 1.33\n"
        "1700.0 1500.0 100.0 100.0 10.0 0.0 0.0 1.2\n")
    text = "TURBINES {\nnum_x = 2\nnum_y = 1\nread_param = .true.\n}\n"
    kw, _, _ = read_conf(write(tmp_path, text))
    t = kw["turbines"]
    assert [(x["xloc"], x["yloc"], x["height"], x["dia"], x["thk"], x["theta1"], x["Ct_prime"]) for x in t] == \
        [(1.0, 0.5, 0.1, 0.1, 0.01, 5.0, 1.33), (1.7, 1.5, 0.1, 0.1, 0.01, 0.0, 1.2)]
    with pytest.raises(LesgoError):
        read_conf(write(tmp_path, "TURBINES {\nnum_x = 3\nnum_y = 1\nread_param = T\n}\n"))


def test_dynamic_turbine_flags_and_schedules(built_lib, tmp_path):
    """dyn_theta1 / dyn_theta2 / dyn_Ct_prime are reported; the control files
    (read_control_files, turbines.f90:872-931) hold one row per line: the
    dimensional time and one value per turbine, list-directed."""
    from lesgo_gb300.solver import read_turbine_schedule
    text = ("TURBINES {\nnum_x = 2\nnum_y = 1\ndyn_theta1 = .true.\ndyn_Ct_prime = T\n}\n")
    _, run, _ = read_conf(write(tmp_path, text))
    assert (run["dyn_theta1"], run["dyn_theta2"], run["dyn_ct_prime"]) == (1, 0, 1)
    (tmp_path / "input_turbines").mkdir()
    (tmp_path / "input_turbines" / "theta1.dat").write_text("0.0 0.0 5.0\n\n10.0, 20.0, -5d0\n 25 1.5D1 0\n")
    rows = read_turbine_schedule(str(tmp_path) + os.sep, "theta1", 2)
    assert rows.tolist() == [[0.0, 0.0, 5.0], [10.0, 20.0, -5.0], [25.0, 15.0, 0.0]]
    (tmp_path / "input_turbines" / "Ct_prime.dat").write_text("0.0 1.33\n")
    with pytest.raises(LesgoError) as ei:
        read_turbine_schedule(str(tmp_path) + os.sep, 2, 2)
    assert ei.value.code == L.LESGO_ERR_ARG and "Ct_prime.dat:1" in str(ei.value)
    with pytest.raises(LesgoError):
        read_turbine_schedule(str(tmp_path) + os.sep, "theta2", 2)
    from lesgo_gb300.solver import conf_turbine_schedules
    (tmp_path / "input_turbines" / "Ct_prime.dat").write_text("0.0 1.33 1.2\n5.0 1.0 1.1\n")
    sch = conf_turbine_schedules(str(tmp_path) + os.sep, run, 2)
    assert sorted(sch) == ["Ct_prime", "theta1"] and sch["Ct_prime"].shape == (2, 3)


def test_schedule_interpolation_semantics():
    """binary_search + linear_interp (functions.f90:712-860): clamped to the
    first / last value outside the table, exact at the samples, linear in
    between; a repeated time takes the bracket the bisection finds."""
    from oracle.lesgo_oracle import sched_interp
    x, v = [0.0, 1.0, 3.0, 3.0, 7.0], [10.0, 20.0, 0.0, 8.0, -4.0]
    assert sched_interp(x, v, -1.0) == 10.0 and sched_interp(x, v, 8.0) == -4.0
    assert sched_interp(x, v, 0.5) == 15.0
    assert sched_interp(x, v, 2.0) == 10.0
    assert sched_interp(x, v, 1.0) == 20.0
    assert sched_interp(x, v, 5.0) == 8.0 + 2.0 * (-12.0) / 4.0
    assert sched_interp(x, v, 7.0) == -4.0
    assert sched_interp([2.0], [5.0], 2.0) == 5.0 and sched_interp([2.0], [5.0], 9.0) == 5.0
