"""Checkpoint / restart files (io.f90:1173-1267; initial.f90:20-380;
io.f90:60-96; time_average.f90:114-150, :665-716).

CPU tests pin the oracle's restatement of the file formats (gfortran record
framing with subrecords, total_time.dat as list-directed text) and of the
ic_interp regrid (exact on a matching grid, exact for fields linear in z and
on coarse-grid nodes in x-y).  GPU tests check the library against it:
files the library writes read back in the oracle field for field; a run
restarted from its own checkpoint equals the uninterrupted run bit for bit
(FP64 and mixed); regrids from a coarser checkpoint and from a two-rank MPI
checkpoint equal the oracle's ic_interp; the time-average sums carried
through tavg.out equal the oracle's restarted TimeAverage.
"""
import os
import struct

import numpy as np
import pytest

from oracle.lesgo_oracle import (SUBMAX, TAVG_FILE, VEL_FIELDS, Oracle, Params, TimeAverage, binary_search,
                                 fortran_record_bytes, fortran_records, ic_interp, oracle_state, read_checkpoint,
                                 write_checkpoint)


def test_record_framing_small():
    rec = fortran_record_bytes(b"abcdefgh")
    assert rec == struct.pack("<i", 8) + b"abcdefgh" + struct.pack("<i", 8)
    assert fortran_records(rec + fortran_record_bytes(b"")) == [b"abcdefgh", b""]


def test_record_framing_subrecords():
    """A payload split into 3 subrecords: leading markers -10, -10, 5;
    trailing markers 10, -10, -5."""
    payload = bytes(range(25))
    rec = fortran_record_bytes(payload, submax=10)
    lead = [struct.unpack_from("<i", rec, o)[0] for o in (0, 18, 36)]
    trail = [struct.unpack_from("<i", rec, o)[0] for o in (14, 32, 45)]
    assert lead == [-10, -10, 5] and trail == [10, -10, -5]
    assert fortran_records(rec) == [payload]
    assert SUBMAX == 2 ** 31 - 9


def test_binary_search_reference_semantics():
    a = [0.0, 1.0, 2.0, 3.0]
    assert binary_search(a, -0.1) == 0 and binary_search(a, 3.5) == 4
    assert binary_search(a, 0.0) == 1 and binary_search(a, 0.5) == 1
    assert binary_search(a, 2.0) == 3 and binary_search(a, 2.5) == 3
    assert binary_search(a, 3.0) == 3


def test_ic_interp_same_grid_and_linear_fields():
    p = Params(nx=16, ny=8, Nz=8)
    rng = np.random.default_rng(1)
    f = [rng.standard_normal((p.nz, p.ny, p.ld)) for _ in range(3)]
    u, v, w = ic_interp(p, (p.nx, p.ny, p.nz, p.L_x, p.L_y, p.L_z), *f)
    for a, b in zip((u, v, w), f):
        assert np.allclose(a[:, :, :p.nx], b[:, :, :p.nx], rtol=0, atol=1e-12)
    # a coarser file grid, fields linear in z (reproduced exactly inside the
    # file's range) and constant in x, y
    pf = Params(nx=8, ny=4, Nz=4)
    zc = (np.arange(1, pf.nz + 1) - 0.5) * pf.dz
    zw = (np.arange(1, pf.nz + 1) - 1.0) * pf.dz
    uf = np.broadcast_to((2.0 + 3.0 * zc)[:, None, None], (pf.nz, pf.ny, pf.ld)).copy()
    wf = np.broadcast_to((1.0 - zw)[:, None, None], (pf.nz, pf.ny, pf.ld)).copy()
    u, v, w = ic_interp(p, (pf.nx, pf.ny, pf.nz, pf.L_x, pf.L_y, pf.L_z), uf, uf, wf)
    z = (np.arange(1, p.nz + 1) - 0.5) * p.dz
    inside = (z >= zc[0]) & (z <= zc[-1])
    assert np.allclose(u[inside, :, :p.nx], (2.0 + 3.0 * z[inside])[:, None, None], atol=1e-12)
    assert np.allclose(w[:, :, :p.nx], (1.0 - (np.arange(p.nz) * p.dz))[:, None, None], atol=1e-12)


def test_oracle_checkpoint_roundtrip(tmp_path):
    p = Params(nx=16, ny=8, Nz=8)
    o = Oracle(p)
    o.set_ic(4)
    o.jt_total, o.time = 37, 0.0074
    rng = np.random.default_rng(2)
    for n in VEL_FIELDS[3:]:
        oracle_state(o, n)[:] = rng.standard_normal(oracle_state(o, n).shape)
    pre = str(tmp_path) + os.sep
    write_checkpoint(o, pre)
    o2 = Oracle(Params(nx=16, ny=8, Nz=8))
    assert read_checkpoint(o2, pre) is True
    for n in VEL_FIELDS:
        assert np.array_equal(oracle_state(o2, n)[1:], oracle_state(o, n)[1:]), n
    assert (o2.jt_total, o2.time, o2.jt, o2.p.initu) == (37, 0.0074, 0, True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
BASE = dict(nx=32, ny=32, Nz=16, dyn_init=3, cs_count=3)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp64dw", "mixed"])
def test_gpu_restart_is_bitwise(built_lib, tmp_path, precision):
    """10 steps straight == 5 steps, checkpoint, restart in a new handle, 5 steps."""
    from lesgo_gb300.solver import LesgoGPU
    a = LesgoGPU(precision=precision, **BASE)
    a.init_ic(5)
    a.step(10)
    b = LesgoGPU(precision=precision, **BASE)
    b.init_ic(5)
    b.step(5)
    pre = str(tmp_path) + os.sep
    b.checkpoint_write(pre)
    b.close()
    c = LesgoGPU(precision=precision, **BASE)
    assert c.checkpoint_read(pre) is True
    assert c.counters() == (0, 5)
    c.step(5)
    assert c.counters() == (5, 10)
    assert c.sim_time() == pytest.approx(a.sim_time(), rel=1e-15)
    for f in ("u", "v", "w", "p", "RHSx", "Cs_opt2", "F_LM", "F_QN"):
        assert np.array_equal(a.get(f)[1:a.nz], c.get(f)[1:c.nz]), f
    a.close()
    c.close()


@pytest.mark.gpu
def test_gpu_checkpoint_files_read_by_oracle(built_lib, tmp_path):
    from lesgo_gb300.solver import LesgoGPU
    g = LesgoGPU(**BASE)
    g.init_ic(6)
    g.step(4)
    pre = str(tmp_path) + os.sep
    g.checkpoint_write(pre, mpi_names=True)
    assert os.path.exists(pre + "vel.out.c0")
    p = Params(**BASE)
    o = Oracle(p)
    assert read_checkpoint(o, pre) is True
    for n in VEL_FIELDS:
        assert np.array_equal(oracle_state(o, n)[1:], g.get(n)[1:]), n
    assert (o.jt_total, o.time) == (4, pytest.approx(4 * p.dt, rel=1e-15))
    with open(pre + "grid.out", "rb") as f:
        rec, = fortran_records(f.read())
    assert struct.unpack("<4i3d", rec) == (1, p.nx, p.ny, p.nz, p.L_x, p.L_y, p.L_z)
    g.close()


@pytest.mark.gpu
def test_gpu_restart_matches_oracle_restart(built_lib, tmp_path):
    """An oracle-written checkpoint: the GPU and the oracle both restart from
    it (initu) and step 4 more times."""
    from gpu_util import rel_err
    from lesgo_gb300.solver import LesgoGPU
    p = Params(**BASE)
    o = Oracle(p)
    o.set_ic(7)
    for _ in range(4):
        o.step()
    pre = str(tmp_path) + os.sep
    write_checkpoint(o, pre)
    g = LesgoGPU(**BASE)
    assert g.checkpoint_read(pre) is True
    o2 = Oracle(Params(**BASE))
    read_checkpoint(o2, pre)
    for _ in range(4):
        o2.step()
    g.step(4)
    for f in ("u", "v", "w", "p"):
        e = rel_err(o2.p, f, g.get(f), oracle_state(o2, f))
        assert e < 1e-10, (f, e)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("nproc", [1, 2])
def test_gpu_regrid_matches_oracle(built_lib, tmp_path, nproc):
    """A coarser checkpoint (one rank, or two MPI ranks' files) is
    interpolated onto the handle's grid as ic_interp does."""
    from lesgo_gb300.solver import LesgoGPU
    pc = Params(nx=16, ny=16, Nz=8)
    oc = Oracle(pc)
    oc.set_ic(8)
    pre = str(tmp_path) + os.sep
    if nproc == 1:
        write_checkpoint(oc, pre)
    else:
        # two ranks of nz_l = 5 levels each (global 9 = 2 * 4 + 1), the
        # shared level written by both
        nzl = (pc.nz - 1) // 2 + 1
        for c in range(2):
            lev = slice(c * (nzl - 1) + 1, c * (nzl - 1) + nzl + 1)
            payload = b"".join(np.ascontiguousarray(oracle_state(oc, n)[lev]).tobytes() for n in VEL_FIELDS)
            with open(pre + "vel.out.c%d" % c, "wb") as f:
                f.write(fortran_record_bytes(payload))
        with open(pre + "grid.out", "wb") as f:
            f.write(fortran_record_bytes(struct.pack("<4i3d", 2, pc.nx, pc.ny, nzl, pc.L_x, pc.L_y, pc.L_z)))
    g = LesgoGPU(nx=32, ny=24, Nz=12)
    assert g.checkpoint_read(pre) is False
    o = Oracle(Params(nx=32, ny=24, Nz=12))
    assert read_checkpoint(o, pre) is False
    for f in ("u", "v", "w"):
        a, b = g.get(f)[1:, :, :32], getattr(o, f)[1:, :, :32]
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b)), f
    assert np.all(g.get("RHSx")[1:] == 0.0)
    g.step(2)                                    # AB2 from RHS_f = 0, as the reference does
    assert np.isfinite(g.diag()["ke"])
    g.close()


@pytest.mark.gpu
def test_gpu_tavg_restart_matches_oracle(built_lib, tmp_path):
    """tavg.out carries the sums (not the pressure sum) into the restarted
    run, which takes them up at its first sample step."""
    from lesgo_gb300.solver import LesgoGPU
    g = LesgoGPU(**BASE)
    g.init_ic(9)
    g.tavg_config(2, 100, 2)
    g.step(6)
    pre = str(tmp_path) + os.sep
    g.checkpoint_write(pre)
    assert os.path.exists(pre + "tavg.out")
    g.close()
    # restart both from the same files
    g2 = LesgoGPU(**BASE)
    g2.tavg_config(2, 100, 2)
    g2.checkpoint_read(pre)
    o = Oracle(Params(**BASE))
    ta = TimeAverage(o, 2, 100, 2)
    read_checkpoint(o, pre, ta)
    for _ in range(7):
        o.step()
        ta.after_step()
    g2.step(7)
    assert g2.tavg_total_time() == pytest.approx(ta.total_time, rel=1e-14)
    with open(pre + "tavg.out", "rb") as f:
        total0, = struct.unpack("<d", fortran_records(f.read())[0])
    assert ta.total_time > total0 > 0
    for name in ("u", "w", "uw", "txz", "vortz", "p", "upwp"):
        ref = ta.mean(name)[1:o.p.nz]
        a = g2.tavg_get(name)[:o.p.nz - 1, :, :o.p.nx]
        assert np.max(np.abs(a - ref)) <= 1e-10 * max(np.max(np.abs(ref)), 1e-30), name
    g2.close()


@pytest.mark.gpu
def test_gpu_rejects_big_endian_checkpoint(built_lib, tmp_path):
    """The reference's WRITE_ENDIAN=BIG build writes every record marker and
    value big-endian; the reader names that instead of reading a byte-swapped
    record length."""
    from lesgo_gb300.solver import LesgoError, LesgoGPU
    g = LesgoGPU(**BASE)
    ld = 2 * (BASE["nx"] // 2 + 1)
    nzf = BASE["Nz"] + 1
    payload = np.zeros(11 * ld * BASE["ny"] * nzf, dtype=">f8").tobytes()
    rec = struct.pack(">i", len(payload)) + payload + struct.pack(">i", len(payload))
    pre = str(tmp_path) + os.sep
    with open(pre + "vel.out", "wb") as f:
        f.write(rec)
    with pytest.raises(LesgoError) as ei:
        g.checkpoint_read(pre)
    assert "big-endian" in str(ei.value)
    g.close()
