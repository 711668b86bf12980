"""The forward x transforms as tensor-core GEMMs (k_xdft_tc, LESGO_XDFT=1)
against the radix kernels and the FP64 oracle (GPU required).

The GEMM form multiplies each x row by the real DFT matrix on the tcgen05
tensor cores with three-pass TF32 splitting (hi*Whi + hi*Wlo + lo*Whi,
FP32 accumulation), so its values differ from the radix FFT's by FP32
rounding: against the FP64 oracle a filtered-derivative stage stays below
1e-5 of each output's maximum in both forms (the GEMM form's error is up to
5x the radix form's: 2.5e-6 against 4.7e-7 at nx = 128), stepped fields
agree with the radix form's within 5e-5 (pressure 1e-3), and the 10-step
fields stay within the mixed form's 2e-4 bar against the oracle.
"""
import numpy as np
import pytest

from gpu_util import make_pair, oracle_field, rel_err

pytestmark = pytest.mark.gpu

GRIDS = [(32, 32, 16), (48, 32, 24), (64, 64, 40), (96, 48, 9), (128, 64, 16)]
# 195 tiles of the three-field passes: blocks take two tiles each, so the
# stage ring wraps several times and both accumulator sets are reused
MULTI_TILE = (128, 128, 64)


def _pair(monkeypatch, grid, **kw):
    from lesgo_gb300.solver import LesgoGPU
    nx, ny, Nz = grid
    args = dict(nx=nx, ny=ny, Nz=Nz, precision="mixed", dyn_init=3, cs_count=3)
    args.update(kw)
    monkeypatch.setenv("LESGO_XDFT", "0")
    a = LesgoGPU(**args)
    monkeypatch.setenv("LESGO_XDFT", "1")
    b = LesgoGPU(**args)
    monkeypatch.delenv("LESGO_XDFT")
    return a, b


def _close(x, y, tol):
    return np.max(np.abs(x - y)) <= tol * np.max(np.abs(x))


@pytest.mark.parametrize("grid", GRIDS)
def test_filtered_derivatives_as_accurate_as_radix(built_lib, monkeypatch, grid):
    """filt_da (x forward as a GEMM, y pass, x inverse) on one field, both
    forms against the FP64 oracle's filt_da of the same FP32 input: both
    stay below 1e-5 of each output's maximum.  The derivatives weight the
    high modes by their wavenumber, so they show the transform's rounding
    most."""
    from oracle.lesgo_oracle import Oracle, Params
    a, b = _pair(monkeypatch, grid)
    nx, ny, Nz = grid
    o = Oracle(Params(nx=nx, ny=ny, Nz=Nz))
    for g in (a, b):
        g.init_ic(7)
    src = a.get("u")
    assert np.array_equal(src, b.get("u"))
    f, dx, dy = src.copy(), np.zeros_like(src), np.zeros_like(src)
    o.filt_da(f, dx, dy)
    for g in (a, b):
        g.filt_da("u", "dudx", "dudy")
    for name, ref in (("u", f), ("dudx", dx), ("dudy", dy)):
        r = ref[1:a.nz, :, :nx]
        scale = np.max(np.abs(r))
        ea = np.max(np.abs(a.get(name)[1:a.nz, :, :nx] - r)) / scale
        eb = np.max(np.abs(b.get(name)[1:b.nz, :, :nx] - r)) / scale
        assert eb < 1e-5 and ea < 1e-5, (grid, name, ea, eb)
    a.close()
    b.close()


@pytest.mark.parametrize("grid", GRIDS + [MULTI_TILE])
def test_stepped_fields_match_radix(built_lib, monkeypatch, grid):
    """Five fused steps (graph-replayed, two dynamic-model updates): every
    forward x pass of the step (filtered derivatives, the convective
    term's vorticity, stress divergence, the Lagrangian test filters, the
    pressure right-hand side) runs as a GEMM."""
    a, b = _pair(monkeypatch, grid)
    nx = grid[0]
    for g in (a, b):
        g.init_ic(11)
        g.step(5)
        g.sync()
    # measured: velocities within 2.1e-5, pressure within 4.6e-4 (the
    # Poisson solve divides each mode by k^2, so the low modes' rounding
    # differences grow most in p)
    for f, tol in (("u", 5e-5), ("v", 5e-5), ("w", 5e-5), ("p", 1e-3)):
        x, y = a.get(f)[1:a.nz, :, :nx], b.get(f)[1:b.nz, :, :nx]
        assert _close(x, y, tol), (grid, f, np.max(np.abs(x - y)) / np.max(np.abs(x)))
    a.close()
    b.close()


def test_batch_matches_instances_alone(built_lib, monkeypatch):
    """Three instances in one batch handle (tiles spanning instances) equal
    each instance run alone with the same transform form, bit for bit."""
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    monkeypatch.setenv("LESGO_XDFT", "1")
    kw = dict(nx=64, ny=48, Nz=20, precision="mixed", dyn_init=3, cs_count=3)
    bt = LesgoBatch(3, **kw)
    ids = [bt.add(1e-4 * (i + 1), 30 + i) for i in range(3)]
    bt.step(4)
    bt.sync()
    for i, iid in enumerate(ids):
        s = LesgoGPU(zo=1e-4 * (i + 1), **kw)
        s.init_ic(30 + i)
        s.step(4)
        for f in ("u", "w"):
            assert np.array_equal(s.get(f), bt.get(iid, f)), (i, f)
        s.close()
    bt.close()


def test_ten_steps_against_oracle(built_lib, monkeypatch):
    monkeypatch.setenv("LESGO_XDFT", "1")
    p, o, g = make_pair(precision="mixed", nx=32, ny=32, Nz=32, dyn_init=5)
    for _ in range(10):
        o.step()
    g.step(10)
    g.sync()
    for f in ("u", "v", "w", "p"):
        e = rel_err(p, f, g.get(f), oracle_field(o, f))
        assert e < 2e-4, (f, e)
    g.close()
