"""Stand-alone entry points through the C ABI against the oracle (GPU
required): the spectral derivatives ddx, ddy and ddxy
(derivatives.f90:37-163), the in-place 2-Delta test filter of one plane
(test_filtermodule.f90:126-147) and the plane-mean bottom wall stress of the
diagnostics (functions.f90:882-905).  Each single stage is held to 1e-12
max relative error over the valid entries, like the stagewise tests."""
import numpy as np
import pytest

from gpu_util import make_pair, oracle_field, rel_err

pytestmark = pytest.mark.gpu

STAGE_TOL = 1e-12


@pytest.mark.parametrize("grid", [(32, 32, 16), (48, 96, 12)])
def test_ddx_ddy_ddxy_match_oracle(built_lib, grid):
    """Each derivative of u, v and w on the seeded initial fields; the
    48 x 96 grid has radix-3 lengths in both directions."""
    nx, ny, Nz = grid
    p, o, g = make_pair(nx=nx, ny=ny, Nz=Nz, L_y=2.0 if ny != nx else np.pi)
    for f in ("u", "v", "w"):
        src = oracle_field(o, f).copy()
        before = g.get(f)
        dx = np.zeros_like(src)
        dy = np.zeros_like(src)
        o.ddx(src.copy(), dx)
        o.ddy(src.copy(), dy)
        ex, ey = "d%sdx" % f, "d%sdy" % f
        g.ddx(f, ex)
        assert rel_err(p, ex, g.get(ex), dx) < STAGE_TOL, (f, "ddx")
        g.ddy(f, ey)
        assert rel_err(p, ey, g.get(ey), dy) < STAGE_TOL, (f, "ddy")
        # ddxy writes both; clear them first so stale values cannot pass
        g.set(ex, np.zeros((g.nz + 1, g.ny, g.ld)))
        g.set(ey, np.zeros((g.nz + 1, g.ny, g.ld)))
        dx2 = np.zeros_like(src)
        dy2 = np.zeros_like(src)
        o.ddxy(src.copy(), dx2, dy2)
        g.ddxy(f, ex, ey)
        assert rel_err(p, ex, g.get(ex), dx2) < STAGE_TOL, (f, "ddxy x")
        assert rel_err(p, ey, g.get(ey), dy2) < STAGE_TOL, (f, "ddxy y")
        # the input field is left as it was (derivatives.f90 keeps f)
        assert np.array_equal(g.get(f)[:, :, :nx], before[:, :, :nx])
    g.close()


@pytest.mark.parametrize("level", [1, 5, 16])
def test_test_filter_plane_matches_oracle(built_lib, level):
    """lesgo_gpu_test_filter filters one plane in place with the 2-Delta
    spectral cut-off G_test (its 1/(nx ny) included); the other planes stay."""
    p, o, g = make_pair(nx=32, ny=32, Nz=16)
    before = g.get("u")
    g.test_filter("u", level)
    after = g.get("u")
    ref = o.test_filter(oracle_field(o, "u")[level].copy())
    a, b = after[level, :, :p.nx], ref[:, :p.nx]
    assert np.max(np.abs(a - b)) / np.max(np.abs(b)) < STAGE_TOL
    others = [k for k in range(g.nz + 1) if k != level]
    assert np.array_equal(after[others][:, :, :p.nx], before[others][:, :, :p.nx])
    g.close()


@pytest.mark.parametrize("lbc", [2, 1])
def test_tau_wall_bot_matches_oracle(built_lib, lbc):
    """The diagnostics' plane-mean bottom wall stress after a few steps
    (log law; DNS no-slip wall with molecular viscosity)."""
    kw = dict(nx=32, ny=32, Nz=16, dyn_init=2, cs_count=2, lbc_mom=lbc)
    if lbc == 1:
        kw["molec"] = True
    p, o, g = make_pair(**kw)
    for _ in range(3):
        o.step()
    g.step(3)
    d = g.diag()
    ref = o.tau_wall_bot()
    assert ref > 0.0
    assert abs(d["tau_bot"] - ref) / ref < STAGE_TOL * 100, (d["tau_bot"], ref)
    g.close()
