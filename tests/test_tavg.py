"""Time-averaging statistics (time_average.f90:176-319, :616-629; schedule
io.f90:557-580).

CPU tests pin the oracle's restatement: the sample weights of the schedule
and the averages of fields whose statistics are known.  GPU tests compare
the device accumulators, Reynolds stresses and plane-mean profiles with the
oracle (FP64 form within 1e-10 of the quantity's scale, mixed form 1e-3),
and a batch instance with the same instance run alone (bit for bit).
"""
import numpy as np
import pytest

from oracle.lesgo_oracle import TAVG_NAMES, TAVG_RS_NAMES, Oracle, Params, TimeAverage

NSTART, NEND, NSKIP, NSTEPS = 2, 11, 3, 13


def _run_schedule(o, ta, nsteps):
    for _ in range(nsteps):
        o.jt_total += 1
        ta.after_step()


def test_schedule_weights():
    """Samples at jt = 2 (start), 5, 8, 11, each weighted by 3 dt; steps after
    nend add nothing."""
    o = Oracle(Params(nx=16, ny=16, Nz=8))
    ta = TimeAverage(o, NSTART, NEND, NSKIP)
    seen = []
    orig = ta.compute

    def spy():
        seen.append((o.jt_total, ta.dt))
        orig()
    ta.compute = spy
    _run_schedule(o, ta, NSTEPS)
    dt = o.p.dt
    assert [j for j, _ in seen] == [5, 8, 11]
    assert np.allclose([w for _, w in seen], 3 * dt, rtol=0, atol=1e-15)
    assert ta.total_time == pytest.approx(9 * dt, rel=1e-15)
    assert ta.dt == 0.0


def test_constant_fields_statistics():
    """Steady fields: averages equal the field, fluctuations vanish, u_w and
    v_w are zero at the wall (lbc_mom = 2) and vortz is zero at level 1."""
    p = Params(nx=16, ny=12, Nz=8)
    o = Oracle(p)
    rng = np.random.default_rng(0)
    for name in ("u", "v", "w", "pres", "dudy", "dvdx", "dwdy", "dvdz", "dudz", "dwdx", "txz"):
        getattr(o, name)[:] = rng.standard_normal(getattr(o, name).shape)
    ta = TimeAverage(o, 1, 100, 2)
    _run_schedule(o, ta, 9)
    nx, nz = p.nx, p.nz
    assert np.allclose(ta.mean("u")[1:], o.u[1:, :, :nx], rtol=1e-14, atol=1e-14)
    assert np.allclose(ta.mean("txz")[1:], o.txz[1:, :, :nx], rtol=1e-14, atol=1e-14)
    for rs in TAVG_RS_NAMES:
        assert np.max(np.abs(ta.mean(rs))) < 1e-12, rs
    assert np.all(ta.mean("u_w")[1] == 0.0) and np.all(ta.mean("vortz")[1] == 0.0)
    exp = 0.5 * (o.u[1:nz, :, :nx] + o.u[2:nz + 1, :, :nx])
    assert np.allclose(ta.mean("u_w")[2:], exp, rtol=1e-14, atol=1e-14)
    w_uv = 0.5 * (o.w[2:nz + 1, :, :nx] + o.w[1:nz, :, :nx])
    assert np.allclose(ta.mean("w_uv")[1:nz], w_uv, rtol=1e-14, atol=1e-14)
    assert np.allclose(ta.mean("w_uv")[nz], w_uv[-1], rtol=1e-14, atol=1e-14)


def test_alternating_field_fluctuation():
    """u alternating between a and b with equal weights: <u'u'> = ((a-b)/2)^2."""
    p = Params(nx=16, ny=12, Nz=8)
    o = Oracle(p)
    ta = TimeAverage(o, 1, 100, 1)
    for step in range(1, 10):
        o.u[:] = 3.0 if step % 2 else 1.0
        o.jt_total = step
        ta.after_step()
    # samples at steps 2..9: four of 3.0, four of 1.0
    assert np.allclose(ta.mean("u")[1:], 2.0, rtol=1e-14)
    assert np.allclose(ta.mean("up2")[1:], 1.0, rtol=1e-13)


# ---------------------------------------------------------------------------
# GPU parity
# ---------------------------------------------------------------------------
def _scale(ta, name):
    """Reynolds stresses are differences of O(u^2) sums: scale by those."""
    base = {"up2": "u2", "vp2": "v2", "wp2": "w2", "upvp": "u2", "upwp": "u2", "vpwp": "v2"}.get(name, name)
    hi = ta.o.p.nz - 1 if base in TOP_UNDEFINED else ta.o.p.nz
    s = np.max(np.abs(ta.mean(base)[1:hi + 1]))
    return s if s > 0 else 1.0


# the uv-grid stresses are defined at levels 1..nz-1 (sgs_stag leaves level
# nz to the BOGUS fill of safety mode); every other sum at levels 1..nz
TOP_UNDEFINED = {"txx", "tyy", "tzz", "txy"}


def _compare(p, ta, get, prof, tol, names=TAVG_NAMES + TAVG_RS_NAMES):
    worst = {}
    for name in names:
        hi = p.nz - 1 if name in TOP_UNDEFINED else p.nz
        ref = ta.mean(name)[1:hi + 1]
        sc = np.max(np.abs(ref)) or 1.0
        if name in TAVG_RS_NAMES:
            sc = max(sc, _scale(ta, name))
        a = get(name)[:hi, :, :p.nx]             # get() starts at level 1
        err = np.max(np.abs(a - ref)) / sc
        worst[name] = err
        assert err < tol, (name, err)
        pr = prof(name)[1:hi + 1]
        perr = np.max(np.abs(pr - ref.mean(axis=(1, 2)))) / sc
        assert perr < tol, (name, "profile", perr)
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp64dw", 1e-10), ("mixed", 1e-3)])
def test_gpu_tavg_matches_oracle(built_lib, precision, tol):
    from gpu_util import make_pair
    p, o, g = make_pair(precision=precision, nx=32, ny=32, Nz=32, dyn_init=5)
    ta = TimeAverage(o, NSTART, NEND, NSKIP)
    g.tavg_config(NSTART, NEND, NSKIP)
    for _ in range(NSTEPS):
        o.step()
        ta.after_step()
    g.step(NSTEPS)
    g.sync()
    assert g.tavg_total_time() == pytest.approx(ta.total_time, rel=1e-14)
    _compare(p, ta, g.tavg_get, g.tavg_profile, tol)
    g.close()


@pytest.mark.gpu
def test_gpu_tavg_turbines_and_dropin(built_lib):
    """Turbine forces enter fx/fy/fz; the drop-in sequence plus
    lesgo_gpu_tavg_sample gives the same sums as the fused step."""
    from lesgo_gb300.solver import LesgoGPU
    from test_gpu_parity import _farm
    ts, farm = _farm(2, 1)
    kw = dict(nx=64, ny=32, Nz=24, dyn_init=5)
    p = Params(turbines=farm, **kw)
    o = Oracle(p)
    o.set_ic(3)
    ta = TimeAverage(o, 1, 50, 2)
    g = LesgoGPU(turbines=ts, **kw)
    g.init_ic(3)
    g.tavg_config(1, 50, 2)
    g2 = LesgoGPU(turbines=ts, **kw)
    g2.init_ic(3)
    g2.tavg_config(1, 50, 2)
    for _ in range(7):
        o.step()
        ta.after_step()
        g2.step_reference_order()
        g2.tavg_sample()
    g.step(7)
    g.sync()
    _compare(p, ta, g.tavg_get, g.tavg_profile, 1e-10)
    for name in ("u", "fx", "fz", "upwp", "p"):
        assert np.max(np.abs(g.tavg_get(name) - g2.tavg_get(name))) <= 1e-11 * _scale(ta, name), name
    assert np.max(np.abs(ta.mean("fx"))) > 0
    g.close()
    g2.close()


@pytest.mark.gpu
def test_gpu_tavg_batch_instance_equals_alone(built_lib):
    """Statistics of a batch instance (admitted late, moved by a removal) are
    bit for bit those of the instance run alone."""
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    base = dict(nx=32, ny=32, Nz=24, dyn_init=3, cs_count=3)
    b = LesgoBatch(capacity=3, **base)
    b.tavg_config(2, 40, 2)
    i0 = b.add(1e-4, 21)
    i1 = b.add(3e-4, 22)
    b.step(3)
    i2 = b.add(5e-4, 23)
    b.step(2)
    b.remove(i0)
    b.step(4)
    for iid, zo, seed, n in [(i1, 3e-4, 22, 9), (i2, 5e-4, 23, 6)]:
        g = LesgoGPU(zo=zo, **base)
        g.init_ic(seed)
        g.tavg_config(2, 40, 2)
        g.step(n)
        assert b.tavg_total_time(iid) == g.tavg_total_time()
        for name in ("u", "w", "p", "upwp", "cs_opt2", "vortz"):
            assert np.array_equal(b.tavg_get(iid, name), g.tavg_get(name)), (iid, name)
            assert np.array_equal(b.tavg_profile(iid, name), g.tavg_profile(name)), (iid, name)
        g.close()
    b.close()
