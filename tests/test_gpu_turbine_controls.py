"""Time-varying turbine controls (turbines.f90:500-515): yaw theta1, tilt
theta2 and Ct' interpolated every step at total_time_dim, the disk nodes
re-selected on the device when the yaw or tilt moves (turbines_nodes,
turbines.f90:275-462), against the oracle; a constant schedule against the
static path; batch instances with their own schedules against their runs
alone; total_time_dim through a checkpoint."""
import numpy as np
import pytest

KW = dict(nx=64, ny=32, Nz=24, dyn_init=4, cs_count=2)
# dt = 2e-4, z_i = 1000, u_star = 0.45: one step is 0.444 dimensional time units
THETA1 = [[0.0, 0.0, 0.0], [1.5, 12.0, -8.0], [3.0, 30.0, 4.0]]
THETA2 = [[0.0, 0.0, 0.0], [3.5, 6.0, -3.0]]
CTP = [[0.0, 1.33, 1.2], [2.0, 1.0, 1.6]]


def _pair(precision="fp64", scheds=((0, THETA1), (1, THETA2), (2, CTP))):
    from oracle.lesgo_oracle import Oracle, Params
    from lesgo_gb300.solver import LesgoGPU
    from test_gpu_parity import _farm
    ts, farm = _farm(2, 1)
    farm.sched = {w: np.array(r) for w, r in scheds}
    p = Params(turbines=farm, **KW)
    o = Oracle(p)
    o.set_ic(6)
    g = LesgoGPU(turbines=ts, precision=precision, **KW)
    g.init_ic(6)
    for w, r in scheds:
        g.turbine_schedule(w, r)
    return p, o, g


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 2e-4)])
def test_dynamic_controls_match_oracle(built_lib, precision, tol):
    from gpu_util import oracle_field, rel_err
    p, o, g = _pair(precision)
    for _ in range(8):
        o.step()
    g.step(8)
    c = g.turbine_controls()
    for s, t in enumerate(o.farm.turbines):
        assert c["theta1"][s] == pytest.approx(t.theta1, rel=1e-14, abs=1e-14)
        assert c["theta2"][s] == pytest.approx(t.theta2, rel=1e-14, abs=1e-14)
        assert c["Ct_prime"][s] == pytest.approx(t.Ct_prime, rel=1e-14)
    assert abs(o.farm.turbines[0].theta1) > 20.0     # the yaw moved through the run
    for f in ("u", "v", "w", "fxa", "fya", "fza"):
        e = rel_err(p, f, g.get(f), oracle_field(o, f))
        assert e < tol, (f, e)
    po = o.turbine_power()
    assert np.max(np.abs(g.turbine_state()["power"] - po)) <= 50 * tol * np.max(np.abs(po))
    g.close()


@pytest.mark.gpu
def test_constant_schedule_equals_static(built_lib):
    """A yaw schedule that holds the static yaw: the device-selected nodes give
    the forces of the static node lists (round-off of the normalisation sum
    apart)."""
    from lesgo_gb300.solver import LesgoGPU
    from test_gpu_parity import _farm
    ts, _ = _farm(2, 1)
    a = LesgoGPU(turbines=ts, **KW)
    b = LesgoGPU(turbines=ts, **KW)
    b.turbine_schedule("theta1", [[0.0, 0.0, 0.0], [100.0, 0.0, 0.0]])
    for h in (a, b):
        h.init_ic(7)
        h.step(5)
    for f in ("u", "w", "fxa", "fza"):
        x, y = a.get(f)[1:a.nz, :, :a.nx], b.get(f)[1:b.nz, :, :b.nx]
        assert np.max(np.abs(x - y)) <= 1e-12 * np.max(np.abs(y)), f
    pa, pb = a.turbine_state()["power"], b.turbine_state()["power"]
    assert np.max(np.abs(pa - pb)) <= 1e-12 * np.max(np.abs(pa))
    a.close()
    b.close()


@pytest.mark.gpu
def test_batch_instances_with_own_schedules_equal_alone(built_lib):
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    from test_gpu_parity import _farm
    ts, _ = _farm(2, 1)
    specs = [(1e-4, 41, THETA1), (3e-4, 42, None), (2e-4, 43, [[0.0, -10.0, 10.0]])]
    b = LesgoBatch(capacity=3, **KW)
    ids = [b.add(zo, seed, turbines=ts) for zo, seed, _ in specs]
    for iid, (_, _, sch) in zip(ids, specs):
        if sch is not None:
            b.turbine_schedule(iid, "theta1", sch)
    b.turbine_schedule(ids[1], "Ct_prime", CTP)
    b.step(6)
    for iid, (zo, seed, sch) in zip(ids, specs):
        g = LesgoGPU(turbines=ts, zo=zo, **KW)
        g.init_ic(seed)
        if sch is not None:
            g.turbine_schedule("theta1", sch)
        if iid == ids[1]:
            g.turbine_schedule("Ct_prime", CTP)
        g.step(6)
        for f in ("u", "v", "w", "fxa"):
            assert np.array_equal(b.get(iid, f)[1:g.nz], g.get(f)[1:g.nz]), (iid, f)
        assert np.array_equal(b.turbine_controls(iid)["theta1"], g.turbine_controls()["theta1"])
        g.close()
    b.close()


@pytest.mark.gpu
def test_total_time_dim_through_checkpoint(built_lib, tmp_path):
    """total_time.dat carries total_time_dim (io.f90:77): a restarted run
    continues the schedule where the uninterrupted one is."""
    import os
    from lesgo_gb300.solver import LesgoGPU
    from test_gpu_parity import _farm
    ts, _ = _farm(2, 1)
    pre = str(tmp_path) + os.sep
    kw = dict(KW, dyn_init=2, cs_count=1)
    a = LesgoGPU(turbines=ts, **kw)
    a.turbine_schedule("theta1", THETA1)
    a.init_ic(8)
    a.step(4)
    a.checkpoint_write(pre)
    with open(pre + "total_time.dat") as f:
        vals = [float(x.replace("D", "E")) for x in f.read().split()]
    assert vals[2] == pytest.approx(4 * 2e-4 * 1000 / 0.45, rel=1e-14)
    c = LesgoGPU(turbines=ts, **kw)
    c.turbine_schedule("theta1", THETA1)
    c.checkpoint_read(pre)
    a.step(3)
    c.step(3)
    assert np.array_equal(a.turbine_controls()["theta1"], c.turbine_controls()["theta1"])
    a.close()
    c.close()


@pytest.mark.gpu
def test_disks_leaving_a_batch_leave_no_forcing(built_lib):
    """The last instance with disks leaves and another joins at the same
    instance count: its steps carry no disk forcing (the captured steps of
    the earlier disk layout are dropped at every rebuild) and equal its run
    alone."""
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    from test_gpu_parity import _farm
    ts, _ = _farm(2, 1)
    b = LesgoBatch(capacity=2, **KW)
    a = b.add(1e-4, 51, turbines=ts)
    k = b.add(2e-4, 52)
    b.step(3)
    b.remove(a)
    c = b.add(3e-4, 53)
    b.step(3)
    for iid, zo, seed, n in ((k, 2e-4, 52, 6), (c, 3e-4, 53, 3)):
        # k moved into the slot the disks' instance held
        assert not np.any(b.get(iid, "fxa")) and not np.any(b.get(iid, "fza")), iid
        g = LesgoGPU(zo=zo, **KW)
        g.init_ic(seed)
        g.step(n)
        for f in ("u", "v", "w"):
            assert np.array_equal(b.get(iid, f)[1:g.nz], g.get(f)[1:g.nz]), (iid, f)
        g.close()
    b.close()
