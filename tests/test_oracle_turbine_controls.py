"""The oracle's time-varying turbine controls (turbines.f90:500-515), host
only: every step each turbine takes its yaw, tilt and Ct' interpolated at
total_time_dim (the sum of dt z_i / u_star, main.f90:139-150), and a yaw or
tilt schedule re-selects the disk nodes (turbines_nodes,
turbines.f90:275-462) with the indicator normalised to integrate to one."""
import math

import numpy as np
import pytest

from oracle.lesgo_oracle import Oracle, Params, Turbine, TurbineFarm, sched_interp


def _farm(sched):
    ts = [Turbine(xloc=1.0 + 0.7 * i, yloc=1.0, height=0.1, dia=0.1, thk=0.001, Ct_prime=1.33) for i in range(2)]
    return TurbineFarm(ts, alpha1=1.5, alpha2=1.5, filter_cutoff=1e-2, adm_correction=True, sched=sched)


def test_controls_follow_schedules_and_nodes_move():
    theta1 = np.array([[0.0, 0.0, 0.0], [1.0, 20.0, -30.0], [2.0, 45.0, -40.0]])
    ctp = np.array([[0.0, 1.33, 1.2], [1.5, 1.0, 1.6]])
    p = Params(nx=64, ny=32, Nz=16, dyn_init=100, turbines=_farm({0: theta1, 2: ctp}))
    o = Oracle(p)
    o.set_ic(2)
    nodes0 = [(set(zip(*[a.tolist() for a in t.nodes])), t.ind.copy()) for t in o.farm.turbines]
    dt_dim = p.dt * p.z_i / p.u_star
    for step in range(1, 5):
        o.step()
        assert o.time_dim == pytest.approx(step * dt_dim, rel=1e-14)
        for s, t in enumerate(o.farm.turbines):
            assert t.theta1 == sched_interp(theta1[:, 0], theta1[:, 1 + s], o.time_dim)
            assert t.Ct_prime == sched_interp(ctp[:, 0], ctp[:, 1 + s], o.time_dim)
            assert t.theta2 == 0.0
            # normalised indicator (turbines.f90:454-457) and the yawed normal
            assert np.sum(t.ind) * p.dx * p.dy * p.dz == pytest.approx(1.0, rel=1e-12)
            c = math.cos(math.pi * t.theta1 / 180.0)
            assert t.nhat[0] == pytest.approx(-c, rel=1e-15)
    # a disk about one cell wide: the yaw moves the node set or, on the same
    # nodes, the indicator values
    moved = [set(zip(*[a.tolist() for a in t.nodes])) != n0 or not np.array_equal(t.ind, i0)
             for t, (n0, i0) in zip(o.farm.turbines, nodes0)]
    assert all(moved)
    assert np.all(np.isfinite(o.u)) and np.any(o.fxa != 0.0)


def test_constant_schedule_keeps_static_nodes():
    """A yaw schedule that holds the static yaw re-selects the same nodes
    with the same indicator values."""
    a = Oracle(Params(nx=64, ny=32, Nz=16, dyn_init=100, turbines=_farm({})))
    b = Oracle(Params(nx=64, ny=32, Nz=16, dyn_init=100,
                      turbines=_farm({0: np.array([[0.0, 0.0, 0.0], [10.0, 0.0, 0.0]])})))
    for o in (a, b):
        o.set_ic(3)
        o.step()
    for ta, tb in zip(a.farm.turbines, b.farm.turbines):
        assert all(np.array_equal(x, y) for x, y in zip(ta.nodes, tb.nodes))
        assert np.array_equal(ta.ind, tb.ind)
    assert np.array_equal(a.u, b.u)
