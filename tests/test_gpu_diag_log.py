"""Diagnostics log on the device (main.f90:359-436: the wbase / nenergy
output of rmsdiv, kinetic energy, CFL and wall stress): rows written every
`every` steps without host synchronisation equal lesgo_gpu_diag taken at
the same steps, the ring keeps the newest rows, and batch instances log
their own rows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BASE = dict(nx=32, ny=32, Nz=16, dyn_init=5, cs_count=5)


def _host_rows(steps, every, **kw):
    from lesgo_gb300.solver import LesgoGPU
    g = LesgoGPU(**kw)
    g.init_ic(2)
    rows = []
    for s in range(1, steps + 1):
        g.step(1)
        if s % every == 0:
            d = g.diag()
            rows.append([s, g.sim_time(), d["rmsdiv"], d["ke"], d["cfl"], d["tau_bot"]])
    g.close()
    return np.array(rows)


@pytest.mark.parametrize("cfl", [False, True])
def test_diag_log_equals_host_diag(built_lib, cfl):
    from lesgo_gb300.solver import LesgoGPU
    kw = dict(BASE, use_cfl_dt=cfl, cfl=0.05)
    g = LesgoGPU(**kw)
    g.init_ic(2)
    g.diag_log_config(3, 3)
    g.step(14)                       # rows at 3, 6, 9, 12; the ring keeps 6, 9, 12
    log = g.diag_log()
    ref = _host_rows(14, 3, **kw)[1:]
    assert log.shape == (3, 6)
    assert np.array_equal(log[:, 0], ref[:, 0])
    assert np.allclose(log[:, 1:], ref[:, 1:], rtol=1e-14, atol=0)
    assert np.all(log[:, 3] > 0)
    g.close()


def test_diag_log_batch_instances(built_lib):
    from lesgo_gb300.solver import LesgoBatch, LesgoGPU
    b = LesgoBatch(capacity=2, **BASE)
    b.diag_log_config(2, 8)
    i0 = b.add(1e-4, 2)
    b.step(2)
    i1 = b.add(5e-4, 3)
    b.step(4)
    l0, l1 = b.diag_log(i0), b.diag_log(i1)
    assert list(l0[:, 0]) == [2, 4, 6] and list(l1[:, 0]) == [2, 4]
    g = LesgoGPU(zo=5e-4, **BASE)
    g.init_ic(3)
    g.diag_log_config(2, 8)
    g.step(4)
    assert np.array_equal(g.diag_log(), l1)
    g.close()
    b.close()
