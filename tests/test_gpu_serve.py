"""Served requests give the same result in the mix as alone (GPU)."""
import numpy as np
import pytest

from lesgo_gb300.serve import GpuBackend, Server, poisson_requests

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(built_lib):
    from lesgo_gb300.solver import LesgoGPU
    base = dict(dyn_init=5, cs_count=5)
    reqs = poisson_requests(7, rate=400.0, grids=[(32, 32, 16), (48, 32, 24)], steps_range=(6, 14), seed=3,
                            turbines_max=2)
    srv = Server(GpuBackend("mixed", **base), budget_bytes=8e9, chunk_slots=3, cs_count=5)
    rep = srv.run(reqs)
    assert rep["requests"] == 7 and rep["p99_s"] >= rep["p50_s"]
    for r in srv.done:
        nx, ny, nz = r.grid
        g = LesgoGPU(turbines=r.turbines, nx=nx, ny=ny, Nz=nz, zo=r.zo, precision="mixed", **base)
        g.init_ic(r.seed)
        g.step(r.steps)
        prof = g.get("u")[1:g.nz, :, :nx].mean(axis=(1, 2))
        assert np.array_equal(prof, r.result["u_profile"]), r.rid
        if r.turbines:
            assert np.array_equal(g.turbine_state()["power"], r.result["power"])
        g.close()
