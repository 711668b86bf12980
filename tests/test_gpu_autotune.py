"""The tile-shape autotuner leaves the simulation state alone, and tile
shapes do not change results: every row and column transform is computed
the same way whatever the tile, so a tuned run equals an untuned one bit for
bit (FP64 and mixed)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "p", "RHSx", "Cs_opt2", "F_LM")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_state_and_results(built_lib, precision):
    from lesgo_gb300.solver import LesgoGPU
    kw = dict(nx=48, ny=32, Nz=24, dyn_init=3, cs_count=3, precision=precision)
    a = LesgoGPU(**kw)
    a.init_ic(1)
    a.step(3)
    before = {f: a.get(f) for f in FIELDS}
    cfg = a.autotune()
    assert cfg["xtarget"] in (1024, 2048, 4096) and cfg["ybudget"] in (32768, 49152, 65536, 112640)
    for f in FIELDS:
        assert np.array_equal(a.get(f), before[f]), f
    a.step(4)
    b = LesgoGPU(**kw)
    b.init_ic(1)
    b.step(7)
    for f in FIELDS:
        x, y = a.get(f)[1:a.nz, :, :a.nx], b.get(f)[1:b.nz, :, :b.nx]
        assert np.array_equal(x, y), f
    a.close()
    b.close()
