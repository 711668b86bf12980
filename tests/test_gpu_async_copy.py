"""Stream-ordered field copies (lesgo_gpu_set_field_async, ..._inst_async):
a loop of queued uploads, steps and downloads through page-locked host
buffers, with one host synchronisation at the end, gives bit-for-bit the
fields of the same loop with synchronous copies.  Both forms; two grid
classes stepping on their own streams, as the batched ensemble does."""
import numpy as np
import pytest

KW = dict(ny=32, Nz=24, dyn_init=2, cs_count=2)


def _loop(torch, batches, steps, wait):
    bufs = []
    for b, ids in batches:
        for iid in ids:
            shape = (b.nz + 1, b.ny, b.ld)
            d = {k: torch.empty(shape, dtype=torch.float64, pin_memory=True) for k in ("u", "v", "w")}
            for k, t in d.items():
                b.get_ptr(iid, k, t.data_ptr(), 0, b.nz)
            bufs.append((b, iid, d))
    for _ in range(steps):
        for b, ids in batches:
            mine = [x for x in bufs if x[0] is b]
            for _, iid, d in mine:
                for k, t in d.items():
                    b.set_ptr(iid, k, t.data_ptr(), 0, b.nz, wait=wait)
            b.step(1)
            for _, iid, d in mine:
                for k, t in d.items():
                    b.get_ptr(iid, k, t.data_ptr(), 0, b.nz, wait=wait)
    for b, _ in batches:   # the only host synchronisation of the queued loop
        b.sync()
    return [{k: t.numpy().copy() for k, t in d.items()} for _, _, d in bufs]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_copies_equal_synchronous(built_lib, precision):
    import torch
    from lesgo_gb300.solver import LesgoBatch
    out = []
    for wait in (True, False):
        batches = []
        for nx, seeds in ((32, (11, 12)), (48, (13,))):
            b = LesgoBatch(capacity=len(seeds), nx=nx, precision=precision, **KW)
            batches.append((b, [b.add(1e-4 * (i + 1), s) for i, s in enumerate(seeds)]))
        out.append(_loop(torch, batches, 4, wait))
        for b, _ in batches:
            b.close()
    assert len(out[0]) == 3
    for a, c in zip(*out):
        for k in ("u", "v", "w"):
            assert np.array_equal(a[k], c[k]), k
            assert np.all(np.isfinite(a[k]))


@pytest.mark.gpu
def test_async_single_handle_round_trip(built_lib):
    """set_field_async then get_field_async on one handle: the values come
    back (FP64 form: exactly)."""
    import torch
    from lesgo_gb300.solver import LesgoGPU
    g = LesgoGPU(nx=32, **KW)
    shape = (g.nz + 1, g.ny, g.ld)
    src = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    src.copy_(torch.from_numpy(np.random.default_rng(3).standard_normal(shape)))
    dst = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
    g.set_ptr("u", src.data_ptr(), 0, g.nz, wait=False)
    g.get_ptr("u", dst.data_ptr(), 0, g.nz, wait=False)
    g.sync()
    assert torch.equal(src, dst)
    g.close()
