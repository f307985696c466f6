"""vxl_voxelize_noalloc, the voxelizer entry point for callers that cannot
allocate device memory (it uses the library's fixed static device table as
its only scratch), checked through the C ABI against vxl_voxelize on two
calls in a row, and checked to allocate no device memory once the library's
kernels are loaded.

The file name makes pytest collect it after every other test file, so a run
that stops at the first failure (-x) has run all other tests before this
one. It depends on no earlier test: it passes alone in a fresh process too."""
import numpy as np
import pytest

from tests import vox_cases
from tests.gpu_util import dev, export_r8

pytestmark = pytest.mark.gpu


def _instances(rng, nmodels, count, n, clear_every):
    out = []
    for i in range(count):
        op = 0 if (clear_every and i % clear_every == clear_every - 1) else 1
        out.append((vox_cases.world_matrix(rng, -0.5, n / 10.0), int(rng.integers(0, nmodels)), op))
    return out


def test_voxelize_noalloc_matches_voxelize(vxl, ctx):
    import torch

    rng = np.random.default_rng(20261203)
    models = [vox_cases.random_model(rng, *rng.integers(3, 40, 3)) for _ in range(6)]
    d_models = [dev(m) for m in models]
    mdesc = [(d.data_ptr(),) + m.shape[::-1] for m, d in zip(models, d_models)]
    n = 160
    ref = vxl.Grid(ctx, n, n, n)          # updated by vxl_voxelize
    tgt = vxl.Grid(ctx, n, n, n)          # updated by vxl_voxelize_noalloc
    desc = tgt.describe()
    S = n // 2
    for call, (count, clear_every) in enumerate([(90, 0), (70, 3)]):
        insts = _instances(rng, len(models), count, n, clear_every)
        a0 = np.tile(np.array([S - 1, S - 1, S - 1, 0, 0, 0], np.int32), (count, 1))
        aabb_ref, aabb_na = dev(a0), dev(a0)
        vxl.voxelize(ctx, ref, mdesc, insts, aabb_ref)
        vxl.voxelize_noalloc(desc, mdesc, insts, aabb_na)
        torch.cuda.synchronize()
        g_ref, g_na = export_r8(ref), export_r8(tgt)
        assert g_ref.any(), call
        assert np.array_equal(g_na, g_ref), "call %d: grids differ in %d bytes" % (call, int((g_na != g_ref).sum()))
        assert torch.equal(aabb_na, aabb_ref), call
        assert tgt.count() == ref.count()


def test_voxelize_noalloc_allocates_nothing(vxl, ctx):
    """After a warm-up call (which loads the kernels and looks up the table's
    address), further calls leave the device's free memory and torch's
    allocator unchanged."""
    import torch

    rng = np.random.default_rng(7)
    models = [vox_cases.random_model(rng, *rng.integers(3, 30, 3)) for _ in range(4)]
    d_models = [dev(m) for m in models]
    mdesc = [(d.data_ptr(),) + m.shape[::-1] for m, d in zip(models, d_models)]
    n = 96
    g = vxl.Grid(ctx, n, n, n)
    desc = g.describe()
    aabb = dev(np.zeros((200, 6), np.int32))
    vxl.voxelize_noalloc(desc, mdesc, _instances(rng, len(models), 50, n, 0), aabb)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for count, clear_every in [(200, 0), (120, 4), (10, 2)]:
        vxl.voxelize_noalloc(desc, mdesc, _instances(rng, len(models), count, n, clear_every), aabb)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
    assert torch.cuda.memory_allocated() == alloc0
    assert g.count() > 0


def test_voxelize_noalloc_rejects_oversize(vxl, ctx):
    n = 16
    g = vxl.Grid(ctx, n, n, n)
    m = dev(np.full((2, 2, 2), 20, np.uint8))
    too_many = [(np.eye(4, dtype=np.float32).reshape(16), 0, 1)] * (16384 + 1)
    with pytest.raises(vxl.VxlError) as e:
        vxl.voxelize_noalloc(g.describe(), [(m.data_ptr(), 2, 2, 2)], too_many)
    assert e.value.status == 5 and "exceed" in str(e.value)
