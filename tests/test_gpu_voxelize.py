"""GPU voxelizer vs the oracle's restatement of ShadowVoxSystem (bit-exact
grids, per-instance AABBs and dirty regions)."""
import numpy as np
import pytest

import oracle
from tests import vox_cases
from tests.gpu_util import dev, export_r8

pytestmark = pytest.mark.gpu


def _models(rng, k):
    ms = [vox_cases.random_model(rng, *rng.integers(3, 48, 3)) for _ in range(k)]
    return ms, [dev(m) for m in ms]


def test_voxelize_set_runs(vxl, ctx):
    import torch

    rng = np.random.default_rng(1)
    ms, dms = _models(rng, 5)
    n = 192
    G = vxl.Grid(ctx, n, n, n)
    insts = []
    for i in range(60):
        mi = int(rng.integers(0, len(ms)))
        insts.append((vox_cases.world_matrix(rng, -1.0, n / 10.0), mi, vxl.OP_SET))
    S = n // 2
    aabb0 = np.tile(np.array([S - 1, S - 1, S - 1, 0, 0, 0], np.int32), (len(insts), 1))
    d_aabb = dev(aabb0)
    vxl.voxelize(ctx, G, [(dm.data_ptr(),) + m.shape[::-1] for m, dm in zip(ms, dms)], insts, d_aabb)
    torch.cuda.synchronize()
    want = np.zeros((S, S, S), np.uint8)
    want_aabb = aabb0.copy()
    for k, (M, mi, op) in enumerate(insts):
        oracle.voxelize_model(want, ms[mi], M, 1, want_aabb[k])
    got = export_r8(G)
    assert np.array_equal(got, want)
    assert np.array_equal(d_aabb.cpu().numpy(), want_aabb)
    assert got.any()


def test_voxelize_mixed_ops_in_order(vxl, ctx):
    import torch

    rng = np.random.default_rng(2)
    ms, dms = _models(rng, 4)
    n = 96
    G = vxl.Grid(ctx, n, n, n)
    S = n // 2
    want = np.zeros((S, S, S), np.uint8)
    insts = []
    for i in range(40):
        mi = int(rng.integers(0, len(ms)))
        op = vxl.OP_SET if (i % 3 != 2) else vxl.OP_CLEAR
        insts.append((vox_cases.world_matrix(rng, 0.0, n / 10.0 - 1), mi, op))
    vxl.voxelize(ctx, G, [(dm.data_ptr(),) + m.shape[::-1] for m, dm in zip(ms, dms)], insts)
    torch.cuda.synchronize()
    for M, mi, op in insts:
        oracle.voxelize_model(want, ms[mi], M, op)
    assert np.array_equal(export_r8(G), want)


def test_shadowvox_update_and_destroy(vxl, ctx):
    import torch

    rng = np.random.default_rng(3)
    ms, dms = _models(rng, 4)
    n = 128
    G = vxl.Grid(ctx, n, n, n)
    S = n // 2
    want = np.zeros((S, S, S), np.uint8)
    mdesc = [(dm.data_ptr(),) + m.shape[::-1] for m, dm in zip(ms, dms)]
    for frame in range(3):
        ents = []
        for e in range(12):
            prev = vox_cases.world_matrix(rng, -0.5, n / 10.0)
            cur = prev.copy() if e % 4 == 0 else vox_cases.world_matrix(rng, -0.5, n / 10.0)
            cur[12] += 0.25
            ents.append((prev, cur, rng.uniform(-1, 1, 3).astype(np.float32), int(rng.integers(0, len(ms)))))
        regions = vxl.shadowvox_update(ctx, G, mdesc, ents)
        wreg = oracle.shadowvox_update(want, [ms[e[3]] for e in ents], np.stack([e[0] for e in ents]),
                                       np.stack([e[1] for e in ents]), np.stack([e[2] for e in ents]))
        assert np.array_equal(export_r8(G), want)
        assert np.array_equal(regions, wreg)
    M = ents[0][1]
    reg = vxl.vox_destroyed(ctx, G, mdesc[ents[0][3]], M)
    wr = oracle.vox_destroyed(want, ms[ents[0][3]], M)
    assert np.array_equal(export_r8(G), want)
    assert np.array_equal(reg, wr)
