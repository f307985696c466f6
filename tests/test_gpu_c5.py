"""Stress configuration: 2048^3 grid (1 GiB of bits) with a heightfield
terrain (amplitude 512) and 50,000 Vox-model instances of edge 16-128,
3840x2160 G-buffer, 1 shadow + 16 AO (L = 64) + 1 specular rays per pixel.

At this size the oracle checks samples, plus size-independent properties:
  - the terrain generator bit for bit on a small grid, and at full size
    against the oracle's column heights;
  - the voxelizer on a 96-instance subset, bit for bit, into a fresh 2048^3 grid;
  - SET-only voxelization is order-independent (shuffled instance order gives
    the same grid) and idempotent (voxelizing again changes nothing);
  - 1024 sampled pixels (32 runs of 32) of the full frame: every output and
    every per-ray record (hit cell, t bits, fetch count, flags) bit-exact.
"""
import numpy as np
import pytest

import oracle
from tests.gpu_util import assert_recs_equal, export_r8, rec_buffer, recs_np, same_bits

pytestmark = pytest.mark.gpu


def test_terrain_matches_oracle(vxl, ctx):
    import torch

    n = 96
    G = vxl.Grid(ctx, n, n, n)
    d_h = torch.empty((n, n), dtype=torch.float32, device="cuda")
    G.scene_terrain(11, 6.0, 40.0, 1.0 / 24.0, 5, d_height=d_h)
    got = export_r8(G)
    want = np.zeros((n // 2, n // 2, n // 2), np.uint8)
    h = oracle.scene_terrain(want, 11, 6.0, 40.0, 1.0 / 24.0, 5)
    assert np.array_equal(got, want)
    assert np.array_equal(d_h.cpu().numpy().view(np.int32), h.view(np.int32))
    assert 0.1 < oracle.r8_to_fine(got).mean() < 0.6


@pytest.fixture(scope="module")
def c5(vxl, ctx):
    from voxelengine_gb300 import scenes

    return scenes.make_terrain_scene(ctx, 2048, 3840, 2160, seed=5, n_instances=50000)


def test_c5_terrain_heights(vxl, ctx, c5):
    n = c5["n"]
    # the oracle's column heights over the whole 2048 x 2048 map (a 4-voxel-high
    # grid is enough to get them)
    h = oracle.scene_terrain(np.zeros((n // 2, 2, n // 2), np.uint8), 5, n / 16.0, 512.0, 1.0 / (n / 4.0), 6)
    got = c5["heights"].cpu().numpy()
    assert np.array_equal(got.view(np.int32), h.view(np.int32))
    assert h.max() - h.min() > 200.0


def test_c5_voxelizer_subset_matches_oracle(vxl, ctx, c5):
    import torch

    n = c5["n"]
    rng = np.random.default_rng(3)
    pick = rng.choice(len(c5["instances"]), 96, replace=False)
    insts = [c5["instances"][i] for i in pick]
    G = vxl.Grid(ctx, n, n, n)
    vxl.voxelize(ctx, G, c5["mdesc"], insts)
    torch.cuda.synchronize()
    got = export_r8(G)
    want = np.zeros((n // 2, n // 2, n // 2), np.uint8)
    for M, mi, op in insts:
        oracle.voxelize_model(want, c5["models"][mi], M, 1)
    assert np.array_equal(got, want)
    assert got.any()
    del G


def test_c5_voxelize_order_independent_and_idempotent(vxl, ctx, c5):
    import torch

    n = c5["n"]
    rng = np.random.default_rng(4)
    pick = rng.choice(len(c5["instances"]), 2000, replace=False)
    insts = [c5["instances"][i] for i in pick]
    A = vxl.Grid(ctx, n, n, n)
    B = vxl.Grid(ctx, n, n, n)
    vxl.voxelize(ctx, A, c5["mdesc"], insts)
    vxl.voxelize(ctx, B, c5["mdesc"], [insts[i] for i in rng.permutation(len(insts))])
    ca = A.count()
    assert ca == B.count() and ca > 0
    ra = torch.empty((n // 2) ** 3, dtype=torch.uint8, device="cuda")
    rb = torch.empty_like(ra)
    A.export_r8(ra)
    B.export_r8(rb)
    assert torch.equal(ra, rb)
    vxl.voxelize(ctx, A, c5["mdesc"], insts)
    assert A.count() == ca
    A.export_r8(rb)
    assert torch.equal(ra, rb)


def test_c5_sampled_pixels_bit_exact(vxl, ctx, c5):
    import torch

    npix, P = c5["npix"], c5["params"]
    R = P.n_shadow + P.n_ao + P.n_spec
    assert R == 18
    outs = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                                  "spec_t")}
    rec = rec_buffer(npix * R)
    vxl.trace_occlusion(ctx, c5["grid"], c5["pos"], c5["nrm"], c5["rough"], npix, P, records=rec, **outs)
    # the same frame without records (the timed configuration) gives the same outputs
    outs2 = {k: torch.empty_like(v) for k, v in outs.items()}
    vxl.trace_occlusion(ctx, c5["grid"], c5["pos"], c5["nrm"], c5["rough"], npix, P, width=c5["W"],
                        height=c5["H"], **outs2)
    torch.cuda.synchronize()
    for k in outs:
        assert torch.equal(outs[k], outs2[k]), k
    g = export_r8(c5["grid"])
    pos = c5["pos"].cpu().numpy()
    nrm = c5["nrm"].cpu().numpy()
    rough = c5["rough"].cpu().numpy()
    got_recs = recs_np(rec)
    got = {k: v.cpu().numpy() for k, v in outs.items()}
    from voxelengine_gb300 import scenes

    OP = oracle.make_params(light_dir=scenes.light_dir(c5["seed"]), cam_pos=list(P.cam_pos), bias=P.bias,
                            shadow_len=P.shadow_len, ao_len=P.ao_len, spec_len=P.spec_len, n_shadow=P.n_shadow,
                            n_ao=P.n_ao, n_spec=P.n_spec, seed=P.seed)
    rng = np.random.default_rng(9)
    starts = np.sort(rng.choice(npix // 32, 32, replace=False)) * 32
    traced = 0
    for p0 in starts:
        p1 = int(p0) + 32
        want = oracle.occlusion_range(g, pos, nrm, rough, OP, int(p0), p1)
        assert_recs_equal(got_recs[p0 * R:p1 * R], want["recs"], "records @%d" % p0)
        for k in got:
            assert same_bits(got[k][p0:p1], want[k]).all(), (k, p0)
        traced += int((want["recs"]["steps"] > 0).sum())
    assert traced > 5000
    # the frame sees terrain and instances, some shadowed, some lit
    sh = got["shadow"]
    assert 0.02 < float((sh == 0).mean()) < 0.98
