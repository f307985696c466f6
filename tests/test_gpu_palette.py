"""The grid's 4-bit palette plane (vxl_grid_palette_alloc, vxl_grid_export_palette,
vxl_scene_palette, and vxl_grid_import_palette on a grid that has the plane),
through the C ABI.

The plane has no counterpart in the reference: its ShadowVox image holds
occupancy only (ShadowVoxSystem.cpp:56-79), and the palette index only decides
occupancy (index >= 16, ShadowVoxSystem.cpp:145). The checks are therefore
against numpy on the same inputs: occupancy as the reference sets it, the
index's low 4 bits kept for set voxels, and occlusion outputs that do not
change when a grid carries the plane."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, export_r8

pytestmark = pytest.mark.gpu


def test_import_palette_keeps_low_bits(vxl, ctx):
    import torch

    rng = np.random.default_rng(7)
    nx, ny, nz = 38, 30, 22
    vol = rng.integers(0, 256, size=(nz, ny, nx), dtype=np.uint8)
    G = vxl.Grid(ctx, nx, ny, nz)
    G.palette_alloc()
    G.palette_alloc()  # a second call keeps the plane
    G.import_palette(dev(vol), opaque_min=16)
    out = torch.full((nz * ny * nx,), 255, dtype=torch.uint8, device="cuda")
    G.export_palette(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(nz, ny, nx)
    want = np.where(vol >= 16, vol & 15, 0).astype(np.uint8)
    assert np.array_equal(got, want)
    # occupancy is the reference's: set where the index is >= 16
    assert np.array_equal(oracle.r8_to_fine(export_r8(G)), vol >= 16)
    # vxl_grid_clear zeroes the plane with the words
    G.clear()
    G.export_palette(out)
    torch.cuda.synchronize()
    assert int(out.max().item()) == 0
    G.close()


def test_scene_palette_marks_set_voxels(vxl, ctx):
    import torch

    n = 64
    G = vxl.Grid(ctx, n, n, n)
    G.palette_alloc()
    G.scene_noise(11, 0.55, 1.0 / 16.0, 6)
    G.scene_palette(11)
    out = torch.empty(n ** 3, dtype=torch.uint8, device="cuda")
    G.export_palette(out)
    torch.cuda.synchronize()
    pal = out.cpu().numpy().reshape(n, n, n)
    occ = oracle.r8_to_fine(export_r8(G))
    assert 0.05 < occ.mean() < 0.95
    assert np.array_equal(pal != 0, occ)
    assert pal.max() <= 15 and pal[occ].min() >= 1
    assert len(np.unique(pal[occ])) == 15
    # seeded: the same seed gives the same plane, another seed another one
    G.scene_palette(11)
    again = torch.empty_like(out)
    G.export_palette(again)
    G.scene_palette(12)
    other = torch.empty_like(out)
    G.export_palette(other)
    torch.cuda.synchronize()
    assert torch.equal(out, again) and not torch.equal(out, other)
    G.close()


def test_plane_does_not_change_occlusion(vxl, ctx):
    import torch

    from voxelengine_gb300 import scenes as S

    n, W, H = 96, 96, 64
    grids = []
    for with_plane in (False, True):
        G = vxl.Grid(ctx, n, n, n)
        if with_plane:
            G.palette_alloc()
        G.scene_noise(3, 0.55, 1.0 / 32.0, 8)
        G.scene_boxes(3, 30, 4, 24)
        if with_plane:
            G.scene_palette(3)
        grids.append(G)
    cam, tgt = S.camera(n)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    vxl.scene_gbuffer(ctx, grids[0], cam, tgt, W, H, 3, pos, nrm, rough)
    P = vxl.make_params(cam_pos=cam, n_ao=8, ao_len=32.0, n_spec=1, seed=3)
    outs = []
    for G in grids:
        o = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                                 "spec_t")}
        vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **o)
        outs.append(o)
    torch.cuda.synchronize()
    for k in outs[0]:
        assert torch.equal(outs[0][k].view(torch.int32), outs[1][k].view(torch.int32)), k
    for G in grids:
        G.close()


def test_export_without_plane_is_an_error(vxl, ctx):
    import torch

    G = vxl.Grid(ctx, 8, 8, 8)
    out = torch.empty(512, dtype=torch.uint8, device="cuda")
    with pytest.raises(vxl.VxlError):
        G.export_palette(out)
    with pytest.raises(vxl.VxlError):
        G.scene_palette(1)
    G.close()
